// FP32 stream-collide in the reference's exact floating-point expression
// order, plus the FP32 equilibrium initialisers.
//
// This translation unit is compiled with --fmad=false: no multiply-add is
// contracted, so every expression rounds exactly as written. The collision
// (collide_exact in collide_common.cuh) and the equilibrium reproduce the
// expression tree of the reference kernel (src/sim/lbm_core.cu:65-73,
// 241-283, 386-474) with the terms whose lattice coefficient is 0 left out
// (adding the exact zero 0*f changes no result) and multiplications by +-1
// folded (exact). The FP32 drop-in therefore produces bit-identical
// populations to the reference step evaluated without FMA contraction -- the
// CPU build of the reference kernels and the oracle -- rather than drifting
// by accumulated reordering rounding (~1e-5 relative in u after 1000 steps).
#include "collide_common.cuh"

namespace fcfd {
namespace {

constexpr int kBlock1D = 256;

__global__ void init_eq_f32_kernel(float* __restrict__ f, const std::uint8_t* __restrict__ kind, long long n,
                                   float uIn) {
    const long long c = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const float ux = ((kind[c] & kFlagMask) == kSolid) ? 0.0f : uIn;
    float feq[kQ];
    eq19(1.0f, ux, 0.0f, 0.0f, feq);
#pragma unroll
    for (int q = 0; q < kQ; ++q) f[q * n + c] = feq[q];
}

__global__ void init_macro_f32_kernel(float* __restrict__ f, const std::uint8_t* __restrict__ kind,
                                      long long n, const float* __restrict__ rho, const float* __restrict__ u,
                                      const float* __restrict__ v, const float* __restrict__ w) {
    const long long c = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const bool solid = (kind[c] & kFlagMask) == kSolid;
    float feq[kQ];
    eq19(solid ? 1.0f : rho[c], solid ? 0.0f : u[c], solid ? 0.0f : v[c], solid ? 0.0f : w[c], feq);
#pragma unroll
    for (int q = 0; q < kQ; ++q) f[q * n + c] = feq[q];
}

} // namespace

bool staged_applies(LevelDims d, Storage s) {
    return s == Storage::F32 ? staged_plan<StoreF32>(d).stages >= 2 : staged_plan<StoreF16>(d).stages >= 2;
}

cudaError_t launch_collide_f32_ref(const float* src, float* dst, const std::uint8_t* kind, LevelDims d,
                                   const CollideParams& p, float* rho, float* u, float* v, float* w,
                                   SlipField slip, cudaStream_t st) {
    return launch_collide_impl<StoreF32, true>(src, dst, kind, d, p, rho, u, v, w, slip, st);
}

cudaError_t launch_collide_aa_f32(float* f, LevelDims d, const CollideParams& p, int odd, float* rho, float* u,
                                  float* v, float* w, cudaStream_t st) {
    return launch_collide_aa_impl<StoreF32, true>(f, d, p, odd, rho, u, v, w, st);
}

cudaError_t launch_collide_child_f32(const float* src, float* dst, const std::uint8_t* kind, LevelDims d,
                                     const CollideParams& p, SlipField slip, const ChildFuse& cf, cudaStream_t st) {
    return launch_collide_child_impl<StoreF32, true>(src, dst, kind, d, p, slip, cf, st);
}

cudaError_t launch_apply_flag_edits_f32(float* fA, float* fB, const std::uint8_t* flags, const std::uint8_t* mask,
                                        LevelDims d, cudaStream_t st) {
    return launch_apply_flag_edits_impl<StoreF32>(fA, fB, flags, mask, d, st);
}

cudaError_t launch_init_eq_f32(float* f, const std::uint8_t* kind, long long n, float uIn, cudaStream_t st) {
    init_eq_f32_kernel<<<static_cast<unsigned>((n + kBlock1D - 1) / kBlock1D), kBlock1D, 0, st>>>(f, kind, n, uIn);
    return cudaGetLastError();
}

cudaError_t launch_init_macro_f32(float* f, const std::uint8_t* kind, long long n, const float* rho,
                                  const float* u, const float* v, const float* w, cudaStream_t st) {
    init_macro_f32_kernel<<<static_cast<unsigned>((n + kBlock1D - 1) / kBlock1D), kBlock1D, 0, st>>>(
        f, kind, n, rho, u, v, w);
    return cudaGetLastError();
}

} // namespace fcfd
