// FP32 stream-collide in the reference's exact floating-point expression
// order, plus the FP32 equilibrium initialisers.
//
// This translation unit is compiled with --fmad=false: no multiply-add is
// contracted, so every expression rounds exactly as written. Each sum,
// product and relaxation below reproduces the expression tree of the
// reference kernel (src/sim/lbm_core.cu:65-73, 241-283, 386-474) with the
// terms whose lattice coefficient is 0 left out (adding the exact zero
// 0*f changes no result) and multiplications by +-1 folded (exact). The FP32
// drop-in therefore produces bit-identical populations to the reference
// step evaluated without FMA contraction -- the CPU build of the reference
// kernels and the oracle -- rather than drifting by accumulated reordering
// rounding (which reaches ~1e-5 relative in u after 1000 steps).
//
// Boundary selection, the kind byte and the periodic index wrap are the same
// as in the re-associated kernel of step_kernels.cu.
#include "d3q19.cuh"
#include "kernels.h"

#include <cuda_runtime.h>

namespace fcfd {
namespace {

constexpr int kBlockX = 128;
constexpr int kBlock1D = 256;

struct Args {
    int nx, ny, nz;
    long long n;
    float tau0, lambda, smagPre, uIn;
    int writeMacro;
    float *rho, *u, *v, *w;
    const std::uint16_t *uwx, *uwy, *uwz;
};

/// Reference equilibrium19 (lbm_core.cu:65-73), same rounding.
__device__ __forceinline__ void eq19(float rho, float ux, float uy, float uz, float (&feq)[kQ]) {
    const float usq = 1.5f * (ux * ux + uy * uy + uz * uz);
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        // cu = 3 * ((cx ux + cy uy) + cz uz), zero terms dropped.
        float dot = 0.0f;
        bool any = false;
        if (cx(q) != 0) { dot = cx(q) > 0 ? ux : -ux; any = true; }
        if (cy(q) != 0) {
            const float t = cy(q) > 0 ? uy : -uy;
            dot = any ? dot + t : t;
            any = true;
        }
        if (cz(q) != 0) {
            const float t = cz(q) > 0 ? uz : -uz;
            dot = any ? dot + t : t;
            any = true;
        }
        const float cu = 3.0f * dot;
        feq[q] = (wgt(q) * rho) * (1.0f + cu + 0.5f * cu * cu - usq);
    }
}

template <bool WM>
__global__ void __launch_bounds__(kBlockX)
collide_ref_kernel(const float* __restrict__ src, float* __restrict__ dst,
                   const std::uint8_t* __restrict__ kind, Args a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= a.nx) return;
    const int y = blockIdx.y, z = blockIdx.z;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const long long n = a.n;
    const unsigned unx = static_cast<unsigned>(nx), uny = static_cast<unsigned>(ny);
    const unsigned cell = static_cast<unsigned>(x) + unx * (static_cast<unsigned>(y) + uny * z);
    const std::uint8_t k = kind[cell];
    const int flag = k & kFlagMask;
    const int xm = wrap_dec(x, nx), xp = wrap_inc(x, nx);
    const unsigned sx[3] = {static_cast<unsigned>(xp), static_cast<unsigned>(x), static_cast<unsigned>(xm)};
    const unsigned sy[3] = {static_cast<unsigned>(wrap_inc(y, ny)), static_cast<unsigned>(y),
                            static_cast<unsigned>(wrap_dec(y, ny))};
    const unsigned sz[3] = {static_cast<unsigned>(wrap_inc(z, nz)), static_cast<unsigned>(z),
                            static_cast<unsigned>(wrap_dec(z, nz))};

    if (flag != kFluid) {
        if (flag == kInlet) {
            float feq[kQ];
            eq19(1.0f, a.uIn, 0.0f, 0.0f, feq);
#pragma unroll
            for (int q = 0; q < kQ; ++q) dst[q * n + cell] = feq[q];
            if (a.writeMacro) {
                a.rho[cell] = 1.0f; a.u[cell] = a.uIn; a.v[cell] = 0.0f; a.w[cell] = 0.0f;
            }
        } else if (flag == kOutlet || flag == kOutletEq) {
            const unsigned up = static_cast<unsigned>(xm) + unx * (static_cast<unsigned>(y) + uny * z);
            float g[kQ];
            float r = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
            for (int q = 0; q < kQ; ++q) {
                g[q] = src[q * n + up];
                r += g[q];
                if (cx(q) != 0) jx = cx(q) > 0 ? jx + g[q] : jx - g[q];
                if (cy(q) != 0) jy = cy(q) > 0 ? jy + g[q] : jy - g[q];
                if (cz(q) != 0) jz = cz(q) > 0 ? jz + g[q] : jz - g[q];
            }
            const float inv = 1.0f / r;
            const float ux = jx * inv, uy = jy * inv, uz = jz * inv;
            if (flag == kOutletEq) {
                eq19(1.0f, ux, uy, uz, g);
                r = 1.0f;
            }
#pragma unroll
            for (int q = 0; q < kQ; ++q) dst[q * n + cell] = g[q];
            if (a.writeMacro) {
                a.rho[cell] = r; a.u[cell] = ux; a.v[cell] = uy; a.w[cell] = uz;
            }
        } else if (a.writeMacro) {
            a.rho[cell] = 1.0f; a.u[cell] = 0.0f; a.v[cell] = 0.0f; a.w[cell] = 0.0f;
        }
        return;
    }

    float fpop[kQ];
    if (!(k & kNearWall)) {
#pragma unroll
        for (int q = 0; q < kQ; ++q)
            fpop[q] = __ldg(src + q * n + (sx[1 + cx(q)] + unx * (sy[1 + cy(q)] + uny * sz[1 + cz(q)])));
    } else {
        float uwx = 0.0f, uwy = 0.0f, uwz = 0.0f;
        bool uwLoaded = false;
        fpop[0] = __ldg(src + cell);
#pragma unroll
        for (int q = 1; q < kQ; ++q) {
            const unsigned X = sx[1 + cx(q)], Y = sy[1 + cy(q)], Z = sz[1 + cz(q)];
            const unsigned pn = X + unx * (Y + uny * Z);
            const int nf = kind[pn] & kFlagMask;
            const bool solid = nf == kSolid;
            const bool slipY = is_slip_y(nf);
            const bool slipZ = is_slip_z(nf);
            const unsigned pY = X + unx * (static_cast<unsigned>(y) + uny * Z);
            const unsigned pZ = X + unx * (Y + uny * static_cast<unsigned>(z));
            const int qs = solid ? opp(q) : (slipY ? mir_y(q) : (slipZ ? mir_z(q) : q));
            const unsigned cs = solid ? cell : (slipY ? pY : (slipZ ? pZ : pn));
            float fq = __ldg(src + static_cast<long long>(qs) * n + cs);
            if constexpr (WM) {
                if (solid) {
                    if (!uwLoaded) {
                        uwx = __half2float(__ushort_as_half(a.uwx[cell]));
                        uwy = __half2float(__ushort_as_half(a.uwy[cell]));
                        uwz = __half2float(__ushort_as_half(a.uwz[cell]));
                        uwLoaded = true;
                    }
                    // 6 w_q ((cx uwx + cy uwy) + cz uwz), zero terms dropped.
                    float dot = 0.0f;
                    bool any = false;
                    if (cx(q) != 0) { dot = cx(q) > 0 ? uwx : -uwx; any = true; }
                    if (cy(q) != 0) { const float t = cy(q) > 0 ? uwy : -uwy; dot = any ? dot + t : t; any = true; }
                    if (cz(q) != 0) { const float t = cz(q) > 0 ? uwz : -uwz; dot = any ? dot + t : t; any = true; }
                    fq += (6.0f * wgt(q)) * dot;
                }
            }
            fpop[q] = fq;
        }
    }

    // Moments, left to right over q (lbm_core.cu:386-393).
    float rho = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        rho += fpop[q];
        if (cx(q) != 0) jx = cx(q) > 0 ? jx + fpop[q] : jx - fpop[q];
        if (cy(q) != 0) jy = cy(q) > 0 ? jy + fpop[q] : jy - fpop[q];
        if (cz(q) != 0) jz = cz(q) > 0 ? jz + fpop[q] : jz - fpop[q];
    }
    rho = fmaxf(rho, kRhoFloor);
    const float invRho = 1.0f / rho;
    float ux = jx * invRho, uy = jy * invRho, uz = jz * invRho;
    const float u2 = ux * ux + uy * uy + uz * uz;
    if (u2 > kMaxSimSpeed * kMaxSimSpeed) {
        // 1/sqrt rounded as IEEE operations (not the approximate rsqrt).
        const float s = kMaxSimSpeed * (1.0f / sqrtf(u2));
        ux *= s; uy *= s; uz *= s;
    }
    float feq[kQ];
    eq19(rho, ux, uy, uz, feq);

    float tauEff = a.tau0;
    if (a.smagPre > 0.0f) {
        float pxx = 0.0f, pyy = 0.0f, pzz = 0.0f, pxy = 0.0f, pxz = 0.0f, pyz = 0.0f;
#pragma unroll
        for (int q = 0; q < kQ; ++q) {
            const float fneq = fpop[q] - feq[q];
            if (cx(q) != 0) pxx += fneq;
            if (cy(q) != 0) pyy += fneq;
            if (cz(q) != 0) pzz += fneq;
            if (cx(q) * cy(q) != 0) pxy = cx(q) * cy(q) > 0 ? pxy + fneq : pxy - fneq;
            if (cx(q) * cz(q) != 0) pxz = cx(q) * cz(q) > 0 ? pxz + fneq : pxz - fneq;
            if (cy(q) * cz(q) != 0) pyz = cy(q) * cz(q) > 0 ? pyz + fneq : pyz - fneq;
        }
        const float qbar = sqrtf(pxx * pxx + pyy * pyy + pzz * pzz
                                 + 2.0f * (pxy * pxy + pxz * pxz + pyz * pyz));
        tauEff = 0.5f * (a.tau0 + sqrtf(a.tau0 * a.tau0 + a.smagPre * qbar * invRho));
    }
    const float omP = 1.0f / tauEff;
    const float tauM = 0.5f + a.lambda / (tauEff - 0.5f);
    const float omM = 1.0f / tauM;

    dst[cell] = fpop[0] - omP * (fpop[0] - feq[0]);
#pragma unroll
    for (int p = 1; p <= 9; ++p) {
        const int qa = 2 * p - 1, qb = 2 * p;
        const float symRelax = omP * (0.5f * (fpop[qa] + fpop[qb]) - 0.5f * (feq[qa] + feq[qb]));
        const float asymRelax = omM * (0.5f * (fpop[qa] - fpop[qb]) - 0.5f * (feq[qa] - feq[qb]));
        dst[qa * n + cell] = fpop[qa] - symRelax - asymRelax;
        dst[qb * n + cell] = fpop[qb] - symRelax + asymRelax;
    }
    if (a.writeMacro) {
        a.rho[cell] = rho; a.u[cell] = ux; a.v[cell] = uy; a.w[cell] = uz;
    }
}

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

cudaError_t launch_collide_f32_ref(const float* src, float* dst, const std::uint8_t* kind, LevelDims d,
                                   const CollideParams& p, float* rho, float* u, float* v, float* w,
                                   SlipField slip, cudaStream_t st) {
    Args a;
    a.nx = d.nx; a.ny = d.ny; a.nz = d.nz; a.n = d.cells();
    a.tau0 = p.tau; a.lambda = p.magicLambda; a.smagPre = p.smagPrefactor; a.uIn = p.uInlet;
    a.writeMacro = (p.writeMacro && rho && u && v && w) ? 1 : 0;
    a.rho = rho; a.u = u; a.v = v; a.w = w;
    a.uwx = slip.uwx; a.uwy = slip.uwy; a.uwz = slip.uwz;
    const int bx = d.nx >= kBlockX ? kBlockX : ((d.nx + 31) / 32) * 32;
    const dim3 grid(static_cast<unsigned>((d.nx + bx - 1) / bx), static_cast<unsigned>(d.ny),
                    static_cast<unsigned>(d.nz));
    if (slip.active()) collide_ref_kernel<true><<<grid, bx, 0, st>>>(src, dst, kind, a);
    else collide_ref_kernel<false><<<grid, bx, 0, st>>>(src, dst, kind, a);
    return cudaGetLastError();
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
