// Momentum-exchange force on the solid (reference forceReductionKernel,
// src/sim/lbm_core.cu:573-637): every fluid cell with a solid neighbour at
// +c_q hands the wall c_q (2 f_q - 6 w_q (c_q . u_w)) per step, f_q being the
// post-collision population and u_w the wall-model slip velocity (zero when
// the model is off).
//
// GB300 design: instead of sweeping every cell and reading 18 neighbour flags
// (the reference), the kernel walks a compact list of wall-adjacent cells with
// a per-cell solid-link bit mask, built once per flag upload. Per-link terms
// are formed in FP32 as the reference does, then summed in FP64: per thread,
// per warp (shuffles), per block, and finally in a single-block pass over the
// block partials in a fixed order, so the result is deterministic run to run.
#include "d3q19.cuh"
#include "kernels.h"

#include <cuda_runtime.h>

namespace fcfd {
namespace {

constexpr int kForceBlock = 256;
constexpr int kMaxForceBlocks = 1024;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

/// Block-wide FP64 sum of (a, b, c); the result is valid in thread 0.
__device__ __forceinline__ void block_sum3(double& a, double& b, double& c) {
    __shared__ double sh[3][kForceBlock / 32];
    a = warp_sum(a); b = warp_sum(b); c = warp_sum(c);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { sh[0][warp] = a; sh[1][warp] = b; sh[2][warp] = c; }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        a = lane < nw ? sh[0][lane] : 0.0;
        b = lane < nw ? sh[1][lane] : 0.0;
        c = lane < nw ? sh[2][lane] : 0.0;
        a = warp_sum(a); b = warp_sum(b); c = warp_sum(c);
    }
}

template <class S, bool WM>
__global__ void __launch_bounds__(kForceBlock)
force_partial_kernel(const typename S::T* __restrict__ f, long long n,
                     const std::uint32_t* __restrict__ cells,
                     const std::uint32_t* __restrict__ masks, int count,
                     const std::uint16_t* __restrict__ uwxA,
                     const std::uint16_t* __restrict__ uwyA,
                     const std::uint16_t* __restrict__ uwzA,
                     double* __restrict__ partials) {
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const std::uint32_t c = cells[i];
        const std::uint32_t m = masks[i];
        float uwx = 0.0f, uwy = 0.0f, uwz = 0.0f;
        if constexpr (WM) {
            uwx = __half2float(__ushort_as_half(uwxA[c]));
            uwy = __half2float(__ushort_as_half(uwyA[c]));
            uwz = __half2float(__ushort_as_half(uwzA[c]));
        }
#pragma unroll
        for (int q = 1; q < kQ; ++q) {
            if (!(m & (1u << q))) continue;
            const float fq = S::ld(f + q * n, c, wgt(q));
            float corr = 0.0f;
            if constexpr (WM) corr = 6.0f * wgt(q) * (cx(q) * uwx + cy(q) * uwy + cz(q) * uwz);
            const float t = 2.0f * fq - corr;
            fx += static_cast<double>(cx(q) * t);
            fy += static_cast<double>(cy(q) * t);
            fz += static_cast<double>(cz(q) * t);
        }
    }
    block_sum3(fx, fy, fz);
    if (threadIdx.x == 0) {
        partials[3 * blockIdx.x + 0] = fx;
        partials[3 * blockIdx.x + 1] = fy;
        partials[3 * blockIdx.x + 2] = fz;
    }
}

__global__ void __launch_bounds__(kForceBlock)
force_final_kernel(const double* __restrict__ partials, int nblocks, double* __restrict__ out) {
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        fx += partials[3 * b + 0];
        fy += partials[3 * b + 1];
        fz += partials[3 * b + 2];
    }
    block_sum3(fx, fy, fz);
    if (threadIdx.x == 0) { out[0] = fx; out[1] = fy; out[2] = fz; }
}

} // namespace

int force_blocks(int count) {
    int b = (count + kForceBlock - 1) / kForceBlock;
    if (b < 1) b = 1;
    if (b > kMaxForceBlocks) b = kMaxForceBlocks;
    return b;
}

cudaError_t launch_force(Storage s, const void* f, long long cells, const std::uint32_t* linkCells,
                         const std::uint32_t* linkMasks, int count, SlipField slip,
                         double* partials, double* out, cudaStream_t st) {
    if (!f || !partials || !out || cells <= 0 || count < 0) return cudaErrorInvalidValue;
    const int nb = force_blocks(count);
    if (count == 0) return cudaMemsetAsync(out, 0, 3 * sizeof(double), st);
    const bool wm = slip.active();
    if (s == Storage::F32) {
        auto* p = static_cast<const float*>(f);
        if (wm) force_partial_kernel<StoreF32, true><<<nb, kForceBlock, 0, st>>>(p, cells, linkCells, linkMasks, count, slip.uwx, slip.uwy, slip.uwz, partials);
        else force_partial_kernel<StoreF32, false><<<nb, kForceBlock, 0, st>>>(p, cells, linkCells, linkMasks, count, nullptr, nullptr, nullptr, partials);
    } else {
        auto* p = static_cast<const __half*>(f);
        if (wm) force_partial_kernel<StoreF16, true><<<nb, kForceBlock, 0, st>>>(p, cells, linkCells, linkMasks, count, slip.uwx, slip.uwy, slip.uwz, partials);
        else force_partial_kernel<StoreF16, false><<<nb, kForceBlock, 0, st>>>(p, cells, linkCells, linkMasks, count, nullptr, nullptr, nullptr, partials);
    }
    if (auto e = cudaGetLastError(); e != cudaSuccess) return e;
    force_final_kernel<<<1, kForceBlock, 0, st>>>(partials, nb, out);
    return cudaGetLastError();
}

} // namespace fcfd
