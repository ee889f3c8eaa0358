// Allocation-free variant of the momentum-exchange force reduction.
//
// Some callers cannot call cudaMalloc: a frame loop with a hard per-frame
// time budget (cudaMalloc may synchronise the whole device and stall the
// frame), an engine whose memory manager owns every device allocation, or a
// host thread that must not take the driver's allocation locks. For them this
// entry point computes the same FP64 force as the solver's reduction from
// buffers the caller already owns, and keeps its only scratch -- the FP64
// block partials -- in a file-scope device array instead of allocating it.
//
// The array is part of the library's module image: every GPU that loads the
// library holds its 96 KB until the process exits. Host code cannot use the
// array's name as a device address, so every call looks the address up with
// cudaGetSymbolAddress on the current device. The first call on a device may
// load the module there, so make it before any stream capture on that
// device; later lookups are cheap, and because nothing is cached, a call
// after cudaDeviceReset (a new context, possibly a new address) finds the
// array where the new context put it. All calls share the array: each call
// writes the partials of its own blocks before reading them, so nothing has
// to be cleared between calls, but two calls that overlap on the GPU
// (different streams, no ordering) race on the array and must be serialised
// by the caller.
#include "../../include/foilcfd_step.h"
#include "d3q19.cuh"

#include <cuda_runtime.h>

// Block partials (Fx, Fy, Fz per block of a call): 3 doubles for every 256
// links of the largest accepted list, 96 KB per device.
static __device__ __align__(256) double g_force_partials[3 * (FCFD_FORCE_NOALLOC_MAX_LINKS / 256)];

namespace fcfd {
namespace {

constexpr int kNoAllocBlock = 256;

static_assert(FCFD_FORCE_NOALLOC_MAX_LINKS % kNoAllocBlock == 0, "link limit must fill whole blocks");

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void block_sum3(double& a, double& b, double& c) {
    __shared__ double sh[3][kNoAllocBlock / 32];
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

/// One link-list entry per thread; block b writes partials[3b .. 3b+2].
__global__ void __launch_bounds__(kNoAllocBlock)
noalloc_partial_kernel(const float* __restrict__ f, long long n, const std::uint32_t* __restrict__ cells,
                       const std::uint32_t* __restrict__ masks, int count, const std::uint16_t* __restrict__ uwxA,
                       const std::uint16_t* __restrict__ uwyA, const std::uint16_t* __restrict__ uwzA,
                       double* __restrict__ partials) {
    double fx = 0.0, fy = 0.0, fz = 0.0;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) {
        const std::uint32_t c = cells[i];
        const std::uint32_t m = masks[i];
        const bool wm = uwxA != nullptr;
        const float uwx = wm ? __half2float(__ushort_as_half(uwxA[c])) : 0.0f;
        const float uwy = wm ? __half2float(__ushort_as_half(uwyA[c])) : 0.0f;
        const float uwz = wm ? __half2float(__ushort_as_half(uwzA[c])) : 0.0f;
#pragma unroll
        for (int q = 1; q < kQ; ++q) {
            if (!(m & (1u << q))) continue;
            const float fq = f[q * n + c];
            const float corr = wm ? 6.0f * wgt(q) * (cx(q) * uwx + cy(q) * uwy + cz(q) * uwz) : 0.0f;
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

/// Sums the partials of blocks 0..nb-1 in a fixed order into out[3].
__global__ void __launch_bounds__(kNoAllocBlock)
noalloc_final_kernel(const double* __restrict__ partials, int nb, double* __restrict__ out) {
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        fx += partials[3 * b + 0];
        fy += partials[3 * b + 1];
        fz += partials[3 * b + 2];
    }
    block_sum3(fx, fy, fz);
    if (threadIdx.x == 0) { out[0] = fx; out[1] = fy; out[2] = fz; }
}

/// Device address of the partials array in the current device's context
/// (looked up on every call: no address outlives its context).
cudaError_t partials_address(double** out) {
    void* p = nullptr;
    if (auto e = cudaGetSymbolAddress(&p, g_force_partials); e != cudaSuccess) return e;
    *out = static_cast<double*>(p);
    return cudaSuccess;
}

} // namespace
} // namespace fcfd

extern "C" int fcfd_force_links_noalloc(const float* f, long long ncells, const uint32_t* link_cells,
                                        const uint32_t* link_masks, int count, const uint16_t* uwx,
                                        const uint16_t* uwy, const uint16_t* uwz, double* out, void* stream) {
    using namespace fcfd;
    if (!f || !out || ncells <= 0 || count < 0) return cudaErrorInvalidValue;
    if (count > FCFD_FORCE_NOALLOC_MAX_LINKS) return cudaErrorInvalidValue; // beyond the scratch array
    if (count > 0 && (!link_cells || !link_masks)) return cudaErrorInvalidValue;
    const bool wm = uwx || uwy || uwz;
    if (wm && !(uwx && uwy && uwz)) return cudaErrorInvalidValue;
    auto st = static_cast<cudaStream_t>(stream);
    if (count == 0) return cudaMemsetAsync(out, 0, 3 * sizeof(double), st);
    double* partials = nullptr;
    if (auto e = partials_address(&partials); e != cudaSuccess) return e;
    const int nb = (count + kNoAllocBlock - 1) / kNoAllocBlock;
    noalloc_partial_kernel<<<nb, kNoAllocBlock, 0, st>>>(f, ncells, link_cells, link_masks, count,
                                                         wm ? uwx : nullptr, wm ? uwy : nullptr,
                                                         wm ? uwz : nullptr, partials);
    if (auto e = cudaGetLastError(); e != cudaSuccess) return e;
    noalloc_final_kernel<<<1, kNoAllocBlock, 0, st>>>(partials, nb, out);
    return cudaGetLastError();
}
