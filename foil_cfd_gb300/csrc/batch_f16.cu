// Batched collide, FP16 deviation storage (half(f - w_q)), with the same
// collision body as the single-tunnel FP16 solver.
#include "batch_kernels.cuh"

namespace fcfd {

cudaError_t launch_batch_collide_f16(const BatchTable& tab, unsigned itemBase, unsigned nItems, int parity,
                                     BatchShape sh, cudaStream_t st) {
    return launch_batch_impl<StoreF16, false>(tab, itemBase, nItems, parity, sh, st);
}

int batch_occupancy_f16(BatchShape sh) { return batch_occupancy_impl<StoreF16, false>(sh); }

/// Append the current per-tunnel forces (3 doubles each) to a ring of
/// force samples and advance its device-side count.
__global__ void force_append_kernel(const double* __restrict__ cur, int n3, double* __restrict__ hist, int cap,
                                    int* __restrict__ count) {
    const int c = *count;
    double* slot = hist + static_cast<long long>(c % cap) * n3;
    for (int i = threadIdx.x; i < n3; i += blockDim.x) slot[i] = cur[i];
    __syncthreads();
    if (threadIdx.x == 0) *count = c + 1;
}

/// Largest speed |j| / rho over the non-solid cells of one tunnel (float
/// bits, atomicMax: speeds are non-negative) and the count of cells whose
/// density is not finite.
template <class S>
__global__ void health_kernel(const typename S::T* __restrict__ f, const std::uint8_t* __restrict__ kind, long long n,
                              int* __restrict__ maxSpeedBits, int* __restrict__ nonFinite) {
    float best = 0.0f;
    int bad = 0;
    for (long long c = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        if ((kind[c] & kFlagMask) == kSolid) continue;
        float r = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
        for (int q = 0; q < kQ; ++q) {
            const float v = S::ld(f + q * n, c, wgt(q));
            r += v; jx += cx(q) * v; jy += cy(q) * v; jz += cz(q) * v;
        }
        if (!isfinite(r) || !isfinite(jx) || !isfinite(jy) || !isfinite(jz)) {
            ++bad;
            continue;
        }
        best = fmaxf(best, sqrtf(jx * jx + jy * jy + jz * jz) / fmaxf(r, kRhoFloor));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        best = fmaxf(best, __shfl_down_sync(0xffffffffu, best, o));
        bad += __shfl_down_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(maxSpeedBits, __float_as_int(best));
        if (bad) atomicAdd(nonFinite, bad);
    }
}

cudaError_t launch_batch_health(bool fp32, const void* f, const std::uint8_t* kind, long long n, int* maxSpeedBits,
                                int* nonFinite, cudaStream_t st) {
    const unsigned nb = static_cast<unsigned>(std::min<long long>(4096, (n + 255) / 256));
    if (fp32)
        health_kernel<StoreF32><<<nb, 256, 0, st>>>(static_cast<const float*>(f), kind, n, maxSpeedBits, nonFinite);
    else
        health_kernel<StoreF16><<<nb, 256, 0, st>>>(static_cast<const __half*>(f), kind, n, maxSpeedBits, nonFinite);
    return cudaGetLastError();
}

/// Latch every running tunnel whose health scan found a non-finite cell
/// (verdict 1) or a speed at the limiter (verdict 2, |u| >= cap); latch[ntun
/// + t] records the force-sample count at that moment.
__global__ void batch_latch_kernel(const int* __restrict__ maxSpeedBits, const int* __restrict__ nonFinite, int ntun,
                                   float cap, const int* __restrict__ samples, int* __restrict__ latch) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntun || latch[t] != 0) return;
    const int v = nonFinite[t] > 0 ? 1 : (__int_as_float(maxSpeedBits[t]) >= cap ? 2 : 0);
    if (v) {
        latch[t] = v;
        latch[ntun + t] = *samples;
    }
}

cudaError_t launch_batch_latch(const int* maxSpeedBits, const int* nonFinite, int ntun, float cap,
                               const int* samples, int* latch, cudaStream_t st) {
    batch_latch_kernel<<<(ntun + 63) / 64, 64, 0, st>>>(maxSpeedBits, nonFinite, ntun, cap, samples, latch);
    return cudaGetLastError();
}

cudaError_t launch_force_append(const double* cur, int n3, double* hist, int cap, int* count, cudaStream_t st) {
    force_append_kernel<<<1, 256, 0, st>>>(cur, n3, hist, cap, count);
    return cudaGetLastError();
}

} // namespace fcfd
