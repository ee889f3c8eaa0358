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

cudaError_t launch_force_append(const double* cur, int n3, double* hist, int cap, int* count, cudaStream_t st) {
    force_append_kernel<<<1, 256, 0, st>>>(cur, n3, hist, cap, count);
    return cudaGetLastError();
}

} // namespace fcfd
