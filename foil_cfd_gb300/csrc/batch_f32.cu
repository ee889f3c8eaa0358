// Batched collide, FP32 storage, in the reference expression order. Built
// with --fmad=false like collide_f32.cu, so each tunnel of a batch steps bit
// for bit as the single-tunnel FP32 solver (and the reference) does.
#include "batch_kernels.cuh"

namespace fcfd {

cudaError_t launch_batch_collide_f32(const BatchTable& tab, unsigned itemBase, unsigned nItems, int parity,
                                     BatchShape sh, cudaStream_t st) {
    return launch_batch_impl<StoreF32, true>(tab, itemBase, nItems, parity, sh, st);
}

int batch_occupancy_f32(BatchShape sh) { return batch_occupancy_impl<StoreF32, true>(sh); }

} // namespace fcfd
