// The iMEM wall-model update (wall_common.cuh) for FP16 storage, built with
// nvcc's default multiply-add contraction, and the harvest of wall samples
// for the learned seed. FP32 storage runs wall_kernels_x.cu's build of the
// same kernels (no contraction), so its slip velocities round like the
// reference's expressions as written, as every FP32 kernel does.
#include "wall_common.cuh"

namespace fcfd {

cudaError_t launch_wall_update(Storage s, const void* f, long long cells, WallListDev list,
                               std::uint16_t* uwx, std::uint16_t* uwy, std::uint16_t* uwz,
                               float nuLat, float utCutoff, float emaAlpha, WallStatsDev* stats,
                               cudaStream_t st, int method, const wallnet::NetDev* net) {
    if (s == Storage::F32)
        return launch_wall_update_f32_x(f, cells, list, uwx, uwy, uwz, nuLat, utCutoff, emaAlpha, stats, st, method,
                                        net);
    return wall_update_launch<StoreF16>(s, f, cells, list, uwx, uwy, uwz, nuLat, utCutoff, emaAlpha, stats, st,
                                        method, net);
}
cudaError_t launch_wall_harvest(Storage s, const void* f, long long cells, WallListDev list, float utCutoff,
                                float* utOut, float* ysOut, cudaStream_t st) {
    if (list.count <= 0 || !f || !utOut || !ysOut) return cudaErrorInvalidValue;
    const unsigned nb = static_cast<unsigned>((list.count + kWallBlock - 1) / kWallBlock);
    if (s == Storage::F32)
        wall_harvest_kernel<StoreF32><<<nb, kWallBlock, 0, st>>>(static_cast<const float*>(f), cells, list, utCutoff,
                                                                 utOut, ysOut);
    else
        wall_harvest_kernel<StoreF16><<<nb, kWallBlock, 0, st>>>(static_cast<const __half*>(f), cells, list, utCutoff,
                                                                 utOut, ysOut);
    return cudaGetLastError();
}

} // namespace fcfd
