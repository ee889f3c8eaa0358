// The FP32 iMEM wall-model update (wall_common.cuh) built with
// --fmad=false: the reference's expressions (src/sim/lbm_wallmodel.cu:31-196)
// rounded as written, like every FP32 kernel of the solver step.
#include "wall_common.cuh"

namespace fcfd {

cudaError_t launch_wall_update_f32_x(const void* f, long long cells, WallListDev list, std::uint16_t* uwx,
                                     std::uint16_t* uwy, std::uint16_t* uwz, float nuLat, float utCutoff,
                                     float emaAlpha, WallStatsDev* stats, cudaStream_t st, int method,
                                     const wallnet::NetDev* net) {
    return wall_update_launch<StoreF32>(Storage::F32, f, cells, list, uwx, uwy, uwz, nuLat, utCutoff, emaAlpha,
                                        stats, st, method, net);
}

} // namespace fcfd
