// What the snapshot code (snapshot.cpp) reads from a solver: the current
// population buffer of every active level, its storage, the host copy of the
// coarse flags and the scaling.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/foilcfd_step.h"
#include "kernels.h"

namespace fcfd {

struct SolverFieldView {
    int levels = 0;                 ///< active levels: coarse, fine, finer
    void* f[3] = {nullptr, nullptr, nullptr};
    size_t bytes[3] = {0, 0, 0};
    LevelDims dims[3];
    /// Wall-model state of each level (null / 0 without a wall model):
    /// u_tau per wall cell and the three slip-velocity arrays (one uint16
    /// per cell each). The collide reads the slip arrays, so an exact
    /// snapshot carries them with the populations.
    void* wm[3][4] = {};
    size_t wmBytes[3][4] = {};
    int storage = FCFD_STORE_FP32;
    cudaStream_t stream = nullptr;
    std::uint64_t flagsHash = 0;    ///< FNV-1a of the coarse flags (cached)
    fcfd_scaling scaling{};
};

/// 0, or cudaErrorNotReady when the solver is not initialised.
int solver_field_view(fcfd_solver* s, SolverFieldView* v);
/// FNV-1a 64 of a byte array (the snapshot flag hash).
std::uint64_t fnv1a64(const void* p, size_t n);

} // namespace fcfd
