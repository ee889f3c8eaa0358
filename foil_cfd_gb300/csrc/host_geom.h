// Host-side list and geometry builders of the solver step (pure C++, no CUDA).
#pragma once

#include <cstdint>
#include <vector>

#include "kernels.h"

namespace fcfd {

constexpr std::uint8_t kFlagFluidHost = 0;
constexpr std::uint8_t kFlagSolidHost = 1;
constexpr int kHostCx[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
constexpr int kHostCy[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
constexpr int kHostCz[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};
constexpr int kWallSampleCoarse = 2; ///< Sample distance on the base grid.
constexpr int kWallSampleFine = 3;   ///< Sample distance on a refined level.
constexpr int kInterfaceShell = 2;   ///< Fine interface shell width.

/// Wall-model cell list, SoA (one entry per wall-adjacent fluid cell).
struct WallList {
    std::vector<long long> cellIdx, sampleIdx;
    std::vector<float> nX, nY, nZ, ys;
    std::vector<std::uint32_t> linkMask;
    size_t size() const { return cellIdx.size(); }
};
struct WallListStats {
    int listed = 0, excludedVG = 0, degenerate = 0;
};

/// Fluid cells of `active` with a solid pull neighbour; excluded when any
/// such neighbour is solid only in `active` (a vane); normals from the 5^3
/// occupancy gradient of `clean`; sample cell k..1 normals out.
WallList build_wall_list(const LevelDims& d, const std::uint8_t* active,
                         const std::uint8_t* clean, int sampleCells,
                         WallListStats* stats);

void boundary_flags(const LevelDims& d, std::uint8_t* flags);
int naca4(const char* digits, int pointsPerSurface, std::vector<float>& xy);
constexpr int kMinOutlinePoints = 20;  ///< smallest valid section outline
/// Cosine and sine of the outline rotation (-AoA about the quarter chord),
/// evaluated as the reference's rotated(p, -aoaRad) does (src/core/vec.h:42-46).
void foil_rotation(float aoaDeg, float& c, float& s);
/// voxelizeAirfoil: only Fluid cells inside the outline become Solid.
void voxelize_airfoil(const LevelDims& d, const float* xy, int npts, float aoaDeg,
                      int chordCells, float anchorX, float anchorY,
                      std::uint8_t* flags);
/// closeTrailingEdgeGaps: returns the number of cells closed.
int close_trailing_edge_gaps(const LevelDims& d, std::uint8_t* flags);
void stamp_interface_shell(const LevelDims& d, std::uint8_t* flags, int shell);
void derive_patch_box(const LevelDims& d, const std::uint8_t* flags, int mx0,
                      int mx1, int my0, int my1, int clearance, int out[4]);

} // namespace fcfd
