// ORACLE - test infrastructure only. C entry point over the reference's host
// wall-cell list builder (src/sim/wall_model.cpp, compiled unmodified from
// the reference tree by ref_build.py) for golden-vector generation.
#include <cstring>

#include "wall_model.h"

extern "C" long long ref_build_wall_list(int nx, int ny, int nz, const unsigned char* active,
                                         const unsigned char* clean, int sample, long long* ci, long long* si,
                                         float* nX, float* nY, float* nZ, float* ys, unsigned* mask,
                                         long long cap, int* stats) {
    foilcfd::GridDims d;
    d.nx = nx; d.ny = ny; d.nz = nz;
    const size_t n = static_cast<size_t>(d.cellCount());
    std::vector<std::uint8_t> a(active, active + n), c(clean, clean + n);
    foilcfd::WallListStats st{};
    const foilcfd::WallCellList l = foilcfd::buildWallCellList(d, a, c, sample, &st);
    stats[0] = st.listed; stats[1] = st.excludedVG; stats[2] = st.degenerate;
    const long long m = static_cast<long long>(l.size());
    if (m > cap) return -1;
    for (long long i = 0; i < m; ++i) {
        ci[i] = l.cellIdx[i]; si[i] = l.sampleIdx[i];
        nX[i] = l.normalX[i]; nY[i] = l.normalY[i]; nZ[i] = l.normalZ[i];
        ys[i] = l.sampleDist[i]; mask[i] = l.linkMask[i];
    }
    return m;
}
