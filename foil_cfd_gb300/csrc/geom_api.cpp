// C ABI of the on-device geometry builders (include/foilcfd_geom.h): argument
// checks and the host-side parts (outline rotation, patch-box clamping) around
// the kernels of geom_kernels.cu.
#include "../../include/foilcfd_geom.h"

#include <cuda_runtime.h>

#include <algorithm>

#include "host_geom.h"
#include "kernels.h"

using namespace fcfd;

namespace {

bool dims_ok(const fcfd_dims* d) {
    return d && d->nx > 0 && d->ny > 0 && d->nz > 0
           && static_cast<long long>(d->nx) * d->ny * d->nz < (1LL << 31);
}

} // namespace

extern "C" {

int fcfd_device_build_flags(const fcfd_dims* dims, int base, const uint8_t* d_in, const fcfd_foil* foil,
                            int close_gaps, int shell_cells, uint8_t* d_out, void* stream, int* closed) {
    if (!dims_ok(dims) || !d_out || shell_cells < 0) return cudaErrorInvalidValue;
    const LevelDims d{dims->nx, dims->ny, dims->nz};
    FoilRaster r;
    const FoilRaster* rp = nullptr;
    // voxelizeAirfoil stamps nothing for an invalid section or a grid under 3x3.
    if (foil && foil->xy && foil->npts >= kMinOutlinePoints && d.nx >= 3 && d.ny >= 3) {
        r.xy = foil->xy;
        r.npts = foil->npts;
        foil_rotation(foil->aoa_deg, r.cosA, r.sinA);
        r.chord = static_cast<float>(foil->chord_cells);
        r.anchorX = foil->anchor_x;
        r.anchorY = foil->anchor_y;
        rp = &r;
    }
    const bool closeOk = close_gaps && d.nx >= 3 && d.ny >= 3;
    int c = 0;
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    const cudaError_t e = device_build_flags(d, base, d_in, rp, closeOk ? 1 : 0, shell_cells, d_out, st, &c);
    if (e == cudaSuccess && closed) *closed = c;
    return static_cast<int>(e);
}

int fcfd_device_derive_patch_box(const fcfd_dims* dims, const uint8_t* d_flags, int mx0, int mx1, int my0, int my1,
                                 int clearance, void* stream, fcfd_patch_box* box) {
    if (!dims_ok(dims) || !d_flags || !box) return cudaErrorInvalidValue;
    *box = fcfd_patch_box{};
    int b[4];
    const LevelDims d{dims->nx, dims->ny, dims->nz};
    if (auto e = device_solid_bbox(d, d_flags, static_cast<cudaStream_t>(stream), b); e != cudaSuccess)
        return static_cast<int>(e);
    if (b[2] < 0) return 0;
    // Pad by the margins; keep `clearance` cells to every domain face.
    box->x0 = std::max(clearance, b[0] - mx0);
    box->x1 = std::min(d.nx - clearance, b[2] + 1 + mx1);
    box->y0 = std::max(clearance, b[1] - my0);
    box->y1 = std::min(d.ny - clearance, b[3] + 1 + my1);
    return 0;
}

int fcfd_device_force_links(const fcfd_dims* dims, const uint8_t* d_flags, uint32_t* d_cells, uint32_t* d_masks,
                            long long cap, long long* count, void* stream) {
    if (!dims_ok(dims) || !d_flags || !count || cap < 0 || (cap > 0 && (!d_cells || !d_masks)))
        return cudaErrorInvalidValue;
    const LevelDims d{dims->nx, dims->ny, dims->nz};
    return static_cast<int>(device_force_links(d, d_flags, d_cells, d_masks, cap, count,
                                               static_cast<cudaStream_t>(stream)));
}

int fcfd_device_build_wall_list(const fcfd_dims* dims, const uint8_t* d_active, const uint8_t* d_clean,
                                int sample_cells, uint32_t* d_cell, uint32_t* d_sample, float* d_nx, float* d_ny,
                                float* d_nz, float* d_ys, uint32_t* d_link_mask, long long cap, long long* count,
                                int* stats, void* stream) {
    if (!dims_ok(dims) || !d_active || !count || cap < 0 || sample_cells < 0) return cudaErrorInvalidValue;
    if (cap > 0 && (!d_cell || !d_sample || !d_nx || !d_ny || !d_nz || !d_ys || !d_link_mask))
        return cudaErrorInvalidValue;
    const LevelDims d{dims->nx, dims->ny, dims->nz};
    WallListOut o;
    o.cell = d_cell; o.sample = d_sample; o.mask = d_link_mask;
    o.nX = d_nx; o.nY = d_ny; o.nZ = d_nz; o.ys = d_ys;
    int st3[3] = {0, 0, 0};
    const cudaError_t e = device_wall_list(d, d_active, d_clean, sample_cells, o, cap, count, st3,
                                           static_cast<cudaStream_t>(stream));
    if (e == cudaSuccess && stats) { stats[0] = st3[0]; stats[1] = st3[1]; stats[2] = st3[2]; }
    return static_cast<int>(e);
}

} // extern "C"
