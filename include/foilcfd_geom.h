/*
 * foilcfd_geom.h - C ABI of the on-device geometry builders.
 *
 * The reference prepares every flag field and cell list on the host
 * (src/geom/voxelizer.cpp, src/sim/wall_model.cpp) and uploads them; an
 * angle-of-attack sweep rebuilds them for every geometry. These entry points
 * build the same bytes in device memory with CUDA kernels on the caller's
 * stream: the result of each equals, byte for byte, the host builder of
 * foilcfd_step.h it names (fcfd_boundary_flags, fcfd_voxelize_airfoil,
 * fcfd_close_trailing_edge_gaps, fcfd_stamp_interface_shell,
 * fcfd_derive_patch_box, fcfd_build_wall_list).
 *
 * Pointers prefixed d_ are device memory; the outline (fcfd_foil.xy) is host
 * memory. The solver entry points that take flags (fcfd_init, fcfd_set_flags,
 * fcfd_apply_edited_flags, fcfd_init_refinement, fcfd_set_refined_flags,
 * fcfd_init_finer_refinement, fcfd_set_refined_finer_flags) accept a flag
 * field in device memory as well: the solver then copies it on the device and
 * builds its force-link, wall-model, shell and seed lists with these kernels.
 *
 * Return convention: 0 or a cudaError_t value. The list builders and the
 * patch box synchronise the stream before they return; the flag builder
 * does when it rasterises an outline (row-crossing check) or reports the
 * closure count.
 */
#ifndef FOILCFD_GEOM_H
#define FOILCFD_GEOM_H

#include <stddef.h>
#include <stdint.h>

#include "foilcfd_step.h"

#ifdef __cplusplus
extern "C" {
#endif

/* A section placed in the lattice (DomainLayout, src/geom/voxelizer.h:57-90,
 * with the anchor in cells): the outline of fcfd_naca4 (HOST memory, npts
 * (x, y) pairs in chord units), rotated about the quarter chord by -aoa_deg,
 * scaled by chord_cells and moved to the anchor. */
typedef struct fcfd_foil {
    const float* xy;
    int npts;
    float aoa_deg;
    int chord_cells;
    float anchor_x, anchor_y;
} fcfd_foil;

/* Base of a built flag field. */
enum {
    FCFD_BASE_BOUNDARY = 0, /* buildBoundaryFlags: inlet, outlet, slip faces */
    FCFD_BASE_FLUID = 1,    /* all fluid (a refinement level)                */
    FCFD_BASE_INPUT = 2     /* the device field d_in (d_in != d_out)          */
};

/* Build a flag field of dims into d_out: the base, then the foil (nullable;
 * voxelizeAirfoil), then, when close_gaps, closeTrailingEdgeGaps over the
 * whole field, then, when shell_cells > 0, the interface shell
 * (stampInterfaceShell). buildCleanFoilFlags is (BOUNDARY, foil, 1, 0);
 * buildFinePatchFlags is (FLUID, the fine placement, 1, 2). *closed
 * (nullable) <- cells closed. A lattice row crossed by more than 64 outline
 * edges is refused (cudaErrorInvalidValue). */
int fcfd_device_build_flags(const fcfd_dims* dims, int base, const uint8_t* d_in, const fcfd_foil* foil,
                            int close_gaps, int shell_cells, uint8_t* d_out, void* stream, int* closed);

/* derivePatchBox (voxelizer.cpp:265-301) of a device flag field; an all-zero
 * box when the field has no solid cell. */
int fcfd_device_derive_patch_box(const fcfd_dims* dims, const uint8_t* d_flags, int mx0, int mx1, int my0, int my1,
                                 int clearance, void* stream, fcfd_patch_box* box);

/* Fluid cells with a solid neighbour at x + c_q (all axes periodic) and that
 * neighbour mask (bit q), in ascending cell order - the momentum-exchange
 * link list. *count <- the list length; nothing is written when it exceeds
 * cap (size the buffers with a first call of cap 0). */
int fcfd_device_force_links(const fcfd_dims* dims, const uint8_t* d_flags, uint32_t* d_cells, uint32_t* d_masks,
                            long long cap, long long* count, void* stream);

/* buildWallCellList (wall_model.h:107-111) on device fields (d_clean
 * nullable = d_active), the same entries in the same order as
 * fcfd_build_wall_list, cell and sample indices as uint32. *count, cap and
 * stats[3] = {listed, excluded_vg, degenerate} as above. */
int fcfd_device_build_wall_list(const fcfd_dims* dims, const uint8_t* d_active, const uint8_t* d_clean,
                                int sample_cells, uint32_t* d_cell, uint32_t* d_sample, float* d_nx, float* d_ny,
                                float* d_nz, float* d_ys, uint32_t* d_link_mask, long long cap, long long* count,
                                int* stats, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FOILCFD_GEOM_H */
