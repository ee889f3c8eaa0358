/*
 * foilcfd_step.h - C ABI of the GB300-native FoilCFD solver step.
 *
 * One opaque solver object owns every device buffer of one wind tunnel (the
 * coarse lattice, an optional 2:1 refinement patch, the wall-model lists and
 * the force-reduction scratch) and runs the D3Q19 TRT + Smagorinsky step on a
 * single CUDA stream. Plain C types only: pointers, sizes, ints, floats. The
 * stream is passed as `void*` (a cudaStream_t, or NULL for the legacy default
 * stream) so a caller needs no CUDA header to bind this file.
 *
 * Each entry point names the reference interface it replaces
 * (src/sim/lbm_solver.h unless stated otherwise). Return convention, kept from
 * the reference: functions returning `int` give 0 on success or a cudaError_t
 * value (nonzero) on failure; `fcfd_init` / `fcfd_init_refinement` also write a
 * human-readable reason into `err` (always NUL-terminated when errlen > 0).
 *
 * Threading: not thread-safe; one host thread drives one solver, exactly like
 * foilcfd::LBMSolver (lbm_solver.h:129-132).
 */
#ifndef FOILCFD_STEP_H
#define FOILCFD_STEP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- lattice contract (src/sim/lbm_core.cuh:20-130) -------------------- */

/* CellFlag byte values (frozen numbering, lbm_core.cuh:114-130) plus one
 * addition: FCFD_FLAG_OUTLET_EQ, an equilibrium outflow (feq(1, u) of the
 * upstream column) that the reference does not have. */
enum {
    FCFD_FLAG_FLUID = 0,
    FCFD_FLAG_SOLID = 1,
    FCFD_FLAG_INLET = 2,
    FCFD_FLAG_OUTLET = 3,
    FCFD_FLAG_SLIP_TOP = 4,
    FCFD_FLAG_SLIP_BOTTOM = 5,
    FCFD_FLAG_SLIP_FRONT = 6,
    FCFD_FLAG_SLIP_BACK = 7,
    FCFD_FLAG_INTERFACE = 8,
    FCFD_FLAG_OUTLET_EQ = 9
};

/* Population storage precision of a solver (chosen at init). */
enum {
    FCFD_STORE_FP32 = 0, /* f stored as float: 153 B per lattice update   */
    FCFD_STORE_FP16 = 1  /* f - w_q stored as IEEE half: 77 B per update  */
};

/* Grid dimensions; cell index = x + nx*(y + ny*z). Replaces GridDims
 * (lbm_core.cuh:139-158). Unlike the reference, buffers are NOT padded with
 * ghost z planes: all three axes wrap periodically in the index math. */
typedef struct fcfd_dims {
    int nx, ny, nz;
} fcfd_dims;

/* Lattice scaling, field for field the reference LatticeScaling
 * (src/sim/units.h:115-174). Build it with fcfd_compute_scaling. */
typedef struct fcfd_scaling {
    float chord_m, airspeed_ms, nu_m2s; /* PhysicalParams            */
    int chord_cells;                    /* N_c                       */
    float u_lat;                        /* clamped to 0.12           */
    float dx, dt;
    float nu_lat_target, nu_lat, tau;
    int tau_clamped;
    float re_target, re_effective;
} fcfd_scaling;

/* Options of one solver; zero-initialise and set what you need.
 * les_cs / magic_lambda default (when 0) to the reference constants
 * kSmagorinskyCs = 0.1733 and kTRTMagicLambda = 3/16 (units.h:37,46);
 * les_cs < 0 disables the LES term. */
typedef struct fcfd_options {
    int storage;        /* FCFD_STORE_FP32 (default) or FCFD_STORE_FP16   */
    float les_cs;       /* Smagorinsky constant                          */
    float magic_lambda; /* TRT magic parameter                           */
    int use_graphs;     /* 1: replay steady-state batches as CUDA graphs */
    int collide_kernel; /* 0 automatic (= 1), 1 one cell per thread,
                           2 staged rows (bulk async copies into shared
                           memory; slower on GB300, kept selectable) */
    int layout;         /* FCFD_LAYOUT_AB (default) or FCFD_LAYOUT_AA     */
} fcfd_options;

/* Streaming layouts. AB: two population arrays, each step pulls from one
 * into the other (the reference's ping-pong, lbm_solver.cpp:1156-1160). AA:
 * one array updated in place, odd and even steps alternating between a
 * swapped and a streamed slot layout (half the population memory; same
 * results bit for bit). The AA layout serves all-fluid periodic lattices
 * (every flag FCFD_FLAG_FLUID, no refinement, no link fields): fcfd_init
 * refuses other flag fields with cudaErrorNotSupported, as do
 * fcfd_set_flags, fcfd_apply_edited_flags, fcfd_init_refinement and
 * fcfd_set_q_links. Every read of the populations through this interface
 * (export, lattice view, fcfd_active_f, snapshots) sees the A/B state; the
 * solver converts in place and back around such reads. */
enum { FCFD_LAYOUT_AB = 0, FCFD_LAYOUT_AA = 1 };

/* Refinement patch in coarse cells, [x0,x1) x [y0,y1) x [0,nz)
 * (PatchBox, src/sim/lbm_refine.cuh:54-61). */
typedef struct fcfd_patch_box {
    int x0, y0, x1, y1;
} fcfd_patch_box;

/* ForceReadout (lbm_solver.h:28-50), coefficients from the EMA force.
 * fcfd_forces reads the force samples whose asynchronous read-back has
 * completed (as the reference's const forces() reads the state its last
 * poll folded): it never waits on the stream. */
typedef struct fcfd_force_readout {
    float cl, cd, lift_to_drag;
    int valid;
    float flow_throughs;
    float cl_avg, cl_min, cl_max, cl_median;
    float cd_avg, cd_min, cd_max, cd_median;
    float ld_avg, ld_min, ld_max, ld_median;
} fcfd_force_readout;

/* WallModelReadout (lbm_solver.h:82-91). */
typedef struct fcfd_wm_readout {
    int enabled, from_fine, cells;
    float mean_yplus, max_yplus, clamped_frac;
    int excluded_vg, degenerate;
} fcfd_wm_readout;

/* SolverPerfStats (lbm_solver.h:68-74): updates counted as coarse + m*fine,
 * as lbm_solver.cpp:1696-1716 counts them. */
typedef struct fcfd_perf {
    double last_step_ms;
    double mlups;
    double updates_per_step;
} fcfd_perf;

/* Refinement info (RefinementInfo, lbm_solver.h:95-115, level-2 subset). */
typedef struct fcfd_refine_info {
    int active, factor;
    fcfd_patch_box box;
    fcfd_dims fine_dims;
    int forces_from_fine;
    double vram_bytes;
} fcfd_refine_info;

typedef struct fcfd_solver fcfd_solver;

/* ---- units (src/sim/units.h:192-318) ------------------------------------ */

/* computeScaling (units.h:192-219). */
fcfd_scaling fcfd_compute_scaling(float chord_m, float airspeed_ms,
                                  float nu_m2s, int chord_cells, float u_lat);
/* refinedScaling (units.h:242-254). */
fcfd_scaling fcfd_refined_scaling(const fcfd_scaling* parent, int factor);
/* rampedTau / rampedU (units.h:274-283, 310-318). */
float fcfd_ramped_tau(const fcfd_scaling* s, long long step, int nx);
float fcfd_ramped_u(const fcfd_scaling* s, long long step, int nx);
/* LatticeScaling::forceToCoefficient (units.h:168-173). */
float fcfd_force_to_coefficient(const fcfd_scaling* s, float force_lat,
                                int span_cells);

/* ---- lifecycle (lbm_solver.h:133-170) ----------------------------------- */

/* LBMSolver::LBMSolver (lbm_solver.cpp:889). */
fcfd_solver* fcfd_create(void);
/* LBMSolver::~LBMSolver + shutdown (lbm_solver.cpp:890, 868). */
void fcfd_destroy(fcfd_solver* s);
/* LBMSolver::init (lbm_solver.h:151-154, lbm_solver.cpp:803-887): allocates,
 * uploads flags (n == nx*ny*nz bytes), resets. opts may be NULL. */
int fcfd_init(fcfd_solver* s, const fcfd_dims* dims,
              const fcfd_scaling* scaling, const uint8_t* flags, size_t n,
              void* stream, const fcfd_options* opts, char* err,
              size_t errlen);
/* LBMSolver::reset (lbm_solver.cpp:893-944). */
void fcfd_reset(fcfd_solver* s);
/* LBMSolver::setFlags (lbm_solver.cpp:946-952): upload + cold restart. */
int fcfd_set_flags(fcfd_solver* s, const uint8_t* flags, size_t n);
/* LBMSolver::applyEditedFlags (lbm_solver.cpp:1086-1126) with the
 * applyFlagEditsKernel fixup (lbm_core.cu:644-717): warm restart after a
 * geometry edit of the coarse level. Cells whose SOLID state changed are
 * fixed in both population buffers - newly solid zeroed, newly fluid set to
 * the equilibrium of the mean density and velocity of their unedited fluid
 * neighbours (rest state when there are none) - the new flags, force links
 * and wall list are uploaded, and the run continues without ramp; the force
 * average restarts and the force gate reopens half a flow-through later.
 * *edited (nullable) <- number of cells changed. */
int fcfd_apply_edited_flags(fcfd_solver* s, const uint8_t* flags, size_t n, long long* edited);
/* LBMSolver::setStartupRampEnabled (lbm_solver.h:269). */
void fcfd_set_startup_ramp(fcfd_solver* s, int enabled);
/* LBMSolver::setForceEmaWindow (lbm_solver.h:490). */
void fcfd_set_force_ema_window(fcfd_solver* s, float flow_throughs);

/* ---- stepping (lbm_solver.cpp:1132-1390) --------------------------------- */

/* LBMSolver::stepN: n steps with the reference cadence (per-step collide and
 * refinement sub-steps; one force reduction and one wall-model update per
 * batch). Returns 0 with no work while the watchdog is latched. */
int fcfd_step_n(fcfd_solver* s, int n);
/* Blocks until the solver's stream is idle; returns the stream status. */
int fcfd_synchronize(fcfd_solver* s);
long long fcfd_step_count(const fcfd_solver* s);
float fcfd_current_tau(const fcfd_solver* s);
float fcfd_flow_throughs(const fcfd_solver* s);

/* ---- read-back (lbm_solver.h:371-465) ------------------------------------- */

/* forces() (lbm_solver.cpp:1414-1509). Waits for the pending reduction. */
int fcfd_forces(fcfd_solver* s, fcfd_force_readout* out);
/* Raw momentum-exchange force of the last batch in FP64 lattice units
 * (replaces reading DeviceForceAccumulator after launchForceReduction,
 * lbm_core.cuh:341-343; the sum is FP64 and deterministic). */
int fcfd_force_raw(fcfd_solver* s, double out[3]);
/* Runs the force reduction now on the current state (no stepping). */
int fcfd_force_now(fcfd_solver* s, double out[3]);

/* Largest wall-link list fcfd_force_links_noalloc accepts (1,048,576
 * entries): its scratch is a fixed device array of one FP64 triple per 256
 * links, 96 KB, held by every GPU that loads the library. */
#define FCFD_FORCE_NOALLOC_MAX_LINKS (4096 * 256)

/* No counterpart in the reference. The momentum-exchange force of a caller's
 * FP32 population buffer (unpadded SoA, 19*ncells floats on the device) over
 * a caller's compact wall-link list (link_cells[i]: fluid cell index,
 * link_masks[i]: bit q set when the neighbour at +c_q is solid), optionally
 * with a half-bit slip field (uwx/uwy/uwz, all three or none), summed in FP64
 * into out[3] (device memory), enqueued on `stream`. For callers that cannot
 * allocate device memory -- a frame loop with a hard time budget, where
 * cudaMalloc may synchronise the device, or a host whose memory manager owns
 * every allocation: it calls no cudaMalloc/cudaFree; its scratch lives in a
 * static device array. Each call looks that array's address up on the
 * current device (cudaGetSymbolAddress); the first call on a device may load
 * the module, so make it before any stream capture. Calls share the array,
 * so calls that overlap on the GPU race. The buffer must hold FP32
 * populations: fcfd_active_f of a solver created with FCFD_STORE_FP16 holds
 * half-precision deviations (fcfd_f_bytes = 38 * ncells instead of
 * 76 * ncells) and would be read past its end; check fcfd_f_bytes first.
 * Returns cudaErrorInvalidValue (1) when count exceeds
 * FCFD_FORCE_NOALLOC_MAX_LINKS or an argument is missing. */
int fcfd_force_links_noalloc(const float* f, long long ncells,
                             const uint32_t* link_cells,
                             const uint32_t* link_masks, int count,
                             const uint16_t* uwx, const uint16_t* uwy,
                             const uint16_t* uwz, double* out, void* stream);
/* velocityField() / deviceRho() (lbm_solver.h:423-429): device pointers of
 * the unpadded macroscopic arrays, written on each batch's last step. */
int fcfd_macro(fcfd_solver* s, const float** rho, const float** u,
               const float** v, const float** w);
/* Synchronous copy of the four macroscopic arrays to host memory. */
int fcfd_download_macro(fcfd_solver* s, float* rho, float* u, float* v,
                        float* w);
/* deviceFlags() (lbm_solver.h:431-437): device CellFlag bytes of a level
 * (0 coarse, 1 fine, 2 finer), cellCount bytes, unpadded x + nx*(y + ny*z)
 * -- here the same layout the kernels index, since nothing is padded. */
int fcfd_device_flags(fcfd_solver* s, int level, const uint8_t** flags);
/* latticeView() (lbm_solver.h:439-444): the current source buffer of a
 * level with everything an external kernel needs to read it -- the
 * population base (unpadded SoA f[q*cells + cell] in the storage precision:
 * float for FCFD_STORE_FP32, half(f - w_q) for FCFD_STORE_FP16), the flag
 * bytes, the grid and, with the wall model on, the level's half-bit slip
 * field (else NULL). Valid until the next step, flag change or refinement
 * change. fcfd_force_links_noalloc takes an FP32 view's f and slip arrays. */
typedef struct fcfd_lattice {
    void* f;
    const uint8_t* flags;
    fcfd_dims dims;
    long long cells;
    int storage;
    const uint16_t *uwx, *uwy, *uwz;
} fcfd_lattice;
int fcfd_lattice_view(fcfd_solver* s, int level, fcfd_lattice* out);
/* Device pointer of the current population buffer and its size
 * (activeDeviceF / fBufferBytes, lbm_solver.h:446-458). The layout is
 * unpadded SoA f[q*ncells + cell] in the solver's storage precision. */
void* fcfd_active_f(fcfd_solver* s);
size_t fcfd_f_bytes(const fcfd_solver* s);
/* notifySnapshotRestored (lbm_solver.cpp:1750-1771). */
void fcfd_notify_restored(fcfd_solver* s, int full_state);
/* Unpadded FP32 SoA import/export, f[q*ncells + cell], 19*ncells floats,
 * whatever the storage precision (the uploadF / downloadMoments harness of
 * tests/lbm_test_util.h:116-204). Import calls fcfd_notify_restored(s, 1). */
int fcfd_import_f32(fcfd_solver* s, const float* host_f, size_t count);
int fcfd_export_f32(fcfd_solver* s, float* host_f, size_t count);
/* Copy every level's current population buffer into its other A/B buffer.
 * Cells a step never writes (solid, slip planes, interface shell) keep the
 * other buffer's contents, as in the reference's ping-pong pair; after
 * importing a state that holds only the current buffer, this makes both
 * buffers carry it. No reference counterpart. */
int fcfd_mirror_buffers(fcfd_solver* s);
/* Two-phase FP32 import, so that the host copy of the next state overlaps
 * the stepping of the current one (no reference counterpart: the reference
 * restores with blocking copies). fcfd_stage_f32 queues the host -> device
 * copy of one level's FP32 SoA state (level 0 coarse, 1 fine, 2 finer;
 * 19*ncells floats, pinned host memory for the copy to be asynchronous) into
 * a device staging buffer on a copy stream of the solver's own; the host
 * buffer must stay valid until the commit. fcfd_commit_staged orders the
 * solver stream after the staged copies and makes them the levels' current
 * state: the same state as fcfd_import_f32 / fcfd_import_fine_f32 /
 * fcfd_import_finer_f32 of that data (with fcfd_notify_restored(s, 1) when
 * the coarse level was staged). A stage issued after a commit waits for the
 * commit to have read the staging buffer. cudaErrorNotReady: nothing staged. */
int fcfd_stage_f32(fcfd_solver* s, int level, const float* host_f, size_t count);
int fcfd_commit_staged(fcfd_solver* s);
/* restoreFromMacroscopic (lbm_solver.cpp:1773-1803), host arrays. */
int fcfd_restore_from_macro(fcfd_solver* s, const float* rho, const float* u,
                            const float* v, const float* w);
/* perfStats (lbm_solver.cpp:1696-1716). */
int fcfd_perf_stats(const fcfd_solver* s, fcfd_perf* out);
/* nanDetected / nanDiagnosis (lbm_solver.h:401-404). Kind 1/2: NaN or
 * velocity runaway on the coarse grid, 3/4 on the fine grid (the reference's
 * codes), 9: a staged collide's copy wait timed out (the step's results are
 * incomplete; the solver pauses like on a watchdog trip). */
int fcfd_nan_detected(fcfd_solver* s);
int fcfd_nan_kind(fcfd_solver* s);

/* ---- wall model (lbm_solver.h:280-307, lbm_wallmodel.cuh) ---------------- */

/* setWallModelEnabled (lbm_solver.cpp:968-980). */
int fcfd_set_wall_model(fcfd_solver* s, int enabled);
/* setSurfaceReference (lbm_solver.cpp:955-966): clean (VG-free) flags. */
int fcfd_set_surface_reference(fcfd_solver* s, const uint8_t* clean,
                               size_t n);
/* setRefinedSurfaceReference (lbm_solver.cpp:984-991). */
int fcfd_set_refined_surface_reference(fcfd_solver* s, const uint8_t* clean,
                                       size_t n);
/* wallModelReadout (lbm_solver.cpp:993-1022). */
int fcfd_wall_model_readout(fcfd_solver* s, fcfd_wm_readout* out);
/* Wall-cell count and state export of one level (0 coarse, 1 fine): u_tau
 * per listed cell (count floats) and the slip field as half bits (3*ncells
 * uint16: uwx, then uwy, then uwz). Test/inspection hooks. */
int fcfd_wall_count(fcfd_solver* s, int level);
int fcfd_export_wall_state(fcfd_solver* s, int level, float* utau,
                           size_t n_utau, uint16_t* slip, size_t n_slip);
int fcfd_import_wall_state(fcfd_solver* s, int level, const float* utau,
                           size_t n_utau, const uint16_t* slip,
                           size_t n_slip);
/* Runs one wall-model update now (launchWallModelUpdate,
 * lbm_wallmodel.cu:200-225) on a level with the given lattice viscosity. */
int fcfd_wall_update_now(fcfd_solver* s, int level, float nu_lat,
                         float ut_cutoff);

/* ---- interpolated bounce-back (q-LIBB) link fields ----------------------- */

/* setCoarseQLinks / setFineQLinks (lbm_solver.h:330-340, lbm_solver.cpp:
 * 1041-1056): per cell and direction the cut fraction of a resolved surface
 * on a solid link (byte b -> q = b/255, 0 = plain half-way bounce-back),
 * q_frac[cell * 19 + q] (count = 19 * cells), and per cell the bits of the
 * links whose second fluid node x + c_q exists, ff_mask[cell]. The collide
 * then applies Bouzidi's linear interpolation on those links
 * (lbm_core.cu:332-364). level 0 coarse, 1 fine, 2 finer; nq == 0 clears.
 * links / fallback are the caller's counts, kept for fcfd_q_link_info. */
int fcfd_set_q_links(fcfd_solver* s, int level, const uint8_t* q_frac, size_t nq,
                     const uint32_t* ff_mask, size_t nm, int links, int fallback);
int fcfd_q_link_info(fcfd_solver* s, int level, int* active, int* links, int* fallback);

/* ---- refinement (lbm_solver.h:192-246) ------------------------------------ */

/* initRefinement (lbm_solver.cpp:1812-1888). */
int fcfd_init_refinement(fcfd_solver* s, const fcfd_patch_box* box,
                         int factor, const uint8_t* fine_flags, size_t n,
                         char* err, size_t errlen);
void fcfd_shutdown_refinement(fcfd_solver* s);
/* setRefinedFlags (lbm_solver.cpp:1894-1912). */
int fcfd_set_refined_flags(fcfd_solver* s, const uint8_t* fine_flags,
                           size_t n);
int fcfd_refinement_info(const fcfd_solver* s, fcfd_refine_info* out);
/* FP32 SoA import/export of the fine level's current buffer. */
int fcfd_import_fine_f32(fcfd_solver* s, const float* host_f, size_t count);
int fcfd_export_fine_f32(fcfd_solver* s, float* host_f, size_t count);
/* Factor-2 patches: form the restriction's child averages inside the last
 * fine sub-step's collide (1) instead of re-reading the fine level in a
 * separate pass (0; lbm_refine.cu:274-429 reads it in the restriction).
 * Negative (the default): 1 with FP32 storage, 0 with FP16, the faster of
 * the two for each. With FP32 storage both give the same populations bit
 * for bit. */
int fcfd_set_fused_restriction(fcfd_solver* s, int enabled);

/* ---- nested finer level (lbm_solver.h:118-124, 207-243) ----------------- */

/* Finer level state (the RefinementInfo finer* fields). */
typedef struct fcfd_finer_info {
    int active;
    int factor;
    fcfd_patch_box box;   /* in FINE cells */
    fcfd_dims dims;       /* factor * box extent, factor * fine nz */
    double vram_bytes;
} fcfd_finer_info;

/* initFinerRefinement (lbm_solver.cpp:1916-2000): a nested patch inside the
 * fine level, box in FINE cells, factor 2..4, finer flags with their
 * INTERFACE shell; the finer level is seeded from the fine field. Each fine
 * sub-step then runs `factor` finer sub-steps and a finer -> fine
 * restriction (lbm_solver.cpp:1209-1270). Forces stay on the fine level. */
int fcfd_init_finer_refinement(fcfd_solver* s, const fcfd_patch_box* box, int factor,
                               const uint8_t* finer_flags, size_t n, char* err, size_t errlen);
void fcfd_shutdown_finer_refinement(fcfd_solver* s);
/* setRefinedFinerFlags / setRefinedFinerSurfaceReference. */
int fcfd_set_refined_finer_flags(fcfd_solver* s, const uint8_t* finer_flags, size_t n);
int fcfd_set_refined_finer_surface_reference(fcfd_solver* s, const uint8_t* clean, size_t n);
int fcfd_finer_refinement_info(const fcfd_solver* s, fcfd_finer_info* out);
/* FP32 SoA import/export of the finer level's current buffer. */
int fcfd_import_finer_f32(fcfd_solver* s, const float* host_f, size_t count);
int fcfd_export_finer_f32(fcfd_solver* s, float* host_f, size_t count);

/* ---- host fixture builders (src/sim/wall_model.h, src/geom/) ------------- */

/* buildWallCellList (wall_model.h:107-111): host-only, no GPU. Output
 * arrays sized `cap`; returns the listed count (or -1 if cap is too small),
 * stats[3] = {listed, excludedVG, degenerate}. */
long long fcfd_build_wall_list(const fcfd_dims* dims, const uint8_t* active,
                               const uint8_t* clean, int sample_cells,
                               long long* cell_idx, long long* sample_idx,
                               float* nx, float* ny, float* nz, float* ys,
                               uint32_t* link_mask, long long cap,
                               int* stats);

/* buildBoundaryFlags (src/geom/voxelizer.h:97). */
int fcfd_boundary_flags(const fcfd_dims* dims, uint8_t* flags, size_t n);
/* generateNACA4 (src/geom/airfoil.h:73): 2*pps-1 points (x,y) into xy.
 * Returns the point count, or -1 on a bad digit string / small buffer. */
int fcfd_naca4(const char* digits, int points_per_surface, float* xy,
               int cap_points);
/* voxelizeAirfoil (voxelizer.h:99-116, voxelizer.cpp:62-153) with the
 * DomainLayout anchor given in lattice cells: Fluid cells whose centres lie
 * inside the rotated, scaled outline become Solid (x in 1..nx-2, y in
 * 1..ny-2, every z). An outline of fewer than 20 points stamps nothing. */
int fcfd_voxelize_airfoil(const fcfd_dims* dims, const float* xy, int npts,
                          float aoa_deg, int chord_cells, float anchor_x,
                          float anchor_y, uint8_t* flags, size_t n);
/* closeTrailingEdgeGaps (voxelizer.h:118-125, voxelizer.cpp:155-183):
 * returns the number of single-cell gaps closed. */
int fcfd_close_trailing_edge_gaps(const fcfd_dims* dims, uint8_t* flags,
                                  size_t n);
/* stampInterfaceShell (voxelizer.h:181). */
int fcfd_stamp_interface_shell(const fcfd_dims* dims, uint8_t* flags,
                               size_t n);
/* derivePatchBox (voxelizer.h:196). */
fcfd_patch_box fcfd_derive_patch_box(const fcfd_dims* dims,
                                     const uint8_t* flags, int mx0, int mx1,
                                     int my0, int my1, int clearance);

/* ---- diagnostics ----------------------------------------------------------- */

/* Kernel launches issued by this solver since creation (all kernels). */
long long fcfd_kernel_launches(const fcfd_solver* s);
/* Per-kernel timing on the solver stream with CUDA events: when enabled,
 * every stream-collide launch (both levels) is bracketed by events and
 * fcfd_collide_time_ms returns, for the plain collides, the total ms, the
 * launch count, the cells
 * those launches covered and their algorithmic DRAM bytes (per cell class:
 * read+write cells 2*19 populations + kind byte, inlet cells 19 + 1,
 * untouched solid/slip/interface cells 1) since the last call. */
int fcfd_enable_collide_timing(fcfd_solver* s, int enabled);
int fcfd_collide_time_ms(fcfd_solver* s, double* total_ms, long long* count,
                         double* cells, double* alg_bytes);
/* The same for the fine collides that form the restriction's child averages
 * (fcfd_set_fused_restriction): their bytes add the 96-byte scratch record
 * of every coarse cell of the restricted box. No reference counterpart. */
int fcfd_fused_collide_time_ms(fcfd_solver* s, double* total_ms, long long* count,
                               double* cells, double* alg_bytes);
/* Event pair on the solver stream: start, then stop returns elapsed ms. */
int fcfd_timer_start(fcfd_solver* s);
int fcfd_timer_stop(fcfd_solver* s, double* ms);
/* Page-locked host memory (cudaMallocHost / cudaFreeHost) for staging. */
void* fcfd_host_alloc(size_t bytes);
void fcfd_host_free(void* p);
/* Library version string. */
const char* fcfd_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FOILCFD_STEP_H */
