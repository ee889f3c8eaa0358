// Host-callable launch functions of the GB300 solver-step kernels. Plain C++
// (no CUDA-only syntax), so the orchestrator compiles as ordinary host code.
// Every launcher returns the cudaGetLastError() of its launch, the contract of
// the reference launch wrappers (src/sim/lbm_core.cuh:249-254).
#pragma once

#include <cstdint>
#include <cuda_runtime_api.h>

#include "batch_types.h"
#include "wallnet_types.h"

struct fcfd_wallnet;

#ifdef __CUDACC__
#define FCFD_HD __host__ __device__
#else
#define FCFD_HD
#endif

namespace fcfd {

/// Geometry of one lattice level: unpadded SoA, cell = x + nx*(y + ny*z).
struct LevelDims {
    int nx = 0, ny = 0, nz = 0;
    FCFD_HD long long cells() const { return static_cast<long long>(nx) * ny * nz; }
};

/// Per-step collision parameters (reference StepParams, lbm_core.cuh:233-241).
struct CollideParams {
    float tau = 0.6f;
    float magicLambda = 3.0f / 16.0f;
    float smagPrefactor = 0.0f; ///< 18*sqrt(2)*Cs^2; 0 disables LES.
    float uInlet = 0.08f;
    int writeMacro = 0;
    int* status = nullptr;  ///< Device int set nonzero if a staged copy wait timed out.
    int kernel = 0;         ///< 0 automatic, 1 one-cell kernel, 2 staged kernel.
    /// Interpolated bounce-back (q-LIBB) link field of the level, or null:
    /// cut bytes [cell * 19 + q] (q = byte / 255) and two-node bits [cell].
    const std::uint8_t* qFrac = nullptr;
    const std::uint32_t* ffMask = nullptr;
    /// Link classes of each fluid cell's pull neighbours (launch_classify),
    /// or null: the near-wall gather then reads the neighbours' flags.
    const uint2* links = nullptr;
};

/// Half-bit slip field of a level (WallSlipView, lbm_core.cuh:201-208).
struct SlipField {
    const std::uint16_t* uwx = nullptr;
    const std::uint16_t* uwy = nullptr;
    const std::uint16_t* uwz = nullptr;
    bool active() const { return uwx && uwy && uwz; }
};

enum class Storage : int { F32 = 0, F16 = 1 };

// ---- step kernels (step_kernels.cu) ---------------------------------------
/// Kind bytes, and (links not null) per fluid cell the classes of its 18
/// pull links x - c_q as one 64-bit word (low half in .x): bit q - 1 solid,
/// bit 17 + q free-slip y wall, bit 35 + q free-slip z wall; 0 for cells
/// that are not fluid.
cudaError_t launch_classify(const std::uint8_t* flags, std::uint8_t* kind,
                            LevelDims d, cudaStream_t st, uint2* links = nullptr);
cudaError_t launch_collide(Storage s, const void* src, void* dst,
                           const std::uint8_t* kind, LevelDims d,
                           const CollideParams& p, float* rho, float* u,
                           float* v, float* w, SlipField slip, cudaStream_t st);
cudaError_t launch_init_equilibrium(Storage s, void* f, const std::uint8_t* kind,
                                    LevelDims d, float uInlet, cudaStream_t st);
cudaError_t launch_speck(Storage s, void* f, const std::uint8_t* kind, LevelDims d,
                         float amplitude, unsigned seed, cudaStream_t st);
cudaError_t launch_init_from_macro(Storage s, void* f, const std::uint8_t* kind,
                                   LevelDims d, const float* rho, const float* u,
                                   const float* v, const float* w, cudaStream_t st);
cudaError_t launch_watchdog(Storage s, const void* f, LevelDims d, int* flag,
                            long long offset, int flagBase, cudaStream_t st);
cudaError_t launch_f32_to_store(Storage s, const float* in, void* out,
                                long long cells, cudaStream_t st);
cudaError_t launch_store_to_f32(Storage s, const void* in, float* out,
                                long long cells, cudaStream_t st);
cudaError_t launch_fill(float* dst, long long n, float v, cudaStream_t st);

/// AA-pattern in-place step of an all-fluid periodic level (one population
/// array): odd steps read the swapped layout and leave the streamed one, even
/// steps the reverse (collide_common.cuh).
cudaError_t launch_collide_aa(Storage s, void* f, LevelDims d, const CollideParams& p, int odd, float* rho,
                              float* u, float* v, float* w, cudaStream_t st);
/// A/B state <-> swapped layout, in place.
cudaError_t launch_aa_pair_swap(Storage s, void* f, long long cells, cudaStream_t st);
/// Streamed layout -> A/B state (toAB 1) or back (0), in place through a
/// one-slice scratch buffer (cells elements of the storage type).
cudaError_t launch_aa_shift(Storage s, void* f, void* slice, LevelDims d, int toAB, cudaStream_t st);

/// The restriction's child-average pass fused into the last fine sub-step
/// (factor 2): scratch records of the coarse cells of the restricted sub-box.
struct ChildFuse {
    float* scratch = nullptr;
    int boxX0 = 0, boxY0 = 0;       ///< patch origin (coarse cells)
    int rx0 = 0, ry0 = 0, rw = 0, rh = 0;  ///< restricted sub-box (coarse cells)
};
cudaError_t launch_collide_child(Storage s, const void* src, void* dst, const std::uint8_t* kind, LevelDims d,
                                 const CollideParams& p, SlipField slip, const ChildFuse& cf, cudaStream_t st);
/// Warm-restart flag-edit fixup of both buffers (mask 1 newly solid, 2 newly
/// fluid; flags = the new CellFlag bytes).
cudaError_t launch_apply_flag_edits(Storage s, void* fA, void* fB, const std::uint8_t* flags,
                                    const std::uint8_t* mask, LevelDims d, cudaStream_t st);
cudaError_t launch_apply_flag_edits_f32(float* fA, float* fB, const std::uint8_t* flags, const std::uint8_t* mask,
                                        LevelDims d, cudaStream_t st);

// ---- FP32 reference-order kernels (collide_f32.cu, built with --fmad=false)
cudaError_t launch_collide_f32_ref(const float* src, float* dst, const std::uint8_t* kind,
                                   LevelDims d, const CollideParams& p, float* rho,
                                   float* u, float* v, float* w, SlipField slip,
                                   cudaStream_t st);
cudaError_t launch_collide_aa_f32(float* f, LevelDims d, const CollideParams& p, int odd, float* rho, float* u,
                                  float* v, float* w, cudaStream_t st);
/// Whether the staged kernel serves a level (16-byte rows, >= 2 stages fit).
bool staged_applies(LevelDims d, Storage s);
cudaError_t launch_init_eq_f32(float* f, const std::uint8_t* kind, long long n, float uIn,
                               cudaStream_t st);
cudaError_t launch_collide_child_f32(const float* src, float* dst, const std::uint8_t* kind, LevelDims d,
                                     const CollideParams& p, SlipField slip, const ChildFuse& cf, cudaStream_t st);
cudaError_t launch_init_macro_f32(float* f, const std::uint8_t* kind, long long n,
                                  const float* rho, const float* u, const float* v,
                                  const float* w, cudaStream_t st);

// ---- force reduction (force_kernels.cu) ------------------------------------
/// Momentum exchange over a compact wall-link list: entry i is fluid cell
/// cells[i] with bit q of masks[i] set when the neighbour at +c_q is solid.
/// Block partials go to `partials` (3 doubles per block, blocks =
/// force_blocks(count)); a second single-block pass sums them in a fixed
/// order into out[3]. Deterministic, FP64 from the per-link terms up.
int force_blocks(int count);
cudaError_t launch_force(Storage s, const void* f, long long cells,
                         const std::uint32_t* linkCells,
                         const std::uint32_t* linkMasks, int count,
                         SlipField slip, double* partials, double* out,
                         cudaStream_t st);

// ---- wall model (wall_kernels.cu) ------------------------------------------
struct WallListDev {
    const std::uint32_t* cellIdx = nullptr;
    const std::uint32_t* sampleIdx = nullptr;
    const float* nX = nullptr;
    const float* nY = nullptr;
    const float* nZ = nullptr;
    const float* ys = nullptr;
    const std::uint32_t* linkMask = nullptr;
    float* uTau = nullptr;
    int count = 0;
};
struct WallStatsDev {
    float sumYplus;
    int maxYplusBits;
    int activeCells;
    int clampedCells;
    int fallbackCells;            // learned u_tau solve: FP64 fallbacks
    int pad;
    unsigned long long newtonIters; // FP64 Newton iterations summed
};
/// u_tau solve of a wall update: the FCFD_UTAU_* values of
/// include/foilcfd_wallnet.h (0 reference, 1 FP64 Newton, 2 learned).
/// `net` is the device view of a learned seed (BF16 weights + normalisation),
/// required by the learned method.
cudaError_t launch_wall_update(Storage s, const void* f, long long cells,
                               WallListDev list, std::uint16_t* uwx,
                               std::uint16_t* uwy, std::uint16_t* uwz,
                               float nuLat, float utCutoff, float emaAlpha,
                               WallStatsDev* stats, cudaStream_t st,
                               int method = 0, const wallnet::NetDev* net = nullptr);
/// The FP32 update, built without contraction (wall_kernels_x.cu): FP32
/// storage rounds the wall model's expressions as written, like every other
/// FP32 kernel; launch_wall_update routes FP32 storage here.
cudaError_t launch_wall_update_f32_x(const void* f, long long cells, WallListDev list,
                                     std::uint16_t* uwx, std::uint16_t* uwy, std::uint16_t* uwz,
                                     float nuLat, float utCutoff, float emaAlpha, WallStatsDev* stats,
                                     cudaStream_t st, int method, const wallnet::NetDev* net);
/// Device view (BF16 weights + normalisation) of a learned seed network.
wallnet::NetDev wallnet_view(const fcfd_wallnet* net);
/// Sampled tangential speed (0 below the cut-off) and sample distance of
/// every wall-list entry.
cudaError_t launch_wall_harvest(Storage s, const void* f, long long cells, WallListDev list,
                                float utCutoff, float* utOut, float* ysOut, cudaStream_t st);

// ---- batched multi-tunnel step (batch_f32.cu, batch_f16.cu) ---------------
/// One step of the tunnels owning work items [itemBase, itemBase + nItems):
/// src = f[parity], dst = f[parity ^ 1]. The table goes by value into the
/// kernel's parameters. Shapes: block 64/128/256, rows 1/2/4; grid 0 = one
/// block per work item.
cudaError_t launch_batch_collide_f32(const BatchTable& tab, unsigned itemBase, unsigned nItems, int parity,
                                     BatchShape sh, cudaStream_t st);
cudaError_t launch_batch_collide_f16(const BatchTable& tab, unsigned itemBase, unsigned nItems, int parity,
                                     BatchShape sh, cudaStream_t st);
/// Resident blocks per SM of a batched collide shape (0: unknown shape).
int batch_occupancy_f32(BatchShape sh);
int batch_occupancy_f16(BatchShape sh);
cudaError_t launch_force_append(const double* cur, int n3, double* hist, int cap, int* count, cudaStream_t st);
/// Per-tunnel health: max speed over non-solid cells (float bits into
/// *maxSpeedBits, which must start at 0) and non-finite cell count.
cudaError_t launch_batch_health(bool fp32, const void* f, const std::uint8_t* kind, long long n, int* maxSpeedBits,
                                int* nonFinite, cudaStream_t st);
/// Set latch[t] (1 non-finite, 2 speed >= cap) of every running tunnel from
/// its health scan (maxSpeedBits[t], nonFinite[t]), and latch[ntun + t] to the
/// force-sample count *samples when it does.
cudaError_t launch_batch_latch(const int* maxSpeedBits, const int* nonFinite, int ntun, float cap,
                               const int* samples, int* latch, cudaStream_t st);

// ---- refinement (refine_kernels.cu) ----------------------------------------
struct RefineGeom {
    LevelDims coarse, fine;
    int boxX0 = 0, boxY0 = 0, boxX1 = 0, boxY1 = 0;
    int factor = 2;
};
cudaError_t launch_fill_c2f(Storage s, const void* cT0, const void* cT1,
                            const std::uint8_t* coarseKind, void* fineF,
                            const std::uint32_t* targets, int count,
                            const RefineGeom& g, float timeWeight,
                            float neqScale, cudaStream_t st);
/// Fine-to-coarse restriction. `scratch` holds 24 floats per coarse cell of
/// the restricted sub-box (child-averaged fneq[19], rho, ux, uy, uz, valid).
long long restrict_scratch_floats(const RefineGeom& g);
/// Restricted sub-box of a patch (the patch minus its 2-cell coarse band).
void restrict_sub_box(const RefineGeom& g, int& rx0, int& ry0, int& rw, int& rh);
/// childDone: the scratch records are already written (fused fine collide).
cudaError_t launch_restrict_f2c(Storage s, const void* fineF,
                                const std::uint8_t* fineKind, void* coarseF,
                                const std::uint8_t* coarseKind,
                                const RefineGeom& g, float neqScaleInv,
                                float* scratch, float* rho, float* u, float* v,
                                float* w, cudaStream_t st, bool childDone = false);

// ---- on-device geometry builders (geom_kernels.cu) ----------------------------
/// An outline to rasterise: HOST xy pairs (normalised chord, Selig loop), the
/// cosine/sine of the rotation (-AoA), chord in cells and the anchor (cells).
struct FoilRaster {
    const float* xy = nullptr;
    int npts = 0;
    float cosA = 1.0f, sinA = 0.0f, chord = 0.0f, anchorX = 0.0f, anchorY = 0.0f;
};
/// Device SoA outputs of the wall-model cell list.
struct WallListOut {
    std::uint32_t *cell = nullptr, *sample = nullptr, *mask = nullptr;
    float *nX = nullptr, *nY = nullptr, *nZ = nullptr, *ys = nullptr;
};
/// Flag field into device `out`: base 0 domain faces, 1 all fluid, 2 the
/// device field `in`; then the rasterised foil (nullable), the trailing-edge
/// closure and the interface shell (width `shell`, 0 for none). A non-null
/// closedOut synchronises and receives the closure count.
cudaError_t device_build_flags(LevelDims d, int base, const std::uint8_t* in, const FoilRaster* foil, int closeGaps,
                               int shell, std::uint8_t* out, cudaStream_t st, int* closedOut);
/// Solid bounding box {x0, y0, x1, y1} (inclusive; x1 < 0 when no solid).
cudaError_t device_solid_bbox(LevelDims d, const std::uint8_t* flags, cudaStream_t st, int box[4]);
/// Cells whose flag is read and written / inlet / neither.
cudaError_t device_flag_classes(LevelDims d, const std::uint8_t* flags, cudaStream_t st, long long out[3]);
/// True for a pointer into device memory (cudaPointerGetAttributes).
bool is_device_pointer(const void* p);
/// Ordered cell lists. *count <- the list length; nothing is written when it
/// exceeds cap (size with a first call of capacity 0). All synchronise.
cudaError_t device_force_links(LevelDims d, const std::uint8_t* flags, std::uint32_t* cells, std::uint32_t* masks,
                               long long cap, long long* count, cudaStream_t st);
cudaError_t device_cells_where(LevelDims d, const std::uint8_t* flags, std::uint8_t value, bool equal,
                               std::uint32_t* cells, long long cap, long long* count, cudaStream_t st);
/// Interface cells with a fluid or outlet cell among their 18 neighbours
/// (the shell cells a stream-collide reads), ascending; as device_cells_where.
cudaError_t device_shell_pulled(LevelDims d, const std::uint8_t* flags, std::uint32_t* cells, long long cap,
                                long long* count, cudaStream_t st);
cudaError_t device_wall_list(LevelDims d, const std::uint8_t* active, const std::uint8_t* clean, int sampleCells,
                             const WallListOut& out, long long cap, long long* count, int stats[3],
                             cudaStream_t st);

} // namespace fcfd
