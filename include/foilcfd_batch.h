/*
 * foilcfd_batch.h - C ABI of the batched multi-tunnel solver step.
 *
 * An angle-of-attack polar is a set of independent, unevenly sized tunnels
 * (2.5-D: a few spanwise cells, periodic in z). Stepping each with its own
 * solver leaves most of the GPU idle and pays launch latency per tunnel; a
 * batch owns all of them in one device arena and advances every tunnel by
 * one step with ONE kernel launch: a grid-stride walk over work items (row
 * groups of each tunnel in x chunks) that is persistent across tunnels when
 * the grid is a few blocks per SM. Chunks of steps, with a per-tunnel
 * momentum-exchange force sample at their end, are captured once as CUDA
 * graphs and replayed. A project-written autotuner times the launch shapes
 * (threads per block, rows per work item, persistent vs one-item grids) on
 * the batch itself and keeps the fastest.
 *
 * Per tunnel the physics is the single-tunnel step's (fcfd_step_n of
 * foilcfd_step.h) without wall model and refinement patch: TRT + Smagorinsky,
 * half-way bounce-back, free-slip, inlet feq(1, u), zero-gradient or
 * equilibrium outflow; uniform-flow start (no ramps). Each tunnel produces
 * the same populations, bit for bit, as a single-tunnel solver with the same
 * storage, flags and parameters. The reference steps one tunnel per solver
 * (src/sim/lbm_solver.cpp:1132-1390); there is no batched counterpart.
 *
 * Return convention: 0 or a cudaError_t value. Not thread-safe.
 */
#ifndef FOILCFD_BATCH_H
#define FOILCFD_BATCH_H

#include <stddef.h>
#include <stdint.h>

#include "foilcfd_step.h"

#ifdef __cplusplus
extern "C" {
#endif

#define FCFD_BATCH_MAX_TUNNELS 64

typedef struct fcfd_batch fcfd_batch;

/* One tunnel: dims, flags (nx*ny*nz CellFlag bytes, copied; host memory or
 * device memory, e.g. built by fcfd_device_build_flags), lattice relaxation
 * time, inlet speed, and the chord in cells (force coefficients). */
typedef struct fcfd_batch_tunnel {
    fcfd_dims dims;
    const uint8_t* flags;
    float tau;
    float u_lat;
    int chord_cells;
} fcfd_batch_tunnel;

/* Launch shape of the batched collide. block: 64, 128 or 256 threads (one x
 * cell each); rows: 1, 2 or 4 rows per work item; ctas_per_sm: blocks per SM
 * of a persistent grid, 0 for one block per work item. group_mb: 0 steps all
 * tunnels with one launch per step; > 0 packs consecutive tunnels into groups
 * of at most that many MB of population buffers, and a graph-replayed chunk
 * then runs all its steps group after group (tunnels are independent), so a
 * group small enough for the L2 cache streams from it instead of HBM. */
typedef struct fcfd_batch_config {
    int block;
    int rows;
    int ctas_per_sm;
    int group_mb;
} fcfd_batch_config;

fcfd_batch* fcfd_batch_create(void);
void fcfd_batch_destroy(fcfd_batch* b);

/* Allocate and initialise `count` tunnels (<= FCFD_BATCH_MAX_TUNNELS) with
 * storage FCFD_STORE_FP32 / FCFD_STORE_FP16, Smagorinsky constant les_cs
 * (<= 0 disables LES) and TRT magic parameter (0: 3/16); uniform-flow
 * state as fcfd_reset. force_every: steps between force samples (even,
 * >= 2; also the length of a captured graph chunk). */
int fcfd_batch_init(fcfd_batch* b, const fcfd_batch_tunnel* tunnels, int count, int storage, float les_cs,
                    float magic_lambda, int force_every, void* stream, char* err, size_t errlen);
/* Uniform-flow start (feq(1, u) + the reference's speck), step count 0,
 * force history cleared. */
int fcfd_batch_reset(fcfd_batch* b);

int fcfd_batch_set_config(fcfd_batch* b, const fcfd_batch_config* cfg);
int fcfd_batch_get_config(const fcfd_batch* b, fcfd_batch_config* cfg);
/* Two stages: time every launch shape with all tunnels in one launch for
 * trial_steps direct steps; then, with the fastest shape, time one
 * graph-replayed chunk per grouping (group_mb 0, 48, 96, 192). The steps
 * advance the tunnels like any others. Keeps the fastest; its ms per step ->
 * *ms (nullable). candidates (nullable, capacity max_candidates) receives
 * every timed configuration and *n_candidates their number, with ms per step
 * in ms_each. */
int fcfd_batch_autotune(fcfd_batch* b, int trial_steps, fcfd_batch_config* chosen, float* ms,
                        fcfd_batch_config* candidates, float* ms_each, int max_candidates, int* n_candidates);

/* n steps of every tunnel: whole graph chunks replayed when `use_graphs`
 * (steps aligned to force_every), the rest launched directly. */
int fcfd_batch_step_n(fcfd_batch* b, int n, int use_graphs);
int fcfd_batch_synchronize(fcfd_batch* b);
long long fcfd_batch_step_count(const fcfd_batch* b);
/* Lattice updates per step (sum of the tunnels' cells). */
long long fcfd_batch_updates_per_step(const fcfd_batch* b);
long long fcfd_batch_kernel_launches(const fcfd_batch* b);

/* Force samples taken so far (one per force_every steps) and the last
 * `max_samples` of them (oldest first), 3 doubles (Fx, Fy, Fz) per tunnel
 * per sample. */
int fcfd_batch_force_samples(fcfd_batch* b, int* total);
int fcfd_batch_force_history(fcfd_batch* b, double* out, int max_samples, int* written);
/* Momentum-exchange force of every tunnel now (3 doubles per tunnel). */
int fcfd_batch_forces_now(fcfd_batch* b, double* out);

/* Health of every tunnel at the current state: largest speed |u| over the
 * non-solid cells (max_speed, count floats) and the number of cells with a
 * non-finite density or momentum (non_finite, count ints). */
int fcfd_batch_health(fcfd_batch* b, float* max_speed, int* non_finite);
/* Per-tunnel watchdog (the batch counterpart of the solver's NaN watchdog,
 * lbm_core.cu:508-559): after every force sample (each force_every steps)
 * the same full-field scan latches each tunnel that reached 0.95 x the 0.3
 * limiter speed (verdict 2) or holds a non-finite cell (verdict 1); a
 * latched tunnel stops stepping (its work items are skipped, its state
 * freezes; its force samples repeat the frozen state) until
 * fcfd_batch_reset. verdicts: count ints, 0 for a tunnel still running;
 * steps_run (count long longs, may be NULL): the steps a tunnel has taken
 * since the reset (up to its latch). Synchronises the batch stream. */
int fcfd_batch_latched(fcfd_batch* b, int* verdicts, long long* steps_run);

/* FP32 SoA populations of one tunnel (19 * cells floats). */
int fcfd_batch_export_f32(fcfd_batch* b, int tunnel, float* f, size_t n);
int fcfd_batch_import_f32(fcfd_batch* b, int tunnel, const float* f, size_t n);

/* CUDA-event time of the last fcfd_batch_step_n (ms). */
int fcfd_batch_last_ms(const fcfd_batch* b, double* ms);

#ifdef __cplusplus
}
#endif

#endif /* FOILCFD_BATCH_H */
