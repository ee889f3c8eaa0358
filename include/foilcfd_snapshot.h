/*
 * foilcfd_snapshot.h - C ABI of the warm-start snapshots for the solver's
 * storage layouts (src/sim/snapshot.h:17-217 of the reference).
 *
 * - Cache key (SnapshotKey): geometry id, AoA in 0.5-degree buckets, lattice
 *   inflow speed, grid dims and solver version; its 64-bit FNV-1a hash names
 *   the disk-cache file ("%016llx.fcs"). The flag-field FNV-1a hash is kept
 *   with every snapshot so a restore can check the geometry it lands on.
 * - VRAM snapshot (VramSnapshot): a device-resident exact copy of the current
 *   population buffer of every active level (coarse, fine patch, nested finer
 *   patch) in the solver's own storage (FP32 or FP16 deviation, unpadded
 *   SoA), with each level's wall-model state (u_tau and the slip-velocity
 *   arrays the collide reads); capture and restore are device-to-device
 *   copies, and a run continued from a restore repeats the original bit for
 *   bit. The reference keeps the coarse buffer only; with a refinement patch
 *   or the wall model on, the rest is part of the state and is captured too.
 * - Compact snapshot (CompactSnapshot): the coarse macroscopic fields (rho,
 *   u, v, w; 16 bytes per cell) in host memory, restored by an equilibrium
 *   re-init (fcfd_restore_from_macro) and a settling transient. Its file
 *   format "FCS1" is the reference's byte for byte: little-endian fields,
 *   magic 0x31534346, format 1, key, flags hash, scaling echo, payload tag 0
 *   (raw FP32), cell count, then the four arrays.
 * - Disk cache (DiskSnapshotCache): a directory of .fcs files with a byte
 *   budget, least-recently-used eviction by file time (a hit refreshes it;
 *   the file just stored is never evicted), writes through a temporary file
 *   and a rename, and an optional background writer thread.
 *
 * Return convention: 0 on success; a cudaError_t value for CUDA failures and
 * -1 for the rest (a reason goes to err when given). Not thread-safe except
 * the disk cache, whose calls are serialised internally.
 */
#ifndef FOILCFD_SNAPSHOT_H
#define FOILCFD_SNAPSHOT_H

#include <stddef.h>
#include <stdint.h>

#include "foilcfd_step.h"

#ifdef __cplusplus
extern "C" {
#endif

/* kSolverVersion (snapshot.h:22): stamped into every key and file. */
#define FCFD_SOLVER_VERSION 1

typedef struct fcfd_snapshot_key {
    const char* geometry_id; /* "naca:2412", "dat:<file>" or "stl:<hash>" */
    int aoa_bucket;          /* fcfd_aoa_bucket(aoa_deg)                  */
    float u_lat;             /* exact match                               */
    fcfd_dims dims;
    int solver_version;      /* FCFD_SOLVER_VERSION                       */
} fcfd_snapshot_key;

/* SnapshotKey::bucketForAoA: lround(aoa_deg * 2). */
int fcfd_aoa_bucket(float aoa_deg);
/* SnapshotKey::hash (snapshot.cpp:89-100). */
uint64_t fcfd_snapshot_key_hash(const fcfd_snapshot_key* key);
/* SnapshotKey::toString, e.g. "naca-2412_a6.0_u0.0800_640x192x192_v1".
 * Returns the length written (excluding NUL), or -1. */
int fcfd_snapshot_key_string(const fcfd_snapshot_key* key, char* buf, size_t len);
/* hashFlags: FNV-1a 64 of a HOST flag field. */
uint64_t fcfd_hash_flags(const uint8_t* flags, size_t n);

/* ---- VRAM snapshot (VramSnapshot, snapshot.h:70-115) ---------------------- */
typedef struct fcfd_vram_snapshot fcfd_vram_snapshot;
fcfd_vram_snapshot* fcfd_vram_snapshot_create(void);
void fcfd_vram_snapshot_destroy(fcfd_vram_snapshot* v);
/* Device copy of the current buffers on the solver's stream; the device
 * allocation is reused while its size fits. */
int fcfd_vram_snapshot_capture(fcfd_vram_snapshot* v, fcfd_solver* s, const fcfd_snapshot_key* key, char* err,
                               size_t errlen);
/* Copy back and fcfd_notify_restored(s, 1). Fails (-1) when empty or when
 * the solver's storage, levels or dims differ from the captured ones. */
int fcfd_vram_snapshot_restore(const fcfd_vram_snapshot* v, fcfd_solver* s);
int fcfd_vram_snapshot_has_data(const fcfd_vram_snapshot* v);
uint64_t fcfd_vram_snapshot_flags_hash(const fcfd_vram_snapshot* v);
size_t fcfd_vram_snapshot_bytes(const fcfd_vram_snapshot* v);
/* The captured key; key->geometry_id points into v (valid while v lives). */
int fcfd_vram_snapshot_key(const fcfd_vram_snapshot* v, fcfd_snapshot_key* key);
void fcfd_vram_snapshot_release(fcfd_vram_snapshot* v);

/* ---- compact snapshot (CompactSnapshot, snapshot.h:126-167) --------------- */
typedef struct fcfd_compact_snapshot fcfd_compact_snapshot;
fcfd_compact_snapshot* fcfd_compact_snapshot_create(void);
void fcfd_compact_snapshot_destroy(fcfd_compact_snapshot* c);
/* Download the coarse rho, u, v, w (refreshed on each batch's last step)
 * with the key, the flags hash and the scaling. */
int fcfd_compact_snapshot_capture(fcfd_compact_snapshot* c, fcfd_solver* s, const fcfd_snapshot_key* key,
                                  char* err, size_t errlen);
/* fcfd_restore_from_macro of the held fields; -1 when empty or the grid
 * differs. */
int fcfd_compact_snapshot_restore(const fcfd_compact_snapshot* c, fcfd_solver* s);
int fcfd_compact_snapshot_save(const fcfd_compact_snapshot* c, const char* path, char* err, size_t errlen);
/* Rejects a bad magic, format, solver version, header or payload size. */
int fcfd_compact_snapshot_load(fcfd_compact_snapshot* c, const char* path, char* err, size_t errlen);
int fcfd_compact_snapshot_has_data(const fcfd_compact_snapshot* c);
uint64_t fcfd_compact_snapshot_flags_hash(const fcfd_compact_snapshot* c);
int fcfd_compact_snapshot_key(const fcfd_compact_snapshot* c, fcfd_snapshot_key* key);
int fcfd_compact_snapshot_scaling(const fcfd_compact_snapshot* c, fcfd_scaling* scaling);
/* The held arrays (host memory owned by c) and the cell count. */
int fcfd_compact_snapshot_fields(const fcfd_compact_snapshot* c, const float** rho, const float** u,
                                 const float** v, const float** w, size_t* ncells);

/* ---- disk cache (DiskSnapshotCache, snapshot.h:174-214) ------------------- */
typedef struct fcfd_disk_cache fcfd_disk_cache;
/* Create the directory if missing and size the existing .fcs entries. */
fcfd_disk_cache* fcfd_disk_cache_open(const char* directory, uint64_t budget_bytes);
/* Finishes queued background writes, then frees the cache. */
void fcfd_disk_cache_close(fcfd_disk_cache* c);
/* 1 and the file path on a hit (its time refreshed), 0 on a miss. */
int fcfd_disk_cache_find(fcfd_disk_cache* c, const fcfd_snapshot_key* key, char* path, size_t len);
int fcfd_disk_cache_store(fcfd_disk_cache* c, const fcfd_compact_snapshot* snap, char* err, size_t errlen);
/* Queue a store on the cache's writer thread; the cache takes ownership of
 * snap and destroys it after the write. */
int fcfd_disk_cache_store_async(fcfd_disk_cache* c, fcfd_compact_snapshot* snap);
/* Block until every queued background store has been written. */
void fcfd_disk_cache_wait(fcfd_disk_cache* c);
/* A smaller budget evicts at once (nothing protected). */
void fcfd_disk_cache_set_budget(fcfd_disk_cache* c, uint64_t budget_bytes);
uint64_t fcfd_disk_cache_used_bytes(fcfd_disk_cache* c);

#ifdef __cplusplus
}
#endif

#endif /* FOILCFD_SNAPSHOT_H */
