"""Warm-start snapshots (include/foilcfd_snapshot.h): cache keys, the
device-resident exact snapshot, the host macroscopic snapshot with its FCS1
file format, and the LRU disk cache (src/sim/snapshot.h of the reference)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .solver import SolverError

SOLVER_VERSION = 1


def aoa_bucket(aoa_deg: float) -> int:
    """AoA quantised to 0.5-degree buckets: lround(aoa * 2)."""
    return capi.load().fcfd_aoa_bucket(aoa_deg)


class SnapshotKey:
    """Identity of a cached flow state (geometry id, AoA bucket, u_lat,
    dims, solver version); equal keys may share a snapshot."""

    def __init__(self, geometry_id: str, aoa_bucket: int, u_lat: float, dims, solver_version: int = SOLVER_VERSION):
        self.geometry_id = geometry_id
        self.aoa_bucket = int(aoa_bucket)
        self.u_lat = float(np.float32(u_lat))
        self.dims = tuple(int(v) for v in dims)
        self.solver_version = int(solver_version)

    def c(self) -> capi.SnapshotKey:
        self._id = self.geometry_id.encode()
        return capi.SnapshotKey(self._id, self.aoa_bucket, self.u_lat, capi.Dims(*self.dims), self.solver_version)

    @classmethod
    def from_c(cls, k: capi.SnapshotKey) -> "SnapshotKey":
        return cls(k.geometry_id.decode(), k.aoa_bucket, k.u_lat, (k.dims.nx, k.dims.ny, k.dims.nz),
                   k.solver_version)

    def hash(self) -> int:
        return capi.load().fcfd_snapshot_key_hash(C.byref(self.c()))

    def __str__(self) -> str:
        buf = C.create_string_buffer(512)
        capi.load().fcfd_snapshot_key_string(C.byref(self.c()), buf, 512)
        return buf.value.decode()

    def __eq__(self, o) -> bool:
        return isinstance(o, SnapshotKey) and (self.geometry_id, self.aoa_bucket, self.u_lat, self.dims,
                                               self.solver_version) == (o.geometry_id, o.aoa_bucket, o.u_lat,
                                                                        o.dims, o.solver_version)


def hash_flags(flags) -> int:
    f = np.ascontiguousarray(flags, np.uint8)
    return capi.load().fcfd_hash_flags(capi.ptr(f), f.size)


class VramSnapshot:
    """Exact device copy of every active level's current populations."""

    def __init__(self):
        self._lib = capi.load()
        self._h = self._lib.fcfd_vram_snapshot_create()

    def capture(self, solver, key: SnapshotKey):
        err = C.create_string_buffer(256)
        rc = self._lib.fcfd_vram_snapshot_capture(self._h, solver._h, C.byref(key.c()), err, 256)
        if rc:
            raise SolverError(err.value.decode() or f"VRAM capture failed ({rc})")

    def restore(self, solver) -> bool:
        return self._lib.fcfd_vram_snapshot_restore(self._h, solver._h) == 0

    @property
    def has_data(self) -> bool:
        return bool(self._lib.fcfd_vram_snapshot_has_data(self._h))

    @property
    def flags_hash(self) -> int:
        return self._lib.fcfd_vram_snapshot_flags_hash(self._h)

    @property
    def nbytes(self) -> int:
        return self._lib.fcfd_vram_snapshot_bytes(self._h)

    def key(self) -> SnapshotKey:
        k = capi.SnapshotKey()
        if self._lib.fcfd_vram_snapshot_key(self._h, C.byref(k)):
            raise SolverError("empty snapshot")
        return SnapshotKey.from_c(k)

    def release(self):
        self._lib.fcfd_vram_snapshot_release(self._h)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fcfd_vram_snapshot_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class CompactSnapshot:
    """Coarse rho, u, v, w in host memory; FCS1 files; equilibrium restore."""

    def __init__(self, handle=None):
        self._lib = capi.load()
        self._h = handle or self._lib.fcfd_compact_snapshot_create()

    def capture(self, solver, key: SnapshotKey):
        err = C.create_string_buffer(256)
        rc = self._lib.fcfd_compact_snapshot_capture(self._h, solver._h, C.byref(key.c()), err, 256)
        if rc:
            raise SolverError(err.value.decode() or f"compact capture failed ({rc})")

    def restore(self, solver) -> bool:
        return self._lib.fcfd_compact_snapshot_restore(self._h, solver._h) == 0

    def save(self, path):
        err = C.create_string_buffer(512)
        if self._lib.fcfd_compact_snapshot_save(self._h, str(path).encode(), err, 512):
            raise SolverError(err.value.decode())

    def load(self, path):
        err = C.create_string_buffer(512)
        if self._lib.fcfd_compact_snapshot_load(self._h, str(path).encode(), err, 512):
            raise SolverError(err.value.decode())

    @property
    def has_data(self) -> bool:
        return bool(self._lib.fcfd_compact_snapshot_has_data(self._h))

    @property
    def flags_hash(self) -> int:
        return self._lib.fcfd_compact_snapshot_flags_hash(self._h)

    def key(self) -> SnapshotKey:
        k = capi.SnapshotKey()
        if self._lib.fcfd_compact_snapshot_key(self._h, C.byref(k)):
            raise SolverError("empty snapshot")
        return SnapshotKey.from_c(k)

    def scaling(self) -> capi.Scaling:
        s = capi.Scaling()
        if self._lib.fcfd_compact_snapshot_scaling(self._h, C.byref(s)):
            raise SolverError("empty snapshot")
        return s

    def fields(self):
        """(rho, u, v, w) copies as float32 arrays."""
        ptrs = [C.POINTER(C.c_float)() for _ in range(4)]
        n = C.c_size_t(0)
        if self._lib.fcfd_compact_snapshot_fields(self._h, *[C.byref(p) for p in ptrs], C.byref(n)):
            raise SolverError("empty snapshot")
        return tuple(np.ctypeslib.as_array(p, shape=(n.value,)).copy() for p in ptrs)

    def detach(self):
        """Hand the native object over (to the disk cache's writer)."""
        h, self._h = self._h, None
        return h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fcfd_compact_snapshot_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class DiskSnapshotCache:
    """Directory of .fcs files under a byte budget, LRU by file time."""

    def __init__(self, directory, budget_bytes: int = 10 << 30):
        self._lib = capi.load()
        self._h = self._lib.fcfd_disk_cache_open(str(directory).encode(), budget_bytes)
        if not self._h:
            raise SolverError(f"cannot open cache directory {directory}")

    def find(self, key: SnapshotKey):
        buf = C.create_string_buffer(4096)
        return buf.value.decode() if self._lib.fcfd_disk_cache_find(self._h, C.byref(key.c()), buf, 4096) else None

    def store(self, snap: CompactSnapshot):
        err = C.create_string_buffer(512)
        if self._lib.fcfd_disk_cache_store(self._h, snap._h, err, 512):
            raise SolverError(err.value.decode())

    def store_async(self, snap: CompactSnapshot):
        """The cache takes the snapshot over; `snap` is empty afterwards."""
        if self._lib.fcfd_disk_cache_store_async(self._h, snap.detach()):
            raise SolverError("store_async failed")

    def wait(self):
        self._lib.fcfd_disk_cache_wait(self._h)

    def set_budget(self, budget_bytes: int):
        self._lib.fcfd_disk_cache_set_budget(self._h, budget_bytes)

    @property
    def used_bytes(self) -> int:
        return self._lib.fcfd_disk_cache_used_bytes(self._h)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fcfd_disk_cache_close(self._h)
            self._h = None

    def __del__(self):
        self.close()
