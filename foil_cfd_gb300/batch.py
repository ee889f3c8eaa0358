"""Batched multi-tunnel step (include/foilcfd_batch.h) and the angle-of-attack
polar built on it: NACA 4-digit sections (camber 0/2/4 % at 40 % chord, 12 %
thick) at -4..16 deg in 2.5 deg steps, first 24 (camber, angle) pairs, chord
resolution drawn uniformly from 96-192 cells, domain 2.5 x 1.5 chords, span
16 cells periodic, equilibrium outflow, Reynolds number 1000 on the chord.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import capi
from .solver import STORE, SolverError, boundary_flags, layout_anchor, naca4, voxelize_airfoil

Q = 19
FLAG_OUTLET, FLAG_OUTLET_EQ = 3, 9


@dataclass
class PolarTunnel:
    digits: str
    aoa: float
    chord: int
    dims: tuple
    flags: np.ndarray
    tau: float
    u_lat: float

    @property
    def cells(self) -> int:
        return int(np.prod(self.dims))


def polar_tunnels(count: int = 24, seed: int = 0, span: int = 16, u_lat: float = 0.08, chord_range=(96, 192),
                  cambers=(0, 2, 4), aoas=None, reynolds: float = 1000.0, outlet_eq: bool = True,
                  device: bool = False):
    """The polar's tunnels in (camber, angle) order; chord cells seeded.
    Reynolds number on the chord (tau = 1/2 + 3 u c / Re). With `device`
    the flag fields are built by the device geometry kernels (uint8 CUDA
    tensors, the same bytes) instead of the host builders."""
    if device:
        from . import geometry
    aoas = [-4.0 + 2.5 * k for k in range(9)] if aoas is None else list(aoas)
    pairs = [(m, a) for m in cambers for a in aoas][:count]
    rng = np.random.default_rng(seed)
    chords = rng.integers(chord_range[0], chord_range[1] + 1, len(pairs))
    out = []
    for (m, aoa), c in zip(pairs, chords):
        c = int(c)
        digits = f"{m}{4 if m else 0}12"
        dims = (int(round(2.5 * c)), int(round(1.5 * c)), span)
        if device:
            placed = geometry.foil(naca4(digits, 200), aoa, c, *layout_anchor(dims))
            flags = geometry.build_flags(dims, "boundary", placed, True, 0, count_closed=False)[0]
            if outlet_eq:   # voxels and closures never touch the outlet column
                flags.masked_fill_(flags == FLAG_OUTLET, FLAG_OUTLET_EQ)
        else:
            flags = boundary_flags(dims)
            if outlet_eq:
                flags[flags == FLAG_OUTLET] = FLAG_OUTLET_EQ
            voxelize_airfoil(dims, flags, naca4(digits, 200), aoa, c, *layout_anchor(dims))
        tau = float(np.float32(0.5 + 3.0 * u_lat * c / reynolds))
        out.append(PolarTunnel(digits, aoa, c, dims, flags, tau, u_lat))
    return out


class BatchSolver:
    """All tunnels of a polar in one device arena, stepped by one launch."""

    def __init__(self):
        self._lib = capi.load()
        self._h = self._lib.fcfd_batch_create()
        self.tunnels = []

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fcfd_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def init(self, tunnels, storage: str = "fp16", les_cs: float = 0.1, magic_lambda: float = 0.0,
             force_every: int = 100, stream=None):
        self.tunnels = list(tunnels)
        # Host bytes, or uint8 CUDA tensors (device-built flags).
        self._flags = [t.flags if getattr(t.flags, "is_cuda", False) else np.ascontiguousarray(t.flags, np.uint8)
                       for t in self.tunnels]
        arr = (capi.BatchTunnel * len(self.tunnels))()
        for i, (t, f) in enumerate(zip(self.tunnels, self._flags)):
            fp = C.c_void_p(f.data_ptr()) if getattr(f, "is_cuda", False) else f.ctypes.data_as(C.c_void_p)
            arr[i] = capi.BatchTunnel(capi.Dims(*t.dims), fp, t.tau, t.u_lat, t.chord)
        err = C.create_string_buffer(512)
        rc = self._lib.fcfd_batch_init(self._h, arr, len(self.tunnels), STORE[storage],
                                       les_cs if les_cs > 0 else -1.0, magic_lambda, force_every, stream, err, 512)
        if rc:
            raise SolverError(err.value.decode() or f"batch init failed ({rc})")
        self.force_every = force_every

    def reset(self):
        self._check(self._lib.fcfd_batch_reset(self._h), "reset")

    @staticmethod
    def _check(rc, what):
        if rc:
            raise SolverError(f"batch {what} failed ({rc})")

    def set_config(self, block: int, rows: int, ctas_per_sm: int, group_mb: int = 0):
        c = capi.BatchConfig(block, rows, ctas_per_sm, group_mb)
        self._check(self._lib.fcfd_batch_set_config(self._h, C.byref(c)), "set_config")

    def config(self):
        c = capi.BatchConfig()
        self._lib.fcfd_batch_get_config(self._h, C.byref(c))
        return (c.block, c.rows, c.ctas_per_sm, c.group_mb)

    def autotune(self, trial_steps: int = 10):
        """Returns (chosen (block, rows, ctas_per_sm, group_mb), ms/step,
        [(config, ms/step), ...])."""
        chosen = capi.BatchConfig()
        ms = C.c_float()
        cap = 128
        cands = (capi.BatchConfig * cap)()
        each = (C.c_float * cap)()
        n = C.c_int()
        self._check(self._lib.fcfd_batch_autotune(self._h, trial_steps, C.byref(chosen), C.byref(ms), cands, each,
                                                  cap, C.byref(n)), "autotune")
        table = [((cands[i].block, cands[i].rows, cands[i].ctas_per_sm, cands[i].group_mb), each[i])
                 for i in range(n.value)]
        return (chosen.block, chosen.rows, chosen.ctas_per_sm, chosen.group_mb), ms.value, table

    def step_n(self, n: int, use_graphs: bool = True) -> int:
        return self._lib.fcfd_batch_step_n(self._h, n, int(use_graphs))

    def synchronize(self):
        return self._lib.fcfd_batch_synchronize(self._h)

    def step_count(self) -> int:
        return self._lib.fcfd_batch_step_count(self._h)

    def updates_per_step(self) -> int:
        return self._lib.fcfd_batch_updates_per_step(self._h)

    def kernel_launches(self) -> int:
        return self._lib.fcfd_batch_kernel_launches(self._h)

    def last_ms(self) -> float:
        ms = C.c_double()
        self._lib.fcfd_batch_last_ms(self._h, C.byref(ms))
        return ms.value

    def force_history(self, max_samples: int = 4096) -> np.ndarray:
        """(samples, tunnels, 3) FP64 force samples, oldest first."""
        nt = len(self.tunnels)
        out = np.zeros((max_samples, nt, 3), np.float64)
        w = C.c_int()
        self._check(self._lib.fcfd_batch_force_history(self._h, capi.ptr(out), max_samples, C.byref(w)), "history")
        return out[:w.value]

    def forces_now(self) -> np.ndarray:
        out = np.zeros((len(self.tunnels), 3), np.float64)
        self._check(self._lib.fcfd_batch_forces_now(self._h, capi.ptr(out)), "forces")
        return out

    def health(self):
        """(max speed per tunnel, non-finite cells per tunnel)."""
        nt = len(self.tunnels)
        sp = np.zeros(nt, np.float32)
        bad = np.zeros(nt, np.int32)
        self._check(self._lib.fcfd_batch_health(self._h, capi.ptr(sp), capi.ptr(bad)), "health")
        return sp, bad

    def latched(self, with_steps: bool = False):
        """Watchdog verdict per tunnel: 0 running, 1 non-finite cell, 2 speed
        at the limiter (the tunnel stopped stepping when it was latched);
        with_steps also the steps each tunnel has taken since the reset."""
        v = np.zeros(len(self.tunnels), np.int32)
        st = np.zeros(len(self.tunnels), np.int64)
        self._check(self._lib.fcfd_batch_latched(self._h, capi.ptr(v), capi.ptr(st)), "latch read-back")
        return (v, st) if with_steps else v

    def export_f32(self, i: int) -> np.ndarray:
        f = np.empty(Q * int(np.prod(self.tunnels[i].dims)), np.float32)
        self._check(self._lib.fcfd_batch_export_f32(self._h, i, capi.ptr(f), f.size), "export")
        return f

    def import_f32(self, i: int, f):
        f = np.ascontiguousarray(f, np.float32)
        self._check(self._lib.fcfd_batch_import_f32(self._h, i, capi.ptr(f), f.size), "import")

    def coefficients(self, last_fraction: float = 0.5):
        """Time-averaged (Cl, Cd) per tunnel over the last fraction of the
        force samples: C = F / (1/2 u^2 chord span)."""
        h = self.force_history()
        if len(h) == 0:
            return np.zeros(0), np.zeros(0)
        k = max(1, int(round(len(h) * last_fraction)))
        avg = h[-k:].mean(0)
        q = np.array([0.5 * t.u_lat ** 2 * t.chord * t.dims[2] for t in self.tunnels])
        return avg[:, 1] / q, avg[:, 0] / q
