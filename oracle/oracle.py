"""ORACLE - test infrastructure only (tests/, smoke() and bench.py's
cpu_baseline leg). numpy/ctypes front end of the C++ restatement in
``lbm_oracle.cpp`` plus the host cadence of the reference solver
(src/sim/lbm_solver.cpp:1132-1390, stepN): per step one collide, then m fine
sub-steps of fill + collide and one restriction when a patch is active; one
force reduction and one wall-model update per batch.

The product never imports this module; it only checks the product.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
SRC = HERE / "lbm_oracle.cpp"
FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]

Q = 19
CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1])
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


def build(force: bool = False) -> Path:
    """Compile the oracle library (g++, OpenMP, no FMA contraction)."""
    digest = hashlib.sha256((" ".join(FLAGS)).encode() + SRC.read_bytes()).hexdigest()
    stamp = BUILD / "digest.txt"
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == digest:
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    tmp = BUILD / "liboracle.so.tmp"
    r = subprocess.run(["g++", *FLAGS, str(SRC), "-o", str(tmp)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr)
    os.replace(tmp, LIB)
    stamp.write_text(digest)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        P = C.c_void_p
        i, f, d = C.c_int, C.c_float, C.c_double
        _lib.oracle_collide_f32.argtypes = [i, i, i, P, P, P, f, f, f, f, i, P, P, P, P, P, P, P, P, P]
        _lib.oracle_collide_f64.argtypes = [i, i, i, P, P, P, d, d, d, d, i, P, P, P, P, P, P, P, P, P]
        _lib.oracle_force_f32.argtypes = [i, i, i, P, P, P, P, P, P]
        _lib.oracle_force_f64.argtypes = [i, i, i, P, P, P, P, P, P]
        _lib.oracle_init_eq.argtypes = [i, i, i, P, P, f]
        _lib.oracle_speck.argtypes = [i, i, i, P, P, f, C.c_uint]
        _lib.oracle_wall_update.argtypes = [i, i, i, P, i, P, P, P, P, P, P, P, P, P, P, P, f, f, f, P]
        _lib.oracle_utau_newton_f64.argtypes = [i, P, P, P, d, i, P]
        _lib.oracle_apply_flag_edits.argtypes = [i, i, i, P, P, P, P]
        _lib.oracle_f2h.argtypes = [f]
        _lib.oracle_f2h.restype = C.c_uint16
        _lib.oracle_h2f.argtypes = [C.c_uint16]
        _lib.oracle_h2f.restype = f
        _lib.oracle_fill_c2f.argtypes = [i, i, i, P, P, P, i, i, i, P, P, i, i, i, f, f, i]
        _lib.oracle_restrict_f2c.argtypes = [i, i, i, P, P, i, i, i, P, P, i, i, i, i, i, f, P, P, P, P]
        _lib.oracle_tunnel_create.argtypes = [i, i, i, P, P, f, f, f, f]
        _lib.oracle_tunnel_create.restype = P
        _lib.oracle_tunnel_destroy.argtypes = [P]
        _lib.oracle_tunnel_refine.argtypes = [P, i, i, i, i, i, P]
        _lib.oracle_tunnel_wall.argtypes = [P, i, i, P, P, P, P, P, P, P]
        _lib.oracle_tunnel_step.argtypes = [P, i]
        _lib.oracle_tunnel_state.argtypes = [P, i, P]
        _lib.oracle_tunnel_force.argtypes = [P, P]
        _lib.oracle_threads.restype = i
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def smag_prefactor(cs: float) -> float:
    """18 sqrt(2) Cs^2 in FP32, as the reference launch wrapper forms it."""
    if cs <= 0:
        return 0.0
    return float(np.float32(18.0) * np.float32(1.41421356) * np.float32(cs) * np.float32(cs))


def collide(dims, src, flags, tau, lam, smag_pre, u_in, write_macro=False, slip=None, dst=None, qlinks=None):
    """One reference stream-collide over the whole grid; returns (dst, macro).
    ``qlinks`` = (qFrac uint8 [cell * 19 + q], ffMask uint32 [cell]) turns on
    the interpolated bounce-back (q-LIBB) on solid links.

    ``dst`` is the other buffer of an A/B pair and is written in place; the
    cells a step does not write (solid, slip, interface) keep its previous
    contents, exactly as in the solver's ping-pong buffers. Without ``dst`` a
    copy of ``src`` stands in for it."""
    nx, ny, nz = dims
    n = nx * ny * nz
    dtype = src.dtype
    if dst is None:
        dst = src.copy()
    macro = [np.zeros(n, dtype) for _ in range(4)] if write_macro else [None] * 4
    sx = [None] * 3 if slip is None else [np.ascontiguousarray(s) for s in slip]
    fn = lib().oracle_collide_f32 if dtype == np.float32 else lib().oracle_collide_f64
    ql = (None, None) if qlinks is None else (np.ascontiguousarray(qlinks[0], np.uint8),
                                               np.ascontiguousarray(qlinks[1], np.uint32))
    fn(nx, ny, nz, _p(src), _p(dst), _p(flags), tau, lam, smag_pre, u_in, int(write_macro),
       *[_p(m) for m in macro], *[_p(s) for s in sx], _p(ql[0]), _p(ql[1]))
    return dst, (macro if write_macro else None)


def force(dims, f, flags, slip=None):
    out = np.zeros(3, np.float64)
    sx = [None] * 3 if slip is None else [np.ascontiguousarray(s) for s in slip]
    fn = lib().oracle_force_f32 if f.dtype == np.float32 else lib().oracle_force_f64
    fn(*dims, _p(f), _p(flags), *[_p(s) for s in sx], _p(out))
    return out


def init_equilibrium(dims, flags, u_in):
    n = int(np.prod(dims))
    f = np.empty(Q * n, np.float32)
    lib().oracle_init_eq(*dims, _p(f), _p(flags), u_in)
    return f


def speck(dims, f, flags, amp, seed=0x5EED):
    lib().oracle_speck(*dims, _p(f), _p(flags), amp, seed)
    return f


def reset_state(dims, flags, u_lat):
    """LBMSolver::reset with the ramps off (lbm_solver.cpp:893-944):
    equilibrium at (1, u_lat) -- solids at rest -- plus the speck of
    amplitude 1e-3 u_lat, seed 0x5eed."""
    f = init_equilibrium(dims, flags, np.float32(u_lat))
    return speck(dims, f, flags, np.float32(1e-3) * np.float32(u_lat))


def f2h(x: float) -> int:
    return int(lib().oracle_f2h(x))


def h2f(h: int) -> float:
    return float(lib().oracle_h2f(h))


def apply_flag_edits(dims, fA, fB, flags, mask):
    """Warm-restart flag-edit fixup of both buffers (in place)."""
    lib().oracle_apply_flag_edits(*dims, _p(fA), _p(fB), _p(np.ascontiguousarray(flags, np.uint8)),
                                  _p(np.ascontiguousarray(mask, np.uint8)))
    return fA, fB


def utau_newton_f64(ut, ys, nu, tol=1e-8, max_iter=100):
    ut = np.ascontiguousarray(ut, np.float64)
    ys = np.ascontiguousarray(np.broadcast_to(ys, ut.shape), np.float64)
    nu = np.ascontiguousarray(np.broadcast_to(nu, ut.shape), np.float64)
    out = np.zeros_like(ut)
    lib().oracle_utau_newton_f64(ut.size, _p(ut), _p(ys), _p(nu), tol, max_iter, _p(out))
    return out


class WallList:
    """Host wall-cell list (SoA) as the reference builds it."""

    def __init__(self, cell, sample, nx, ny, nz, ys, mask):
        self.cell = np.ascontiguousarray(cell, np.int64)
        self.sample = np.ascontiguousarray(sample, np.int64)
        self.nx = np.ascontiguousarray(nx, np.float32)
        self.ny = np.ascontiguousarray(ny, np.float32)
        self.nz = np.ascontiguousarray(nz, np.float32)
        self.ys = np.ascontiguousarray(ys, np.float32)
        self.mask = np.ascontiguousarray(mask, np.uint32)
        self.utau = np.zeros(len(self.cell), np.float32)

    def __len__(self):
        return len(self.cell)


def wall_update(dims, f, wl: WallList, slip, nu, ut_cut, ema=0.25):
    """One reference wall-model update; mutates wl.utau and the slip arrays."""
    stats = np.zeros(4, np.float32)
    lib().oracle_wall_update(*dims, _p(f), len(wl), _p(wl.cell), _p(wl.sample), _p(wl.nx), _p(wl.ny),
                             _p(wl.nz), _p(wl.ys), _p(wl.mask), _p(wl.utau), _p(slip[0]), _p(slip[1]),
                             _p(slip[2]), nu, ut_cut, ema, _p(stats))
    return stats


def fill_c2f(cdims, cT0, cT1, cflags, fdims, ff, fflags, box, factor, tw, neq_scale, full_volume):
    lib().oracle_fill_c2f(*cdims, _p(cT0), _p(cT1), _p(cflags), *fdims, _p(ff), _p(fflags), box[0], box[1],
                          factor, tw, neq_scale, int(full_volume))


def restrict_f2c(fdims, ff, fflags, cdims, fc, cflags, box, factor, neq_inv, macro=None):
    m = [None] * 4 if macro is None else macro
    lib().oracle_restrict_f2c(*fdims, _p(ff), _p(fflags), *cdims, _p(fc), _p(cflags), box[0], box[1], box[2],
                              box[3], factor, neq_inv, *[_p(x) for x in m])


def moments(f, n):
    """rho, u, v, w of an FP32/FP64 SoA population array (host reduction)."""
    f = f.reshape(Q, n).astype(np.float64)
    rho = f.sum(0)
    inv = np.where(rho > 1e-12, 1.0 / np.where(rho > 1e-12, rho, 1.0), 0.0)
    return rho, (CX @ f) * inv, (CY @ f) * inv, (CZ @ f) * inv


def equilibrium(rho, ux, uy, uz, dtype=np.float32):
    """Second-order D3Q19 equilibrium of per-cell fields, SoA [19*n]."""
    rho = np.asarray(rho, np.float64)
    ux, uy, uz = (np.asarray(a, np.float64) for a in (ux, uy, uz))
    usq = 1.5 * (ux * ux + uy * uy + uz * uz)
    out = []
    for q in range(Q):
        cu = 3.0 * (CX[q] * ux + CY[q] * uy + CZ[q] * uz)
        out.append(W[q] * rho * (1.0 + cu + 0.5 * cu * cu - usq))
    return np.concatenate(out).astype(dtype)


class OracleSolver:
    """Reference stepN cadence over the oracle kernels (coarse level, optional
    2:1 patch, force per batch, wall model per batch). Ramps are off: the
    caller uploads a state (the test harness path of the reference)."""

    def __init__(self, dims, flags, tau, u_lat, cs=0.1733, lam=3.0 / 16.0, dtype=np.float32):
        self.dims = tuple(dims)
        self.n = int(np.prod(dims))
        self.flags = np.ascontiguousarray(flags, np.uint8)
        self.tau, self.u_lat, self.lam = tau, u_lat, lam
        self.smag = smag_prefactor(cs)
        self.dtype = dtype
        # Both A/B buffers start from the solver's reset state (ramps off):
        # equilibrium at u_lat plus the spanwise speck.
        self.f = reset_state(self.dims, self.flags, u_lat).astype(dtype)
        self.g = self.f.copy()
        self.macro = None
        self.fine = None
        self.finer = None
        self.wall = None
        self.slip = None
        self.last_force = np.zeros(3)
        self.steps = 0

    def set_state(self, f):
        """Import into the current buffer only (the solver's import path)."""
        self.f = np.ascontiguousarray(f, self.dtype).copy()

    def enable_wall_model(self, wl: WallList):
        self.wall = wl
        self.slip = [np.zeros(self.n, np.uint16) for _ in range(3)]

    def enable_refinement(self, box, factor, fine_flags):
        fd = (factor * (box[2] - box[0]), factor * (box[3] - box[1]), factor * self.dims[2])
        self.fine = dict(dims=fd, box=tuple(box), m=factor, flags=np.ascontiguousarray(fine_flags, np.uint8),
                         f=np.zeros(Q * int(np.prod(fd)), np.float32))
        tc = self.tau
        tf = factor * (tc - 0.5) + 0.5
        fine = self.fine
        fill_c2f(self.dims, self.f, self.f, self.flags, fd, fine["f"], fine["flags"], box, factor, 0.0,
                 np.float32(tf) / (np.float32(factor) * np.float32(tc)), True)
        fine["g"] = fine["f"].copy()

    def enable_finer_refinement(self, box, factor, finer_flags):
        """Nested patch inside the fine level (box in fine cells), seeded from
        the fine field (lbm_solver.cpp:1916-2000, 523-545)."""
        fine = self.fine
        fd0 = fine["dims"]
        rd = (factor * (box[2] - box[0]), factor * (box[3] - box[1]), factor * fd0[2])
        self.finer = dict(dims=rd, box=tuple(box), m=factor, flags=np.ascontiguousarray(finer_flags, np.uint8),
                          f=np.zeros(Q * int(np.prod(rd)), np.float32))
        tf = np.float32(fine["m"]) * (np.float32(self.tau) - np.float32(0.5)) + np.float32(0.5)
        tr = np.float32(factor) * (tf - np.float32(0.5)) + np.float32(0.5)
        fill_c2f(fd0, fine["f"], fine["f"], fine["flags"], rd, self.finer["f"], self.finer["flags"], box, factor,
                 0.0, tr / (np.float32(factor) * tf), True)
        self.finer["g"] = self.finer["f"].copy()

    def _finer_substeps(self, tf, fine_t1):
        """m2 finer sub-steps between the fine pair's time levels, then the
        finer -> fine restriction into fine_t1 (lbm_solver.cpp:1209-1270)."""
        fr, fine = self.finer, self.fine
        rd, m2, box = fr["dims"], fr["m"], fr["box"]
        tr = np.float32(m2) * (tf - np.float32(0.5)) + np.float32(0.5)
        for q in range(m2):
            fill_c2f(fine["dims"], fine["f"], fine_t1, fine["flags"], rd, fr["f"], fr["flags"], box, m2,
                     np.float32(q) / np.float32(m2), tr / (np.float32(m2) * tf), False)
            nr, _ = collide(rd, fr["f"], fr["flags"], tr, self.lam, self.smag, self.u_lat, False, None, dst=fr["g"])
            fr["g"], fr["f"] = fr["f"], nr
        restrict_f2c(rd, fr["f"], fr["flags"], fine["dims"], fine_t1, fine["flags"], box, m2,
                     (np.float32(m2) * tf) / tr, None)

    def step_n(self, n):
        tau = np.float32(self.tau)
        for i in range(n):
            wm = i == n - 1
            dst, macro = collide(self.dims, self.f, self.flags, tau, self.lam, self.smag, self.u_lat, wm,
                                 self.slip, dst=self.g)
            if self.fine is not None:
                fd, m, box = self.fine["dims"], self.fine["m"], self.fine["box"]
                tf = np.float32(m) * (tau - np.float32(0.5)) + np.float32(0.5)
                for k in range(m):
                    fill_c2f(self.dims, self.f, dst, self.flags, fd, self.fine["f"], self.fine["flags"], box, m,
                             np.float32(k) / np.float32(m), tf / (np.float32(m) * tau), False)
                    nf, _ = collide(fd, self.fine["f"], self.fine["flags"], tf, self.lam, self.smag,
                                    self.u_lat, False, None, dst=self.fine["g"])
                    if self.finer is not None:
                        self._finer_substeps(tf, nf)
                    self.fine["g"], self.fine["f"] = self.fine["f"], nf
                restrict_f2c(fd, self.fine["f"], self.fine["flags"], self.dims, dst, self.flags, box, m,
                             (np.float32(m) * tau) / tf, macro)
            self.g, self.f = self.f, dst
            if macro is not None:
                self.macro = macro
            self.steps += 1
        self.last_force = force(self.dims, self.f, self.flags, self.slip)
        if self.wall is not None:
            nu = (np.float32(self.tau) - np.float32(0.5)) / np.float32(3.0)
            wall_update(self.dims, self.f, self.wall, self.slip, nu, np.float32(1e-3) * np.float32(self.u_lat))
        return self.last_force


class OracleTunnel:
    """C++ ping-pong driver of a whole tunnel (reference stepN cadence); the
    timed CPU baseline. No per-step Python or array copies."""

    def __init__(self, dims, flags, f0, tau, u, cs=0.1733, lam=3.0 / 16.0):
        self.dims = tuple(dims)
        self.n = int(np.prod(dims))
        self._flags = np.ascontiguousarray(flags, np.uint8)
        f0 = np.ascontiguousarray(f0, np.float32)
        self._h = lib().oracle_tunnel_create(*self.dims, _p(self._flags), _p(f0), tau, u, smag_prefactor(cs), lam)
        self.fine_n = 0

    def refine(self, box, factor, fine_flags):
        ff = np.ascontiguousarray(fine_flags, np.uint8)
        lib().oracle_tunnel_refine(self._h, box[0], box[1], box[2], box[3], factor, _p(ff))
        self.fine_n = ff.size

    def wall(self, level, wl):
        a = {k: np.ascontiguousarray(wl[k]) for k in ("cell", "sample", "nx", "ny", "nz", "ys", "mask")}
        lib().oracle_tunnel_wall(self._h, level, len(a["cell"]), *[_p(a[k]) for k in
                                 ("cell", "sample", "nx", "ny", "nz", "ys", "mask")])

    def step_n(self, n):
        lib().oracle_tunnel_step(self._h, n)

    def state(self, level=0):
        out = np.empty(Q * (self.n if level == 0 else self.fine_n), np.float32)
        lib().oracle_tunnel_state(self._h, level, _p(out))
        return out

    def force(self):
        out = np.zeros(3)
        lib().oracle_tunnel_force(self._h, _p(out))
        return out

    def close(self):
        if self._h:
            lib().oracle_tunnel_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def threads() -> int:
    return int(lib().oracle_threads())
