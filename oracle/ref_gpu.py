"""ORACLE - measurement and test infrastructure only (tests/ and bench.py's
reference arm). Front end of ``ref_gpu_harness.cu``: the reference's own CUDA
solver-step kernels (src/sim/lbm_core.cu, lbm_refine.cu, lbm_wallmodel.cu),
compiled from the reference tree into ``oracle/_ref/*.cubin`` by ref_build.py
in the build container -- as the reference's build makes them ("asbuilt":
nvcc's default multiply-add contraction) and once more without contraction
("nofma") -- loaded and launched on this GPU through the driver API. The
harness library itself is compiled wherever it runs (nvcc, -lcuda).

The harness holds one build variant at a time; asking for the other one
unloads the modules first.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF = HERE / "_ref"
CUBIN = REF / "ref_core_sm103a.cubin"            # as the reference builds it
CUBIN_NOFMA = REF / "ref_core_sm103a_nofma.cubin"  # no contraction: exact twin
CUBIN_REFINE = REF / "ref_refine_sm103a.cubin"     # fill and restriction
CUBIN_REFINE_NOFMA = REF / "ref_refine_sm103a_nofma.cubin"
CUBIN_WALL = REF / "ref_wall_sm103a.cubin"         # wall-model update
CUBIN_WALL_NOFMA = REF / "ref_wall_sm103a_nofma.cubin"
VARIANTS = {"asbuilt": (CUBIN, CUBIN_REFINE, CUBIN_WALL),
            "nofma": (CUBIN_NOFMA, CUBIN_REFINE_NOFMA, CUBIN_WALL_NOFMA)}
SRC = HERE / "ref_gpu_harness.cu"
LIB = HERE / "_build" / "libref_gpu.so"
FLAGS = ["-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-shared"]
WATCHDOG_PERIOD = 200   # lbm_solver.cpp:25


def available(variant: str = "asbuilt", need=("core",)) -> bool:
    core, refine, wall = VARIANTS[variant]
    paths = {"core": core, "refine": refine, "wall": wall}
    return all(paths[k].exists() for k in need) and shutil.which("nvcc") is not None


def build(force: bool = False) -> Path:
    digest = hashlib.sha256(" ".join(FLAGS).encode() + SRC.read_bytes()).hexdigest()
    stamp = LIB.with_suffix(".digest")
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == digest:
        return LIB
    LIB.parent.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    r = subprocess.run(["nvcc", *FLAGS, str(SRC), "-o", str(tmp), "-lcuda"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference GPU harness build failed:\n" + r.stderr[-3000:])
    os.replace(tmp, LIB)
    stamp.write_text(digest)
    return LIB


class LevelIn(C.Structure):
    """RefLevelIn of the harness."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("flags", C.c_void_p), ("f0", C.c_void_p),
                ("wallCount", C.c_int), ("wallCell", C.c_void_p), ("wallSample", C.c_void_p),
                ("wallNx", C.c_void_p), ("wallNy", C.c_void_p), ("wallNz", C.c_void_p), ("wallYs", C.c_void_p),
                ("wallMask", C.c_void_p), ("outF", C.c_void_p), ("outUTau", C.c_void_p)]


class RunIn(C.Structure):
    """RefRunIn of the harness."""
    _fields_ = [("coarse", LevelIn), ("fine", LevelIn), ("refined", C.c_int), ("bx0", C.c_int), ("by0", C.c_int),
                ("bx1", C.c_int), ("by1", C.c_int), ("factor", C.c_int), ("tau", C.c_float), ("lam", C.c_float),
                ("cs", C.c_float), ("u_in", C.c_float), ("wm", C.c_int), ("warmup", C.c_int), ("steps", C.c_int),
                ("batch", C.c_int), ("forces", C.c_int), ("watchdog", C.c_int), ("wallReps", C.c_int)]


class RunOut(C.Structure):
    """RefRunOut of the harness."""
    _fields_ = [("ms", C.c_double), ("trip_step", C.c_longlong), ("trip_flag", C.c_int), ("checks", C.c_int),
                ("force", C.c_float * 3), ("steps_run", C.c_longlong), ("wall_ms", C.c_double * 2),
                ("force_ms", C.c_double)]


_lib = None
_variant = None


def lib(variant: str = "asbuilt", need=("core",)):
    """The harness with the `variant` cubins in `need` loaded (one variant
    per process)."""
    global _lib, _variant
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _lib.refgpu_error.restype = C.c_char_p
        for fn in ("refgpu_load", "refgpu_load_refine", "refgpu_load_wall"):
            getattr(_lib, fn).argtypes = [C.c_char_p]
        _lib.refgpu_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_float,
                                    C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double), C.c_int]
        _lib.refgpu_run_full.argtypes = [C.POINTER(RunIn), C.POINTER(RunOut)]
    if _variant is not None and _variant != variant:
        _lib.refgpu_unload()
    core, refine, wall = VARIANTS[variant]
    for kind, path, fn in (("core", core, "refgpu_load"), ("refine", refine, "refgpu_load_refine"),
                           ("wall", wall, "refgpu_load_wall")):
        if kind not in need:
            continue
        if not path.exists():
            raise RuntimeError(f"reference cubin missing ({path}); build it with oracle/ref_build.py")
        if getattr(_lib, fn)(str(path).encode()) != 0:
            raise RuntimeError(_lib.refgpu_error().decode())
    _variant = variant
    return _lib


def _variant_of(cubin) -> str:
    return "nofma" if Path(cubin) == CUBIN_NOFMA else "asbuilt"


def run(dims, flags, f0, tau, u_in, cs=0.1733, lam=3.0 / 16.0, warmup=0, steps=1, batch=100, cubin=CUBIN,
        both_buffers=False):
    """Reference steps (stream-collide + ghost refresh) from the unpadded FP32
    state f0 (with both_buffers, the other A/B buffer starts equal to f0
    instead of zero); returns (final state, timed ms)."""
    f = np.ascontiguousarray(f0, np.float32).copy()
    fl = np.ascontiguousarray(flags, np.uint8)
    ms = C.c_double(0.0)
    L = lib(_variant_of(cubin))
    rc = L.refgpu_run(*dims, fl.ctypes.data_as(C.c_void_p), f.ctypes.data_as(C.c_void_p), tau, lam, cs, u_in,
                      warmup, steps, batch, C.byref(ms), int(both_buffers))
    if rc != 0:
        raise RuntimeError(L.refgpu_error().decode())
    return f, ms.value


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _level(dims, flags, f0, wall, keep, out_f, out_utau):
    fl = np.ascontiguousarray(flags, np.uint8)
    keep.append(fl)
    lv = LevelIn(*dims, _p(fl), None, 0)
    if f0 is not None:
        a = np.ascontiguousarray(f0, np.float32)
        keep.append(a)
        lv.f0 = _p(a)
    if wall is not None and len(wall["cell"]) > 0:
        arrs = dict(cell=np.ascontiguousarray(wall["cell"], np.int64),
                    sample=np.ascontiguousarray(wall["sample"], np.int64),
                    nx=np.ascontiguousarray(wall["nx"], np.float32), ny=np.ascontiguousarray(wall["ny"], np.float32),
                    nz=np.ascontiguousarray(wall["nz"], np.float32), ys=np.ascontiguousarray(wall["ys"], np.float32),
                    mask=np.ascontiguousarray(wall["mask"], np.uint32))
        keep.extend(arrs.values())
        lv.wallCount = len(arrs["cell"])
        lv.wallCell, lv.wallSample = _p(arrs["cell"]), _p(arrs["sample"])
        lv.wallNx, lv.wallNy, lv.wallNz = _p(arrs["nx"]), _p(arrs["ny"]), _p(arrs["nz"])
        lv.wallYs, lv.wallMask = _p(arrs["ys"]), _p(arrs["mask"])
    lv.outF, lv.outUTau = _p(out_f), _p(out_utau)
    return lv


def run_full(dims, flags, tau, u_in, cs=0.1, lam=3.0 / 16.0, f0=None, wall=None, fine=None, wm=True,
             warmup=0, steps=100, batch=100, forces=True, watchdog=True, variant="asbuilt", states=False,
             wall_reps=0):
    """The reference's stepN (lbm_solver.cpp:1132-1390) in calls of `batch`
    steps: collide + ghost refresh, with `fine` = dict(dims, flags, box,
    factor, f0, wall) the 2:1 patch's fills, fine collides and restriction;
    the watchdog every 200 steps, the force reduction and the wall-model
    updates (levels with a `wall` list) once per call. f0 (unpadded FP32 SoA)
    seeds both A/B buffers of a level; None starts from feq(1, u_in)
    everywhere. Returns a dict with the timed ms, the watchdog's first trip
    (step and verdict), the last force and, with `states`, the final
    populations and u_tau of each level; with `wall_reps` > 0, after the
    timed steps, the mean ms of that many back-to-back wall-model updates
    per level on the state they left (wall_ms: coarse, fine) and, with
    `forces`, of as many force reductions (force_ms)."""
    keep = []
    n = int(np.prod(dims))
    outs = {}
    if states:
        outs["f"] = np.empty(19 * n, np.float32)
        outs["utau"] = np.empty(len(wall["cell"]), np.float32) if wall is not None else None
    rin = RunIn()
    rin.coarse = _level(dims, flags, f0, wall, keep, outs.get("f"), outs.get("utau"))
    need = ["core"]
    if fine is not None:
        nf = int(np.prod(fine["dims"]))
        fw = fine.get("wall")
        if states:
            outs["fine_f"] = np.empty(19 * nf, np.float32)
            outs["fine_utau"] = np.empty(len(fw["cell"]), np.float32) if fw is not None else None
        rin.fine = _level(fine["dims"], fine["flags"], fine.get("f0"), fw, keep, outs.get("fine_f"),
                          outs.get("fine_utau"))
        b = fine["box"]
        rin.refined, rin.bx0, rin.by0, rin.bx1, rin.by1, rin.factor = 1, b.x0, b.y0, b.x1, b.y1, fine["factor"]
        need.append("refine")
        if fw is not None:
            need.append("wall")
    if wall is not None and "wall" not in need:
        need.append("wall")
    rin.tau, rin.lam, rin.cs, rin.u_in = tau, lam, cs, u_in
    rin.wm, rin.warmup, rin.steps, rin.batch = int(wm), warmup, steps, batch
    rin.forces, rin.watchdog, rin.wallReps = int(forces), int(watchdog), int(wall_reps)
    out = RunOut()
    L = lib(variant, tuple(need))
    if L.refgpu_run_full(C.byref(rin), C.byref(out)) != 0:
        raise RuntimeError(L.refgpu_error().decode())
    res = dict(ms=out.ms, trip_step=int(out.trip_step), trip_flag=int(out.trip_flag), checks=int(out.checks),
               force=tuple(out.force), steps=int(out.steps_run), wall_ms=tuple(out.wall_ms),
               force_ms=float(out.force_ms))
    res.update(outs)
    return res


def run_refined(cdims, cflags, fdims, fflags, box, factor, tau, u_in, cs=0.1, lam=3.0 / 16.0, wall_model=True,
                warmup=10, steps=100, batch=50, refine_cubin=None, states=False, walls=None):
    """The reference's refined step from the uniform start feq(1, u_in):
    coarse collide, m fine sub-steps with fills, restriction, ghost
    refreshes; with `walls` = (coarse list, fine list) also its wall-model
    updates, force reduction and watchdog. Returns the timed ms, and with
    `states` also the final coarse and fine populations (unpadded SoA)."""
    variant = "nofma" if refine_cubin == CUBIN_REFINE_NOFMA else "asbuilt"
    wc, wf = walls if walls is not None else (None, None)
    r = run_full(cdims, cflags, tau, u_in, cs=cs, lam=lam, wall=wc,
                 fine=dict(dims=fdims, flags=fflags, box=box, factor=factor, wall=wf), wm=wall_model,
                 warmup=warmup, steps=steps, batch=batch, forces=walls is not None, watchdog=walls is not None,
                 variant=variant, states=states)
    return (r["ms"], r["f"], r["fine_f"]) if states else r["ms"]
