"""ORACLE - measurement and test infrastructure only (tests/ and bench.py's
reference arm). Front end of ``ref_gpu_harness.cu``: the reference's own CUDA
stream-collide (src/sim/lbm_core.cu), compiled from the reference tree into
``oracle/_ref/ref_core_sm103a.cubin`` by ref_build.py in the build container,
loaded and launched on this GPU through the driver API. The harness library
itself is compiled wherever it runs (nvcc, -lcuda).
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
CUBIN = HERE / "_ref" / "ref_core_sm103a.cubin"            # as the reference builds it
CUBIN_NOFMA = HERE / "_ref" / "ref_core_sm103a_nofma.cubin"  # no contraction: exact twin
CUBIN_REFINE = HERE / "_ref" / "ref_refine_sm103a.cubin"     # fill and restriction
CUBIN_REFINE_NOFMA = HERE / "_ref" / "ref_refine_sm103a_nofma.cubin"
SRC = HERE / "ref_gpu_harness.cu"
LIB = HERE / "_build" / "libref_gpu.so"
FLAGS = ["-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-shared"]


def available() -> bool:
    return CUBIN.exists() and shutil.which("nvcc") is not None


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


_lib = None
_loaded = None


def lib(cubin: Path = CUBIN):
    """The harness with `cubin` loaded (one module per process)."""
    global _lib, _loaded
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _lib.refgpu_error.restype = C.c_char_p
        _lib.refgpu_load.argtypes = [C.c_char_p]
        _lib.refgpu_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_float,
                                    C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
        _lib.refgpu_load_refine.argtypes = [C.c_char_p]
        i, f, P = C.c_int, C.c_float, C.c_void_p
        _lib.refgpu_run_refined.argtypes = [i, i, i, P, i, i, i, P, i, i, i, i, i, f, f, f, f, i, i, i, i,
                                            C.POINTER(C.c_double), P, P]
    if _loaded is None:
        if not cubin.exists():
            raise RuntimeError(f"reference cubin missing ({cubin}); build it with oracle/ref_build.py")
        if _lib.refgpu_load(str(cubin).encode()) != 0:
            raise RuntimeError(_lib.refgpu_error().decode())
        _loaded = cubin
    elif _loaded != cubin:
        raise RuntimeError(f"harness already holds {_loaded.name}")
    return _lib


def run(dims, flags, f0, tau, u_in, cs=0.1733, lam=3.0 / 16.0, warmup=0, steps=1, batch=100, cubin=CUBIN):
    """Reference steps (stream-collide + ghost refresh) from the unpadded FP32
    state f0; returns (final state, timed ms)."""
    f = np.ascontiguousarray(f0, np.float32).copy()
    fl = np.ascontiguousarray(flags, np.uint8)
    ms = C.c_double(0.0)
    rc = lib(cubin).refgpu_run(*dims, fl.ctypes.data_as(C.c_void_p), f.ctypes.data_as(C.c_void_p), tau, lam, cs, u_in,
                          warmup, steps, batch, C.byref(ms))
    if rc != 0:
        raise RuntimeError(lib(cubin).refgpu_error().decode())
    return f, ms.value


def run_refined(cdims, cflags, fdims, fflags, box, factor, tau, u_in, cs=0.1, lam=3.0 / 16.0, wall_model=True,
                warmup=10, steps=100, batch=50, refine_cubin=None, states=False):
    """The reference's refined step (coarse collide, m fine sub-steps with
    fills, restriction; ghost refreshes) from the uniform start feq(1, u_in)
    on every cell; returns the timed ms for `steps` coarse steps, and with
    `states` also the final coarse and fine populations (unpadded SoA)."""
    L = lib(CUBIN_NOFMA if refine_cubin == CUBIN_REFINE_NOFMA else CUBIN)
    if L.refgpu_load_refine(str(refine_cubin or CUBIN_REFINE).encode()) != 0:
        raise RuntimeError(L.refgpu_error().decode())
    cf = np.ascontiguousarray(cflags, np.uint8)
    ff = np.ascontiguousarray(fflags, np.uint8)
    oc = np.empty(19 * int(np.prod(cdims)), np.float32) if states else None
    of = np.empty(19 * int(np.prod(fdims)), np.float32) if states else None
    ms = C.c_double(0.0)
    ptr = (lambda a: None if a is None else a.ctypes.data_as(C.c_void_p))
    rc = L.refgpu_run_refined(*cdims, ptr(cf), *fdims, ptr(ff), box.x0, box.y0, box.x1, box.y1, factor, tau, lam,
                              cs, u_in, int(wall_model), warmup, steps, batch, C.byref(ms), ptr(oc), ptr(of))
    if rc != 0:
        raise RuntimeError(L.refgpu_error().decode())
    return (ms.value, oc, of) if states else ms.value
