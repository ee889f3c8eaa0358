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
