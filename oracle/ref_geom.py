"""ORACLE - test infrastructure only. The reference's own host geometry
builders (src/geom/voxelizer.cpp, airfoil.cpp), wall-cell list builder
(src/sim/wall_model.cpp) and lattice scaling (src/sim/units.h), for the
benchmark's reference arm: it builds its tunnels and wall lists with the
reference's code, not with this library.

`stage()` runs in the build container, where the reference tree is
mounted: it copies the handful of files these builders compile from into
oracle/_ref/geomkit/ (git-ignored; it travels with the working tree to the
GPU machine, where the reference tree is absent). `build()` compiles them,
with ref_geom_driver.cpp and ref_walllist_driver.cpp, into a shared library
for the machine it runs on (g++, no other dependency). The builders produce
the same bytes as this library's (tests/test_ref_geom_kit.py).
"""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from collections import namedtuple
from pathlib import Path
from types import SimpleNamespace

import numpy as np

HERE = Path(__file__).resolve().parent
KIT = HERE / "_ref" / "geomkit"
OUT = HERE / "_build"
SO = OUT / "libref_geomkit.so"
FILES = ["src/geom/voxelizer.cpp", "src/geom/voxelizer.h", "src/geom/airfoil.cpp", "src/geom/airfoil.h",
         "src/geom/vg.cpp", "src/geom/vg.h", "src/platform/platform.cpp", "src/platform/platform.h",
         "src/sim/wall_model.cpp", "src/sim/wall_model.h", "src/sim/lbm_core.cuh", "src/sim/lbm_refine.cuh",
         "src/sim/units.h", "src/core/vec.h"]
_lib = None
PatchBox = namedtuple("PatchBox", "x0 y0 x1 y1")


def staged() -> bool:
    return all((KIT / f).exists() for f in FILES)


def stage(reference: Path) -> Path:
    """Copy the builders' sources from the reference tree into the kit."""
    for f in FILES:
        src = Path(reference) / f
        if not src.exists():
            raise RuntimeError(f"reference file missing: {src}")
        dst = KIT / f
        dst.parent.mkdir(parents=True, exist_ok=True)
        if not dst.exists() or dst.read_bytes() != src.read_bytes():
            shutil.copyfile(src, dst)
    return KIT


def _cuda_include() -> str:
    nvcc = shutil.which("nvcc")
    root = Path(nvcc).resolve().parent.parent if nvcc else Path("/usr/local/cuda")
    return str(root / "include")


def build() -> Path:
    """The kit's shared library for this machine (rebuilt when missing)."""
    if not staged():
        raise RuntimeError("reference geometry sources not staged (oracle/ref_build.py, build container)")
    if SO.exists():
        return SO
    OUT.mkdir(parents=True, exist_ok=True)
    cmd = ["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w", "-pthread",
           *[str(KIT / f) for f in ("src/geom/voxelizer.cpp", "src/geom/airfoil.cpp", "src/geom/vg.cpp",
                                    "src/platform/platform.cpp", "src/sim/wall_model.cpp")],
           str(HERE / "ref_geom_driver.cpp"), str(HERE / "ref_walllist_driver.cpp"),
           "-I", str(KIT / "src" / "geom"), "-I", str(KIT / "src" / "sim"), "-I", _cuda_include(),
           "-o", str(SO)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference geometry kit build failed:\n" + r.stderr[-4000:])
    return SO


def available() -> bool:
    try:
        build()
        return True
    except (RuntimeError, OSError):
        return False


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(str(build()))
        P = C.c_void_p
        L.ref_naca4.argtypes = [C.c_char_p, C.c_int, P, C.c_int]
        L.ref_clean_foil_flags.argtypes = [C.c_char_p, C.c_int, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int,
                                           C.c_float, C.c_float, P]
        L.ref_fine_patch_flags.argtypes = [C.c_char_p, C.c_int, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int,
                                           C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, P]
        L.ref_derive_patch_box.argtypes = [C.c_int, C.c_int, C.c_int, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                           P]
        L.ref_derive_patch_box.restype = None
        L.ref_compute_scaling.argtypes = [C.c_float, C.c_float, C.c_float, C.c_int, C.c_float, P, P]
        L.ref_compute_scaling.restype = None
        L.ref_build_wall_list.argtypes = [C.c_int, C.c_int, C.c_int, P, P, C.c_int, P, P, P, P, P, P, P,
                                          C.c_longlong, P]
        L.ref_build_wall_list.restype = C.c_longlong
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def scaling(chord_m: float, airspeed_ms: float, nu_m2s: float, chord_cells: int, u_lat: float):
    """computeScaling (units.h): (tau, u_lat)."""
    tau, u = np.zeros(1, np.float32), np.zeros(1, np.float32)
    lib().ref_compute_scaling(chord_m, airspeed_ms, nu_m2s, chord_cells, u_lat, _p(tau), _p(u))
    return float(tau[0]), float(u[0])


def wall_list(dims, active, clean=None, sample_cells: int = 2) -> dict:
    """buildWallCellList (wall_model.cpp) as SoA arrays."""
    nx, ny, nz = dims
    active = np.ascontiguousarray(active, np.uint8)
    clean = active if clean is None else np.ascontiguousarray(clean, np.uint8)
    cap = int(np.count_nonzero(active == 0)) + 1
    out = dict(cell=np.zeros(cap, np.int64), sample=np.zeros(cap, np.int64), nx=np.zeros(cap, np.float32),
               ny=np.zeros(cap, np.float32), nz=np.zeros(cap, np.float32), ys=np.zeros(cap, np.float32),
               mask=np.zeros(cap, np.uint32))
    stats = np.zeros(3, np.int32)
    m = lib().ref_build_wall_list(nx, ny, nz, _p(active), _p(clean), sample_cells, _p(out["cell"]),
                                  _p(out["sample"]), _p(out["nx"]), _p(out["ny"]), _p(out["nz"]), _p(out["ys"]),
                                  _p(out["mask"]), cap, _p(stats))
    if m < 0:
        raise RuntimeError("wall list capacity exceeded")
    return {k: v[:m].copy() for k, v in out.items()}


def airfoil_tunnel(nx=640, ny=192, nz=192, chord=256, aoa=6.0, digits="0012", margin_chord=0.1, factor=2,
                   u_lat=0.08, patch=True, anchor=(0.3, 0.5)):
    """The benchmark's airfoil tunnel from the reference's builders:
    buildCleanFoilFlags at the anchor fractions, derivePatchBox with a
    margin of `margin_chord` chords and clearance 3, the box widened to a
    multiple of 4 coarse cells (the benchmark's patch, as this library's
    tunnel builder widens it) and buildFinePatchFlags."""
    L = lib()
    dims = (nx, ny, nz)
    flags = np.zeros(nx * ny * nz, np.uint8)
    if L.ref_clean_foil_flags(digits.encode(), 200, aoa, nx, ny, nz, chord, anchor[0], anchor[1], _p(flags)) < 0:
        raise RuntimeError(f"bad NACA digits {digits!r}")
    t = SimpleNamespace(name=f"naca{digits}_{aoa:g}deg_{nx}x{ny}x{nz}", dims=dims, flags=flags, chord_cells=chord,
                        u_lat=u_lat, factor=factor, box=None, fine_dims=None, fine_flags=None)
    if patch:
        m = int(round(margin_chord * chord))
        b = np.zeros(4, np.int32)
        L.ref_derive_patch_box(nx, ny, nz, _p(flags), m, m, m, m, 3, _p(b))
        x0, y0, x1, y1 = (int(v) for v in b)
        extra = (-(x1 - x0)) % 4
        grow = min(extra, nx - 3 - x1)
        x0, x1 = x0 - (extra - grow), x1 + grow
        t.box = PatchBox(x0, y0, x1, y1)
        t.fine_dims = (factor * (x1 - x0), factor * (y1 - y0), factor * nz)
        t.fine_flags = np.zeros(int(np.prod(t.fine_dims)), np.uint8)
        L.ref_fine_patch_flags(digits.encode(), 200, aoa, nx, ny, nz, chord, anchor[0], anchor[1], x0, y0, x1, y1,
                               factor, _p(t.fine_flags))
    cells = float(np.prod(dims)) + (factor * float(np.prod(t.fine_dims)) if patch else 0.0)
    t.updates_per_step = lambda: cells
    return t
