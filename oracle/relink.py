"""ORACLE - test infrastructure only. The reference's own solver tests, relinked
against this library through the LBMSolver shim.

FoilCFD's GPU tests (tests/m0_taylor_green.cpp, tests/m3_refine.cpp of the
reference) drive foilcfd::LBMSolver exactly as the app does. Relinking them
with foil_cfd_gb300/shim/lbm_solver_shim.cpp and libfoilcfd_gb300.so in place
of the reference's lbm_*.cu / lbm_solver.cpp shows the drop-in on the
reference's own callers. Two more of its solver tests run the same way:
tests/m1_cavity.cpp (the lid-driven cavity against Ghia et al.) and
tests/m4_finer.cpp (the nested finer level).

`stage()` runs in the build container, where the reference tree is mounted:
it copies the handful of files those tests compile from (their test
headers and the src/sim headers they include) into oracle/_ref/relink/, a
git-ignored build directory that travels with the working tree to the GPU
machine (the reference tree itself is not there). `build()` compiles and
links one program with g++ wherever it runs; `run()` executes one.
Nothing here is part of the product.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
KIT = HERE / "_ref" / "relink"
OUT = HERE / "_build"
SHIM = ROOT / "foil_cfd_gb300" / "shim" / "lbm_solver_shim.cpp"
TESTS = ("m0_taylor_green", "m3_refine", "m1_cavity", "m4_finer")
# What the tests compile from (reference-relative paths).
COMMON = ["src/sim/lbm_solver.h", "src/sim/lbm_core.cuh", "src/sim/lbm_refine.cuh", "src/sim/units.h",
          "tests/lbm_test_util.h", "tests/test_util.h"]
FILES = COMMON + [f"tests/{t}.cpp" for t in TESTS]


def staged(test: str | None = None) -> bool:
    """The shared headers and one test's source (default: every test's)."""
    tests = (test,) if test else TESTS
    return all((KIT / f).exists() for f in COMMON + [f"tests/{t}.cpp" for t in tests])


def stage(reference: Path) -> Path:
    """Copy the tests' sources from the reference tree into the build kit."""
    for f in FILES:
        src = reference / f
        if not src.exists():
            raise RuntimeError(f"reference file missing: {src}")
        dst = KIT / f
        dst.parent.mkdir(parents=True, exist_ok=True)
        if not dst.exists() or dst.read_bytes() != src.read_bytes():
            shutil.copyfile(src, dst)
    return KIT


def _cuda() -> Path:
    env = os.environ.get("CUDA_HOME")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    return Path(nvcc).resolve().parent.parent if nvcc else Path("/usr/local/cuda")


def build(test: str) -> Path:
    """Compile and link one relinked reference test; returns the program."""
    if not staged(test):
        raise RuntimeError("reference test sources not staged (oracle/relink.py stage, build container)")
    from foil_cfd_gb300 import build_lib
    lib = build_lib.build()
    cuda = _cuda()
    lib64 = next((p for p in (cuda / "lib64", cuda / "lib", cuda / "targets" / "sbsa-linux" / "lib") if p.exists()),
                 cuda / "lib64")
    OUT.mkdir(parents=True, exist_ok=True)
    exe = OUT / f"relinked_{test}"
    cmd = ["g++", "-std=c++20", "-O2", "-w", "-I", str(KIT / "src"), "-I", str(KIT / "src" / "sim"),
           "-I", str(KIT / "tests"), "-I", str(ROOT / "include"), "-I", str(cuda / "include"),
           str(SHIM), str(KIT / "tests" / f"{test}.cpp"),
           "-L", str(lib.parent), "-lfoilcfd_gb300", f"-Wl,-rpath,{lib.parent}",
           "-L", str(lib64), "-lcudart", f"-Wl,-rpath,{lib64}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("relink build failed:\n" + r.stderr[-4000:])
    return exe


def run(test: str, timeout: float = 600.0):
    """(exit code, output) of one relinked reference test."""
    exe = build(test)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=timeout)
    return r.returncode, r.stdout + r.stderr
