"""ORACLE - test infrastructure only. Recipe that compiles the reference's
own solver-step kernels for the CPU into ``oracle/_ref/`` (git-ignored).

For each of src/sim/lbm_core.cu, lbm_wallmodel.cu and lbm_refine.cu the
kernel section (everything up to the close of the file's anonymous
namespace, i.e. all kernels and device helpers, without the ``<<<>>>``
launch wrappers) is read from the reference tree where it lies and streamed
through a pipe into g++, preceded by ``ref_shim.h`` / ``ref_launch.h`` (CUDA
built-in stand-ins, fiber-emulated blocks) and followed by a driver of ours
(``ref_driver_*.inc``) that exposes extern "C" entry points. No reference
text is written to disk. Contraction is off (-ffp-contract=off) so the CPU
build evaluates the reference expressions exactly as written.

Used only in this container, to pin the C++ restatement (lbm_oracle.cpp)
and to generate the golden fixtures under tests/golden/.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
# The reference checkout this recipe reads: FOILCFD_REFERENCE, else the
# build container's read-only mount.
REFERENCE = Path(os.environ.get("FOILCFD_REFERENCE") or "/root/reference")
SIM = REFERENCE / "src" / "sim"
UNITS = {
    "core": ("lbm_core.cu", "ref_driver_core.inc"),
    "wall": ("lbm_wallmodel.cu", "ref_driver_wall.inc"),
    "refine": ("lbm_refine.cu", "ref_driver_refine.inc"),
}
FLAGS = ["-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-w"]


def available() -> bool:
    """True when the reference tree with the sources is present."""
    return (all((SIM / src).exists() for src, _ in UNITS.values()) and (SIM / "wall_model.cpp").exists()
            and (REFERENCE / "src" / "geom" / "voxelizer.cpp").exists() and (SIM / "snapshot.cpp").exists())


def _kernel_section(path: Path) -> str:
    lines = path.read_text().splitlines(keepends=True)
    for i, line in enumerate(lines):
        if line.rstrip() == "} // namespace":
            return "".join(lines[: i + 1])
    raise RuntimeError(f"no anonymous-namespace close found in {path}")


def _cuda_include() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and Path(c, "include", "cuda_runtime_api.h").exists():
            return str(Path(c, "include"))
    raise RuntimeError("CUDA headers not found")


def build(force: bool = False) -> dict:
    """Build the three reference CPU libraries; returns {unit: path}."""
    if not available():
        raise RuntimeError(f"reference sources not found under {REFERENCE} (set FOILCFD_REFERENCE)")
    OUT.mkdir(parents=True, exist_ok=True)
    libs = {}
    for unit, (src, drv) in UNITS.items():
        so = OUT / f"libref_{unit}.so"
        libs[unit] = so
        if so.exists() and not force:
            continue
        text = _kernel_section(SIM / src) + "\n" + (HERE / drv).read_text()
        cmd = ["g++", *FLAGS, "-include", str(HERE / "ref_shim.h"), "-include", str(HERE / "ref_launch.h"),
               "-I", str(SIM), "-I", _cuda_include(), "-x", "c++", "-", "-o", str(so)]
        r = subprocess.run(cmd, input=text, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference CPU build of {src} failed:\n{r.stderr[-4000:]}")
    # The host wall-cell list builder is plain C++: compiled unmodified.
    so = OUT / "libref_walllist.so"
    libs["walllist"] = so
    if force or not so.exists():
        cmd = ["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
               str(SIM / "wall_model.cpp"), str(HERE / "ref_walllist_driver.cpp"),
               "-I", str(SIM), "-I", _cuda_include(), "-o", str(so)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference wall_model.cpp build failed:\n{r.stderr[-4000:]}")
    # The host geometry builders (NACA outline, voxeliser, patch flags) are
    # plain C++ too; vg.cpp and platform.cpp only resolve their symbols.
    so = OUT / "libref_geom.so"
    libs["geom"] = so
    if force or not so.exists():
        geom = REFERENCE / "src" / "geom"
        cmd = ["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w",
               str(geom / "voxelizer.cpp"), str(geom / "airfoil.cpp"), str(geom / "vg.cpp"),
               str(REFERENCE / "src" / "platform" / "platform.cpp"), str(HERE / "ref_geom_driver.cpp"),
               "-I", str(geom), "-I", str(SIM), "-I", _cuda_include(), "-o", str(so)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference geometry build failed:\n{r.stderr[-4000:]}")
    # The reference's CUDA stream-collide as an sm_103a cubin (device code
    # only, loaded through the driver API by ref_gpu_harness.cu), built as
    # the reference builds it (C++20, default contraction).
    # A second one without contraction is the exact-parity twin of the CPU
    # build (the check that the harness passes the parameters right).
    for key, src, name, extra in (("cubin", "lbm_core.cu", "ref_core_sm103a.cubin", []),
                                  ("cubin_nofma", "lbm_core.cu", "ref_core_sm103a_nofma.cubin", ["--fmad=false"]),
                                  ("cubin_refine", "lbm_refine.cu", "ref_refine_sm103a.cubin", []),
                                  ("cubin_refine_nofma", "lbm_refine.cu", "ref_refine_sm103a_nofma.cubin",
                                   ["--fmad=false"]),
                                  ("cubin_wall", "lbm_wallmodel.cu", "ref_wall_sm103a.cubin", []),
                                  ("cubin_wall_nofma", "lbm_wallmodel.cu", "ref_wall_sm103a_nofma.cubin",
                                   ["--fmad=false"])):
        cubin = OUT / name
        libs[key] = cubin
        if (force or not cubin.exists()) and shutil.which("nvcc"):
            cmd = ["nvcc", "-cubin", "-std=c++20", "-O3", *extra, "-gencode", "arch=compute_103a,code=sm_103a",
                   "-I", str(SIM), str(SIM / src), "-o", str(cubin)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"reference cubin build failed:\n{r.stderr[-4000:]}")
    # The snapshot code (keys, flag hash, FCS1 reader/writer); the solver
    # methods it names are stubbed by the driver.
    so = OUT / "libref_snapshot.so"
    libs["snapshot"] = so
    if force or not so.exists():
        cuda = Path(_cuda_include()).parent
        lib64 = next((str(p) for p in (cuda / "lib64", cuda / "lib") if p.exists()), str(cuda / "lib64"))
        cmd = ["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w", "-pthread",
               str(SIM / "snapshot.cpp"), str(REFERENCE / "src" / "platform" / "platform.cpp"),
               str(HERE / "ref_snapshot_driver.cpp"), "-I", str(SIM), "-I", _cuda_include(),
               "-L", lib64, "-lcudart", "-Wl,-rpath," + lib64, "-o", str(so)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference snapshot build failed:\n{r.stderr[-4000:]}")
    # The reference's own solver tests, staged for relinking against this
    # library through the LBMSolver shim (oracle/relink.py).
    from oracle import ref_geom, relink
    libs["relink"] = relink.stage(REFERENCE)
    # The host geometry builders, staged the same way for the benchmark's
    # reference arm on the GPU machine (oracle/ref_geom.py).
    libs["geomkit"] = ref_geom.stage(REFERENCE)
    return libs


if __name__ == "__main__":
    for k, v in build(force="--force" in sys.argv).items():
        print(k, v)
