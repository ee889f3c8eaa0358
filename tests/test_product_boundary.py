"""The product path stands on its own: the package and its CUDA library
neither import, include nor link anything under oracle/ (the CPU
restatement and the reference builds are test infrastructure), the library
needs no shared object beyond the C/C++ runtime (the CUDA runtime is linked
statically; only the driver is loaded at run time), and a missing library
is a loud error, never a CPU fallback."""
from __future__ import annotations

import ast
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "foil_cfd_gb300"


def test_package_imports_nothing_from_the_oracle():
    offenders = []
    for py in sorted(PKG.rglob("*.py")):
        for node in ast.walk(ast.parse(py.read_text(), filename=str(py))):
            names = []
            if isinstance(node, ast.Import):
                names = [a.name for a in node.names]
            elif isinstance(node, ast.ImportFrom) and node.level == 0 and node.module:
                names = [node.module]
            offenders += [f"{py.relative_to(ROOT)}: {n}" for n in names if n.split(".")[0] in ("oracle", "tests")]
    assert not offenders, offenders


def test_native_sources_include_nothing_from_the_oracle():
    pat = re.compile(r'^\s*#\s*include\s*[<"]([^>"]+)[>"]', re.M)
    offenders = []
    for src in sorted(list(PKG.rglob("*.cu")) + list(PKG.rglob("*.cuh")) + list(PKG.rglob("*.cpp"))
                      + list(PKG.rglob("*.h")) + list((ROOT / "include").glob("*.h"))):
        for inc in pat.findall(src.read_text()):
            if "oracle" in inc or "_ref" in inc:
                offenders.append(f"{src.relative_to(ROOT)}: {inc}")
    assert not offenders, offenders


@pytest.mark.skipif(shutil.which("readelf") is None or shutil.which("nm") is None, reason="needs binutils")
def test_library_links_no_oracle_and_no_cuda_shared_object(built_lib):
    dyn = subprocess.run(["readelf", "-d", str(built_lib)], capture_output=True, text=True, check=True).stdout
    needed = re.findall(r"\(NEEDED\)\s+Shared library: \[([^\]]+)\]", dyn)
    assert needed, dyn
    allowed = re.compile(r"^(libstdc\+\+|libm|libgcc_s|libc|libdl|libpthread|librt|ld-linux[-\w]*)\.so")
    assert all(allowed.match(n) for n in needed), needed
    undef = subprocess.run(["nm", "-D", "--undefined-only", str(built_lib)], capture_output=True, text=True,
                           check=True).stdout
    assert not re.search(r"\b(oracle_|ref_)\w*", undef), undef


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from foil_cfd_gb300 import capi
    monkeypatch.setattr(capi, "_lib", None)
    monkeypatch.setattr(capi, "LIB_PATH", tmp_path / "absent" / "libfoilcfd_gb300.so")
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        capi.load()
