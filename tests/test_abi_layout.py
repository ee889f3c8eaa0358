"""The C ABI as the headers in include/ declare it, against the ctypes table
in foil_cfd_gb300/capi.py that every Python caller (tests, bench, the batch
and wall-seed wrappers) binds through.

A ctypes prototype that disagrees with its C declaration does not fail at
load time: a missing argument or a 4-byte integer where the library reads 8
bytes passes garbage silently, and a struct field out of place shifts every
field after it. So this file checks, with the host compiler and no GPU:

* every header compiles on its own as C11 and as C++17 (what a reference-side
  caller includes);
* each struct the ctypes table mirrors has the C struct's size and each
  field the C field's offset (gcc prints sizeof/offsetof);
* each declared function has the ctypes prototype's arity, and each argument
  and the return value the same class and width (pointer, integer of N
  bytes, float, double, struct by value of the same type, void)."""
from __future__ import annotations

import ctypes as C
import re
import shutil
import subprocess
import tempfile
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
INCLUDE = ROOT / "include"
HEADERS = sorted(INCLUDE.glob("*.h"))

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None, reason="needs the host C compiler")


def _capi():
    from foil_cfd_gb300 import capi
    return capi


def _struct_map(capi):
    """ctypes mirror -> C typedef name."""
    return {capi.Dims: "fcfd_dims", capi.Scaling: "fcfd_scaling", capi.Options: "fcfd_options",
            capi.Lattice: "fcfd_lattice", capi.PatchBox: "fcfd_patch_box", capi.SnapshotKey: "fcfd_snapshot_key",
            capi.Foil: "fcfd_foil", capi.ForceReadout: "fcfd_force_readout", capi.WMReadout: "fcfd_wm_readout",
            capi.Perf: "fcfd_perf", capi.RefineInfo: "fcfd_refine_info", capi.FinerInfo: "fcfd_finer_info",
            capi.WallNetNorm: "fcfd_wallnet_norm", capi.TrainOpts: "fcfd_wallnet_train_opts",
            capi.UtauStats: "fcfd_utau_stats", capi.BatchTunnel: "fcfd_batch_tunnel",
            capi.BatchConfig: "fcfd_batch_config"}


def _compile_and_run(src: str, lang: str = "c") -> str:
    with tempfile.TemporaryDirectory() as d:
        cfile = Path(d) / ("probe.c" if lang == "c" else "probe.cpp")
        exe = Path(d) / "probe"
        cfile.write_text(src)
        cc = ["gcc", "-std=c11"] if lang == "c" else ["g++", "-std=c++17"]
        r = subprocess.run(cc + ["-Wall", "-Werror", "-I", str(INCLUDE), str(cfile), "-o", str(exe)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        return subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout


@pytest.mark.parametrize("lang", ["c", "c++"])
@pytest.mark.parametrize("header", [h.name for h in HEADERS])
def test_header_is_self_contained(header, lang):
    if lang == "c++" and shutil.which("g++") is None:
        pytest.skip("no g++")
    out = _compile_and_run(f'#include "{header}"\n#include <stdio.h>\nint main(void) {{ puts("ok"); return 0; }}\n',
                           "c" if lang == "c" else "cpp")
    assert out.strip() == "ok"


def test_struct_sizes_and_offsets_match_ctypes():
    capi = _capi()
    smap = _struct_map(capi)
    lines = ["#include <stdio.h>", "#include <stddef.h>"] + [f'#include "{h.name}"' for h in HEADERS]
    lines.append("int main(void) {")
    for cls, cname in smap.items():
        lines.append(f'    printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'    printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    got = dict(line.split() for line in _compile_and_run("\n".join(lines) + "\n").splitlines())
    bad = []
    for cls, cname in smap.items():
        if int(got[cname]) != C.sizeof(cls):
            bad.append(f"sizeof {cname}: C {got[cname]} vs ctypes {C.sizeof(cls)}")
        for fname, _ in cls._fields_:
            off = getattr(cls, fname).offset
            if int(got[f"{cname}.{fname}"]) != off:
                bad.append(f"{cname}.{fname}: C offset {got[cname + '.' + fname]} vs ctypes {off}")
    assert not bad, bad


# --- prototypes ----------------------------------------------------------

_C_SCALARS = {"int": ("int", 4), "unsigned": ("int", 4), "unsigned int": ("int", 4), "long long": ("int", 8),
              "unsigned long long": ("int", 8), "size_t": ("int", 8), "int64_t": ("int", 8),
              "uint64_t": ("int", 8), "int32_t": ("int", 4), "uint32_t": ("int", 4), "float": ("float", 4),
              "double": ("float", 8), "void": ("void", 0)}


def _classify_c(decl: str, struct_names: set[str]):
    """(class, detail) of one C parameter or return type (name stripped)."""
    t = re.sub(r"\b(const|volatile|restrict|struct)\b", " ", decl)
    if "*" in t or "[" in t:
        base = " ".join(t.replace("*", " ").replace("[", " ").replace("]", " ").split())
        return ("ptr", (base, t.count("*") + t.count("[")))
    words = t.split()
    for n in (3, 2, 1):     # longest type spelling first ("unsigned long long", "long long", "int")
        if len(words) >= n and " ".join(words[:n]) in _C_SCALARS:
            return _C_SCALARS[" ".join(words[:n])]
    if words and words[0] in struct_names:
        return ("struct", words[0])
    raise AssertionError(f"unclassified C type: {decl!r}")


def _strip_param_name(p: str) -> str:
    p = p.strip()
    if p in ("", "void"):
        return p
    # "const float* f" -> "const float*"; "int n" -> "int"; "double out[3]" -> "double *"
    p = re.sub(r"\[[^\]]*\]$", "", p).strip() + (" *" if p.endswith("]") else "")
    m = re.match(r"^(.*?[\s\*])([A-Za-z_]\w*)(\s*\*?)$", p)
    if m and m.group(2) not in _C_SCALARS and not m.group(2).startswith("fcfd_"):
        return (m.group(1) + m.group(3)).strip()
    return p


def _classify_ctypes(t, smap):
    if t is None:
        return ("void", 0)
    if t in (C.c_void_p, C.c_char_p) or (isinstance(t, type) and issubclass(t, C._Pointer)):
        return ("ptr", t)
    if isinstance(t, type) and issubclass(t, C.Structure):
        return ("struct", smap.get(t))
    if t in (C.c_float,):
        return ("float", 4)
    if t in (C.c_double,):
        return ("float", 8)
    return ("int", C.sizeof(t))


def _declarations():
    src = "\n".join(f'#include "{h.name}"' for h in HEADERS) + "\n"
    r = subprocess.run(["gcc", "-E", "-P", "-I", str(INCLUDE), "-x", "c", "-"], input=src,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # System-header statements declare no fcfd_ function, so they never match.
    decls = {}
    for stmt in " ".join(r.stdout.split()).split(";"):
        stmt = stmt.strip()
        stmt = stmt[stmt.rfind("}") + 1:].strip() if "}" in stmt else stmt
        if stmt.startswith("typedef") or "{" in stmt:
            continue
        m = re.match(r"^(.*?)\b(fcfd_\w+)\s*\((.*)\)$", stmt)
        if m:
            decls[m.group(2)] = (m.group(1).strip(), [p for p in m.group(3).split(",")])
    return decls


def test_prototypes_match_the_ctypes_table():
    capi = _capi()
    smap = _struct_map(capi)
    struct_names = set(smap.values()) | {"fcfd_solver", "fcfd_batch", "fcfd_wallnet", "fcfd_vram_snapshot",
                                         "fcfd_compact_snapshot", "fcfd_disk_cache"}
    decls = _declarations()
    assert set(decls) == set(capi._SIGS), (sorted(set(decls) ^ set(capi._SIGS)))
    bad = []
    for name, (ret_c, params_c) in decls.items():
        res_t, args_t = capi._SIGS[name]
        params = [_strip_param_name(p) for p in params_c]
        if params in ([""], ["void"]):
            params = []
        if len(params) != len(args_t):
            bad.append(f"{name}: {len(params)} C parameters vs {len(args_t)} ctypes")
            continue
        pairs = [("return", ret_c, res_t)] + [(f"arg {i}", p, a) for i, (p, a) in enumerate(zip(params, args_t))]
        for where, ctype, pytype in pairs:
            kc, dc = _classify_c(ctype, struct_names)
            kp, dp = _classify_ctypes(pytype, smap)
            if kc != kp:
                bad.append(f"{name} {where}: C {ctype!r} vs ctypes {pytype}")
            elif kc in ("int", "float") and dc != dp:
                bad.append(f"{name} {where}: C {ctype!r} is {dc} bytes, ctypes {pytype} {dp}")
            elif kc == "struct" and dc != dp:
                bad.append(f"{name} {where}: C struct {dc} vs ctypes {pytype}")
            elif kc == "ptr" and isinstance(dp, type) and issubclass(dp, C._Pointer):
                pointee = dp._type_
                base, stars = dc
                if stars > 1:       # pointer to a pointer: the pointee must be one
                    ok = pointee in (C.c_void_p, C.c_char_p) or issubclass(pointee, C._Pointer)
                elif issubclass(pointee, C.Structure):
                    ok = smap.get(pointee) == base
                else:
                    ok = C.sizeof(pointee) == _C_SCALARS.get(base, ("", -1))[1]
                if not ok:
                    bad.append(f"{name} {where}: C {ctype!r} vs ctypes pointer to {pointee}")
            elif kc == "ptr" and dp is C.c_char_p and dc != ("char", 1):
                bad.append(f"{name} {where}: C {ctype!r} vs ctypes c_char_p")
    assert not bad, "\n".join(bad)
