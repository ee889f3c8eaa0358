"""Host-side logic of the solver step, no GPU: the C-ABI library loads and
exports every symbol the include/*.h headers declare; units; the host
wall-cell list builder against the reference builder's own output and the
exact expectations of the reference's tests/test_wallmodel.cpp; geometry
fixture builders (boundary flags, NACA 4-digit, voxeliser, patch shell)."""
import math
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def fc(built_lib):
    import foil_cfd_gb300 as fc
    return fc


def test_library_exports_every_declared_symbol(built_lib, fc):
    from foil_cfd_gb300 import capi
    header = "".join(h.read_text() for h in sorted((ROOT / "include").glob("*.h")))
    declared = set(re.findall(r"\b(fcfd_[a-z0-9_]+)\s*\(", header))
    assert declared, "no declarations parsed"
    out = subprocess.run(["nm", "-D", "--defined-only", str(built_lib)], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert declared <= exported, sorted(declared - exported)
    assert declared == set(capi.declared_symbols())
    lib = capi.load()
    for name in declared:
        assert getattr(lib, name) is not None
    assert b"sm_103a" in lib.fcfd_version()


def test_units_contract(fc):
    s = fc.compute_scaling(1.2, 30.0, 1.48e-5, 256, 0.08)
    assert math.isclose(s.dx, 1.2 / 256, rel_tol=1e-6)
    assert math.isclose(s.dt, 0.08 * (1.2 / 256) / 30.0, rel_tol=1e-6)
    assert s.tau_clamped == 1 and math.isclose(s.tau, 0.5005, rel_tol=1e-7)
    nu_min = (0.5005 - 0.5) / 3
    assert math.isclose(s.nu_lat, nu_min, rel_tol=1e-4)
    assert math.isclose(s.re_effective, 0.08 * 256 / nu_min, rel_tol=1e-3)
    s2 = fc.compute_scaling(1.0, 1.0, 1e-3, 128, 0.08)  # Re 1000 at 128 cells
    assert s2.tau_clamped == 0
    assert math.isclose(s2.tau, 3 * 0.08 * 128 / 1000 + 0.5, rel_tol=1e-4)
    assert math.isclose(s2.re_effective, 1000.0, rel_tol=1e-3)
    s3 = fc.compute_scaling(1.0, 1.0, 1e-3, 128, 0.5)
    assert math.isclose(s3.u_lat, 0.12, rel_tol=1e-7)
    from foil_cfd_gb300 import capi
    import ctypes as C
    lib = capi.load()
    nx = 768
    assert math.isclose(lib.fcfd_ramped_tau(C.byref(s), 0, nx), 3 * 4 * s.nu_lat + 0.5, rel_tol=1e-5)
    assert math.isclose(lib.fcfd_ramped_tau(C.byref(s), 2 * nx, nx), s.tau, rel_tol=1e-6)
    assert lib.fcfd_ramped_u(C.byref(s), 0, nx) == 0.0
    assert math.isclose(lib.fcfd_ramped_u(C.byref(s), nx, nx), s.u_lat, rel_tol=1e-7)
    qref = 0.5 * s.u_lat ** 2 * 256 * 96
    assert math.isclose(fc.force_to_coefficient(s, 1.5 * qref, 96), 1.5, rel_tol=1e-5)
    f2 = fc.refined_scaling(s, 2)
    assert math.isclose(f2.tau, 2 * (s.tau - 0.5) + 0.5, rel_tol=1e-6) and f2.chord_cells == 512


@pytest.mark.parametrize("geom", ["slab", "wedge", "sphere", "vane"])
@pytest.mark.parametrize("sample", [2, 3])
def test_wall_list_matches_reference_builder(fc, golden, geom, sample):
    import importlib.util
    spec = importlib.util.spec_from_file_location("mg", ROOT / "tests" / "golden" / "make_golden.py")
    # geometry definitions only (no reference needed)
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    d, active, clean = mg.wall_list_geometries()[geom]
    g = golden("wall_list")
    res = fc.build_wall_list(d, active, clean, sample)
    key = f"{geom}_{sample}"
    assert res["stats"]["listed"] == int(g[key + "_stats"][0])
    assert res["stats"]["excluded_vg"] == int(g[key + "_stats"][1])
    assert res["stats"]["degenerate"] == int(g[key + "_stats"][2])
    for k in ("cell", "sample", "mask"):
        assert np.array_equal(res[k], g[f"{key}_{k}"]), k
    for k in ("nx", "ny", "nz", "ys"):
        assert np.array_equal(res[k], g[f"{key}_{k}"]), k


def test_wall_list_flat_slab_expectations(fc):
    """tests/test_wallmodel.cpp:44-85 of the reference."""
    d = (32, 32, 8)
    f = np.zeros(d[::-1], np.uint8)
    f[:, :16, :] = 1
    res = fc.build_wall_list(d, f.ravel())
    assert res["stats"]["listed"] == 32 * 8
    expect = (1 << 3) | (1 << 7) | (1 << 11) | (1 << 14) | (1 << 17)
    x = res["cell"] % 32
    inner = (x >= 2) & (x < 30)
    assert np.all(res["mask"][inner] == expect)
    assert np.allclose(res["ys"][inner], 2.5)
    assert np.all(res["sample"][inner] == res["cell"][inner] + 64)
    assert np.allclose(res["ny"][inner], 1.0, atol=1e-6)


def test_boundary_flags(fc):
    d = (10, 6, 3)
    f = fc.boundary_flags(d).reshape(d[::-1])
    assert np.all(f[:, :, 0] == 2)
    assert np.all(f[:, 1:-1, -1] == 3)
    assert np.all(f[:, 0, 1:] == 5) and np.all(f[:, -1, 1:] == 4)
    assert np.all(f[:, 1:-1, 1:-1] == 0)


def test_naca4_section(fc):
    xy = fc.naca4("0012", 200)
    assert xy.shape == (399, 2)
    assert np.allclose(xy[199], [0.0, 0.0], atol=1e-7)   # LE
    assert abs(xy[0, 1]) < 1e-6 and abs(xy[-1, 1]) < 1e-6  # closed TE
    assert math.isclose(xy[:, 1].max() - xy[:, 1].min(), 0.12, rel_tol=2e-2)
    cam = fc.naca4("4412", 100)
    assert cam[:, 1].max() > 0.09
    with pytest.raises(Exception):
        fc.naca4("1012")


def test_voxelize_airfoil_area(fc):
    d = (200, 80, 2)
    flags = fc.boundary_flags(d)
    xy = fc.naca4("0012", 200)
    fc.voxelize_airfoil(d, flags, xy, 0.0, 128, 60.0, 40.0)
    solid = (flags.reshape(d[::-1]) == 1)
    area = 0.0822 * 128 * 128  # NACA 0012 section area ~ 0.0822 c^2 (closed TE)
    assert abs(solid[0].sum() - area) / area < 0.05
    assert np.array_equal(solid[0], solid[1])
    # 6 degrees: the TE drops below the anchor row, the LE rises above it.
    f6 = fc.boundary_flags(d)
    fc.voxelize_airfoil(d, f6, xy, 6.0, 128, 60.0, 40.0)
    ys, xs = np.nonzero(f6.reshape(d[::-1])[0] == 1)
    assert ys[xs.argmax()] < 40 < ys[xs.argmin()] + 1


@pytest.mark.parametrize("digits", ["0012", "2412", "4415", "6409"])
@pytest.mark.parametrize("pps", [200, 50])
def test_naca4_matches_reference(fc, golden, digits, pps):
    """generateNACA4 (src/geom/airfoil.cpp:177-266): every outline point."""
    assert np.array_equal(fc.naca4(digits, pps), golden("geometry")[f"naca_{digits}_{pps}"])


@pytest.mark.parametrize("case", [0, 1, 2])
def test_clean_foil_flags_match_reference(fc, golden, mg, case):
    """buildCleanFoilFlags: boundary flags, voxelised foil, closure."""
    from foil_cfd_gb300.solver import layout_anchor
    g = golden("geometry")
    dims, chord, aoa, digits = mg.FOIL_CASES[case]
    f = fc.boundary_flags(dims)
    closed = fc.voxelize_airfoil(dims, f, fc.naca4(digits, 200), aoa, chord, *layout_anchor(dims))
    assert closed == int(g[f"foil{case}_closed"])
    assert np.array_equal(f, g[f"foil{case}"])


@pytest.mark.parametrize("k", [0, 1])
def test_patch_box_and_fine_flags_match_reference(fc, golden, mg, k):
    """derivePatchBox + buildFinePatchFlags (makeFineLayout anchor)."""
    from foil_cfd_gb300.solver import fine_anchor, layout_anchor
    g = golden("geometry")
    i, margins, factor = mg.PATCH_CASES[k]
    dims, chord, aoa, digits = mg.FOIL_CASES[i]
    box = fc.derive_patch_box(dims, g[f"foil{i}"], *margins)
    assert [box.x0, box.y0, box.x1, box.y1] == list(g[f"patch{k}_box"])
    fd = (factor * (box.x1 - box.x0), factor * (box.y1 - box.y0), factor * dims[2])
    ff = np.zeros(int(np.prod(fd)), np.uint8)
    fc.voxelize_airfoil(fd, ff, fc.naca4(digits, 200), aoa, factor * chord,
                        *fine_anchor(layout_anchor(dims), box, factor))
    fc.stamp_interface_shell(fd, ff)
    assert np.array_equal(ff, g[f"patch{k}"])


def test_voxelize_outline_and_closure_match_reference(fc, golden):
    """voxelizeAirfoil of an arbitrary outline over a field holding other
    flags (only fluid becomes solid, faces untouched), and
    closeTrailingEdgeGaps on a random field (closures do not cascade)."""
    g = golden("geometry")
    f = g["wedge_base"].copy()
    assert fc.voxelize_airfoil((90, 40, 3), f, g["wedge_xy"], 20.0, 70, 30.0, 30.0, close_gaps=False) == 0
    assert np.array_equal(f, g["wedge_vox"])
    t = g["te_in"].copy()
    assert fc.close_trailing_edge_gaps((40, 30, 3), t) == int(g["te_closed"])
    assert np.array_equal(t, g["te_out"])
    # An outline under 20 points is not a section: nothing is stamped.
    f2 = g["wedge_base"].copy()
    fc.voxelize_airfoil((90, 40, 3), f2, g["wedge_xy"][:19], 20.0, 70, 30.0, 30.0, close_gaps=False)
    assert np.array_equal(f2, g["wedge_base"])


def test_interface_shell_and_patch_box(fc):
    d = (20, 12, 2)
    f = np.zeros(int(np.prod(d)), np.uint8)
    fc.stamp_interface_shell(d, f)
    g = f.reshape(d[::-1])
    assert np.all(g[:, :2, :] == 8) and np.all(g[:, :, -2:] == 8)
    assert np.all(g[:, 2:-2, 2:-2] == 0)
    c = np.zeros((2, 30, 40), np.uint8)
    c[:, 10:14, 12:20] = 1
    box = fc.derive_patch_box((40, 30, 2), c.ravel(), 3, 4, 2, 2, 5)
    assert (box.x0, box.y0, box.x1, box.y1) == (9, 8, 24, 16)
