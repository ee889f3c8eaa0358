"""On-device geometry builders (include/foilcfd_geom.h) against the
reference's host builders (golden vectors from src/geom/voxelizer.cpp,
airfoil.cpp and src/sim/wall_model.cpp) and against this library's host
builders, and a solver fed with device-built flags against the same solver
fed with host flags. Flags, boxes and lists are compared exactly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fc(built_lib):
    import foil_cfd_gb300 as fc
    return fc


@pytest.fixture(scope="module")
def geo(fc):
    from foil_cfd_gb300 import geometry
    return geometry


@pytest.fixture(scope="module")
def torch():
    import torch
    assert torch.cuda.is_available()
    return torch


def host(t):
    return t.cpu().numpy()


@pytest.mark.parametrize("case", [0, 1, 2])
def test_clean_foil_flags_vs_reference_golden(fc, geo, golden, mg, case):
    g = golden("geometry")
    dims, chord, aoa, digits = mg.FOIL_CASES[case]
    xy = fc.naca4(digits, 200)
    t, closed = geo.build_flags(dims, "boundary", geo.foil(xy, aoa, chord, *fc.layout_anchor(dims)), True, 0)
    assert np.array_equal(host(t), g[f"foil{case}"])
    assert closed == int(g[f"foil{case}_closed"])
    assert np.array_equal(host(geo.clean_foil_flags(dims, digits, aoa, chord)), g[f"foil{case}"])


@pytest.mark.parametrize("k", [0, 1])
def test_patch_box_and_fine_flags_vs_reference_golden(fc, geo, golden, mg, torch, k):
    g = golden("geometry")
    i, margins, factor = mg.PATCH_CASES[k]
    dims, chord, aoa, digits = mg.FOIL_CASES[i]
    coarse = torch.from_numpy(g[f"foil{i}"]).cuda()
    box = geo.derive_patch_box(dims, coarse, *margins)
    assert [box.x0, box.y0, box.x1, box.y1] == list(g[f"patch{k}_box"])
    fd, ff = geo.fine_patch_flags(dims, box, factor, digits, aoa, chord)
    assert np.array_equal(host(ff), g[f"patch{k}"])


def test_outline_over_input_field_and_closure_vs_reference_golden(geo, golden, torch):
    g = golden("geometry")
    base = torch.from_numpy(g["wedge_base"]).cuda()
    out, closed = geo.build_flags((90, 40, 3), "input", geo.foil(g["wedge_xy"], 20.0, 70, 30.0, 30.0), False, 0,
                                  inp=base)
    assert np.array_equal(host(out), g["wedge_vox"]) and closed == 0
    te = torch.from_numpy(g["te_in"]).cuda()
    out, closed = geo.build_flags((40, 30, 3), "input", None, True, 0, inp=te)
    assert np.array_equal(host(out), g["te_out"]) and closed == int(g["te_closed"])
    # No solid: an all-zero box.
    empty, _ = geo.build_flags((40, 30, 3), "fluid", None, False, 0)
    b = geo.derive_patch_box((40, 30, 3), empty, 2, 2, 2, 2)
    assert (b.x0, b.y0, b.x1, b.y1) == (0, 0, 0, 0)


@pytest.mark.parametrize("geom", ["slab", "wedge", "sphere", "vane"])
@pytest.mark.parametrize("sample", [2, 3])
def test_wall_list_vs_reference_golden(geo, golden, mg, torch, geom, sample):
    d, active, clean = mg.wall_list_geometries()[geom]
    g = golden("wall_list")
    key = f"{geom}_{sample}"
    dclean = None if clean is None else torch.from_numpy(np.ascontiguousarray(clean)).cuda()
    res = geo.wall_list(d, torch.from_numpy(np.ascontiguousarray(active)).cuda(), dclean, sample)
    st = g[key + "_stats"]
    assert (res["stats"]["listed"], res["stats"]["excluded_vg"], res["stats"]["degenerate"]) == tuple(int(v) for v in st)
    for k in ("cell", "sample", "mask"):
        assert np.array_equal(host(res[k]).view(np.uint32).astype(np.int64), g[f"{key}_{k}"].astype(np.int64)), k
    for k in ("nx", "ny", "nz", "ys"):
        assert np.array_equal(host(res[k]), g[f"{key}_{k}"]), k


def test_tunnel_lists_vs_host_builders(fc, geo, torch):
    """The airfoil tunnel's coarse and fine fields: device force links and
    wall lists equal the host builders' lists entry for entry."""
    from foil_cfd_gb300.tunnels import airfoil_tunnel
    t = airfoil_tunnel(160, 64, 16, chord=64, aoa=6.0)
    for dims, flags, sample in ((t.dims, t.flags, 2), (t.fine_dims, t.fine_flags, 3)):
        dflags = torch.from_numpy(flags).cuda()
        wl = fc.build_wall_list(dims, flags, None, sample)
        res = geo.wall_list(dims, dflags, None, sample)
        assert res["stats"] == wl["stats"]
        assert np.array_equal(host(res["cell"]).astype(np.int64), wl["cell"])
        assert np.array_equal(host(res["sample"]).astype(np.int64), wl["sample"])
        for k in ("nx", "ny", "nz", "ys"):
            assert np.array_equal(host(res[k]), wl[k]), k
        cells, masks = geo.force_links(dims, dflags)
        # Host restatement of the link rule: fluid cells with a solid cell
        # at x + c_q (every axis periodic).
        f = flags.reshape(dims[::-1])
        from oracle.oracle import CX, CY, CZ
        m = np.zeros(f.shape, np.uint32)
        for q in range(1, 19):
            nb = np.roll(f, (-CZ[q], -CY[q], -CX[q]), axis=(0, 1, 2))
            m |= ((nb == 1).astype(np.uint32) << q)
        m[f != 0] = 0
        idx = np.flatnonzero(m.ravel())
        assert np.array_equal(host(cells).view(np.uint32), idx.astype(np.uint32))
        assert np.array_equal(host(masks).view(np.uint32), m.ravel()[idx])


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_solver_with_device_built_flags_matches_host_flags(fc, geo, torch, storage):
    """A tunnel whose coarse and fine fields are built on the device steps
    bit for bit like the same tunnel built on the host (wall model on, so
    the device-built wall lists and force links are exercised)."""
    from foil_cfd_gb300.tunnels import airfoil_tunnel
    t = airfoil_tunnel(160, 64, 16, chord=64, aoa=6.0)
    cflags = geo.clean_foil_flags(t.dims, "0012", 6.0, 64)
    assert np.array_equal(host(cflags), t.flags)
    fd, fflags = geo.fine_patch_flags(t.dims, t.box, t.factor, "0012", 6.0, 64)
    assert tuple(fd) == tuple(t.fine_dims) and np.array_equal(host(fflags), t.fine_flags)
    out = {}
    for src in ("host", "device"):
        s = fc.LBMSolver()
        s.init(t.dims, fc.scaling_direct(0.52, t.u_lat, t.chord_cells), t.flags if src == "host" else cflags,
               storage=storage, les_cs=0.1)
        s.set_wall_model_enabled(True)
        s.set_startup_ramp_enabled(False)
        s.reset()
        s.init_refinement(t.box, t.factor, t.fine_flags if src == "host" else fflags)
        assert s.step_n(40) == 0 and not s.nan_detected()
        out[src] = (s.export_f32(), s.export_fine_f32(), s.force_raw(), s.wall_model_readout().cells)
    for a, b in zip(out["host"], out["device"]):
        assert np.array_equal(np.asarray(a), np.asarray(b))
