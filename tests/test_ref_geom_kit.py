"""The reference's own geometry builders, staged for the benchmark's
reference arm (oracle/ref_geom.py): the airfoil tunnel, its patch and the
wall lists they give are this library's bytes, and the reference's
computeScaling gives this library's tau (host only)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def kit():
    from oracle import ref_geom
    if not ref_geom.available():
        pytest.skip("reference geometry sources not staged (needs the reference tree in the build container)")
    return ref_geom


def test_airfoil_tunnel_and_wall_lists_match_the_library(kit):
    import foil_cfd_gb300 as fc
    from foil_cfd_gb300 import tunnels
    ours = tunnels.airfoil_tunnel(nx=320, ny=96, nz=24, chord=128)
    ref = kit.airfoil_tunnel(nx=320, ny=96, nz=24, chord=128)
    assert np.array_equal(ours.flags, ref.flags)
    assert (ours.box.x0, ours.box.y0, ours.box.x1, ours.box.y1) == ref.box
    assert tuple(ours.fine_dims) == ref.fine_dims and np.array_equal(ours.fine_flags, ref.fine_flags)
    assert ours.updates_per_step() == ref.updates_per_step()
    for dims, flags, sample in ((ours.dims, ours.flags, 2), (ours.fine_dims, ours.fine_flags, 3)):
        a = fc.build_wall_list(dims, flags, sample_cells=sample)
        b = kit.wall_list(dims, flags, sample_cells=sample)
        assert len(b["cell"]) > 0
        for k in ("cell", "sample", "nx", "ny", "nz", "ys", "mask"):
            assert np.array_equal(np.asarray(a[k]), b[k]), k


def test_plain_tunnel_and_scaling_match_the_library(kit):
    import foil_cfd_gb300 as fc
    from foil_cfd_gb300 import tunnels
    ours = tunnels.airfoil_tunnel(192, 96, 8, chord=64, aoa=6.0, patch=False)
    ref = kit.airfoil_tunnel(192, 96, 8, chord=64, aoa=6.0, patch=False)
    assert np.array_equal(ours.flags, ref.flags) and ref.box is None
    s = fc.compute_scaling(1.2, 30.0, 1.48e-5, 256, 0.08)
    tau, u = kit.scaling(1.2, 30.0, 1.48e-5, 256, 0.08)
    assert np.float32(s.tau) == np.float32(tau) and np.float32(s.u_lat) == np.float32(u)
