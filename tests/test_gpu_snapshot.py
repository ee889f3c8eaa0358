"""Warm-start snapshots on the device: the exact VRAM snapshot of every
level (FP32 and FP16 deviation storage) restores the captured populations
and the run continues bit for bit; the compact snapshot goes through an FCS1
file and the equilibrium re-init, which matches the reference's
initFromMacroKernel output (golden) bit for bit in FP32."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fc(built_lib):
    import foil_cfd_gb300 as fc
    return fc


@pytest.fixture(scope="module")
def sn(fc):
    from foil_cfd_gb300 import snapshot
    return snapshot


def _tunnel_solver(fc, storage, t):
    s = fc.LBMSolver()
    s.init(t.dims, fc.scaling_direct(0.52, t.u_lat, t.chord_cells), t.flags, storage=storage, les_cs=0.1)
    s.set_wall_model_enabled(True)
    s.set_startup_ramp_enabled(False)
    s.reset()
    s.init_refinement(t.box, t.factor, t.fine_flags)
    return s


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_vram_snapshot_exact_restore_and_replay(fc, sn, storage):
    from foil_cfd_gb300.tunnels import airfoil_tunnel
    t = airfoil_tunnel(160, 64, 16, chord=64, aoa=6.0)
    s = _tunnel_solver(fc, storage, t)
    assert s.step_n(20) == 0
    key = sn.SnapshotKey("naca:0012", sn.aoa_bucket(6.0), t.u_lat, t.dims)
    v = sn.VramSnapshot()
    v.capture(s, key)
    pop = 4 if storage == "fp32" else 2
    cells = int(np.prod(t.dims)) + int(np.prod(t.fine_dims))
    wm = 4 * (s.wall_count(0) + s.wall_count(1)) + 6 * cells   # u_tau + three uint16 slip arrays
    assert v.has_data and v.nbytes == 19 * pop * cells + wm
    assert v.flags_hash == sn.hash_flags(t.flags) and v.key() == key
    f0, g0 = s.export_f32(), s.export_fine_f32()
    assert s.step_n(30) == 0
    f1, g1 = s.export_f32(), s.export_fine_f32()
    assert not np.array_equal(f0, f1)
    assert v.restore(s)
    assert np.array_equal(s.export_f32(), f0) and np.array_equal(s.export_fine_f32(), g0)
    assert s.step_n(30) == 0
    assert np.array_equal(s.export_f32(), f1) and np.array_equal(s.export_fine_f32(), g1)
    # A solver with another storage or without the patch is refused.
    other = fc.LBMSolver()
    other.init(t.dims, fc.scaling_direct(0.52, t.u_lat, t.chord_cells), t.flags,
               storage="fp16" if storage == "fp32" else "fp32")
    assert not v.restore(other)
    plain = fc.LBMSolver()
    plain.init(t.dims, fc.scaling_direct(0.52, t.u_lat, t.chord_cells), t.flags, storage=storage)
    assert not v.restore(plain)
    v.release()
    assert not v.has_data and not v.restore(s)


def test_macro_reinit_vs_reference_golden(fc, golden):
    """restoreFromMacroscopic: feq(rho, u) on every non-solid cell, the rest
    state on solid cells (the reference's initFromMacroKernel)."""
    g = golden("macro_init")
    dims = tuple(int(v) for v in g["dims"])
    s = fc.LBMSolver()
    s.init(dims, fc.scaling_direct(0.52, 0.05, 8), g["flags"])
    s.restore_from_macroscopic(g["rho"], g["u"], g["v"], g["w"])
    assert np.array_equal(s.export_f32(), g["f"])


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_compact_snapshot_file_roundtrip_restore(fc, sn, oracle_mod, storage, tmp_path):
    from foil_cfd_gb300.tunnels import square_cylinder
    t = square_cylinder(96, 48, 8, side=8, cx=24, u_lat=0.05, walls="slip")
    s = fc.LBMSolver()
    s.init(t.dims, fc.scaling_direct(0.55, t.u_lat, t.chord_cells), t.flags, storage=storage)
    s.set_startup_ramp_enabled(False)
    s.reset()
    assert s.step_n(50) == 0
    key = sn.SnapshotKey("stl:00ff12ab34cd56ef", 0, t.u_lat, t.dims)
    c = sn.CompactSnapshot()
    c.capture(s, key)
    rho, u, v, w = s.download_macro()
    for a, b in zip(c.fields(), (rho, u, v, w)):
        assert np.array_equal(a, b)
    path = tmp_path / f"{key.hash():016x}.fcs"
    c.save(path)
    back = sn.CompactSnapshot()
    back.load(path)
    assert back.key() == key and back.flags_hash == sn.hash_flags(t.flags)
    assert back.scaling().tau == s.scaling.tau
    fresh = fc.LBMSolver()
    fresh.init(t.dims, fc.scaling_direct(0.55, t.u_lat, t.chord_cells), t.flags, storage=storage)
    assert back.restore(fresh)
    f = fresh.export_f32()
    solid = t.flags == 1
    expect = oracle_mod.equilibrium(np.where(solid, 1.0, rho), np.where(solid, 0.0, u), np.where(solid, 0.0, v),
                                    np.where(solid, 0.0, w), np.float32)
    # The oracle's equilibrium is evaluated in FP64 (bit-exactness of the
    # FP32 re-init is the golden test above); FP16 adds half an ulp of the
    # stored deviation.
    tol = 5e-7 if storage == "fp32" else 3e-5
    assert np.abs(f - expect).max() <= tol
    assert fresh.step_n(20) == 0 and not fresh.nan_detected()
    # Another grid is refused.
    small = fc.LBMSolver()
    small.init((48, 48, 8), fc.scaling_direct(0.55, t.u_lat, 8), np.zeros(48 * 48 * 8, np.uint8), storage=storage)
    assert not back.restore(small)
