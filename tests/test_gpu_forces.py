"""The force read-back of the drop-in boundary (fcfd_forces, the reference's
LBMSolver::forces): the EMA of the per-batch force samples, the validity gate
and the trailing statistics, against a restatement of the reference's fold
(lbm_solver.cpp:633-653, in pollAsync) and of forces() (lbm_solver.cpp:
1414-1509); that forces() never waits on the stream; and the lattice view
and device flags exports (lbm_solver.h:431-444)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

K_FORCE_GATE_FLOW_THROUGHS = 2.0   # units.h kForceGateFlowThroughs


@pytest.fixture(scope="module")
def fc(built_lib):
    import foil_cfd_gb300 as fc
    return fc


def force_to_coefficient(force, u_lat, chord, span):
    """units.h:168-173 in FP32: F / (0.5 u^2 N_c span)."""
    f32 = np.float32
    qref = f32(f32(f32(f32(0.5) * f32(u_lat)) * f32(u_lat)) * f32(chord)) * f32(span)
    return f32(f32(force) / qref) if qref > 0 else f32(0.0)


def restate(samples, steps, u_lat, chord, span, nx, ema_window=1.0):
    """The reference's EMA fold of each completed sample (step of the force
    launch, fx, fy) and its forces() readout after `steps` steps."""
    f32 = np.float32
    ft = f32(f32(nx) / f32(max(u_lat, 1e-6)))
    window = f32(max(f32(1.0), f32(f32(ema_window) * ft)))
    ema = None
    last = 0
    for step, fx, fy in samples:
        fx, fy = f32(fx), f32(fy)
        alpha = f32(f32(1.0) - f32(np.exp(f32(-f32(step - last) / window))))
        ema = (fx, fy) if ema is None else (f32(ema[0] + f32(alpha * f32(fx - ema[0]))),
                                           f32(ema[1] + f32(alpha * f32(fy - ema[1]))))
        last = step
    r = dict(cd=force_to_coefficient(ema[0], u_lat, chord, span), cl=force_to_coefficient(ema[1], u_lat, chord, span),
             valid=steps >= int(f32(K_FORCE_GATE_FLOW_THROUGHS) * ft))
    keep = [(force_to_coefficient(fy, u_lat, chord, span), force_to_coefficient(fx, u_lat, chord, span))
            for step, fx, fy in samples if step >= int(ft)]
    if not keep:
        return r
    cl = np.array([k[0] for k in keep], np.float32)
    cd = np.array([k[1] for k in keep], np.float32)
    ld = np.array([c / d if abs(d) > 1e-6 else 0.0 for c, d in zip(cl, cd)], np.float32)
    for name, v in (("cl", cl), ("cd", cd), ("ld", ld)):
        acc = f32(0.0)
        for x in v:
            acc = f32(acc + x)
        r[name + "_avg"] = f32(acc / f32(len(v)))
        r[name + "_min"], r[name + "_max"], r[name + "_median"] = v.min(), v.max(), f32(np.median(v))
    return r


def test_forces_ema_gate_and_trailing_statistics(fc):
    """Square cylinder (64x32x8, side 8, slip walls, u 0.1): one flow-through
    is 640 steps, the gate opens after two. Sixteen stepN(100) calls, each
    sample read back before the next call; the readout's EMA coefficients
    agree with the restated fold to FP32 exp rounding (1e-5), the gate and
    the trailing min / max / median / mean to 1e-6."""
    from foil_cfd_gb300 import tunnels
    t = tunnels.square_cylinder(64, 32, 8, side=8, cx=20, u_lat=0.1, walls="slip")
    s = fc.LBMSolver()
    s.init(t.dims, fc.scaling_direct(0.55, 0.1, 8), t.flags)
    s.set_startup_ramp_enabled(False)
    s.reset()
    samples = []
    for k in range(16):
        assert s.step_n(100) == 0
        f = s.force_raw()           # waits for the batch and folds its sample
        samples.append((s.step_count(), float(f[0]), float(f[1])))
        r = s.forces()
        want = restate(samples, s.step_count(), 0.1, 8, t.dims[2], t.dims[0])
        assert bool(r.valid) == want["valid"], (k, r.valid)
        assert np.isclose(r.cd, want["cd"], rtol=1e-5) and np.isclose(r.cl, want["cl"], rtol=1e-5, atol=1e-7)
    assert r.valid
    for name in ("cl", "cd", "ld"):
        for stat in ("avg", "min", "max", "median"):
            got, exp = getattr(r, f"{name}_{stat}"), want[f"{name}_{stat}"]
            assert np.isclose(got, exp, rtol=1e-6, atol=1e-7), (name, stat, got, exp)
    assert np.isclose(r.flow_throughs, 1600 / (64 / np.float32(0.1)), rtol=1e-6)


def test_forces_does_not_wait_on_the_stream(fc):
    """forces() right after an enqueued stepN returns while the GPU is still
    busy (the reference's forces() reads host state only)."""
    from foil_cfd_gb300 import tunnels
    t = tunnels.square_cylinder(384, 128, 64, side=24, u_lat=0.08, walls="slip")
    s = fc.LBMSolver()
    s.init(t.dims, fc.scaling_direct(0.55, 0.08, 24), t.flags)
    s.set_startup_ramp_enabled(False)
    s.reset()
    assert s.step_n(20) == 0
    s.synchronize()
    t0 = time.perf_counter()
    assert s.step_n(200) == 0
    t1 = time.perf_counter()
    s.forces()
    t2 = time.perf_counter()
    s.synchronize()
    t3 = time.perf_counter()
    assert t3 - t1 > 0.005, "the GPU work must outlast the calls for this check to mean anything"
    assert t2 - t1 < 0.25 * (t3 - t1), (t1 - t0, t2 - t1, t3 - t1)


class _DeviceBytes:
    """A device allocation seen through __cuda_array_interface__ (the test
    only copies it to the host)."""

    def __init__(self, ptr, n, typestr="|u1"):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3}


def test_lattice_view_and_device_flags(fc):
    """The lattice view names the current buffer (fcfd_active_f), the flags
    and the grid; the device flags hold the uploaded CellFlag bytes; the
    view's populations are the exported state; the slip arrays appear with
    the wall model."""
    torch = pytest.importorskip("torch")
    from foil_cfd_gb300 import capi
    from foil_cfd_gb300.tunnels import airfoil_tunnel
    t = airfoil_tunnel(160, 64, 16, chord=64, aoa=6.0)
    s = fc.LBMSolver()
    s.init(t.dims, fc.scaling_direct(0.52, t.u_lat, t.chord_cells), t.flags, les_cs=0.1)
    s.set_startup_ramp_enabled(False)
    s.reset()
    s.init_refinement(t.box, t.factor, t.fine_flags)
    assert s.step_n(3) == 0
    s.synchronize()
    n = int(np.prod(t.dims))
    v = s.lattice_view(0)
    assert v.f == capi.load().fcfd_active_f(s._h)
    assert (v.dims.nx, v.dims.ny, v.dims.nz) == t.dims and v.cells == n and v.storage == 0
    assert v.flags == s.device_flags(0) and not v.uwx
    flags = torch.as_tensor(_DeviceBytes(v.flags, n), device="cuda").cpu().numpy()
    assert np.array_equal(flags, t.flags)
    f = torch.as_tensor(_DeviceBytes(v.f, 19 * n, "<f4"), device="cuda").cpu().numpy()
    assert np.array_equal(f, s.export_f32())
    vf = s.lattice_view(1)
    assert vf.cells == int(np.prod(t.fine_dims))
    fine_flags = torch.as_tensor(_DeviceBytes(s.device_flags(1), vf.cells), device="cuda").cpu().numpy()
    assert np.array_equal(fine_flags, t.fine_flags)
    s.set_wall_model_enabled(True)
    vw = s.lattice_view(0)
    assert vw.uwx and vw.uwy and vw.uwz
    with pytest.raises(fc.SolverError):
        s.lattice_view(2)   # no finer level
