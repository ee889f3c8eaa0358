"""The reference's own CUDA stream-collide, compiled from the reference tree
into a cubin (oracle/ref_build.py) and launched on this GPU through the
driver-API harness (oracle/ref_gpu_harness.cu), against this library's
collide on the same flags, state and parameters. Built without contraction
the reference kernel's populations equal ours bit for bit, which checks the
harness as well; bench.py's reference arm times the as-built one."""
import numpy as np
import pytest

from conftest import written_mask

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fc(built_lib):
    import foil_cfd_gb300 as fc
    return fc


def test_reference_cuda_kernel_matches_ours(fc, oracle_mod):
    from oracle import ref_gpu
    if not ref_gpu.CUBIN_NOFMA.exists():
        pytest.skip("reference cubin not built (needs the reference tree in the build container)")
    dims = (48, 24, 8)
    n = int(np.prod(dims))
    fl = np.zeros(dims[::-1], np.uint8)
    fl[:, 0, :] = 5
    fl[:, -1, :] = 4
    fl[:, :, 0] = 2
    fl[:, 1:-1, -1] = 3
    fl[:, 9:15, 12:18] = 1
    flags = fl.ravel().copy()
    rng = np.random.default_rng(11)
    f0 = oracle_mod.equilibrium(1 + 0.005 * rng.standard_normal(n), 0.05 + 0.005 * rng.standard_normal(n),
                                0.005 * rng.standard_normal(n), 0.005 * rng.standard_normal(n))
    ref, _ = ref_gpu.run(dims, flags, f0, 0.52, 0.05, steps=25, cubin=ref_gpu.CUBIN_NOFMA)
    s = fc.LBMSolver()
    s.init(dims, fc.scaling_direct(0.52, 0.05), flags)
    s.set_startup_ramp_enabled(False)
    s.reset()
    s.import_f32(f0)
    assert s.step_n(25) == 0
    m = written_mask(flags)
    assert np.array_equal(s.export_f32().reshape(19, -1)[:, m], ref.reshape(19, -1)[:, m])


def uniform_feq(u):
    """feq(1, u, 0, 0) per direction in FP32 arithmetic, in the expression
    order the harness uses for its uniform start (the reference's
    equilibrium19: (w rho)(1 + cu + cu cu / 2 - usq))."""
    f32 = np.float32
    u = f32(u)
    usq = f32(1.5) * (u * u)
    cx = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0]
    out = np.empty(19, np.float32)
    for q in range(19):
        w = f32(1.0) / f32(3.0) if q == 0 else (f32(1.0) / f32(18.0) if q <= 6 else f32(1.0) / f32(36.0))
        cu = f32(3.0) * (f32(cx[q]) * u)
        out[q] = (w * f32(1.0)) * (((f32(1.0) + cu) + (f32(0.5) * cu) * cu) - usq)
    return out


def test_reference_cuda_refined_step_matches_ours(fc):
    """The reference's refined step (its collide, fill and restriction
    kernels from the reference tree, no contraction) against this library's
    step with the 2:1 patch: coarse and fine fluid populations equal after
    ten coarse steps from the same uniform state."""
    from oracle import ref_gpu
    from foil_cfd_gb300.tunnels import airfoil_tunnel
    if not (ref_gpu.CUBIN_NOFMA.exists() and ref_gpu.CUBIN_REFINE_NOFMA.exists()):
        pytest.skip("reference cubins not built (needs the reference tree in the build container)")
    t = airfoil_tunnel(160, 64, 16, chord=64, aoa=6.0)
    nc, nf = int(np.prod(t.dims)), int(np.prod(t.fine_dims))
    feq = uniform_feq(t.u_lat)
    _, rc, rf = ref_gpu.run_refined(t.dims, t.flags, t.fine_dims, t.fine_flags, t.box, t.factor, 0.52, t.u_lat,
                                    cs=0.1, wall_model=False, warmup=0, steps=10, batch=50,
                                    refine_cubin=ref_gpu.CUBIN_REFINE_NOFMA, states=True)
    s = fc.LBMSolver()
    s.init(t.dims, fc.scaling_direct(0.52, t.u_lat, t.chord_cells), t.flags, les_cs=0.1)
    s.set_startup_ramp_enabled(False)
    s.reset()
    s.init_refinement(t.box, t.factor, t.fine_flags)
    s.import_f32(np.repeat(feq, nc))
    s.import_fine_f32(np.repeat(feq, nf))
    assert s.step_n(10) == 0
    mc = written_mask(t.flags)
    assert np.array_equal(s.export_f32().reshape(19, -1)[:, mc], rc.reshape(19, -1)[:, mc])
    mf = t.fine_flags == 0
    assert np.array_equal(s.export_fine_f32().reshape(19, -1)[:, mf], rf.reshape(19, -1)[:, mf])
