"""The learned wall update against the reference's own wall-model kernel.

The reference's wallModelUpdateKernel (src/sim/lbm_wallmodel.cu:31-196,
as-built sm_103a cubin, launched as its launchWallModelUpdate does by
oracle/ref_gpu_harness.cu) and this library's learned update (network seed,
one FP32 correction, FP64 fallback) run on the same wall lists of the same
tunnel (320x96x96 NACA 0012 at 6 deg, chord 128, 2:1 patch), each on the
state its own step reached 10 steps after the uniform start. The learned
update must take at most half the reference kernel's time on the fine
level's list; its accuracy against FP64 Newton is checked in
test_gpu_wallnet.py.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ref_gpu():
    from oracle import ref_gpu
    if not ref_gpu.available("asbuilt", ("core", "refine", "wall")):
        pytest.skip("reference cubins not built (needs the reference tree in the build container)")
    return ref_gpu


def _trained_net(wn):
    """A network trained as the wall-seed leg trains one, on fewer samples:
    half spanning y+ 1..1e4 broadly, half at the tunnels' lattice
    viscosities and sample distances."""
    ut, ys, nu = wn.synthetic_samples(300_000, 3)
    k = 150_000
    hu, hy, hn = wn.synthetic_samples(k, 2003, yplus=(1.0, 300.0), log10_nu=(-3.78, -3.48), y=(0.5, 3.0))
    ut[:k], ys[:k], nu[:k] = hu, hy, hn
    t = [torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda() for a in (ut, ys, nu)]
    tau, _ = wn.utau_solve(wn.NEWTON64, *t, stats=False)
    net, hist = wn.train_wallnet(*t, tau, epochs=150, batch=2048, seed=0)
    assert hist[-1] < 1e-4
    return net


def test_learned_update_vs_reference_wall_kernel(built_lib, ref_gpu):
    import foil_cfd_gb300 as fc
    from foil_cfd_gb300 import wallnet as wn
    from foil_cfd_gb300.tunnels import airfoil_tunnel
    t = airfoil_tunnel(320, 96, 96, chord=128)
    sc = fc.compute_scaling(1.2, 30.0, 1.48e-5, t.chord_cells, t.u_lat)
    s = fc.LBMSolver()
    s.init(t.dims, sc, t.flags, les_cs=0.1)
    s.set_wall_model_enabled(True)
    s.set_startup_ramp_enabled(False)
    s.reset()
    s.init_refinement(t.box, t.factor, t.fine_flags)
    assert s.step_n(10) == 0
    net = _trained_net(wn)
    s.set_wall_solver(wn.LEARNED, net)
    s.wall_update_timed(1, 3)
    ours, st = s.wall_update_timed(1, 20)
    s.set_wall_solver(wn.REFERENCE)
    ours_restated, _ = s.wall_update_timed(1, 20)
    net.close()
    count = s.wall_count(1)
    del s

    wc = fc.build_wall_list(t.dims, t.flags, None, 2)
    wf = fc.build_wall_list(t.fine_dims, t.fine_flags, None, 3)
    assert len(wf["cell"]) == count
    r = ref_gpu.run_full(t.dims, t.flags, sc.tau, t.u_lat, cs=0.1, wall=wc,
                         fine=dict(dims=t.fine_dims, flags=t.fine_flags, box=t.box, factor=t.factor, wall=wf),
                         wm=True, warmup=0, steps=10, batch=10, forces=True, watchdog=False, variant="asbuilt",
                         wall_reps=20)
    theirs = r["wall_ms"][1]
    print(f"\nfine wall update, {count} cells: learned {ours:.4f} ms ({st['fallbacks']} FP64 fallbacks), "
          f"restated reference solve {ours_restated:.4f} ms, reference wallModelUpdateKernel {theirs:.4f} ms")
    assert theirs > 0.0
    assert st["solved"] > 0.9 * count and st["fallbacks"] <= 0.01 * st["solved"], st
    assert ours <= 0.5 * theirs, (ours, theirs)
