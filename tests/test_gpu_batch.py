"""GPU tests of the batched multi-tunnel step (include/foilcfd_batch.h): each
tunnel of a batch steps bit for bit as a single-tunnel solver with the same
flags, storage and parameters (FP32 and FP16 storage); every launch shape
and the graph-replayed chunks give the same populations; the autotuner keeps
the fastest shape it timed; force samples match a direct reduction."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fc(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import foil_cfd_gb300 as fc
    return fc


def small_polar():
    from foil_cfd_gb300 import batch
    return batch.polar_tunnels(count=4, seed=5, span=4, chord_range=(28, 44), aoas=[-4.0, 6.0, 13.5],
                               cambers=(0, 4))


def make_batch(tunnels, storage, force_every=20):
    from foil_cfd_gb300 import batch
    b = batch.BatchSolver()
    b.init(tunnels, storage=storage, les_cs=0.1, force_every=force_every)
    return b


def single(fc, t, storage):
    s = fc.LBMSolver()
    s.init(t.dims, fc.scaling_direct(t.tau, t.u_lat, t.chord), t.flags, storage=storage, les_cs=0.1)
    s.set_startup_ramp_enabled(False)
    s.reset()
    return s


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_batch_matches_single_tunnel_solvers(fc, storage):
    ts = small_polar()
    b = make_batch(ts, storage)
    assert len({t.dims for t in ts}) >= 3  # unevenly sized
    for i, t in enumerate(ts):  # identical start
        assert np.array_equal(b.export_f32(i), single(fc, t, storage).export_f32())
    assert b.step_n(61, use_graphs=False) == 0
    for i, t in enumerate(ts):
        s = single(fc, t, storage)
        assert s.step_n(61) == 0
        assert np.array_equal(b.export_f32(i), s.export_f32()), (storage, i)
    fb = b.forces_now()
    for i, t in enumerate(ts):
        s = single(fc, t, storage)
        assert s.step_n(61) == 0
        assert np.allclose(fb[i], s.force_now(), rtol=1e-12, atol=1e-12)


def test_shapes_and_graph_replay_are_identical(fc):
    ts = small_polar()
    ref = None
    # group_mb 1: one tunnel per group; 4: two tunnels per group.
    for shape, graphs in [((128, 1, 0, 0), False), ((64, 4, 2, 0), False), ((256, 2, 1, 0), True),
                          ((128, 2, 4, 1), True), ((64, 1, 0, 4), True)]:
        b = make_batch(ts, "fp16")
        b.set_config(*shape)
        assert b.config() == shape
        assert b.step_n(80, use_graphs=graphs) == 0
        out = [b.export_f32(i) for i in range(len(ts))]
        hist = b.force_history()
        assert len(hist) == 4
        if ref is None:
            ref = (out, hist)
        else:
            for a, c in zip(out, ref[0]):
                assert np.array_equal(a, c), shape
            assert np.array_equal(hist, ref[1])
        assert np.allclose(hist[-1], b.forces_now(), rtol=0, atol=0)
        b.close()


def test_graph_chunks_from_odd_step_counts(fc):
    ts = small_polar()
    a = make_batch(ts, "fp32")
    b = make_batch(ts, "fp32")
    for n in (7, 20, 13, 40, 20):  # direct steps, graph chunks, direct tails
        assert a.step_n(n, use_graphs=True) == 0
        assert b.step_n(n, use_graphs=False) == 0
    assert a.step_count() == b.step_count() == 100
    for i in range(len(ts)):
        assert np.array_equal(a.export_f32(i), b.export_f32(i))
    assert np.array_equal(a.force_history(), b.force_history())


def test_autotune_keeps_the_fastest_timed_shape(fc):
    ts = small_polar()
    b = make_batch(ts, "fp16")
    chosen, ms, table = b.autotune(trial_steps=3)
    assert len(table) >= 13 and ms > 0
    groupings = [r for r in table if r[0][:3] == table[-1][0][:3]][-4:]
    assert [r[0][3] for r in groupings] == [0, 48, 96, 192]
    best = min(groupings, key=lambda r: r[1])
    assert chosen == best[0] and abs(ms - best[1]) < 1e-9
    shape_best = min(table[:-4], key=lambda r: r[1])
    assert chosen[:3] == shape_best[0][:3]
    assert b.config() == chosen


def test_bad_arguments(fc):
    from foil_cfd_gb300 import batch
    ts = small_polar()
    b = make_batch(ts, "fp16")
    with pytest.raises(Exception):
        b.set_config(96, 1, 0)
    with pytest.raises(Exception):
        b.set_config(128, 3, 0)
    with pytest.raises(Exception):
        b.set_config(128, 1, 0, -1)
    bb = batch.BatchSolver()
    with pytest.raises(Exception):
        bb.init(ts, storage="fp16", force_every=3)


def test_health_reads_speeds(fc):
    ts = small_polar()
    b = make_batch(ts, "fp16")
    assert b.step_n(40) == 0
    speed, bad = b.health()
    assert (bad == 0).all() and (speed > 0.05).all() and (speed < 0.285).all()


def test_device_built_polar_matches_host_built(fc):
    """Polar tunnels whose flags the device geometry kernels build (CUDA
    tensors handed to the batch) are the host builders' bytes and step bit
    for bit like the host-built batch."""
    from foil_cfd_gb300 import batch
    kw = dict(count=4, seed=5, span=4, chord_range=(28, 44), aoas=[-4.0, 6.0, 13.5], cambers=(0, 4))
    host = batch.polar_tunnels(**kw)
    dev = batch.polar_tunnels(device=True, **kw)
    for h, d in zip(host, dev):
        assert d.flags.is_cuda and np.array_equal(d.flags.cpu().numpy(), h.flags)
    bh, bd = make_batch(host, "fp16"), make_batch(dev, "fp16")
    assert bh.step_n(40) == 0 and bd.step_n(40) == 0
    for i in range(len(host)):
        assert np.array_equal(bh.export_f32(i), bd.export_f32(i))
    assert np.array_equal(np.asarray(bh.forces_now()), np.asarray(bd.forces_now()))



@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_watchdog_latches_and_stops_a_diverged_tunnel(fc, oracle_mod, storage):
    """The batch's per-tunnel watchdog: a tunnel given a block of fluid at
    |u| = 0.6 (twice the 0.3 limiter) is latched with verdict 2 at the next
    force sample (every 2 steps here) and stops stepping (its populations
    freeze, graph replays included), while the other tunnels keep stepping
    exactly as their single-tunnel twins; a reset clears the latch."""
    ts = small_polar()
    b = make_batch(ts, storage, force_every=2)
    f = b.export_f32(0).reshape(19, -1).copy()
    nx, ny, nz = ts[0].dims
    fl = ts[0].flags.reshape(nz, ny, nx)
    hot = np.zeros((nz, ny, nx), bool)
    hot[:, ny // 2 - 8:ny // 2 + 8, nx // 2 + 10:nx // 2 + 26] = True
    hot &= fl == 0
    m = hot.ravel()
    k = int(m.sum())
    assert k > 500
    f[:, m] = oracle_mod.equilibrium(np.ones(k), np.full(k, 0.6), np.zeros(k), np.zeros(k), np.float32).reshape(19, k)
    b.import_f32(0, f.ravel())
    assert b.step_n(2, use_graphs=False) == 0
    v, steps = b.latched(with_steps=True)
    assert v[0] == 2 and not v[1:].any(), v
    assert steps[0] == 2 and (steps[1:] == 2).all()
    frozen = b.export_f32(0)
    assert b.step_n(40, use_graphs=True) == 0
    assert np.array_equal(b.export_f32(0), frozen)
    v, steps = b.latched(with_steps=True)
    assert not v[1:].any() and steps[0] == 2 and (steps[1:] == 42).all()
    for i in range(1, len(ts)):
        s = single(fc, ts[i], storage)
        assert s.step_n(42) == 0
        assert np.array_equal(b.export_f32(i), s.export_f32()), (storage, i)
    b.reset()
    assert not b.latched().any()
