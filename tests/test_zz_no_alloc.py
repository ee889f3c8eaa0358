"""The allocation-free force entry point (fcfd_force_links_noalloc), for
callers that cannot allocate device memory themselves (a frame loop with a
hard time budget, an engine that owns every allocation). Through the C ABI
it must reproduce the solver's own force reduction (fcfd_force_now, which
allocates its scratch) on the same state, on two calls in a row -- the
second call reuses the static scratch the first one left behind -- with and
without the wall-model slip field. The caller's buffers are made with torch.
This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1])


def link_list(dims, flags):
    """Fluid cells with a solid neighbour at +c_q; bit q of the mask."""
    nx, ny, nz = dims
    fl = flags.reshape(nz, ny, nx)
    solid = fl == 1
    mask = np.zeros(fl.shape, np.uint32)
    for q in range(1, 19):
        nb = np.roll(solid, shift=(-CZ[q], -CY[q], -CX[q]), axis=(0, 1, 2))
        mask |= np.where(nb & (fl == 0), np.uint32(1 << q), np.uint32(0))
    cells = np.nonzero(mask.ravel())[0].astype(np.uint32)
    return cells, mask.ravel()[cells].astype(np.uint32)


def test_force_noalloc_matches_solver_reduction(built_lib, oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import foil_cfd_gb300 as fc
    from foil_cfd_gb300 import capi

    lib = capi.load()
    dims = (64, 32, 8)
    n = int(np.prod(dims))
    fl = np.zeros(dims[::-1], np.uint8)
    fl[:, 0, :] = 5
    fl[:, -1, :] = 4
    fl[:, :, 0] = 2
    fl[:, :, -1] = 3
    fl[:, 12:20, 20:30] = 1
    flags = fl.ravel().copy()
    rng = np.random.default_rng(11)
    f0 = oracle_mod.equilibrium(1 + 0.01 * rng.standard_normal(n), 0.05 + 0.01 * rng.standard_normal(n),
                                0.01 * rng.standard_normal(n), 0.01 * rng.standard_normal(n))
    s = fc.LBMSolver()
    s.init(dims, fc.scaling_direct(0.55, 0.05), flags)
    s.set_startup_ramp_enabled(False)
    s.reset()
    s.import_f32(f0)

    # The entry point reads FP32 populations: this solver's buffer is one.
    assert lib.fcfd_f_bytes(s._h) == 19 * 4 * n
    cells, masks = link_list(dims, flags)
    d_cells = torch.from_numpy(cells.view(np.int32)).cuda()
    d_masks = torch.from_numpy(masks.view(np.int32)).cuda()
    out = torch.zeros(3, dtype=torch.float64, device="cuda")

    def call(slip=None):
        f_ptr = lib.fcfd_active_f(s._h)
        sl = [None, None, None] if slip is None else [t.data_ptr() for t in slip]
        torch.cuda.synchronize()
        rc = lib.fcfd_force_links_noalloc(f_ptr, n, d_cells.data_ptr(), d_masks.data_ptr(), len(cells),
                                          sl[0], sl[1], sl[2], out.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        return out.cpu().numpy().copy()

    # Two calls in a row, then two more after the state has moved on.
    for state in range(2):
        ref = s.force_now()
        for _ in range(2):
            got = call()
            assert np.allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max()), (got, ref)
        assert s.step_n(3) == 0

    # With the wall-model slip field.
    s.set_wall_model_enabled(True)
    slip_h = (0.01 * rng.standard_normal((3, n))).astype(np.float16).view(np.uint16)
    s.import_wall_state(0, np.zeros(s.wall_count(0), np.float32), slip_h)
    _, slip_dev = s.export_wall_state(0)
    slip = [torch.from_numpy(slip_dev[k].astype(np.int16, copy=False).view(np.int16).copy()).cuda()
            for k in range(3)]
    ref = s.force_now()
    for _ in range(2):
        got = call(slip)
        assert np.allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max()), (got, ref)

    # A long list (the same links repeated, 300,000 entries = 1,172 blocks) so
    # that the final pass sums several partials per thread, against an FP64
    # host sum of the same per-link terms (t = 2 f_q - corr in FP32, widened).
    reps = 300_000 // len(cells) + 1
    big_cells = np.tile(cells, reps)[:300_000]
    big_masks = np.tile(masks, reps)[:300_000]
    d_big_cells = torch.from_numpy(big_cells.view(np.int32)).cuda()
    d_big_masks = torch.from_numpy(big_masks.view(np.int32)).cuda()
    f_host = s.export_f32().reshape(19, n)
    _, slip_now = s.export_wall_state(0)
    uw = [slip_now[k][big_cells].view(np.float16).astype(np.float32) for k in range(3)]
    acc = np.zeros(3)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, np.float32)
    for q in range(1, 19):
        on = ((big_masks >> q) & 1) == 1
        dot = (np.float32(CX[q]) * uw[0] + np.float32(CY[q]) * uw[1]) + np.float32(CZ[q]) * uw[2]
        corr = (np.float32(6.0) * w[q]) * dot
        t = (np.float32(2.0) * f_host[q, big_cells] - corr).astype(np.float64)
        acc += np.array([CX[q], CY[q], CZ[q]]) * t[on].sum()
    for _ in range(2):
        torch.cuda.synchronize()
        rc = lib.fcfd_force_links_noalloc(lib.fcfd_active_f(s._h), n, d_big_cells.data_ptr(), d_big_masks.data_ptr(),
                                          len(big_cells), slip[0].data_ptr(), slip[1].data_ptr(), slip[2].data_ptr(),
                                          out.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.allclose(got, acc, rtol=1e-10, atol=1e-10 * np.abs(acc).max()), (got, acc)

    # A list longer than the static scratch holds is refused before any work.
    too_many = capi.load().fcfd_force_links_noalloc(lib.fcfd_active_f(s._h), n, d_cells.data_ptr(),
                                                    d_masks.data_ptr(), 4096 * 256 + 1, None, None, None,
                                                    out.data_ptr(), None)
    assert too_many == 1  # cudaErrorInvalidValue
