"""The AA-pattern in-place layout (fcfd_options.layout = FCFD_LAYOUT_AA):
one population array, odd and even steps alternating between the swapped and
the streamed slot layouts. Its populations must equal the A/B ping-pong
step's (the reference's layout, lbm_solver.cpp:1156-1160) bit for bit after
any number of steps, with reads of the state at either phase and stepping
resumed after them; it holds one population array instead of two; and it
refuses lattices it does not serve."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

Q = 19


@pytest.fixture(scope="module")
def fc(built_lib):
    import foil_cfd_gb300 as fc
    return fc


def _state(oracle_mod, dims, seed=7):
    """Taylor-Green equilibrium with a seeded perturbation of every
    population, so that no symmetry hides a slot mix-up."""
    nx, ny, nz = dims
    n = nx * ny * nz
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    u = 0.05 * np.sin(2 * np.pi * x / nx) * np.cos(2 * np.pi * y / ny) * np.cos(2 * np.pi * z / nz)
    v = -0.05 * np.cos(2 * np.pi * x / nx) * np.sin(2 * np.pi * y / ny) * np.cos(2 * np.pi * z / nz)
    f = oracle_mod.equilibrium(np.ones(n), u.ravel(), v.ravel(), np.zeros(n)).astype(np.float32)
    rng = np.random.default_rng(seed)
    return (f * (1.0 + 1e-3 * rng.standard_normal(f.shape))).astype(np.float32)


def _pair(fc, dims, storage, cs=0.1733, tau=0.52):
    out = []
    for layout in ("ab", "aa"):
        s = fc.LBMSolver()
        s.init(dims, fc.scaling_direct(tau, 0.05), np.zeros(int(np.prod(dims)), np.uint8), storage=storage,
               les_cs=cs, layout=layout)
        s.set_startup_ramp_enabled(False)
        s.reset()
        out.append(s)
    return out


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
@pytest.mark.parametrize("dims", [(70, 36, 20), (128, 24, 16)])
def test_aa_equals_ab_bitwise(fc, oracle_mod, storage, dims):
    """Same imported state, same step counts: identical populations and
    macroscopic fields at odd and even step counts (both conversions of the
    AA state), with stepping resumed after every read; rows of 70 cells
    (partial warps) and 128; Smagorinsky on."""
    ab, aa = _pair(fc, dims, storage)
    f0 = _state(oracle_mod, dims)
    ab.import_f32(f0)
    aa.import_f32(f0)
    total = 0
    for k in (1, 2, 1, 7, 6, 40):
        assert ab.step_n(k) == 0 and aa.step_n(k) == 0
        total += k
        fa, fb = aa.export_f32(), ab.export_f32()
        assert np.array_equal(fa.view(np.uint32), fb.view(np.uint32)), (storage, dims, total)
        for x, y in zip(aa.download_macro(), ab.download_macro()):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (storage, dims, total)
    # Steps with no read in between (the layout alternates on the device
    # only), then a read at an odd and at an even count.
    for k in (9, 12):
        assert ab.step_n(k) == 0 and aa.step_n(k) == 0
        total += k
        assert np.array_equal(aa.export_f32().view(np.uint32), ab.export_f32().view(np.uint32)), total
    assert not aa.nan_detected() and not ab.nan_detected()


def test_aa_reset_watchdog_and_snapshot_view(fc):
    """Cold start (equilibrium + spanwise speck) and 450 steps through two
    watchdog checks: identical to the A/B solver; the lattice view shows the
    A/B state and stepping continues exactly after it."""
    torch = pytest.importorskip("torch")
    from foil_cfd_gb300 import capi
    dims = (96, 32, 24)
    ab, aa = _pair(fc, dims, "fp32")
    for s in (ab, aa):
        s.set_startup_ramp_enabled(True)
        s.reset()
    for s in (ab, aa):
        assert s.step_n(225) == 0
    v = aa.lattice_view(0)
    n = int(np.prod(dims))

    class _Dev:
        def __init__(self, ptr, count):
            self.__cuda_array_interface__ = {"shape": (count,), "typestr": "<f4", "data": (ptr, False), "version": 3}

    seen = torch.as_tensor(_Dev(v.f, Q * n), device="cuda").cpu().numpy()
    assert v.f == capi.load().fcfd_active_f(aa._h)
    assert np.array_equal(seen.view(np.uint32), ab.export_f32().view(np.uint32))
    for s in (ab, aa):
        assert s.step_n(225) == 0
    assert np.array_equal(aa.export_f32().view(np.uint32), ab.export_f32().view(np.uint32))
    assert not aa.nan_detected()


def test_aa_holds_one_population_array(fc):
    """Device memory taken by init: the AA solver allocates one population
    array plus a one-slice scratch, the A/B solver two arrays."""
    torch = pytest.importorskip("torch")
    dims = (256, 128, 96)
    n = int(np.prod(dims))
    taken = {}
    for layout in ("ab", "aa"):
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        s = fc.LBMSolver()
        s.init(dims, fc.scaling_direct(0.52, 0.05), np.zeros(n, np.uint8), layout=layout)
        s.synchronize()
        taken[layout] = free0 - torch.cuda.mem_get_info()[0]
        del s
    pop = Q * 4 * n
    # One population array (76 B per cell) saved, less the AA scratch slice;
    # the rest (flags, kind bytes, link classes, macroscopic fields) is common.
    assert taken["ab"] - taken["aa"] >= 0.9 * (pop - 4 * n), taken
    assert taken["aa"] < 0.65 * taken["ab"], taken


def test_aa_refuses_other_lattices(fc):
    from foil_cfd_gb300.solver import Box
    dims = (64, 32, 16)
    n = int(np.prod(dims))
    flags = np.zeros(n, np.uint8)
    flags[n // 2] = 1
    s = fc.LBMSolver()
    with pytest.raises(fc.SolverError, match="AA layout"):
        s.init(dims, fc.scaling_direct(0.52, 0.05), flags, layout="aa")
    s = fc.LBMSolver()
    s.init(dims, fc.scaling_direct(0.52, 0.05), np.zeros(n, np.uint8), layout="aa")
    assert s.set_flags(flags) != 0
    with pytest.raises(fc.SolverError, match="AA layout"):
        s.init_refinement(Box(16, 8, 32, 24), 2, np.zeros(32 * 32 * 32, np.uint8))
    assert s.step_n(3) == 0   # still usable
