"""The oracle (CPU restatement, oracle/lbm_oracle.cpp) against golden vectors
that the reference's own kernels produced (tests/golden/make_golden.py).
Collide, init, wall update and refinement coupling are bit-exact; the force
differs only by the reference's FP32 atomic summation order."""
import numpy as np
import pytest

from conftest import rel_err, written_mask


def _collide_n(o, dims, f, flags, steps, p, slip=None, qlinks=None):
    """A/B stepping: the other buffer starts from the solver's reset state."""
    tau, lam, cs, u_in = (np.float32(x) for x in p)
    macro = None
    other = o.reset_state(dims, flags, u_in)
    for s in range(steps):
        dst, m = o.collide(dims, f, flags, tau, lam, o.smag_prefactor(cs), u_in, s == steps - 1, slip, dst=other,
                           qlinks=qlinks)
        f, other = dst, f
        macro = m if m is not None else macro
    return f, macro


@pytest.mark.parametrize("case,steps,flags_key,slip", [
    ("f1", 1, "flags", False), ("f20", 20, "flags", False),
    ("f20w", 20, "flags", True), ("f20z", 20, "flags_z", False)])
def test_collide_bit_exact(golden, oracle_mod, case, steps, flags_key, slip):
    g = golden("collide")
    dims = tuple(int(x) for x in g["dims"])
    flags = g[flags_key]
    sl = list(g["slip"]) if slip else None
    f, macro = _collide_n(oracle_mod, dims, g["f0"].copy(), flags, steps, g["params"], sl)
    m = written_mask(flags)
    ref = g[case].reshape(19, -1)
    assert np.array_equal(f.reshape(19, -1)[:, m], ref[:, m])
    mkey = {"f1": "m1", "f20": "m20", "f20w": "m20w", "f20z": "m20z"}[case]
    assert np.array_equal(np.stack(macro), g[mkey])


@pytest.mark.parametrize("case,steps,slip", [("f1", 1, False), ("f20", 20, False), ("f20w", 20, True)])
def test_qlibb_collide_bit_exact(golden, oracle_mod, case, steps, slip):
    """Interpolated bounce-back (the reference's streamCollideKernel<WM, true>,
    lbm_core.cu:332-364) around a square block with seeded cut fractions."""
    g = golden("qlibb")
    dims = tuple(int(x) for x in g["dims"])
    flags = g["flags"]
    sl = list(g["slip"]) if slip else None
    f, macro = _collide_n(oracle_mod, dims, g["f0"].copy(), flags, steps, g["params"], sl,
                          qlinks=(g["qfrac"], g["ffmask"]))
    m = written_mask(flags)
    assert np.array_equal(f.reshape(19, -1)[:, m], g[case].reshape(19, -1)[:, m])
    assert np.array_equal(np.stack(macro), g["m" + case[1:]])
    # The interpolation changes the outcome: the plain half-way result differs.
    fp, _ = _collide_n(oracle_mod, dims, g["f0"].copy(), flags, steps, g["params"], sl)
    assert not np.array_equal(fp.reshape(19, -1)[:, m], g[case].reshape(19, -1)[:, m])


def test_taylor_green_1000_steps_bit_exact(golden, oracle_mod):
    g = golden("taylor_green")
    dims = tuple(int(x) for x in g["dims"])
    f, macro = _collide_n(oracle_mod, dims, g["f0"].copy(), g["flags"], 1000, g["params"])
    m = written_mask(g["flags"])
    assert np.array_equal(f.reshape(19, -1)[:, m], g["f1000"].reshape(19, -1)[:, m])


def test_force_matches_reference(golden, oracle_mod):
    g = golden("collide")
    dims = tuple(int(x) for x in g["dims"])
    f = oracle_mod.force(dims, g["f20"], g["flags"])
    assert np.allclose(f, g["force20"], rtol=2e-6, atol=2e-6 * np.abs(g["force20"]).max())
    fw = oracle_mod.force(dims, g["f20w"], g["flags"], list(g["slip"]))
    assert np.allclose(fw, g["force20w"], rtol=2e-6, atol=2e-6 * np.abs(g["force20w"]).max())


def test_init_and_speck(golden, oracle_mod):
    g = golden("init")
    dims = tuple(int(x) for x in g["dims"])
    u_in, amp = (float(x) for x in g["params"])
    f = oracle_mod.init_equilibrium(dims, g["flags"], np.float32(u_in))
    oracle_mod.speck(dims, f, g["flags"], np.float32(amp))
    assert np.array_equal(f, g["f"])


def test_wall_update(golden, oracle_mod):
    g = golden("wall")
    dims = tuple(int(x) for x in g["dims"])
    n = int(np.prod(dims))
    wl = oracle_mod.WallList(g["list_cell"], g["list_sample"], g["list_nx"], g["list_ny"], g["list_nz"],
                             g["list_ys"], g["list_mask"])
    slip = [np.zeros(n, np.uint16) for _ in range(3)]
    nu, cut, ema = (np.float32(x) for x in g["params"])
    for it in range(3):
        oracle_mod.wall_update(dims, g["f"], wl, slip, nu, cut, ema)
        assert np.allclose(wl.utau, g["utau"][it], rtol=1e-6, atol=0)
        d = np.abs(np.stack(slip).astype(np.int32) - g["slip"][it].astype(np.int32))
        assert d.max() <= 1  # at most one half ulp apart


def test_refine_fill_and_restrict(golden, oracle_mod):
    g = golden("refine")
    cd, fd = tuple(int(x) for x in g["cdims"]), tuple(int(x) for x in g["fdims"])
    box, m = tuple(int(x) for x in g["box"]), int(g["factor"])
    tauC, tauF = (np.float32(x) for x in g["taus"])
    ff = g["ff0"].copy()
    oracle_mod.fill_c2f(cd, g["cT0"], g["cT1"], g["cflags"], fd, ff, g["fflags"], box, m, 0.5,
                        tauF / (np.float32(m) * tauC), False)
    assert np.array_equal(ff, g["fill_shell"])
    ff = g["ff0"].copy()
    oracle_mod.fill_c2f(cd, g["cT0"], g["cT0"], g["cflags"], fd, ff, g["fflags"], box, m, 0.0,
                        tauF / (np.float32(m) * tauC), True)
    assert np.array_equal(ff, g["fill_full"])
    fc = g["cT1"].copy()
    cn = int(np.prod(cd))
    mac = [np.zeros(cn, np.float32) for _ in range(4)]
    oracle_mod.restrict_f2c(fd, g["ff0"], g["fflags"], cd, fc, g["cflags"], box, m,
                            (np.float32(m) * tauC) / tauF, mac)
    assert np.array_equal(fc, g["restricted"])
    assert np.array_equal(np.stack(mac), g["rmacro"])


def test_flag_edit_fixup_bit_exact(golden, oracle_mod):
    """applyFlagEditsKernel (lbm_core.cu:644-717): newly solid cells zeroed,
    newly fluid cells equilibrium-filled from their unedited fluid
    neighbours, in both buffers."""
    g = golden("edits")
    dims = tuple(int(x) for x in g["dims"])
    a, b = g["fA"].copy(), g["fB"].copy()
    oracle_mod.apply_flag_edits(dims, a, b, g["flags1"], g["mask"])
    assert np.array_equal(a, g["outA"]) and np.array_equal(b, g["outB"])
