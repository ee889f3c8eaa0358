"""CPU checks of the learned u_tau seed's oracle: the FP64 network gradient
against central finite differences of its own forward pass, the BF16
rounding against torch's, the FP64 Newton judge against Reichardt's law, and
the synthetic sample generator's exactness."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def wo():
    from oracle import wallnet_oracle
    return wallnet_oracle


def _params(seed=0):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.3, 1217)
    return p


def test_oracle_gradient_matches_finite_differences(wo):
    rng = np.random.default_rng(1)
    x = rng.normal(0, 1, (64, 3))
    t = rng.normal(0, 1, 64)
    p = _params()
    loss, g = wo.loss_and_grad(p, x, t)
    idx = list(range(0, 96, 7)) + list(range(96, 128, 5)) + list(range(128, 1152, 37)) + \
        list(range(1152, 1184, 3)) + list(range(1184, 1217, 4)) + [1216]
    fd = wo.finite_difference_grad(p, x, t, idx=idx)
    for i in idx:
        assert abs(fd[i] - g[i]) <= 1e-7 * max(1.0, abs(g[i])), (i, fd[i], g[i])
    assert loss > 0


def test_bf16_rounding_matches_torch(wo):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2)
    v = (rng.normal(0, 1, 10000) * 10.0 ** rng.uniform(-6, 3, 10000)).astype(np.float32)
    ref = torch.from_numpy(v).to(torch.bfloat16).float().numpy()
    assert np.array_equal(wo.bf16_round(v), ref)


def test_newton64_judge_solves_reichardt(oracle_mod):
    from foil_cfd_gb300.wallnet import reichardt_uplus, synthetic_samples
    ut, ys, nu = synthetic_samples(20000, seed=3)
    tau = oracle_mod.utau_newton_f64(ut, ys, nu)
    yp = ys.astype(np.float64) * tau / nu
    res = np.abs(tau * reichardt_uplus(yp) - ut) / ut
    assert res.max() < 1e-12


def test_synthetic_samples_cover_the_yplus_range():
    from foil_cfd_gb300.wallnet import reichardt_uplus, synthetic_samples
    ut, ys, nu = synthetic_samples(50000, seed=4)
    assert ut.dtype == np.float32 and (ut > 0).all() and (ys >= 0.5).all() and (ys <= 4).all()
    # Exact by construction up to the FP32 cast of the inputs.
    from oracle import oracle
    oracle.build()
    tau = oracle.utau_newton_f64(ut, ys, nu)
    yp = ys * tau / nu
    assert yp.min() < 1.2 and yp.max() > 8e3
    assert np.all(np.isfinite(reichardt_uplus(yp)))
