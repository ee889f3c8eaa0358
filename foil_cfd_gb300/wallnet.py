"""Learned friction-velocity seed for the iMEM wall model (config: a 3-32-32-1
tanh network, BF16 weights, FP32 accumulation), over the C ABI of
include/foilcfd_wallnet.h.

Sample arrays are CUDA tensors (torch is used only as device memory); the
forward/backward/Adam kernels, the FP64 Newton label solve and the wall
updates are the library's own. The recipe that trains the shipped-by-bench
network:

* harvested samples: (u_par, y, nu) of the wall cells of NACA 0012 tunnels at
  angles of attack 0-12 deg (coarse level and 2:1 patch), read from running
  solvers every batch of steps (fcfd_wall_harvest);
* synthetic samples: y+ log-uniform in [1, 1e4], nu log-uniform in
  [10^-5.5, 10^-1.5], y uniform in [0.5, 4] cells, u_par = u_tau u+(y+);
* labels: FP64 Newton to a relative step of 1e-8 on the FP32 inputs.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi

REFERENCE, NEWTON64, LEARNED, NEWTON64_NET = 0, 1, 2, 3
PARAMS = 1217
KAPPA, REICHARDT_C = 0.41, 7.8


def _torch():
    import torch
    return torch


def _dev(t):
    torch = _torch()
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
        raise ValueError("sample arrays must be contiguous float32 CUDA tensors")
    return C.c_void_p(t.data_ptr())


def _stream():
    torch = _torch()
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class WallNet:
    """One network: FP32 master weights, BF16 working copy, normalisation."""

    def __init__(self, seed: int = 0):
        self._lib = capi.load()
        self.handle = self._lib.fcfd_wallnet_create()
        if not self.handle:
            raise RuntimeError("fcfd_wallnet_create failed")
        self._check(self._lib.fcfd_wallnet_init_params(self.handle, seed), "init")

    def close(self):
        if getattr(self, "handle", None):
            self._lib.fcfd_wallnet_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()

    @staticmethod
    def _check(rc, what):
        if rc:
            raise RuntimeError(f"wallnet {what} failed ({rc})")

    def fit_norm(self, ut, ys, nu, tau):
        self._check(self._lib.fcfd_wallnet_fit_norm(self.handle, _dev(ut), _dev(ys), _dev(nu), _dev(tau), ut.numel(),
                                                    _stream()), "fit_norm")

    def gradient(self, ut, ys, nu, tau):
        """(mean loss, gradient over all samples) at the current BF16 weights."""
        g = np.zeros(PARAMS, np.float32)
        loss = C.c_double()
        self._check(self._lib.fcfd_wallnet_gradient(self.handle, _dev(ut), _dev(ys), _dev(nu), _dev(tau), ut.numel(),
                                                    C.byref(loss), capi.ptr(g), _stream()), "gradient")
        return loss.value, g

    def train(self, ut, ys, nu, tau, epochs=400, batch=2048, lr_max=3e-3, warmup_frac=0.3, seed=0,
              beta1=0.9, beta2=0.999, eps=1e-8):
        """Adam, one-cycle learning rate; returns the per-epoch loss."""
        o = capi.TrainOpts(epochs, batch, lr_max, warmup_frac, beta1, beta2, eps, seed)
        hist = np.zeros(epochs, np.float32)
        self._check(self._lib.fcfd_wallnet_train(self.handle, _dev(ut), _dev(ys), _dev(nu), _dev(tau), ut.numel(),
                                                 C.byref(o), capi.ptr(hist), _stream()), "train")
        return hist

    def predict(self, ut, ys, nu):
        torch = _torch()
        out = torch.empty_like(ut)
        self._check(self._lib.fcfd_wallnet_predict(self.handle, _dev(ut), _dev(ys), _dev(nu), _dev(out), ut.numel(),
                                                   _stream()), "predict")
        return out

    def params(self):
        """(FP32 master, BF16-rounded as float32, normalisation dict)."""
        m = np.zeros(PARAMS, np.float32)
        b = np.zeros(PARAMS, np.float32)
        nm = capi.WallNetNorm()
        self._check(self._lib.fcfd_wallnet_get_params(self.handle, capi.ptr(m), capi.ptr(b), C.byref(nm)), "get")
        return m, b, {"in_mean": list(nm.in_mean), "in_std": list(nm.in_std), "out_mean": nm.out_mean,
                      "out_std": nm.out_std}

    def set_params(self, params, norm: dict | None = None):
        p = np.ascontiguousarray(params, np.float32)
        assert p.size == PARAMS
        nm = None
        if norm is not None:
            nm = capi.WallNetNorm((C.c_float * 3)(*norm["in_mean"]), (C.c_float * 3)(*norm["in_std"]),
                                  norm["out_mean"], norm["out_std"])
        self._check(self._lib.fcfd_wallnet_set_params(self.handle, capi.ptr(p), None if nm is None else C.byref(nm)),
                    "set")


def utau_solve(method: int, ut, ys, nu, net: WallNet | None = None, warm=None, stats: bool = True):
    """u_tau for each sample by method (REFERENCE, NEWTON64, LEARNED,
    NEWTON64_NET); returns (tensor, stats dict or None)."""
    torch = _torch()
    lib = capi.load()
    out = torch.empty_like(ut)
    st = capi.UtauStats()
    rc = lib.fcfd_utau_solve(method, None if net is None else net.handle, _dev(ut), _dev(ys), _dev(nu),
                             None if warm is None else _dev(warm), _dev(out), ut.numel(),
                             C.byref(st) if stats else None, _stream())
    if rc:
        raise RuntimeError(f"fcfd_utau_solve failed ({rc})")
    return out, ({"solved": st.solved, "fallbacks": st.fallbacks, "newton_iterations": st.newton_iterations}
                 if stats else None)


def reichardt_uplus(yp):
    """Reichardt's law u+(y+) in FP64 (kappa 0.41, C 7.8)."""
    yp = np.asarray(yp, np.float64)
    return np.log1p(KAPPA * yp) / KAPPA + REICHARDT_C * (1 - np.exp(-yp / 11) - (yp / 11) * np.exp(-yp / 3))


def synthetic_samples(n: int, seed: int = 0, yplus=(1.0, 1e4), log10_nu=(-5.5, -1.5), y=(0.5, 4.0)):
    """(u_par, y, nu) as float32 numpy arrays with y+ log-uniform."""
    rng = np.random.default_rng(seed)
    yp = 10 ** rng.uniform(np.log10(yplus[0]), np.log10(yplus[1]), n)
    nu = 10 ** rng.uniform(log10_nu[0], log10_nu[1], n)
    ys = rng.uniform(y[0], y[1], n)
    utau = yp * nu / ys
    ut = utau * reichardt_uplus(yp)
    return ut.astype(np.float32), ys.astype(np.float32), nu.astype(np.float32)


def harvest_airfoil(target: int, aoas=(0.0, 3.0, 6.0, 9.0, 12.0), dims=(320, 96, 32), chord=128, batch=50,
                    warm_steps=100, storage="fp32", log=None):
    """Wall-cell samples (u_par, y, nu) from running NACA 0012 tunnels with
    the wall model and a 2:1 patch, equal shares per angle; CUDA tensors."""
    torch = _torch()
    from .solver import LBMSolver, compute_scaling
    from .tunnels import airfoil_tunnel
    per = -(-target // len(aoas))
    cols = {"ut": [], "ys": [], "nu": []}
    for aoa in aoas:
        t = airfoil_tunnel(*dims, chord=chord, aoa=aoa)
        sc = compute_scaling(1.2, 30.0, 1.48e-5, t.chord_cells, t.u_lat)
        sol = LBMSolver()
        sol.init(t.dims, sc, t.flags, storage=storage, les_cs=0.1)
        sol.set_wall_model_enabled(True)
        sol.set_startup_ramp_enabled(False)
        sol.reset()
        sol.init_refinement(t.box, t.factor, t.fine_flags)
        if sol.step_n(warm_steps):
            raise RuntimeError("harvest tunnel step failed")
        levels = [(0, (sc.tau - 0.5) / 3.0), (1, t.factor * (sc.tau - 0.5) / 3.0)]  # fine tau = m(tau-1/2)+1/2
        cap = max(sol.wall_count(lv) for lv, _ in levels)
        ut_buf = torch.empty(cap, device="cuda")
        ys_buf = torch.empty(cap, device="cuda")
        got = 0
        while got < per:
            for lv, nu in levels:
                cnt = sol.wall_harvest(lv, ut_buf.data_ptr(), ys_buf.data_ptr(), cap)
                ut, ys = ut_buf[:cnt], ys_buf[:cnt]
                keep = ut > 0
                k = int(keep.sum())
                take = min(k, per - got)
                if take <= 0:
                    continue
                cols["ut"].append(ut[keep][:take].clone())
                cols["ys"].append(ys[keep][:take].clone())
                cols["nu"].append(torch.full((take,), nu, device="cuda"))
                got += take
            if got < per and sol.step_n(batch):
                raise RuntimeError("harvest tunnel step failed")
        if log:
            log(f"harvest aoa {aoa:g}: {got} samples, {sol.step_count()} steps")
        del sol
    return tuple(torch.cat(cols[k])[:target].contiguous() for k in ("ut", "ys", "nu"))


def training_set(n_harvest: int, n_synth: int, seed: int = 0, log=None, **harvest_kw):
    """Harvested + synthetic samples with FP64 Newton labels (CUDA tensors)."""
    torch = _torch()
    parts = []
    if n_harvest > 0:
        parts.append(harvest_airfoil(n_harvest, log=log, **harvest_kw))
    if n_synth > 0:
        parts.append(tuple(torch.from_numpy(a).cuda() for a in synthetic_samples(n_synth, seed)))
    ut, ys, nu = (torch.cat([p[k] for p in parts]).contiguous() for k in range(3))
    tau, _ = utau_solve(NEWTON64, ut, ys, nu, stats=False)
    return ut, ys, nu, tau


def train_wallnet(ut, ys, nu, tau, epochs=400, batch=2048, lr_max=3e-3, seed=0):
    """Fit the normalisation, then train a fresh network; returns (net, loss history)."""
    net = WallNet(seed)
    net.fit_norm(ut, ys, nu, tau)
    hist = net.train(ut, ys, nu, tau, epochs=epochs, batch=batch, lr_max=lr_max, seed=seed)
    return net, hist
