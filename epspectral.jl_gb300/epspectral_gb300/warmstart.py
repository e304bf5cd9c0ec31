"""Learned warm start of the scGD0 iteration: a multilayer perceptron that proposes `Σ_init`.

The reference starts the iteration from Σ = -iη_init (iteration 1 is then the one-shot G0D0) or
from a caller's `Σ_init` (src/scgd0.jl:62-66, 204-212). This module supplies that `Σ_init`:

1. one iteration from -iη_init gives the G0D0 self-energy Σ_G0D0[ω, i] and μ;
2. a network maps, per outer state i, the features [Re Σ_G0D0(ω_j), Im Σ_G0D0(ω_j) on all ωs;
   T, μ, coupling scale, ε_i - μ] to the correction Σ_conv - Σ_G0D0 on all ωs;
3. the iteration restarts from Σ_init = Σ_G0D0 + correction, and its own tol check decides when it
   has converged, so the result is the one of the plain iteration (within tol).
If the warm-started run does not converge in maxiter iterations, the plain run from -iη_init is
made (the fallback) and its result returned.

The network (epsp_warmstart_*: forward, backward, Adam on the GPU, BF16 weights, FP32
accumulation) is trained here on (G0D0 Σ, converged Σ) pairs that the method itself produces
(`generate_pairs`). Inputs and outputs are standardised on the host: per-column mean and standard
deviation for the features, per-column mean and one common scale for the targets (so the loss is
the absolute squared error of Σ, the quantity the tol check measures).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import api
from .grids import ArgumentError

_fp = C.POINTER(C.c_float)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def init_params(dims, seed: int = 0, out_scale: float = 0.1) -> np.ndarray:
    """Seeded initial parameters: W ~ N(0, 1/d_in) (the last layer scaled by out_scale), b = 0."""
    rng = np.random.default_rng(seed)
    parts = []
    for l, (din, dout) in enumerate(zip(dims[:-1], dims[1:])):
        W = rng.normal(0.0, 1.0 / math.sqrt(din), size=(dout, din))
        if l == len(dims) - 2:
            W *= out_scale
        parts += [W.ravel(), np.zeros(dout)]
    return np.concatenate(parts).astype(np.float32)


class Network:
    """The GPU multilayer perceptron of the warm start (epsp_warmstart_*)."""

    def __init__(self, dims, *, seed: int = 0, ctx: api.Context | None = None):
        self.ctx = ctx or api.default_context()
        self.dims = [int(d) for d in dims]
        if len(self.dims) < 2:
            raise ArgumentError("a network needs at least an input and an output width")
        self.handle = C.c_void_p()
        d = (C.c_int32 * len(self.dims))(*self.dims)
        self.ctx.check(api.lib().epsp_warmstart_create(self.ctx.handle, len(self.dims) - 1, d, C.byref(self.handle)))
        self.nparams = int(api.lib().epsp_warmstart_nparams(self.handle))
        self.last_train_device_s = 0.0
        self.set_params(init_params(self.dims, seed))

    def set_params(self, p):
        p = _f32(p)
        if p.size != self.nparams:
            raise ArgumentError(f"expected {self.nparams} parameters, got {p.size}")
        self.ctx.check(api.lib().epsp_warmstart_set_params(self.handle, p.ctypes.data_as(_fp)))

    def get_params(self) -> np.ndarray:
        p = np.empty(self.nparams, dtype=np.float32)
        self.ctx.check(api.lib().epsp_warmstart_get_params(self.handle, p.ctypes.data_as(_fp)))
        return p

    def _xy(self, X, Y=None):
        X = _f32(X)
        if X.ndim != 2 or X.shape[1] != self.dims[0]:
            raise ArgumentError(f"X must be [n, {self.dims[0]}], got {X.shape}")
        if Y is None:
            return X, None
        Y = _f32(Y)
        if Y.shape != (X.shape[0], self.dims[-1]):
            raise ArgumentError(f"Y must be [{X.shape[0]}, {self.dims[-1]}], got {Y.shape}")
        return X, Y

    def predict(self, X) -> np.ndarray:
        X, _ = self._xy(X)
        Y = np.empty((X.shape[0], self.dims[-1]), dtype=np.float32)
        self.ctx.check(api.lib().epsp_warmstart_predict(self.handle, X.ctypes.data_as(_fp), X.shape[0],
                                                        Y.ctypes.data_as(_fp)))
        return Y

    def grad(self, X, Y):
        """Mean squared error and its gradient (flat, like the parameters); no update."""
        X, Y = self._xy(X, Y)
        g = np.empty(self.nparams, dtype=np.float32)
        loss = C.c_double()
        self.ctx.check(api.lib().epsp_warmstart_grad(self.handle, X.ctypes.data_as(_fp), Y.ctypes.data_as(_fp),
                                                     X.shape[0], C.byref(loss), g.ctypes.data_as(_fp)))
        return loss.value, g

    def train(self, X, Y, *, epochs: int, batch: int, lr: float, perm=None, seed: int | None = 0) -> np.ndarray:
        """Minibatch Adam; perm [epochs, n] gives the row order (default: a seeded shuffle per epoch)."""
        X, Y = self._xy(X, Y)
        n = X.shape[0]
        if perm is None and seed is not None:
            rng = np.random.default_rng(seed)
            perm = np.stack([rng.permutation(n) for _ in range(epochs)])
        pp = None
        if perm is not None:
            perm = np.ascontiguousarray(perm, dtype=np.int64)
            if perm.shape != (epochs, n):
                raise ArgumentError(f"perm must be [{epochs}, {n}], got {perm.shape}")
            pp = perm.ctypes.data_as(C.POINTER(C.c_int64))
        hist = np.zeros(epochs)
        self.ctx.check(api.lib().epsp_warmstart_train(self.handle, X.ctypes.data_as(_fp), Y.ctypes.data_as(_fp), n,
                                                      int(epochs), int(batch), float(lr), pp,
                                                      hist.ctypes.data_as(C.POINTER(C.c_double))))
        self.last_train_device_s = api.lib().epsp_warmstart_train_ms(self.handle) / 1e3
        return hist

    def close(self):
        if self.handle:
            api.lib().epsp_warmstart_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


N_SCALARS = 4


def _stages(epochs: int, n: int):
    n = max(1, min(int(n), int(epochs)))
    base, extra = divmod(int(epochs), n)
    return [base + (1 if k < extra else 0) for k in range(n)]


def features(sigma_g0d0, T: float, mu: float, scale: float, eps_i) -> np.ndarray:
    """Rows [ni, 2 nω + 4] of one temperature: Re Σ, Im Σ of each state on ωs, then T, μ, coupling
    scale and ε_i - μ (energies in eV)."""
    S = np.asarray(sigma_g0d0)
    nw, ni = S.shape
    eps_i = np.asarray(eps_i, dtype=np.float64)
    X = np.empty((ni, 2 * nw + N_SCALARS), dtype=np.float64)
    X[:, :nw] = S.real.T
    X[:, nw:2 * nw] = S.imag.T
    X[:, 2 * nw] = T
    X[:, 2 * nw + 1] = mu
    X[:, 2 * nw + 2] = scale
    X[:, 2 * nw + 3] = eps_i - mu
    return X


def targets(sigma_g0d0, sigma_conv) -> np.ndarray:
    D = np.asarray(sigma_conv) - np.asarray(sigma_g0d0)
    return np.concatenate([D.real.T, D.imag.T], axis=1)


class WarmStart:
    """Feature standardisation + the network: Σ_G0D0 -> Σ_init."""

    def __init__(self, nw: int, *, width: int = 256, hidden_layers: int = 3, seed: int = 0,
                 ctx: api.Context | None = None):
        self.nw = int(nw)
        self.dims = [2 * self.nw + N_SCALARS] + [int(width)] * int(hidden_layers) + [2 * self.nw]
        self.net = Network(self.dims, seed=seed, ctx=ctx)
        self.x_mean = self.x_std = self.y_mean = None
        self.y_scale = 1.0
        self.loss_history = np.zeros(0)
        self.train_device_s = 0.0

    def fit(self, X, Y, *, epochs: int = 120, batch: int = 256, lr: float = 1e-3, lr_stages: int = 4,
            lr_decay: float = 0.5, seed: int = 0) -> np.ndarray:
        """Standardise and train: `epochs` in `lr_stages` stages, the learning rate times lr_decay
        after each."""
        X = np.asarray(X)
        Y = np.asarray(Y)
        self.x_mean = X.mean(axis=0, dtype=np.float64)
        sd = np.sqrt(np.mean((X - self.x_mean) ** 2, axis=0, dtype=np.float64))
        # columns that barely vary in the training set (the grid's far tails) are not amplified:
        # their scale is at least a tenth of the median column's
        self.x_std = np.maximum(sd, 0.1 * float(np.median(sd)) + 1e-30)
        self.y_mean = Y.mean(axis=0, dtype=np.float64)
        self.y_scale = float(np.sqrt(np.mean((Y - self.y_mean) ** 2, dtype=np.float64))) or 1.0
        Xn = ((X - self.x_mean) / self.x_std).astype(np.float32)
        Yn = ((Y - self.y_mean) / self.y_scale).astype(np.float32)
        self._set_scaling()
        hist = []
        lr_k = lr
        self.train_device_s = 0.0  # the epochs on the device, without the standardisation and uploads
        for k, n_ep in enumerate(_stages(epochs, lr_stages)):
            hist.append(self.net.train(Xn, Yn, epochs=n_ep, batch=batch, lr=lr_k, seed=seed + k))
            self.train_device_s += self.net.last_train_device_s
            lr_k *= lr_decay
        self.loss_history = np.concatenate(hist)
        return self.loss_history

    def _set_scaling(self):
        xm, xs, ym = _f32(self.x_mean), _f32(self.x_std), _f32(self.y_mean)
        self.net.ctx.check(api.lib().epsp_warmstart_set_scaling(self.net.handle, xm.ctypes.data_as(_fp),
                                                                xs.ctypes.data_as(_fp), ym.ctypes.data_as(_fp),
                                                                float(self.y_scale)))

    @property
    def handle(self):
        return self.net.handle

    def predict_rows(self, X) -> np.ndarray:
        if self.x_mean is None:
            raise ArgumentError("the warm start is not trained")
        Xn = (np.asarray(X, dtype=np.float64) - self.x_mean) / self.x_std
        return self.net.predict(Xn).astype(np.float64) * self.y_scale + self.y_mean

    def sigma_init(self, sigma_g0d0, T, mu, scale, eps_i) -> np.ndarray:
        """Σ_init [nω, ni] of one temperature."""
        S = np.asarray(sigma_g0d0)
        D = self.predict_rows(features(S, T, mu, scale, eps_i))
        nw = self.nw
        return S + (D[:, :nw] + 1j * D[:, nw:]).T

    def state(self) -> dict:
        return dict(dims=np.array(self.dims), params=self.net.get_params(), x_mean=self.x_mean, x_std=self.x_std,
                    y_mean=self.y_mean, y_scale=np.array(self.y_scale))

    def save(self, path: str):
        np.savez(path, **self.state())

    @classmethod
    def load(cls, path: str, ctx: api.Context | None = None) -> "WarmStart":
        z = np.load(path)
        dims = [int(d) for d in z["dims"]]
        ws = cls((dims[0] - N_SCALARS) // 2, width=dims[1], hidden_layers=len(dims) - 2, ctx=ctx)
        ws.net.set_params(z["params"])
        ws.x_mean, ws.x_std, ws.y_mean = z["x_mean"], z["x_std"], z["y_mean"]
        ws.y_scale = float(z["y_scale"])
        ws._set_scaling()
        return ws


def run_scgd0_warm(plan: api.Scgd0Plan, occ, warm: WarmStart | None, *, eta_init, tol, maxiter=20,
                   eta_min=None, mu_start=None, scale: float = 1.0) -> dict:
    """The scGD0 iteration with the learned Σ_init, on the device (epsp_scgd0_run_warm).

    Returns the result of Scgd0Plan.run plus `iters_total` (every iteration made, the G0D0 one
    included, and the fallback's if it ran) and `warm` ("used", "fallback" or "off"). With
    warm=None it is the plain run.
    """
    if warm is None:
        r = plan.run(occ, eta_init=eta_init, tol=tol, maxiter=maxiter, eta_min=eta_min, mu_start=mu_start)
        r["iters_total"], r["warm"] = r["niter"], "off"
        return r
    r = plan.run(occ, eta_init=eta_init, tol=tol, maxiter=maxiter, eta_min=eta_min, mu_start=mu_start, warm=warm,
                 coupling_scale=scale)
    r["warm"] = "fallback" if r["fallback"] else "used"
    return r


def run_scgd0_warm_host(plan: api.Scgd0Plan, occ, warm: WarmStart, *, eta_init, tol, maxiter=20, eta_min=None,
                        mu_start=None, scale: float = 1.0) -> dict:
    """The same composition through the public run with `sigma_init` (host round trips): the G0D0
    run, the host-side prediction, the run from Σ_init, the plain fallback."""
    r1 = plan.run(occ, eta_init=eta_init, tol=tol, maxiter=1, eta_min=eta_min, mu_start=mu_start)
    if np.all(r1["converged"]) or maxiter == 1:
        r1["iters_total"], r1["warm"] = 1, "used"
        return r1
    Tlist = np.atleast_1d(occ["Tlist"])
    S0 = r1["sigma"]
    init = np.empty_like(S0)
    for iT, T in enumerate(Tlist):
        init[:, :, iT] = warm.sigma_init(S0[:, :, iT], float(T), float(r1["mu"][iT]), scale, plan.setup["eps_i"])
    r = plan.run(occ, eta_init=eta_init, tol=tol, maxiter=maxiter - 1, eta_min=eta_min, mu_start=r1["mu"],
                 sigma_init=init)
    if np.all(r["converged"]):
        r["iters_total"], r["warm"] = 1 + r["niter"], "used"
        return r
    rp = plan.run(occ, eta_init=eta_init, tol=tol, maxiter=maxiter, eta_min=eta_min, mu_start=mu_start)
    rp["iters_total"], rp["warm"] = 1 + r["niter"] + rp["niter"], "fallback"
    return rp


def sample_runs(n: int, seed: int, *, T_range=(100.0, 800.0), filling_range=(0.5, 1.5),
                scale_range=(0.5, 2.0), group: int = 8):
    """Seeded run parameters: T [K] and filling [e/site] uniform per run, the g2 scale log-uniform
    per group of `group` consecutive runs (one device plan per group)."""
    rng = np.random.default_rng(seed)
    T = rng.uniform(*T_range, size=n)
    fill = rng.uniform(*filling_range, size=n)
    ng = (n + group - 1) // group
    sc = np.exp(rng.uniform(math.log(scale_range[0]), math.log(scale_range[1]), size=ng))
    return [dict(T_K=float(T[k]), filling=float(fill[k]), scale=float(sc[k // group])) for k in range(n)]


def generate_pairs(setup: dict, runs, *, path="gemm_bf16", eta_init=0.01, tol=1e-6, maxiter=50,
                   omega_acoustic=1e-4, spin_degeneracy=2.0, gpu_tile=None, ctx: api.Context | None = None):
    """(features, targets) of each run, from the method itself: the G0D0 iteration and the plain
    iteration to tol. Runs sharing a scale share one plan (g2 scaled on the host: FP32 or FP64 g2;
    g2 of another type, e.g. BF16 bit patterns, only for runs of scale 1). Returns (X list, Y list,
    records), X and Y float32 [ni, ...] per run."""
    g2 = setup["g2"]
    if g2.dtype not in (np.float32, np.float64) and any(run["scale"] != 1.0 for run in runs):
        raise ArgumentError("generate_pairs scales g2 on the host: pass FP32 or FP64 g2, or runs of scale 1")
    from .synthetic import KELVIN, bare_mu
    ctx = ctx or api.default_context()
    Xs, Ys, recs = [], [], []
    plan, plan_scale = None, None
    for run in runs:
        if plan is None or run["scale"] != plan_scale:
            if plan is not None:
                plan.close()
            s = dict(setup)
            if run["scale"] != 1.0:
                s["g2"] = np.asfortranarray(g2 * np.asarray(run["scale"], dtype=g2.dtype))
            plan = api.Scgd0Plan(s, path=path, omega_acoustic=omega_acoustic, gpu_tile=gpu_tile, ctx=ctx)
            plan_scale = run["scale"]
        T = run["T_K"] * KELVIN
        occ = dict(Tlist=[T], nlist=[0.0], nelec=run["filling"], spin_degeneracy=spin_degeneracy, type="metal")
        mu0 = bare_mu(setup, T, run["filling"], spin_degeneracy)
        r1 = plan.run(occ, eta_init=eta_init, tol=tol, maxiter=1, mu_start=[mu0])
        r = plan.run(occ, eta_init=eta_init, tol=tol, maxiter=maxiter, mu_start=[mu0])
        S0, S = r1["sigma"][:, :, 0], r["sigma"][:, :, 0]
        Xs.append(features(S0, T, float(r1["mu"][0]), run["scale"], setup["eps_i"]).astype(np.float32))
        Ys.append(targets(S0, S).astype(np.float32))
        recs.append(dict(run, T=T, mu0=mu0, niter=int(r["niter"]), converged=bool(r["converged"][0]),
                         mu=float(r["mu"][0])))
    if plan is not None:
        plan.close()
    return Xs, Ys, recs
