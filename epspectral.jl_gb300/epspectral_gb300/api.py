"""Python mirror of the reference's loop interface, over the C ABI of libepspectral_gb300.so.

`loop_scgd0(setup, occ; ...)` is `_loop_scgd0` (src/scgd0.jl:189-346), `loop_ladder(setup, Σ, μ,
Tlist, Ωs; ...)` is `_loop_ladder` (src/ladder.jl:303-379) and `apply_ladder_kernel(setup, J, ...)`
is one application of `apply_ladder_kernel!` (src/ladder.jl:245-296), with the same argument meaning
and error behaviour: invalid arguments and a chemical potential with no root raise ArgumentError.
`setup` is a dict with the fields of the reference's `setup` / `ladder` NamedTuples (see abi.py).

The CUDA library is the only compute path. If it is missing or no GPU is present the calls raise
`LibraryUnavailable`; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi
from .abi import (ModelArrays, OccArrays, c_double_p, c_int32_p, epsp_ladder_history, epsp_model, epsp_occ,
                  epsp_options, epsp_scgd0_history, ptr)
from .grids import ArgumentError
from .results import DeviceSigma, LadderOutputs, Scgd0Outputs, as_complex_F, cptr

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libepspectral_gb300.so")


class LibraryUnavailable(RuntimeError):
    """The CUDA library is not built or cannot be loaded."""


class EpspError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


_lib = None


def lib():
    """Load libepspectral_gb300.so (built by build.py); raises LibraryUnavailable if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise LibraryUnavailable(f"{LIB_PATH} is not built: run build.py (or __graft_entry__.build())")
    try:
        L = C.CDLL(LIB_PATH)
    except OSError as e:
        raise LibraryUnavailable(f"cannot load {LIB_PATH}: {e}") from e
    P = C.POINTER
    vp, d, i32, i64, u8p = C.c_void_p, C.c_double, C.c_int32, C.c_int64, P(C.c_uint8)
    sig = {
        "epsp_create": (C.c_int, [P(vp), i32]),
        "epsp_destroy": (None, [vp]),
        "epsp_last_error": (C.c_char_p, [vp]),
        "epsp_kernel_launches": (i64, [vp]),
        "epsp_profile_kernel": (C.c_int, [vp, C.c_char_p]),
        "epsp_profile_read": (C.c_int, [vp, P(d), P(i64)]),
        "epsp_test_fail_alloc": (C.c_int, [vp, C.c_uint64]),
        "epsp_test_gemm_stall": (C.c_int, [vp, C.c_int32, C.c_uint32]),
        "epsp_test_g2_host_gather": (C.c_int, [vp, C.c_int32]),
        "epsp_host_register": (C.c_int, [vp, vp, C.c_uint64]),
        "epsp_host_unregister": (C.c_int, [vp, vp]),
        "epsp_ctx_keep_g2": (C.c_int, [vp, C.c_int32]),
        "epsp_timer_begin": (C.c_int, [vp]),
        "epsp_timer_end": (C.c_int, [vp, P(d)]),
        "epsp_scgd0_setup": (C.c_int, [vp, P(epsp_model), P(epsp_options), P(vp)]),
        "epsp_scgd0_plan_destroy": (None, [vp]),
        "epsp_scgd0_run": (C.c_int, [vp, P(epsp_occ), c_double_p, d, i32, d, i32, c_double_p, c_double_p,
                                     c_double_p, c_double_p, u8p, P(epsp_scgd0_history)]),
        "epsp_scgd0_imsigma": (C.c_int, [vp, c_double_p, d, d, c_double_p]),
        "epsp_ladder_setup": (C.c_int, [vp, P(epsp_model), P(epsp_options), P(vp)]),
        "epsp_ladder_plan_destroy": (None, [vp]),
        "epsp_ladder_run": (C.c_int, [vp, c_double_p, c_double_p, c_double_p, i64, c_double_p, i64, i32, d, i32,
                                      c_double_p, c_double_p, u8p, c_int32_p, P(epsp_ladder_history), c_double_p]),
        "epsp_ladder_apply": (C.c_int, [vp, c_double_p, d, d, d, c_double_p, c_double_p]),
        "epsp_ladder_gemm_config": (C.c_int, [vp, P(i32), P(i32), P(i32), P(d), P(d)]),
        "epsp_ladder_set_gemm_config": (C.c_int, [vp, i32, i32, i32]),
        "epsp_ladder_gemm_persistent": (C.c_int, [vp, P(i32)]),
        "epsp_ladder_set_gemm_persistent": (C.c_int, [vp, i32]),
        "epsp_ladder_gemm_pair": (C.c_int, [vp, P(i32)]),
        "epsp_scgd0_sigma_device": (C.c_int, [vp, P(C.c_void_p), P(C.c_int64)]),
        "epsp_ladder_set_gemm_pair": (C.c_int, [vp, i32]),
        "epsp_ladder_run_batched": (C.c_int, [vp, c_double_p, c_double_p, c_double_p, i64, c_double_p, i64, d, i32, i32,
                                              c_double_p, c_double_p, u8p, c_int32_p, P(epsp_ladder_history),
                                              c_double_p]),
        "epsp_warmstart_create": (C.c_int, [vp, i32, P(i32), P(vp)]),
        "epsp_warmstart_destroy": (None, [vp]),
        "epsp_warmstart_nparams": (i64, [vp]),
        "epsp_warmstart_train_ms": (C.c_double, [vp]),
        "epsp_warmstart_set_params": (C.c_int, [vp, P(C.c_float)]),
        "epsp_warmstart_get_params": (C.c_int, [vp, P(C.c_float)]),
        "epsp_warmstart_predict": (C.c_int, [vp, P(C.c_float), i64, P(C.c_float)]),
        "epsp_warmstart_grad": (C.c_int, [vp, P(C.c_float), P(C.c_float), i64, P(d), P(C.c_float)]),
        "epsp_warmstart_set_scaling": (C.c_int, [vp, P(C.c_float), P(C.c_float), P(C.c_float), C.c_float]),
        "epsp_scgd0_run_warm": (C.c_int, [vp, vp, c_double_p, P(epsp_occ), c_double_p, d, i32, d, i32, c_double_p,
                                          c_double_p, c_double_p, u8p, P(epsp_scgd0_history), P(i32), P(i32)]),
        "epsp_warmstart_train": (C.c_int, [vp, P(C.c_float), P(C.c_float), i64, i32, i32, C.c_float, P(i64),
                                           c_double_p]),
    }
    for name, (res, args) in sig.items():
        if not hasattr(L, name):
            continue
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class Context:
    """A CUDA device and stream for the library (the reference's `backend`)."""

    def __init__(self, device: int = 0):
        self.handle = C.c_void_p()
        st = lib().epsp_create(C.byref(self.handle), int(device))
        if st != abi.EPSP_OK:
            raise LibraryUnavailable(f"epsp_create(device={device}) failed with {abi.STATUS_NAMES.get(st, st)}")

    def check(self, status: int):
        if status == abi.EPSP_OK:
            return
        msg = (lib().epsp_last_error(self.handle) or b"").decode(errors="replace")
        if status in (abi.EPSP_EINVAL, abi.EPSP_ENOROOT_MU):
            raise ArgumentError(msg)
        raise EpspError(status, msg)

    @property
    def kernel_launches(self) -> int:
        return int(lib().epsp_kernel_launches(self.handle))

    def profile(self, name: str | None):
        """Bracket every launch of the kernel family `name` with CUDA events (None: off)."""
        self.check(lib().epsp_profile_kernel(self.handle, (name or "").encode()))

    def profile_read(self):
        ms, n = C.c_double(), C.c_int64()
        self.check(lib().epsp_profile_read(self.handle, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def timer_begin(self):
        self.check(lib().epsp_timer_begin(self.handle))

    def timer_end(self) -> float:
        """Milliseconds on the context's stream since timer_begin (waits for the stream)."""
        ms = C.c_double()
        self.check(lib().epsp_timer_end(self.handle, C.byref(ms)))
        return ms.value

    def fail_next_alloc(self, nbytes: int):
        """Test hook: the next device allocation of at least nbytes fails with ENOMEM."""
        self.check(lib().epsp_test_fail_alloc(self.handle, int(nbytes)))

    def keep_g2(self, on: bool):
        """Keep the last g2 a plan set-up streamed on the device, for a later set-up of the same array
        (an scGD0 plan and a ladder plan of one model); the array must not change in between. False
        frees the copy."""
        self.check(lib().epsp_ctx_keep_g2(self.handle, 1 if on else 0))

    def stall_gemm(self, skip_kblock: int = -1, wait_limit: int = 0):
        """Test hook: the one-CTA tensor-core GEMM skips K block skip_kblock of every tile and gives
        up its pipeline waits after wait_limit tries (EDEVICE_TIMEOUT); stall_gemm() switches it off."""
        self.check(lib().epsp_test_gemm_stall(self.handle, int(skip_kblock), int(wait_limit)))

    def host_register(self, a: np.ndarray):
        """Page-lock the memory of array `a` (epsp_host_register): set-ups then read a g2 there in
        place. Call host_unregister(a) before `a` is freed."""
        self.check(lib().epsp_host_register(self.handle, C.c_void_p(a.ctypes.data), int(a.nbytes)))

    def host_unregister(self, a: np.ndarray):
        self.check(lib().epsp_host_unregister(self.handle, C.c_void_p(a.ctypes.data)))

    def g2_host_gather(self, on: bool = True):
        """Test hook: the set-ups' g2 stream gathers on the host and copies even for a registered g2;
        g2_host_gather(False) restores the device gather."""
        self.check(lib().epsp_test_g2_host_gather(self.handle, 1 if on else 0))

    def close(self):
        if self.handle:
            lib().epsp_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _options(path, gpu_tile, omega_acoustic, verbosity=0):
    p = abi.PATHS[path] if isinstance(path, str) else int(path)
    if gpu_tile is not None and int(gpu_tile) < 1:
        raise ArgumentError(f"gpu_tile must be nothing or a positive number of inner states, got {gpu_tile}")
    return epsp_options(p, int(verbosity), int(gpu_tile or 0), float(omega_acoustic))


class Scgd0Plan:
    """Device-resident tables of one setup (the `setup` half of _loop_scgd0)."""

    def __init__(self, setup, *, path="direct_fp64", gpu_tile=None, omega_acoustic, ctx: Context | None = None,
                 verbosity=0):
        """verbosity >= 2 logs the set-up phases' times and each iteration (err, μ, μ-solve evaluations
        per temperature) to stderr."""
        self.ctx = ctx or default_context()
        self.M = ModelArrays(setup)
        self.setup = setup
        self.opts = _options(path, gpu_tile, omega_acoustic, verbosity)
        self.handle = C.c_void_p()
        self.run_gen = 0  # counts runs: a DeviceSigma is valid for its own run only
        self.ctx.check(lib().epsp_scgd0_setup(self.ctx.handle, C.byref(self.M.struct), C.byref(self.opts),
                                              C.byref(self.handle)))

    def run(self, occ, *, eta_init, tol, maxiter=20, eta_min=None, fix_mu=False, mu_start=None, sigma_init=None,
            warm=None, coupling_scale=1.0, sigma_to_host=True):
        """The iteration of _loop_scgd0 (src/scgd0.jl:246-346).

        With `warm` (a trained warmstart.WarmStart, no Σ_init) the run starts from the network's
        Σ_init after the G0D0 iteration, with the plain start as fallback (epsp_scgd0_run_warm);
        the result then also holds `iters_total` and `fallback`. With sigma_to_host=False Σ stays on
        the device: the result's "sigma" is a DeviceSigma, which LadderPlan.run takes as is."""
        M, O = self.M, OccArrays(occ)
        nT = len(O.Tlist)
        self.run_gen += 1  # the plan's Σ is about to change
        if eta_min is not None and np.ndim(eta_min) > 0 and len(eta_min) != nT:
            raise ArgumentError(f"eta_min must be a scalar or have one entry per temperature ({nT}), got {len(eta_min)}")
        eta_min = np.ascontiguousarray(np.broadcast_to(0.0 if eta_min is None else eta_min, (nT,)), dtype=np.float64)
        if fix_mu and mu_start is None:
            raise ArgumentError("fix_mu = true keeps μ at occ.μlist, which is not given")
        mu0 = np.ascontiguousarray(np.broadcast_to(self.setup.get("mu_start", 0.0) if mu_start is None else mu_start,
                                                   (nT,)), dtype=np.float64)
        if sigma_init is not None and np.shape(sigma_init) != (M.nw, M.ni, nT):
            raise ArgumentError(f"Σ_init must have size (nω, n_i, nT) = {(M.nw, M.ni, nT)}, got {np.shape(sigma_init)}")
        sinit = None if sigma_init is None else as_complex_F(sigma_init, (M.nw, M.ni, nT))
        out = Scgd0Outputs(M.nw, M.ni, nT, maxiter, sigma_to_host)
        if warm is not None:
            if sinit is not None:
                raise ArgumentError("Σ_init and a warm start are exclusive")
            scale = np.ascontiguousarray(np.broadcast_to(coupling_scale, (nT,)), dtype=np.float64)
            it, fb = C.c_int32(), C.c_int32()
            self.ctx.check(lib().epsp_scgd0_run_warm(self.handle, warm.handle, ptr(scale), C.byref(O.struct),
                                                     ptr(eta_min), float(eta_init), int(maxiter), float(tol),
                                                     int(bool(fix_mu)), ptr(mu0), out.sigma_ptr(), ptr(out.mu),
                                                     out.converged.ctypes.data_as(C.POINTER(C.c_uint8)),
                                                     C.byref(out.hist), C.byref(it), C.byref(fb)))
            r = self._result(out)
            r["iters_total"], r["fallback"] = int(it.value), bool(fb.value)
            return r
        self.ctx.check(lib().epsp_scgd0_run(self.handle, C.byref(O.struct), ptr(eta_min), float(eta_init),
                                            int(maxiter), float(tol), int(bool(fix_mu)), ptr(mu0), cptr(sinit),
                                            out.sigma_ptr(), ptr(out.mu),
                                            out.converged.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(out.hist)))
        return self._result(out)

    def _result(self, out):
        r = out.result()
        if out.sigma is None:
            p, n = C.c_void_p(), C.c_int64()
            self.ctx.check(lib().epsp_scgd0_sigma_device(self.handle, C.byref(p), C.byref(n)))
            r["sigma"] = DeviceSigma(self, p.value, (self.M.nw, self.M.ni, int(n.value)), self.run_gen)
        return r

    def imsigma(self, sigma_in, mu, T, imsigma0=None):
        """add_fan_migdal_imsigma! at one temperature (src/scgd0_kernel.jl:59-72)."""
        M = self.M
        sin = as_complex_F(sigma_in, (M.nw, M.ni))
        out = (np.zeros((M.nw, M.ni), order="F") if imsigma0 is None
               else np.array(imsigma0, dtype=np.float64, order="F", copy=True))
        self.ctx.check(lib().epsp_scgd0_imsigma(self.handle, cptr(sin), float(mu), float(T), ptr(out)))
        return out

    def close(self):
        if self.handle:
            lib().epsp_scgd0_plan_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def loop_scgd0(setup, occ, *, eta_init, tol, maxiter=20, eta_min=None, fix_mu=False, mu_start=None,
               sigma_init=None, gpu_tile=None, omega_acoustic, path="direct_fp64", ctx=None):
    """_loop_scgd0 (src/scgd0.jl:189-346) on the GPU: returns Σ[ω, i, T], μ[T], converged[T], history."""
    if maxiter < 1:
        raise ArgumentError(f"maxiter must be at least 1, got {maxiter}")
    plan = Scgd0Plan(setup, path=path, gpu_tile=gpu_tile, omega_acoustic=omega_acoustic, ctx=ctx)
    try:
        return plan.run(occ, eta_init=eta_init, tol=tol, maxiter=maxiter, eta_min=eta_min, fix_mu=fix_mu,
                        mu_start=mu_start, sigma_init=sigma_init)
    finally:
        plan.close()


class LadderPlan:
    """Device-resident tables of one ladder setup (_setup_ladder + _ladder_workspace)."""

    def __init__(self, setup, *, path="direct_fp64", gpu_tile=None, omega_acoustic, ctx: Context | None = None,
                 verbosity=0):
        """verbosity >= 2 logs the set-up phases' times to stderr."""
        if not (omega_acoustic > 0):
            raise ArgumentError(f"ω_acoustic must be positive, got {omega_acoustic}: the shift-grid coupling build "
                                "has no row for a negative phonon frequency")
        self.ctx = ctx or default_context()
        self.M = ModelArrays(setup)
        self.opts = _options(path, gpu_tile, omega_acoustic, verbosity)
        self.handle = C.c_void_p()
        self.ctx.check(lib().epsp_ladder_setup(self.ctx.handle, C.byref(self.M.struct), C.byref(self.opts),
                                               C.byref(self.handle)))

    def gemm_config(self) -> dict:
        """The contraction's tile shape chosen by the autotuner at setup (GEMM_BF16 / GEMM_TF32 plans)."""
        bn, sp, bk, ms, mh = C.c_int32(), C.c_int32(), C.c_int32(), C.c_double(), C.c_double()
        self.ctx.check(lib().epsp_ladder_gemm_config(self.handle, C.byref(bn), C.byref(sp), C.byref(bk), C.byref(ms),
                                                     C.byref(mh)))
        on, pr = C.c_int32(), C.c_int32()
        self.ctx.check(lib().epsp_ladder_gemm_persistent(self.handle, C.byref(on)))
        self.ctx.check(lib().epsp_ladder_gemm_pair(self.handle, C.byref(pr)))
        return dict(bn=bn.value, splits=sp.value, bk=bk.value, persistent=bool(on.value), pair=bool(pr.value),
                    ms=ms.value, ms_heuristic=mh.value)

    def set_gemm_config(self, bn: int, splits: int, bk: int = 64, persistent: bool = False, pair: bool = False):
        """Overrides the autotuner's tile shape of the contraction (GEMM_BF16 / GEMM_TF32 plans);
        persistent: one CTA per SM over all tiles (BF16: bn 256, bk 32 only; TF32: bk 32, either bn);
        pair: CTA pairs computing 256-row tiles (tcgen05 cta_group::2; bn 256, bk 32); both: the
        persistent CTA-pair kernel."""
        self.ctx.check(lib().epsp_ladder_set_gemm_config(self.handle, int(bn), int(splits), int(bk)))
        self.ctx.check(lib().epsp_ladder_set_gemm_persistent(self.handle, 1 if persistent else 0))
        self.ctx.check(lib().epsp_ladder_set_gemm_pair(self.handle, 1 if pair else 0))

    def run(self, sigma, mu, Tlist, Omegas, *, solver="gmres", rtol=1e-2, maxiter=30, store_vertex=False,
            batch_rhs=None):
        """The (T, Ω) loops of _loop_ladder (src/ladder.jl:303-379).

        batch_rhs = R solves up to R (T, Ω) pairs together as GMRES right-hand sides, each from
        x0 = 0 (epsp_ladder_run_batched; GEMM_BF16 / GEMM_TF32 plans); None keeps the reference's order and
        warm starts."""
        M = self.M
        if solver not in ("gmres", "fixed_point"):
            raise ArgumentError(f"solver must be :gmres or :fixed_point, got {solver}")
        if batch_rhs is not None and solver != "gmres":
            raise ArgumentError("batched right-hand sides need solver = :gmres")
        if maxiter < 1:
            raise ArgumentError(f"maxiter must be at least 1, got {maxiter}")
        Tlist = np.ascontiguousarray(Tlist, dtype=np.float64)
        Omegas = np.ascontiguousarray(Omegas, dtype=np.float64)
        if len(Omegas) == 0:
            raise ArgumentError("Ωs must hold at least one probe frequency")
        nT = len(Tlist)
        mu = np.ascontiguousarray(np.broadcast_to(mu, (nT,)), dtype=np.float64)
        if isinstance(sigma, DeviceSigma):  # Σ left on the device by a scGD0 plan
            if sigma.shape != (M.nw, M.ni, nT):
                raise ValueError(f"expected shape {(M.nw, M.ni, nT)}, got {sigma.shape}")
            sig_ptr = sigma.ptr()
        else:
            sig = as_complex_F(sigma, (M.nw, M.ni, nT))
            sig_ptr = cptr(sig)
        out = LadderOutputs(M.nw, M.ni, nT, len(Omegas), maxiter, store_vertex)
        s = {"gmres": abi.EPSP_SOLVER_GMRES, "fixed_point": abi.EPSP_SOLVER_FIXED_POINT}[solver]
        if batch_rhs is not None:
            self.ctx.check(lib().epsp_ladder_run_batched(self.handle, sig_ptr, ptr(mu), ptr(Tlist), nT, ptr(Omegas),
                                                         len(Omegas), float(rtol), int(maxiter), int(batch_rhs),
                                                         ptr(out.sigma_bubble), ptr(out.sigma_ladder),
                                                         out.converged.ctypes.data_as(C.POINTER(C.c_uint8)),
                                                         ptr(out.niter, C.c_int32), C.byref(out.hist), out.J_ptr()))
            return out.result()
        self.ctx.check(lib().epsp_ladder_run(self.handle, sig_ptr, ptr(mu), ptr(Tlist), nT, ptr(Omegas),
                                             len(Omegas), s, float(rtol), int(maxiter), ptr(out.sigma_bubble),
                                             ptr(out.sigma_ladder),
                                             out.converged.ctypes.data_as(C.POINTER(C.c_uint8)),
                                             ptr(out.niter, C.c_int32), C.byref(out.hist), out.J_ptr()))
        return out.result()

    def apply(self, J, sigma_T, mu, T, Omega):
        """LJ = L(J): apply_ladder_kernel! with the propagators of (Σ_T, μ, T, Ω)."""
        M = self.M
        J = as_complex_F(J, (M.nw, 4, 3, 2, M.ni))
        sT = as_complex_F(sigma_T, (M.nw, M.ni))
        LJ = np.zeros_like(J)
        self.ctx.check(lib().epsp_ladder_apply(self.handle, cptr(sT), float(mu), float(T), float(Omega), cptr(J),
                                               cptr(LJ)))
        return LJ

    def close(self):
        if self.handle:
            lib().epsp_ladder_plan_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def loop_ladder(setup, sigma, mu, Tlist, Omegas, *, solver="gmres", rtol=1e-2, maxiter=30, store_vertex=False,
                gpu_tile=None, omega_acoustic, path="direct_fp64", ctx=None):
    """_loop_ladder (src/ladder.jl:303-379) on the GPU."""
    plan = LadderPlan(setup, path=path, gpu_tile=gpu_tile, omega_acoustic=omega_acoustic, ctx=ctx)
    try:
        return plan.run(sigma, mu, Tlist, Omegas, solver=solver, rtol=rtol, maxiter=maxiter, store_vertex=store_vertex)
    finally:
        plan.close()


def apply_ladder_kernel(setup, J, sigma_T, mu, T, Omega, *, omega_acoustic, gpu_tile=None, path="direct_fp64",
                        ctx=None):
    """One application of apply_ladder_kernel! (src/ladder.jl:245-296) on the GPU."""
    plan = LadderPlan(setup, path=path, gpu_tile=gpu_tile, omega_acoustic=omega_acoustic, ctx=ctx)
    try:
        return plan.apply(J, sigma_T, mu, T, Omega)
    finally:
        plan.close()
