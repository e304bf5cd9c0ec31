"""Output buffers and result records of the two loops, shared by every caller of the ABI.

`Scgd0Outputs` holds what `_loop_scgd0` returns (src/scgd0.jl:340-345): Σ[ω, i, T], μ[T],
converged[T] and `history` (err, μ, min_spectral_weight per (T, iteration), wall per iteration,
iter_frozen per T), trimmed to the iterations run. `LadderOutputs` holds what `_loop_ladder`
returns (src/ladder.jl:376-378).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .abi import c_double_p, c_int32_p, epsp_ladder_history, epsp_scgd0_history, ptr


class DeviceSigma:
    """The self-energy of a scGD0 plan's last run left on the device (epsp_scgd0_sigma_device):
    Σ [nω, ni, nT] complex, valid until the plan's next run or close. LadderPlan.run takes it as
    its sigma without a host round trip; a stale one (the plan ran again or was closed) raises
    instead of handing the ladder memory that holds another Σ or none."""

    def __init__(self, plan, address: int, shape, run_gen: int):
        self.plan, self.address, self.shape, self.run_gen = plan, int(address), tuple(shape), int(run_gen)

    def valid(self) -> bool:
        return bool(self.plan.handle) and self.plan.run_gen == self.run_gen

    def ptr(self):
        if not self.valid():
            raise ValueError("this device Σ is stale: its scGD0 plan has run again or was closed")
        return C.cast(C.c_void_p(self.address), c_double_p)


class Scgd0Outputs:
    def __init__(self, nw: int, ni: int, nT: int, maxiter: int, sigma_to_host: bool = True):
        self.sigma = np.zeros((nw, ni, nT), dtype=np.complex128, order="F") if sigma_to_host else None
        self.mu = np.zeros(nT)
        self.converged = np.zeros(nT, dtype=np.uint8)
        self.err = np.full((nT, maxiter), np.nan, order="F")
        self.hmu = np.full((nT, maxiter), np.nan, order="F")
        self.minA = np.full((nT, maxiter), np.nan, order="F")
        self.wall = np.zeros(maxiter)
        self.iter_frozen = np.zeros(nT, dtype=np.int32)
        self.hist = epsp_scgd0_history(ptr(self.err), ptr(self.hmu), ptr(self.minA), ptr(self.wall),
                                       ptr(self.iter_frozen, C.c_int32), 0, 0)

    def sigma_ptr(self):
        return c_double_p() if self.sigma is None else self.sigma.ctypes.data_as(c_double_p)

    def result(self) -> dict:
        n = int(self.hist.niter)
        return dict(
            sigma=self.sigma, mu=self.mu.copy(), converged=self.converged.astype(bool),
            history=dict(err=self.err[:, :n].copy(), mu=self.hmu[:, :n].copy(),
                         min_spectral_weight=self.minA[:, :n].copy(), wall=self.wall[:n].copy(),
                         iter_frozen=self.iter_frozen.copy()),
            niter=n)


class LadderOutputs:
    def __init__(self, nw: int, ni: int, nT: int, nO: int, maxiter: int, store_vertex: bool):
        self.sigma_bubble = np.zeros((3, 3, nO, nT), order="F")
        self.sigma_ladder = np.zeros((3, 3, nO, nT), order="F")
        self.converged = np.zeros((nO, nT), dtype=np.uint8, order="F")
        self.niter = np.zeros((nO, nT), dtype=np.int32, order="F")
        self.norms = np.zeros((maxiter + 1, nO, nT), order="F")
        self.nnorms = np.zeros((nO, nT), dtype=np.int32, order="F")
        self.sigma_iter = np.zeros((3, 3, maxiter, nO, nT), order="F")
        self.nsigma = np.zeros((nO, nT), dtype=np.int32, order="F")
        self.J = (np.zeros((nw, 4, 3, 2, ni, nO, nT), dtype=np.complex128, order="F")
                  if store_vertex else None)
        self.hist = epsp_ladder_history(ptr(self.norms), ptr(self.nnorms, C.c_int32),
                                        ptr(self.sigma_iter), ptr(self.nsigma, C.c_int32))

    def J_ptr(self):
        return self.J.ctypes.data_as(c_double_p) if self.J is not None else c_double_p()

    def result(self) -> dict:
        nO, nT = self.niter.shape
        history = np.empty((nO, nT), dtype=object)
        for iT in range(nT):
            for iO in range(nO):
                history[iO, iT] = dict(
                    norms=self.norms[: self.nnorms[iO, iT], iO, iT].copy(),
                    sigma_iter=[self.sigma_iter[:, :, k, iO, iT].copy()
                                for k in range(self.nsigma[iO, iT])])
        return dict(sigma_bubble=self.sigma_bubble, sigma_ladder=self.sigma_ladder,
                    converged=self.converged.astype(bool), niter=self.niter.astype(np.int64),
                    history=history, J=self.J)


def as_complex_F(a, shape) -> np.ndarray:
    a = np.asfortranarray(np.asarray(a, dtype=np.complex128))
    if a.shape != tuple(shape):
        raise ValueError(f"expected shape {tuple(shape)}, got {a.shape}")
    return a


def cptr(a: np.ndarray | None):
    """Pointer to interleaved complex data as double* (NULL for None)."""
    if a is None:
        return c_double_p()
    return a.ctypes.data_as(c_double_p)


__all__ = ["DeviceSigma", "Scgd0Outputs", "LadderOutputs", "as_complex_F", "cptr", "c_int32_p"]
