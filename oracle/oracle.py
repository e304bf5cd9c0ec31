"""ctypes binding of the CPU oracle (oracle/_build/libepsp_oracle.so).

TEST INFRASTRUCTURE: imported only by tests/, the smoke check and the benchmark's CPU-baseline
leg, as the checker; the product never imports it. The functions take the same setup dictionaries
and keyword arguments as the product's host interface (epspectral_gb300.api), so a parity test
calls both the same way.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.join(os.path.dirname(_HERE), "epspectral.jl_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)

from epspectral_gb300 import abi  # noqa: E402
from epspectral_gb300.abi import (ModelArrays, OccArrays, c_double_p, c_int32_p, epsp_grid,  # noqa: E402
                                  epsp_ladder_history, epsp_model, epsp_occ, epsp_options,
                                  epsp_scgd0_history, ptr)
from epspectral_gb300.grids import ArgumentError  # noqa: E402
from epspectral_gb300.results import LadderOutputs, Scgd0Outputs, as_complex_F, cptr  # noqa: E402

LIB_PATH = os.path.join(_HERE, "_build", "libepsp_oracle.so")


class OracleError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, OpenMP); make rebuilds it when a source is newer
    than the library (force: always)."""
    subprocess.run(["make", "-s", "-C", _HERE] + (["-B"] if force else []), check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        d, i32, i64, u8p = C.c_double, C.c_int32, C.c_int64, P(C.c_uint8)
        msg = [C.c_char_p, i32]
        sig = {
            "epsp_oracle_occ_fermion": (d, [d, d]),
            "epsp_oracle_occ_boson": (d, [d, d]),
            "epsp_oracle_grid_nodes": (None, [P(epsp_grid), c_double_p]),
            "epsp_oracle_trapezoid_weights": (None, [c_double_p, i64, c_double_p]),
            "epsp_oracle_kk_matrix": (None, [c_double_p, i64, c_double_p]),
            "epsp_oracle_interp_table": (None, [c_double_p, i64, c_double_p, i64, c_int32_p, c_double_p]),
            "epsp_oracle_interp_grid": (C.c_int, [P(epsp_grid), c_double_p, i64, c_double_p, i64, c_double_p] + msg),
            "epsp_oracle_ncarrier_spectral": (d, [d, d, c_double_p, c_double_p, i64, d, i32, d, d]),
            "epsp_oracle_imsigma": (C.c_int, [P(epsp_model), P(epsp_options), c_double_p, d, d, c_double_p] + msg),
            "epsp_oracle_scgd0_run": (C.c_int, [P(epsp_model), P(epsp_options), P(epsp_occ), c_double_p, d, i32, d,
                                                i32, c_double_p, c_double_p, c_double_p, c_double_p, u8p,
                                                P(epsp_scgd0_history)] + msg),
            "epsp_oracle_contour_green": (None, [d, d, d, d, d, d, i32, c_double_p]),
            "epsp_oracle_shift_tables": (None, [P(epsp_grid), i64, c_int32_p, c_double_p, c_double_p]),
            "epsp_oracle_nshift": (i64, [P(epsp_model)]),
            "epsp_oracle_bin_coupling": (None, [P(epsp_model), d, d, c_double_p]),
            "epsp_oracle_conductivity": (None, [c_double_p, c_double_p, c_double_p, c_double_p, i64, i64, d, d,
                                                c_double_p]),
            "epsp_oracle_attach_greens": (None, [i64, i64, c_double_p, c_double_p, c_double_p, c_double_p]),
            "epsp_oracle_attach_bare": (None, [i64, i64, c_double_p, c_double_p, c_double_p, c_double_p]),
            "epsp_oracle_ladder_apply": (C.c_int, [P(epsp_model), P(epsp_options), c_double_p, d, d, d, c_double_p,
                                                   c_double_p] + msg),
            "epsp_oracle_ladder_run": (C.c_int, [P(epsp_model), P(epsp_options), c_double_p, c_double_p, c_double_p,
                                                 i64, c_double_p, i64, i32, d, i32, c_double_p, c_double_p, u8p,
                                                 c_int32_p, P(epsp_ladder_history), c_double_p] + msg),
            "epsp_oracle_imsigma_sample": (C.c_int, [P(epsp_model), P(epsp_options), c_double_p, d, d, i64, i64,
                                                     c_double_p] + msg),
            "epsp_oracle_ladder_apply_sample": (C.c_int, [P(epsp_model), P(epsp_options), c_double_p, d, d, d,
                                                          c_double_p, i64, i64, c_double_p] + msg),
            "epsp_oracle_ladder_chunks": (C.c_int, [P(epsp_model), P(epsp_options), P(i64), P(i64), P(i64), i64,
                                                    P(i64)] + msg),
            "epsp_oracle_ladder_chunk_operands": (C.c_int, [P(epsp_model), P(epsp_options), d, c_double_p, i64,
                                                            c_double_p, c_double_p, c_double_p] + msg),
            "epsp_oracle_set_threads": (None, [i32]),
            "epsp_oracle_get_threads": (i32, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _msgbuf():
    return C.create_string_buffer(1024), 1024


def _check(status, buf):
    if status != abi.EPSP_OK:
        m = buf.value.decode(errors="replace")
        if status in (abi.EPSP_EINVAL, abi.EPSP_ENOROOT_MU):
            raise ArgumentError(m)
        raise OracleError(status, m)


def _options(gpu_tile, omega_acoustic):
    return epsp_options(0, 0, int(gpu_tile or 0), float(omega_acoustic))


def set_threads(n: int) -> None:
    lib().epsp_oracle_set_threads(int(n))


def get_threads() -> int:
    return int(lib().epsp_oracle_get_threads())


def occ_fermion(e, T):
    return lib().epsp_oracle_occ_fermion(float(e), float(T))


def occ_boson(e, T):
    return lib().epsp_oracle_occ_boson(float(e), float(T))


def trapezoid_weights(ws):
    ws = np.ascontiguousarray(ws, dtype=np.float64)
    W = np.zeros_like(ws)
    lib().epsp_oracle_trapezoid_weights(ptr(ws), len(ws), ptr(W))
    return W


def kramers_kronig_matrix(ws):
    ws = np.ascontiguousarray(ws, dtype=np.float64)
    K = np.zeros((len(ws), len(ws)), order="F")
    lib().epsp_oracle_kk_matrix(ptr(ws), len(ws), ptr(K))
    return K


def interp_table(ws, xs):
    ws = np.ascontiguousarray(ws, dtype=np.float64)
    xs = np.ascontiguousarray(xs, dtype=np.float64)
    j = np.zeros(len(xs), dtype=np.int32)
    t = np.zeros(len(xs))
    lib().epsp_oracle_interp_table(ptr(ws), len(ws), ptr(xs), len(xs), ptr(j, C.c_int32), ptr(t))
    return j, t


def interp_grid(grid, ys, col, xs):
    """_interp_linear_grid of column `col` of the complex ys[n, ncol] at xs."""
    g = abi.GridArrays(grid)
    ys = np.asfortranarray(ys, dtype=np.complex128)
    xs = np.ascontiguousarray(xs, dtype=np.float64)
    out = np.zeros(len(xs), dtype=np.complex128)
    buf, n = _msgbuf()
    _check(lib().epsp_oracle_interp_grid(C.byref(g.struct), cptr(ys), int(col), ptr(xs), len(xs), cptr(out),
                                         buf, n), buf)
    return out


def ncarrier_spectral(mu, T, wa, D, W, count_holes, nstates_base, spin_degeneracy):
    wa = np.ascontiguousarray(wa, dtype=np.float64)
    D = np.ascontiguousarray(D, dtype=np.float64)
    return lib().epsp_oracle_ncarrier_spectral(float(mu), float(T), ptr(wa), ptr(D), len(wa), float(W),
                                               int(bool(count_holes)), float(nstates_base),
                                               float(spin_degeneracy))


def imsigma(setup, sigma_in, mu, T, imsigma0=None, *, omega_acoustic, gpu_tile=None):
    """add_fan_migdal_imsigma! at one temperature: returns imsigma0 + the Fan-Migdal sum."""
    M = ModelArrays(setup)
    sin = as_complex_F(sigma_in, (M.nw, M.ni))
    out = (np.zeros((M.nw, M.ni), order="F") if imsigma0 is None
           else np.array(imsigma0, dtype=np.float64, order="F", copy=True))
    opts = _options(gpu_tile, omega_acoustic)
    buf, n = _msgbuf()
    _check(lib().epsp_oracle_imsigma(C.byref(M.struct), C.byref(opts), cptr(sin), float(mu), float(T), ptr(out),
                                     buf, n), buf)
    return out


def loop_scgd0(setup, occ, *, eta_init, tol, maxiter=20, eta_min=None, fix_mu=False, mu_start=None,
               sigma_init=None, gpu_tile=None, omega_acoustic):
    """_loop_scgd0 on the CPU (src/scgd0.jl:189-346)."""
    M = ModelArrays(setup)
    O = OccArrays(occ)
    nT = len(O.Tlist)
    eta_min = np.ascontiguousarray(np.broadcast_to(0.0 if eta_min is None else eta_min, (nT,)), dtype=np.float64)
    mu0 = np.ascontiguousarray(np.broadcast_to(setup.get("mu_start", 0.0) if mu_start is None else mu_start, (nT,)),
                               dtype=np.float64)
    sinit = None if sigma_init is None else as_complex_F(sigma_init, (M.nw, M.ni, nT))
    out = Scgd0Outputs(M.nw, M.ni, nT, maxiter)
    opts = _options(gpu_tile, omega_acoustic)
    buf, n = _msgbuf()
    _check(lib().epsp_oracle_scgd0_run(C.byref(M.struct), C.byref(opts), C.byref(O.struct), ptr(eta_min),
                                       float(eta_init), int(maxiter), float(tol), int(bool(fix_mu)), ptr(mu0),
                                       cptr(sinit), out.sigma_ptr(), ptr(out.mu),
                                       out.converged.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(out.hist),
                                       buf, n), buf)
    return out.result()


def contour_green(w, eps, S, mu, T, c12):
    o = np.zeros(2)
    lib().epsp_oracle_contour_green(float(w), float(eps), float(np.real(S)), float(np.imag(S)), float(mu), float(T),
                                    int(c12), ptr(o))
    return complex(o[0], o[1])


def shift_tables(grid, nshift):
    g = abi.GridArrays(grid)
    nw = len(g.offsets)
    klo = np.zeros((nw, nshift, 2), dtype=np.int32, order="F")
    wlo = np.zeros((nw, nshift, 2), order="F")
    whi = np.zeros((nw, nshift, 2), order="F")
    lib().epsp_oracle_shift_tables(C.byref(g.struct), int(nshift), ptr(klo, C.c_int32), ptr(wlo), ptr(whi))
    return klo, wlo, whi


def nshift(setup):
    M = ModelArrays(setup)
    return int(lib().epsp_oracle_nshift(C.byref(M.struct)))


def bin_coupling(setup, T, *, omega_acoustic):
    """B[m, f, i, type] of all inner states in star order (one chunk)."""
    M = ModelArrays(setup)
    ns = int(lib().epsp_oracle_nshift(C.byref(M.struct)))
    B = np.zeros((ns, M.nf, M.ni, 2), order="F")
    lib().epsp_oracle_bin_coupling(C.byref(M.struct), float(omega_acoustic), float(T), ptr(B))
    return B


def conductivity(J, v, w_i, Ww, Omega, T):
    J = np.asfortranarray(J, dtype=np.complex128)
    nw, ni = J.shape[0], J.shape[4]
    v = np.asfortranarray(v, dtype=np.float64)
    w_i = np.ascontiguousarray(w_i, dtype=np.float64)
    Ww = np.ascontiguousarray(Ww, dtype=np.float64)
    s = np.zeros((3, 3), order="F")
    lib().epsp_oracle_conductivity(cptr(J), ptr(v), ptr(w_i), ptr(Ww), nw, ni, float(Omega), float(T), ptr(s))
    return s


def attach_greens(Gm, Gp, X):
    """attach_greens_to_vertex! (src/ladder_kernel.jl:61-67): J = Gm X Gp per (ω, cart, c0, i);
    Gm, Gp [nω, 4, ni], X [nω, 4, 3, 2, ni]."""
    nw, ni = Gm.shape[0], Gm.shape[2]
    Gm, Gp = as_complex_F(Gm, (nw, 4, ni)), as_complex_F(Gp, (nw, 4, ni))
    X = as_complex_F(X, (nw, 4, 3, 2, ni))
    J = np.zeros_like(X)
    lib().epsp_oracle_attach_greens(nw, ni, cptr(Gm), cptr(Gp), cptr(X), cptr(J))
    return J


def attach_bare(Gm, Gp, v):
    """attach_greens_to_bare_vertex! (src/ladder_kernel.jl:70-73): J0 for the velocities v [3, ni]."""
    nw, ni = Gm.shape[0], Gm.shape[2]
    Gm, Gp = as_complex_F(Gm, (nw, 4, ni)), as_complex_F(Gp, (nw, 4, ni))
    v = np.asfortranarray(v, dtype=np.float64)
    J0 = np.zeros((nw, 4, 3, 2, ni), dtype=np.complex128, order="F")
    lib().epsp_oracle_attach_bare(nw, ni, cptr(Gm), cptr(Gp), ptr(v), cptr(J0))
    return J0


def apply_ladder_kernel(setup, J, sigma_T, mu, T, Omega, *, omega_acoustic, gpu_tile=None):
    """apply_ladder_kernel! with the propagators of (sigma_T, mu, T, Omega)."""
    M = ModelArrays(setup)
    J = as_complex_F(J, (M.nw, 4, 3, 2, M.ni))
    sT = as_complex_F(sigma_T, (M.nw, M.ni))
    LJ = np.zeros_like(J)
    opts = _options(gpu_tile, omega_acoustic)
    buf, n = _msgbuf()
    _check(lib().epsp_oracle_ladder_apply(C.byref(M.struct), C.byref(opts), cptr(sT), float(mu), float(T),
                                          float(Omega), cptr(J), cptr(LJ), buf, n), buf)
    return LJ


def loop_ladder(setup, sigma, mu, Tlist, Omegas, *, solver="gmres", rtol=1e-2, maxiter=30, store_vertex=False,
                gpu_tile=None, omega_acoustic):
    """_loop_ladder on the CPU (src/ladder.jl:303-379)."""
    M = ModelArrays(setup)
    Tlist = np.ascontiguousarray(Tlist, dtype=np.float64)
    nT = len(Tlist)
    Omegas = np.ascontiguousarray(Omegas, dtype=np.float64)
    mu = np.ascontiguousarray(np.broadcast_to(mu, (nT,)), dtype=np.float64)
    sig = as_complex_F(sigma, (M.nw, M.ni, nT))
    out = LadderOutputs(M.nw, M.ni, nT, len(Omegas), maxiter, store_vertex)
    s = {"gmres": abi.EPSP_SOLVER_GMRES, "fixed_point": abi.EPSP_SOLVER_FIXED_POINT}.get(solver, -1)
    opts = _options(gpu_tile, omega_acoustic)
    buf, n = _msgbuf()
    _check(lib().epsp_oracle_ladder_run(C.byref(M.struct), C.byref(opts), cptr(sig), ptr(mu), ptr(Tlist), nT,
                                        ptr(Omegas), len(Omegas), s, float(rtol), int(maxiter),
                                        ptr(out.sigma_bubble), ptr(out.sigma_ladder),
                                        out.converged.ctypes.data_as(C.POINTER(C.c_uint8)),
                                        ptr(out.niter, C.c_int32), C.byref(out.hist), out.J_ptr(), buf, n), buf)
    return out.result()


def imsigma_sample(setup, sigma_in, mu, T, i0, i1, *, omega_acoustic, gpu_tile=None):
    """The Fan-Migdal sum of the outer states [i0, i1) only (a bounded CPU-baseline sample)."""
    M = ModelArrays(setup)
    sin = as_complex_F(sigma_in, (M.nw, M.ni))
    out = np.zeros((M.nw, M.ni), order="F")
    opts = _options(gpu_tile, omega_acoustic)
    buf, n = _msgbuf()
    _check(lib().epsp_oracle_imsigma_sample(C.byref(M.struct), C.byref(opts), cptr(sin), float(mu), float(T), int(i0),
                                            int(i1), ptr(out), buf, n), buf)
    return out


def ladder_apply_sample(setup, J, sigma_T, mu, T, Omega, i0, i1, *, omega_acoustic, gpu_tile=None):
    """apply_ladder_kernel! for the output states [i0, i1) only: LJ [nω, 4, 3, 2, i1 - i0], bitwise the
    slice of the full application (a bounded sample at sizes the full application is too slow for)."""
    M = ModelArrays(setup)
    J = as_complex_F(J, (M.nw, 4, 3, 2, M.ni))
    sT = as_complex_F(sigma_T, (M.nw, M.ni))
    LJ = np.zeros((M.nw, 4, 3, 2, int(i1) - int(i0)), dtype=np.complex128, order="F")
    opts = _options(gpu_tile, omega_acoustic)
    buf, n = _msgbuf()
    _check(lib().epsp_oracle_ladder_apply_sample(C.byref(M.struct), C.byref(opts), cptr(sT), float(mu), float(T),
                                                 float(Omega), cptr(J), int(i0), int(i1), cptr(LJ), buf, n), buf)
    return LJ


def ladder_chunks(setup, *, omega_acoustic, gpu_tile=None):
    """The chunks of apply_ladder_kernel! (whole stars within CHUNK_BYTES, src/ladder.jl:180-202):
    ([(i_lo, i_hi), ...], nshift)."""
    M = ModelArrays(setup)
    opts = _options(gpu_tile, omega_acoustic)
    buf, n = _msgbuf()
    cnt, ns = C.c_int64(), C.c_int64()
    cap = M.ni + 1
    lo, hi = (C.c_int64 * cap)(), (C.c_int64 * cap)()
    _check(lib().epsp_oracle_ladder_chunks(C.byref(M.struct), C.byref(opts), C.byref(cnt), lo, hi, cap, C.byref(ns),
                                           buf, n), buf)
    return [(int(lo[c]), int(hi[c])) for c in range(cnt.value)], int(ns.value)


def ladder_chunk_operands(setup, J, T, chunk, *, omega_acoustic, gpu_tile=None):
    """One chunk's operands of C± += X± B̃ (src/ladder.jl:254-290): X+ and X- [16 nω, nk] and B̃
    [nk, 6 ni] (Fortran order, nk = nshift·3·(i_hi - i_lo)), so that the product can run as a BLAS
    DGEMM, as the reference's mul! does."""
    M = ModelArrays(setup)
    J = as_complex_F(J, (M.nw, 4, 3, 2, M.ni))
    chunks, ns = ladder_chunks(setup, omega_acoustic=omega_acoustic, gpu_tile=gpu_tile)
    i_lo, i_hi = chunks[int(chunk)]
    nk = ns * 3 * (i_hi - i_lo)
    Xp = np.empty((16 * M.nw, nk), order="F")
    Xm = np.empty((16 * M.nw, nk), order="F")
    Bt = np.empty((nk, 6 * M.ni), order="F")
    opts = _options(gpu_tile, omega_acoustic)
    buf, n = _msgbuf()
    _check(lib().epsp_oracle_ladder_chunk_operands(C.byref(M.struct), C.byref(opts), float(T), cptr(J), int(chunk),
                                                   ptr(Xp), ptr(Xm), ptr(Bt), buf, n), buf)
    return Xp, Xm, Bt
