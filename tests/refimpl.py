"""Independent references of the reference's own test suite, restated in numpy / plain Python.

These do not call the oracle: each follows the test helper it cites, so a test can pin the oracle
(and through it the GPU library) on the reference's known answers.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.optimize import brentq


def pseudorandom(*dims, seed):
    """sin.(seed .* (1:N).^1.5) reshaped column-major (test/common.jl:11)."""
    n = int(np.prod(dims))
    return np.sin(seed * np.arange(1, n + 1, dtype=np.float64) ** 1.5).reshape(dims, order="F")


def pseudorandom_complex(*dims, seed):
    """test/common.jl:12-13."""
    return pseudorandom(*dims, seed=seed) + 1j * pseudorandom(*dims, seed=seed + 0.5)


def fermi(x, T):
    return 1.0 / (np.exp(x / T) + 1.0)


def kk_matrix(ws):
    """The spline Kramers-Kronig matrix, written from its definition (src/frequency_grids.jl:13-44)."""
    ws = np.asarray(ws, dtype=np.float64)
    N = len(ws)
    xs = np.concatenate([[ws[0] - (ws[1] - ws[0])], ws, [ws[-1] + (ws[-1] - ws[-2])]])

    def xlogx(x):
        with np.errstate(divide="ignore", invalid="ignore"):
            return np.where(x == 0, 0.0, x * np.log(np.abs(x)))

    x = xs[1:N + 1][:, None]
    x1, x2, x3 = xs[None, 0:N], xs[None, 1:N + 1], xs[None, 2:N + 2]
    return (xlogx(x1 - x) / (x2 - x1) - xlogx(x2 - x) * (x3 - x1) / (x2 - x1) / (x3 - x2)
            + xlogx(x3 - x) / (x3 - x2)) / math.pi


def trapezoid(ws):
    ws = np.asarray(ws)
    n = len(ws)
    return np.array([(ws[min(j + 1, n - 1)] - ws[max(j - 1, 0)]) / 2 for j in range(n)])


def interp_flat(ws, ys, x):
    """Gridded(Linear()) with Flat() extrapolation (Interpolations.jl), complex ys."""
    ys = np.asarray(ys)
    return np.interp(x, ws, ys.real) + 1j * np.interp(x, ws, ys.imag)


def holstein_energies(nk, t):
    from epspectral_gb300.synthetic import holstein_1d_energies
    return holstein_1d_energies(nk, t)


def holstein_oneshot_imsigma(ws, *, nk, t, w0, g2, T, mu, eta):
    """Closed-form one-shot Im Σ (test/holstein_1d_reference.jl:27-35)."""
    nB = 1.0 / math.expm1(w0 / T)
    eps = holstein_energies(nk, t)
    out = np.zeros(len(ws))
    for k, w in enumerate(ws):
        s = 0.0
        for e in eps:
            s += (eta / ((w + w0 - e) ** 2 + eta ** 2) * (nB + fermi(w + w0 - mu, T))
                  + eta / ((w - w0 - e) ** 2 + eta ** 2) * (nB + 1 - fermi(w - w0 - mu, T)))
        out[k] = -g2 / nk * s
    return out


def holstein_local_scgd0(ws, wsa, *, nk, t, w0, g2, T, eta_init, mu_start, niter, fix_mu, n_target,
                         spin_degeneracy, eta_min=0.0):
    """The scalar local scGD0 iteration (test/holstein_1d_reference.jl:42-68)."""
    eps = holstein_energies(nk, t)
    nB = 1.0 / math.expm1(w0 / T)
    Wa = trapezoid(wsa)
    K = kk_matrix(ws)
    S = np.full(len(ws), complex(0.0, -eta_init))
    mu = mu_start
    for _ in range(niter):
        Sin = S.real + 1j * np.minimum(S.imag, -eta_min)

        def img_loc(x):
            s = interp_flat(ws, Sin, x)
            return np.imag(np.sum(1.0 / (x[:, None] - eps[None, :] - s[:, None]), axis=1) / nk)

        ImS = g2 * (img_loc(ws + w0) * (nB + fermi(ws + w0 - mu, T))
                    + img_loc(ws - w0) * (nB + 1 - fermi(ws - w0 - mu, T)))
        S = K @ ImS + 1j * ImS
        if fix_mu:
            continue
        Ssp = interp_flat(ws, S, wsa)
        D = np.sum(-np.imag(1.0 / (wsa[:, None] - eps[None, :] - Ssp[:, None])) / math.pi, axis=1) / nk * Wa
        f = lambda m: spin_degeneracy * np.sum(D * fermi(wsa - m, T)) - n_target
        mu = brentq(f, wsa[0] - 0.1, wsa[-1] + 0.1, xtol=1e-15, rtol=1e-15, maxiter=500)
    return S, mu


def naive_imsigma(ws, sigma_in, g2, wq, eps_f, f_to_i, w_f, mu, T, w_ac, imsigma0):
    """Plain (ω, ν, i, f) loop of test/test_scgd0_kernel.jl:133-143 (per-pair ωq[ν, i, f])."""
    nm, ni, nf = g2.shape
    out = imsigma0.copy()
    for f in range(nf):
        for i in range(ni):
            for nu in range(nm):
                q = wq[nu, i, f]
                if q < w_ac:
                    continue
                n = 1.0 / math.expm1(q / T)
                Sp = interp_flat(ws, sigma_in[:, f_to_i[f]], ws + q)
                Sm = interp_flat(ws, sigma_in[:, f_to_i[f]], ws - q)
                out[:, i] += w_f[f] * g2[nu, i, f] * (
                    np.imag(1.0 / (ws + q - eps_f[f] - Sp)) * (n + fermi(ws + q - mu, T))
                    + np.imag(1.0 / (ws - q - eps_f[f] - Sm)) * (n + 1 - fermi(ws - q - mu, T)))
    return out


def hat_value(y, ws, x):
    """Linear interpolation of y on ws, zero outside (test/test_ladder_kernel.jl:68-73)."""
    if x < ws[0] or x > ws[-1]:
        return 0.0 * y[0]
    k = min(int(np.searchsorted(ws, x, side="right")) - 1, len(ws) - 2)
    t = (x - ws[k]) / (ws[k + 1] - ws[k])
    return (1 - t) * y[k] + t * y[k + 1]


def contour_green(w, e, S, mu, T, c12):
    GR = 1.0 / (w - e - S)
    GA = np.conj(GR)
    GK = (GR - GA) * (1 - 2 * fermi(w - mu, T))
    return [(GR + GA + GK) / 2, (GR - GA + GK) / 2, (-GR + GA + GK) / 2, (-GR - GA + GK) / 2][c12]


def propagators(ws, sigma_T, eps_i, mu, T, Omega):
    """ladder_propagators of test/ladder_fixtures.jl:45-53: Gm, Gp [nω, 4, ni]."""
    nw, ni = sigma_T.shape
    Gm = np.zeros((nw, 4, ni), dtype=complex)
    Gp = np.zeros((nw, 4, ni), dtype=complex)
    for i in range(ni):
        sm = interp_flat(ws, sigma_T[:, i], ws - Omega / 2)
        sp = interp_flat(ws, sigma_T[:, i], ws + Omega / 2)
        for c in range(4):
            Gm[:, c, i] = contour_green(ws - Omega / 2, eps_i[i], sm, mu, T, c)
            Gp[:, c, i] = contour_green(ws + Omega / 2, eps_i[i], sp, mu, T, c)
    return Gm, Gp


def naive_apply_ladder(setup, J, Gm, Gp, T, w_ac):
    """L(J) = -Gm (s ⊙ K[J]) Gp by loops (test/test_ladder_kernel.jl:76-116), exact hat-basis
    shifts at ωs[j] ± ωq, no shift grid."""
    g2 = np.asarray(setup["g2"], dtype=np.float64)
    nm, ni, nf = g2.shape
    ws = setup["omegas"].nodes()
    nw = len(ws)
    R, f_to_i, w_f = setup["R"], setup["f_to_i"], setup["w_f"]
    oph, iq, iks_i, iks_f = setup["omega_ph"], setup["iq_kk"], setup["iks_i"], setup["iks_f"]
    F = np.zeros((nw, 4, 3, 2, nf), dtype=complex)
    for f in range(nf):
        F[:, :, :, :, f] = np.einsum("ab,wcbd->wcad", R[:, :, f], J[:, :, :, :, f_to_i[f]])
    Up, Um, Vp, Vm = (np.zeros((nw, 4, 3, 2, ni), dtype=complex) for _ in range(4))
    for i in range(ni):
        for f in range(nf):
            for nu in range(nm):
                q = oph[nu, iq[iks_i[i], iks_f[f]]]
                if q < w_ac:
                    continue
                w = w_f[f] * g2[nu, i, f]
                n = 1.0 / math.expm1(q / T)
                Fy = F[:, :, :, :, f].reshape(nw, -1, order="F")
                up = np.array([hat_value(Fy, ws, ws[j] + q) for j in range(nw)]) * w
                um = np.array([hat_value(Fy, ws, ws[j] - q) for j in range(nw)]) * w
                Up[:, :, :, :, i] += up.reshape(nw, 4, 3, 2, order="F")
                Um[:, :, :, :, i] += um.reshape(nw, 4, 3, 2, order="F")
                Vp[:, :, :, :, i] += n * up.reshape(nw, 4, 3, 2, order="F")
                Vm[:, :, :, :, i] += n * um.reshape(nw, 4, 3, 2, order="F")
    K = kk_matrix(ws)
    KY = (K @ ((Up - Um) / 2).reshape(nw, -1, order="F")).reshape(Up.shape, order="F")
    LJ = np.zeros((nw, 4, 3, 2, ni), dtype=complex)
    s = np.array([[1, -1], [-1, 1]])
    for i in range(ni):
        for c0 in range(2):
            for a in range(3):
                k11 = -1j * KY[:, 0, a, c0, i] - (Up[:, 0, a, c0, i] + Um[:, 0, a, c0, i]) / 2 - (Vp[:, 0, a, c0, i] + Vm[:, 0, a, c0, i])
                k22 = 1j * KY[:, 3, a, c0, i] - (Up[:, 3, a, c0, i] + Um[:, 3, a, c0, i]) / 2 - (Vp[:, 3, a, c0, i] + Vm[:, 3, a, c0, i])
                k21 = -(Vp[:, 1, a, c0, i] + Um[:, 1, a, c0, i] + Vm[:, 1, a, c0, i])
                k12 = -(Up[:, 2, a, c0, i] + Vp[:, 2, a, c0, i] + Vm[:, 2, a, c0, i])
                for j in range(nw):
                    Kab = s * np.array([[k11[j], k12[j]], [k21[j], k22[j]]])
                    gm = Gm[j, :, i].reshape(2, 2, order="F")
                    gp = Gp[j, :, i].reshape(2, 2, order="F")
                    LJ[j, :, a, c0, i] = -(gm @ Kab @ gp).reshape(4, order="F")
    return LJ


def spectral_bubble(ws, sigma_T, eps_i, w_i, v, mu, T, Omega):
    """σ from spectral functions (test/test_ladder_bubble.jl:10-26)."""
    Ww = trapezoid(ws)
    s = np.zeros((3, 3))
    for i in range(len(eps_i)):
        A = lambda w: -np.imag(1.0 / (w - eps_i[i] - interp_flat(ws, sigma_T[:, i], w))) / math.pi
        if Omega == 0:
            fac = fermi(ws - mu, T) * (1 - fermi(ws - mu, T)) / T
        else:
            fac = (fermi(ws - Omega / 2 - mu, T) - fermi(ws + Omega / 2 - mu, T)) / Omega
        win = np.sum(Ww * A(ws - Omega / 2) * A(ws + Omega / 2) * fac)
        s += math.pi * w_i[i] * win * np.outer(v[:, i], v[:, i])
    return s
