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


def hat_matrix(ws, q):
    """S with (S y)[j] = hat_value(y, ws, ws[j] + q): linear interpolation at ωs[j] + q, zero
    outside the grid (test/test_ladder_kernel.jl:68-73)."""
    nw = len(ws)
    S = np.zeros((nw, nw))
    for j in range(nw):
        x = ws[j] + q
        if x < ws[0] or x > ws[-1]:
            continue
        k = min(int(np.searchsorted(ws, x, side="right")) - 1, nw - 2)
        t = (x - ws[k]) / (ws[k + 1] - ws[k])
        S[j, k] += 1 - t
        S[j, k + 1] += t
    return S


def naive_apply_ladder(setup, J, Gm, Gp, T, w_ac):
    """L(J) = -Gm (s ⊙ K[J]) Gp by loops over (i, f, ν) (test/test_ladder_kernel.jl:76-116), with the
    vertex shifted by exact hat-basis interpolation at ωs[j] ± ωq and no shift grid. Terms with the
    same ωq share one interpolation matrix (a regrouping of the same sum)."""
    g2 = np.asarray(setup["g2"], dtype=np.float64)
    nm, ni, nf = g2.shape
    ws = setup["omegas"].nodes()
    nw = len(ws)
    R, f_to_i, w_f = setup["R"], setup["f_to_i"], setup["w_f"]
    oph, iq, iks_i, iks_f = setup["omega_ph"], setup["iq_kk"], setup["iks_i"], setup["iks_f"]
    F = np.zeros((nw, 4, 3, 2, nf), dtype=complex)
    for f in range(nf):
        F[:, :, :, :, f] = np.einsum("ab,wcbd->wcad", R[:, :, f], J[:, :, :, :, f_to_i[f]])
    Ff = F.reshape(nw, 24, nf, order="F")
    U = {s: np.zeros((nw, 24, ni), dtype=complex) for s in (1, -1)}
    V = {s: np.zeros((nw, 24, ni), dtype=complex) for s in (1, -1)}
    cache = {}
    for i in range(ni):
        groups = {}
        for f in range(nf):
            for nu in range(nm):
                q = oph[nu, iq[iks_i[i], iks_f[f]]]
                if q < w_ac:
                    continue
                w = w_f[f] * g2[nu, i, f]
                n = 1.0 / math.expm1(q / T)
                acc = groups.setdefault(q, [np.zeros((nw, 24), dtype=complex), np.zeros((nw, 24), dtype=complex)])
                acc[0] += w * Ff[:, :, f]
                acc[1] += (n * w) * Ff[:, :, f]
        for q, (a, b) in groups.items():
            for s in (1, -1):
                key = s * q
                if key not in cache:
                    cache[key] = hat_matrix(ws, key)
                U[s][:, :, i] += cache[key] @ a
                V[s][:, :, i] += cache[key] @ b
    Up, Um, Vp, Vm = (X.reshape(nw, 4, 3, 2, ni, order="F") for X in (U[1], U[-1], V[1], V[-1]))
    K = kk_matrix(ws)
    KY = (K @ ((Up - Um) / 2).reshape(nw, -1, order="F")).reshape(Up.shape, order="F")
    k11 = -1j * KY[:, 0] - (Up[:, 0] + Um[:, 0]) / 2 - (Vp[:, 0] + Vm[:, 0])
    k22 = 1j * KY[:, 3] - (Up[:, 3] + Um[:, 3]) / 2 - (Vp[:, 3] + Vm[:, 3])
    k21 = -(Vp[:, 1] + Um[:, 1] + Vm[:, 1])
    k12 = -(Up[:, 2] + Vp[:, 2] + Vm[:, 2])
    # s ⊙ K with s = [1 -1; -1 1]; the contour matrix of pair index c12 = c1 + 2 c2.
    Kab = np.stack([k11, -k21, -k12, k22], axis=1)  # [nω, c12, cart, c0, i]
    LJ = np.zeros((nw, 4, 3, 2, ni), dtype=complex)
    for c1 in range(2):
        for c2 in range(2):
            acc = 0
            for a in range(2):
                for b in range(2):
                    acc = acc + (Gm[:, c1 + 2 * a, None, None, :] * Kab[:, a + 2 * b]
                                 * Gp[:, b + 2 * c2, None, None, :])
            LJ[:, c1 + 2 * c2] = -acc
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
