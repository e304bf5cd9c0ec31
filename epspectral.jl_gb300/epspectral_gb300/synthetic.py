"""Seeded synthetic inputs in the layout of the reference's `setup` / `ladder` NamedTuples.

The reference extracts these arrays with ElectronPhonon (src/scgd0.jl:127-184,
src/ladder.jl:112-158). Two models are built here instead, deterministically:

* `holstein_1d_setup`: the 1D Holstein chain exactly as the reference's test fixture builds it by
  hand (test/holstein_1d_reference.jl:80-95): outer states on the wedge j = 0..nk/2 of k -> -k,
  inner states on the full grid, one Einstein mode, constant g2. With `symmetry=False` the outer
  states are the full grid (the `symmetry = nothing` case of test/ladder_fixtures.jl:22-31).
* `cubic_t2g_setup`: a three-band cubic t2g tight-binding model on an N^3 grid with the full O_h
  point group (which contains inversion, so time reversal adds nothing), dispersionless modes and
  log-normal g2 drawn from a seed: the benchmark configurations' model.

Energies are in eV. Index arrays are 0-based. Every array is returned in the reference's index order
and column-major layout (numpy order='F').
"""
from __future__ import annotations

import itertools
import math
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from .grids import FrequencyGrid

KELVIN = 8.617333262e-5  # eV per K


def cospi(x: float) -> float:
    """cos(pi x) with exact zeros at half-integers (Julia's cospi up to an ulp)."""
    r = math.fmod(abs(x), 2.0)
    if r > 1.0:
        r = 2.0 - r
    sign = 1.0
    if r > 0.5:
        r, sign = 1.0 - r, -1.0
    if r == 0.5:
        return 0.0
    if r > 0.25:
        return sign * math.sin(math.pi * (0.5 - r))
    return sign * math.cos(math.pi * r)


def holstein_1d_energies(nk: int, t: float) -> np.ndarray:
    """ε_j = -2t cospi(2j/nk), test/holstein_1d_reference.jl:24."""
    return np.array([-2.0 * t * cospi(2.0 * j / nk) for j in range(nk)])


def spectral_grid_default(ws: FrequencyGrid) -> FrequencyGrid:
    """The default ωs_spectral: uniform on the span of ωs with step ωs.dω_min (src/scgd0.jl:89-92)."""
    w = ws.nodes()
    return FrequencyGrid.uniform(w[0], w[-1], ws.dw_min)


def holstein_1d_setup(nk: int, t: float, omega0: float, g2: float, ws: FrequencyGrid,
                      symmetry: bool = True, omegas_spectral: FrequencyGrid | None = None,
                      g2_dtype=np.float64) -> dict:
    """The hand-built 1D Holstein setup (test/holstein_1d_reference.jl:80-95), with the ladder's
    rotations R (TR-odd: the partner -k of a wedge state carries -1) and velocities v = dε/dk."""
    eps = holstein_1d_energies(nk, t)
    if symmetry:
        ni = nk // 2 + 1
        f_to_i = np.array([min(j, nk - j) for j in range(nk)], dtype=np.int32)
        w_i = np.array([(1.0 if (j == 0 or 2 * j == nk) else 2.0) / nk for j in range(ni)])
    else:
        ni = nk
        f_to_i = np.arange(nk, dtype=np.int32)
        w_i = np.full(nk, 1.0 / nk)
    R = np.zeros((3, 3, nk), order="F")
    for f in range(nk):
        s = -1.0 if (symmetry and f != f_to_i[f]) else 1.0
        R[:, :, f] = s * np.eye(3)
    v = np.zeros((3, ni), order="F")
    for i in range(ni):
        v[0, i] = 2.0 * t * math.sin(2.0 * math.pi * i / nk)
    iq_kk = np.array([[(jf - ji) % nk for jf in range(nk)] for ji in range(ni)], dtype=np.int32)
    return dict(
        g2=np.full((1, ni, nk), g2, dtype=g2_dtype, order="F"),
        omega_ph=np.full((1, nk), omega0, order="F"),
        iq_kk=np.asfortranarray(iq_kk), iks_i=np.arange(ni, dtype=np.int32),
        iks_f=np.arange(nk, dtype=np.int32), eps_i=eps[:ni].copy(), w_i=w_i, eps_f=eps,
        w_f=np.full(nk, 1.0 / nk), f_to_i=f_to_i, W=1.0, nstates_base=0.0, multiplets=[],
        omegas=ws, omegas_spectral=omegas_spectral or spectral_grid_default(ws), R=R, v=v,
        dispersionless=True)


def _t2g_orbital_energies(n, N, t, tp):
    """Orbital energies (xy, yz, zx) and their gradients at k = 2π n / N."""
    c = [math.cos(2.0 * math.pi * n[a] / N) for a in range(3)]
    s = [math.sin(2.0 * math.pi * n[a] / N) for a in range(3)]
    e = (-2.0 * t * (c[0] + c[1]) - 2.0 * tp * c[2],
         -2.0 * t * (c[1] + c[2]) - 2.0 * tp * c[0],
         -2.0 * t * (c[2] + c[0]) - 2.0 * tp * c[1])
    g = ((2.0 * t * s[0], 2.0 * t * s[1], 2.0 * tp * s[2]),
         (2.0 * tp * s[0], 2.0 * t * s[1], 2.0 * t * s[2]),
         (2.0 * t * s[0], 2.0 * tp * s[1], 2.0 * t * s[2]))
    return e, g


def cubic_t2g_setup(N: int = 16, t: float = 0.26, tp: float = 0.08, nmodes: int = 15,
                    wph_min: float = 0.010, wph_max: float = 0.080, g2_logmean: float = math.log(1e-3),
                    g2_logsigma: float = 1.0, g2_scale: float = 1.0, seed: int = 0,
                    ws: FrequencyGrid | None = None, omegas_spectral: FrequencyGrid | None = None,
                    g2_dtype=np.float32, degen_cutoff: float = 1e-8, g2_chunk: int | None = None) -> dict:
    """Three-band cubic t2g model on an N^3 Γ-centred grid with O_h symmetry.

    Outer states: the irreducible k points (folded components sorted, 0 <= n1 <= n2 <= n3 <= N/2)
    times the three bands sorted by energy; inner states: all N^3 k points times three bands. Each
    inner state's IBZ representative has the same sorted band energies, assigned bitwise, and the
    rotation R_f is the signed permutation g with k_f = g k_rep (R_f v_rep = v_f). Multiplets chain
    levels at one k closer than `degen_cutoff` (src/scgd0.jl:144-160). With g2_chunk, g2 is drawn
    g2_chunk inner states at a time, chunk c from the stream seeded by (seed, 1, c), the chunks on
    host threads (for sizes whose FP64 draw would not fit in memory at once).
    """
    rng = np.random.default_rng(seed)
    half = N // 2
    reps = [r for r in itertools.combinations_with_replacement(range(half + 1), 3)]
    rep_index = {r: k for k, r in enumerate(reps)}
    nrep = len(reps)
    ni, nkf = 3 * nrep, N ** 3
    nf = 3 * nkf
    eps_i = np.zeros(ni)
    v = np.zeros((3, ni), order="F")
    orb_of_band = np.zeros((nrep, 3), dtype=np.int64)
    for k, r in enumerate(reps):
        e, g = _t2g_orbital_energies(r, N, t, tp)
        order = sorted(range(3), key=lambda o: (e[o], o))
        orb_of_band[k] = order
        for b, o in enumerate(order):
            eps_i[3 * k + b] = e[o]
            v[:, 3 * k + b] = g[o]
    star_count = np.zeros(nrep, dtype=np.int64)
    f_to_i = np.zeros(nf, dtype=np.int32)
    iks_f = np.zeros(nf, dtype=np.int32)
    R = np.zeros((3, 3, nf), order="F")
    kidx = 0
    for n3 in range(N):
        for n2 in range(N):
            for n1 in range(N):
                n = (n1, n2, n3)
                kidx = n1 + N * (n2 + N * n3)
                m = [min(x, N - x) for x in n]
                sgn = [1.0 if n[c] <= half else -1.0 for c in range(3)]
                perm = sorted(range(3), key=lambda c: (m[c], c))  # rep[r] = m[perm[r]]
                rep = tuple(m[c] for c in perm)
                kr = rep_index[rep]
                star_count[kr] += 1
                inv = [0, 0, 0]
                for r_, c in enumerate(perm):
                    inv[c] = r_
                G = np.zeros((3, 3))
                for c in range(3):
                    G[c, inv[c]] = sgn[c]
                for b in range(3):
                    f = b + 3 * kidx
                    f_to_i[f] = 3 * kr + b
                    iks_f[f] = kidx
                    R[:, :, f] = G
    w_i = np.repeat(star_count / nkf, 3).astype(np.float64)
    eps_f = eps_i[f_to_i].copy()
    w_f = np.full(nf, 1.0 / nkf)
    iks_i = np.repeat(np.arange(nrep, dtype=np.int32), 3)
    # q index of k_f - k_i (the modes are dispersionless, so the table only has to be valid).
    kf = np.arange(nkf)
    kf3 = np.stack([kf % N, (kf // N) % N, kf // (N * N)])
    iq_kk = np.zeros((nrep, nkf), dtype=np.int32, order="F")
    for k, r in enumerate(reps):
        d = (kf3 - np.array(r)[:, None]) % N
        iq_kk[k, :] = d[0] + N * (d[1] + N * d[2])
    wph = np.linspace(wph_min, wph_max, nmodes)
    omega_ph = np.asfortranarray(np.repeat(wph[:, None], nkf, axis=1))
    if g2_chunk:
        dt = np.uint16 if g2_dtype == "bf16" else np.dtype(g2_dtype)
        g2 = np.empty((nmodes, ni, nf), dtype=dt, order="F")

        def draw(c):  # chunk c from its own stream, seeded by (seed, c): the same in any thread order
            f0, f1 = c * g2_chunk, min(nf, (c + 1) * g2_chunk)
            x = np.random.default_rng([seed, 1, c]).standard_normal(size=(nmodes, ni, f1 - f0), dtype=np.float32)
            x = np.float32(g2_scale) * np.exp(np.float32(g2_logmean) + np.float32(g2_logsigma) * x)
            g2[:, :, f0:f1] = float32_to_bf16_bits(x) if g2_dtype == "bf16" else x.astype(dt)

        nchunk = (nf + g2_chunk - 1) // g2_chunk
        with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as pool:
            list(pool.map(draw, range(nchunk)))
    else:
        g2 = (g2_scale * np.exp(rng.normal(g2_logmean, g2_logsigma, size=(nmodes, ni, nf)))).astype(np.float32)
        g2 = np.asfortranarray(g2)
        if g2_dtype == np.float64:
            g2 = np.asfortranarray(g2.astype(np.float64))
        elif g2_dtype == "bf16":
            g2 = np.asfortranarray(float32_to_bf16_bits(g2))
    multiplets = []
    for k in range(nrep):
        es = [eps_i[3 * k + b] for b in range(3)]
        group = [3 * k]
        for b in range(1, 3):
            if es[b] - es[b - 1] < degen_cutoff:
                group.append(3 * k + b)
            else:
                if len(group) > 1:
                    multiplets.append(group)
                group = [3 * k + b]
        if len(group) > 1:
            multiplets.append(group)
    if ws is None:
        ws = c2_output_grid()
    return dict(g2=g2, omega_ph=omega_ph, iq_kk=iq_kk, iks_i=iks_i, iks_f=iks_f, eps_i=eps_i,
                w_i=w_i, eps_f=eps_f, w_f=w_f, f_to_i=f_to_i, W=float(w_i.sum()), nstates_base=0.0,
                multiplets=multiplets, omegas=ws,
                omegas_spectral=omegas_spectral or spectral_grid_default(ws), R=R, v=v,
                dispersionless=True, wph=wph)


def with_dispersion(setup: dict, N: int, amplitude: float) -> dict:
    """The cubic t2g model of cubic_t2g_setup (N^3 q points) with dispersive modes:
    ω_ν(q) = ω_ν (1 + amplitude (cos 2π q1/N + cos 2π q2/N + cos 2π q3/N) / 3), q = (q1, q2, q3)."""
    q = np.arange(N ** 3)
    q3 = np.stack([q % N, (q // N) % N, q // (N * N)])
    shape = np.cos(2 * np.pi * q3 / N).sum(axis=0) / 3.0
    wph = np.asarray(setup["wph"], dtype=np.float64)
    out = dict(setup)
    out["omega_ph"] = np.asfortranarray(wph[:, None] * (1.0 + amplitude * shape[None, :]))
    out["dispersionless"] = False
    return out


def c2_output_grid() -> FrequencyGrid:
    """The graded ωs of the 3-band benchmark configuration: 2 meV on ±0.5 eV, 10 meV on ±3 eV,
    40 meV on ±8 eV (1251 nodes)."""
    from .grids import graded_frequency_grid
    return graded_frequency_grid([(-0.5, 0.5, 0.002), (-3.0, 3.0, 0.010), (-8.0, 8.0, 0.040)])


def float32_to_bf16_bits(x: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even float32 -> bfloat16, returned as uint16 bit patterns."""
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def bf16_bits_to_float32(b: np.ndarray) -> np.ndarray:
    return (np.asarray(b, dtype=np.uint32) << 16).view(np.float32)


def bare_mu(setup: dict, T: float, n_target: float, spin_degeneracy: float = 2.0) -> float:
    """The chemical potential of the bare window bands (the starting μ of src/scgd0.jl:165-170,
    ElectronPhonon's bte_compute_μ!): n(μ) = g Σ_i w_i f(ε_i - μ) + nstates_base = n_target, by
    bisection on the band range ± 1."""
    eps, w = np.asarray(setup["eps_i"]), np.asarray(setup["w_i"])
    base = float(setup.get("nstates_base", 0.0))

    def n(mu):
        x = np.clip((eps - mu) / T, -700, 700)
        return spin_degeneracy * (np.sum(w / (np.exp(x) + 1.0)) + base)

    a, b = eps.min() - 1.0, eps.max() + 1.0
    for _ in range(200):
        m = 0.5 * (a + b)
        if n(m) < n_target:
            a = m
        else:
            b = m
    return 0.5 * (a + b)
