"""The oracle's ladder restatement pinned on the reference's own known answers (CPU only).

Ports test/test_ladder_bubble.jl, test/test_ladder_kernel.jl, test/test_ladder_holstein.jl and the
solver checks of test/test_ladder_pb.jl. The pb artifact of the reference is not available, so its
role (several modes, stars with rotations, multiplets) is taken by a small cubic t2g model.
"""
import math

import numpy as np
import pytest

import refimpl as R
from epspectral_gb300 import ArgumentError, FrequencyGrid, graded_frequency_grid, synthetic

W_AC = 1e-6


def holstein_case(oracle, *, nk=16, w0=0.173, symmetry=True, Tlist=(0.1, 0.2)):
    """holstein_ladder_case (test/ladder_fixtures.jl:22-31): g2 = 2 λ ω0 |t| with λ = 0.5."""
    ws = FrequencyGrid.from_nodes(np.concatenate([np.arange(-4.0, -0.9999, 0.04), np.arange(-0.98, 0.98001, 0.02),
                                                  np.arange(1.0, 4.0001, 0.04)]))
    s = synthetic.holstein_1d_setup(nk, 1.0, w0, w0, ws, symmetry=symmetry)
    occ = dict(Tlist=list(Tlist), nlist=[0.0] * len(Tlist), nelec=1.0, spin_degeneracy=2.0)
    r = oracle.loop_scgd0(s, occ, eta_init=0.05, tol=1e-6, maxiter=100, mu_start=[0.0] * len(Tlist),
                          omega_acoustic=W_AC)
    return dict(setup=s, sigma=r["sigma"], mu=r["mu"], Tlist=np.array(Tlist))


def cubic_case(oracle, *, N=4, unit=0.01, maxiter=2):
    """A small t2g window standing in for the pb fixture (test/ladder_fixtures.jl:33-38): scGD0 run
    for `maxiter` iterations, never converged."""
    ws = graded_frequency_grid([(-0.3, 0.3, unit), (-1.5, 1.5, 5 * unit)])
    s = synthetic.cubic_t2g_setup(N=N, ws=ws, g2_dtype=np.float64, seed=3)
    Tlist = [300 * synthetic.KELVIN, 600 * synthetic.KELVIN]
    occ = dict(Tlist=Tlist, nlist=[0.0, 0.0], nelec=1.0, spin_degeneracy=2.0)
    r = oracle.loop_scgd0(s, occ, eta_init=0.05, eta_min=[0.0, 0.03], tol=0.0, maxiter=maxiter,
                          mu_start=[-0.5, -0.5], omega_acoustic=W_AC)
    return dict(setup=s, sigma=r["sigma"], mu=r["mu"], Tlist=np.array(Tlist))


@pytest.fixture(scope="module")
def hcase(oracle):
    return holstein_case(oracle)


@pytest.fixture(scope="module")
def hcase_nosym(oracle):
    return holstein_case(oracle, symmetry=False)


@pytest.fixture(scope="module")
def ccase(oracle):
    return cubic_case(oracle)


def test_contour_green_identities(oracle):
    # test/test_ladder_bubble.jl:44-60
    for (w, e, S, mu, T) in ((0.3, -0.1, -0.02 - 0.05j, 0.05, 0.1), (-0.7, 0.4, 0.03 - 0.2j, -0.1, 0.25),
                             (1.1, 0.2, -0.1 - 0.01j, 0.3, 0.05)):
        GR = 1 / (w - e - S)
        GA = np.conj(GR)
        G11, G21, G12, G22 = (oracle.contour_green(w, e, S, mu, T, c) for c in range(4))
        f = R.fermi(w - mu, T)
        tol = 1e-14 * abs(GR - GA)
        assert abs(G11 - G12 - GR) <= tol and abs(G21 - G22 - GR) <= tol and abs(G11 - G21 - GA) <= tol
        assert abs(G21 - (1 - f) * (GR - GA)) <= tol and abs(G12 + f * (GR - GA)) <= tol


def test_trapezoid_weights(oracle):
    # test/test_ladder_bubble.jl:62-69
    ws = np.array([-1.0, -0.7, -0.6, 0.0, 0.5, 2.0])
    W = oracle.trapezoid_weights(ws)
    assert abs(W.sum() - (ws[-1] - ws[0])) < 1e-14
    assert abs(np.sum(W * ws) - (ws[-1] ** 2 - ws[0] ** 2) / 2) < 1e-14


def test_attach_greens_against_2x2_matrices(oracle):
    # test/test_ladder_bubble.jl:71-98: the pair index (c1, c2) is column-major, so a four-vector
    # reshaped to 2x2 is the contour matrix and J = Gm X Gp per (ω, cart, c0, i); the bare vertex is
    # the attachment of V^{c1 c2, c0} = δ_{c1 c2} δ_{c1 c0} v_i.
    nw, ni = 5, 3
    Gm = R.pseudorandom_complex(nw, 4, ni, seed=1.1)
    Gp = R.pseudorandom_complex(nw, 4, ni, seed=2.3)
    X = R.pseudorandom_complex(nw, 4, 3, 2, ni, seed=3.7)
    J = oracle.attach_greens(Gm, Gp, X)
    m2 = lambda a: a.reshape(2, 2, order="F")
    J_ref = np.zeros((nw, 4, 3, 2, ni), dtype=complex)
    for i in range(ni):
        for c0 in range(2):
            for a in range(3):
                for w in range(nw):
                    J_ref[w, :, a, c0, i] = (m2(Gm[w, :, i]) @ m2(X[w, :, a, c0, i]) @ m2(Gp[w, :, i])).reshape(
                        4, order="F")
    assert np.linalg.norm(J - J_ref) <= 1e-14 * np.linalg.norm(J_ref)
    v = R.pseudorandom(3, ni, seed=4.1)
    V = np.zeros((nw, 4, 3, 2, ni), dtype=complex)
    for c0 in range(2):
        V[:, c0 + 2 * c0, :, c0, :] = v[None, :, :]
    J_V = oracle.attach_greens(Gm, Gp, V)
    J0 = oracle.attach_bare(Gm, Gp, v)
    assert np.linalg.norm(J0 - J_V) <= 1e-14 * np.linalg.norm(J0)
    assert np.linalg.norm(J0) > 0


@pytest.mark.parametrize("case_name", ["hcase", "ccase"])
def test_bubble_identity(oracle, request, case_name):
    # test/test_ladder_bubble.jl:101-122: the bare-vertex contour bubble equals the spectral bubble.
    c = request.getfixturevalue(case_name)
    s = c["setup"]
    w = s["omegas"].nodes()
    Omegas = [0.0, 0.3] if case_name == "hcase" else [0.0, 0.123]
    out = oracle.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], Omegas, solver="gmres", rtol=1e-2, maxiter=1,
                             omega_acoustic=W_AC)
    for iT in range(len(c["Tlist"])):
        for iO, Om in enumerate(Omegas):
            ref = R.spectral_bubble(w, c["sigma"][:, :, iT], s["eps_i"], s["w_i"], s["v"], c["mu"][iT],
                                    c["Tlist"][iT], Om)
            got = out["sigma_bubble"][:, :, iO, iT]
            assert ref[0, 0] > 0
            assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)


def test_shift_regrouping(oracle):
    # test/test_ladder_kernel.jl:118-143
    g = FrequencyGrid.from_nodes(np.concatenate([np.arange(-1.0, -0.3999, 0.1), np.arange(-0.35, 0.35001, 0.05),
                                                 np.arange(0.4, 1.0001, 0.1)]))
    h, nshift = g.unit, 13
    assert abs(h - 0.05) < 1e-12
    klo, wlo, whi = oracle.shift_tables(g, nshift)
    w = g.nodes()
    y0 = R.pseudorandom_complex(len(w), seed=0.7)
    y = y0.copy()
    y[0] = y[-1] = 0
    for s, sign in ((0, 1), (1, -1)):
        for q in (0.0123, 0.2237, 0.4999, 0.55):
            m = math.floor(q / h)
            r = q / h - m
            sh = lambda yy, mm: wlo[:, mm, s] * yy[klo[:, mm, s]] + whi[:, mm, s] * yy[klo[:, mm, s] + 1]
            reg = (1 - r) * sh(y, m) + r * sh(y, m + 1)
            direct = np.array([R.hat_value(y, w, x + sign * q) for x in w])
            assert np.linalg.norm(reg - direct) <= 1e-14 * np.linalg.norm(direct)
            reg_e = (1 - r) * sh(y0, m) + r * sh(y0, m + 1)
            dir_e = np.array([R.hat_value(y0, w, x + sign * q) for x in w])
            inner = (w > w[0] + q + h) & (w < w[-1] - q - h)
            assert np.linalg.norm((reg_e - dir_e)[inner]) <= 1e-14 * np.linalg.norm(dir_e[inner])


@pytest.mark.parametrize("case_name,unit", [("hcase_nosym", None), ("ccase", 0.0025)])
def test_bin_coupling_bitwise(oracle, request, case_name, unit):
    # test/test_ladder_kernel.jl:163-194: B equals the per-shift sum over modes bitwise, and the last
    # shift row is zero.
    c = request.getfixturevalue(case_name)
    s = dict(c["setup"])
    if unit is not None:
        g = s["omegas"]
        s["omegas"] = FrequencyGrid(g.origin, g.unit / 4, np.asarray(g.offsets) * 4)
    T = c["Tlist"][0]
    B = oracle.bin_coupling(s, T, omega_acoustic=W_AC)
    ns, nf, ni, _ = B.shape
    h = s["omegas"].unit
    order = np.argsort(s["f_to_i"], kind="stable")
    g2 = np.asarray(s["g2"], dtype=np.float64)
    Bref = np.zeros_like(B)
    n = 26  # the first inner states in star order (a plain-Python loop; bitwise in all of them)
    for fc, f in enumerate(order[:n]):
        for i in range(ni):
            for typ in range(2):
                for m in range(ns):
                    acc = 0.0
                    for nu in range(g2.shape[0]):
                        q = s["omega_ph"][nu, s["iq_kk"][s["iks_i"][i], s["iks_f"][f]]]
                        if q < W_AC:
                            continue
                        tent = max(0.0, 1 - abs(q / h - m))
                        cc = g2[nu, i, f] * tent
                        acc += cc if typ == 0 else cc * oracle.occ_boson(q, T)
                    Bref[m, fc, i, typ] = s["w_f"][f] * acc
    assert np.array_equal(B[:, :n], Bref[:, :n])
    assert np.linalg.norm(B) > 0 and np.all(B[-1] == 0)


@pytest.mark.parametrize("case_name,Omega,refine", [("hcase_nosym", 0.2, 1), ("ccase", 0.123, 1), ("ccase", 0.123, 4)])
def test_apply_ladder_against_naive_loop(oracle, request, case_name, Omega, refine):
    # test/test_ladder_kernel.jl:196-234: one application against the loop over (i, f, ν) with the
    # exact hat-basis shift, at 1e-12, on a vertex vanishing at the end nodes; also chunked.
    c = request.getfixturevalue(case_name)
    s = dict(c["setup"])
    if refine > 1:
        g = s["omegas"]
        s["omegas"] = FrequencyGrid(g.origin, g.unit / refine, np.asarray(g.offsets) * refine)
    w = s["omegas"].nodes()
    nw, ni = len(w), s["eps_i"].size
    J = R.pseudorandom_complex(nw, 4, 3, 2, ni, seed=1.3)
    J[0] = 0
    J[-1] = 0
    for iT in range(2):
        Gm, Gp = R.propagators(w, c["sigma"][:, :, iT], s["eps_i"], c["mu"][iT], c["Tlist"][iT], Omega)
        ref = R.naive_apply_ladder(s, J, Gm, Gp, c["Tlist"][iT], W_AC)
        assert np.linalg.norm(ref) > 1e-3 * np.linalg.norm(J)
        for tile in (None, 7):
            LJ = oracle.apply_ladder_kernel(s, J, c["sigma"][:, :, iT], c["mu"][iT], c["Tlist"][iT], Omega,
                                            omega_acoustic=W_AC, gpu_tile=tile)
            assert np.linalg.norm(LJ - ref) <= 1e-12 * np.linalg.norm(ref)


def test_apply_unchanged_on_a_finer_shift_table(oracle, ccase):
    # test/test_ladder_kernel.jl:200-208: the same hat-basis shifts on a table twice as fine; one
    # application on a vertex that vanishes at the end nodes is unchanged to 1e-12 (a non-zero end
    # value is spread over one table step beyond the end, so it makes the result depend on the step).
    c = ccase
    s = c["setup"]
    g = s["omegas"]
    s_half = dict(s, omegas=FrequencyGrid(g.origin, g.unit / 2, np.asarray(g.offsets) * 2))
    assert np.array_equal(s_half["omegas"].nodes(), g.nodes())
    nw, ni = len(g), s["eps_i"].size
    J = R.pseudorandom_complex(nw, 4, 3, 2, ni, seed=0.9)
    J[0] = 0
    J[-1] = 0
    args = (c["sigma"][:, :, 0], c["mu"][0], c["Tlist"][0], 0.123)
    LJ = oracle.apply_ladder_kernel(s, J, *args, omega_acoustic=W_AC)
    LJ_half = oracle.apply_ladder_kernel(s_half, J, *args, omega_acoustic=W_AC)
    assert oracle.nshift(s_half) > oracle.nshift(s)
    assert np.linalg.norm(LJ_half - LJ) <= 1e-12 * np.linalg.norm(LJ)


def test_holstein_current_vertex_correction_vanishes(oracle, hcase):
    # test/test_ladder_holstein.jl:5-26: Σ_f J_f = 0 for J_{-k} = -J_k, so L(J0) = 0 and
    # σ_ladder = σ_bubble; without the sign of the time-reversed partners it does not cancel.
    s = hcase["setup"]
    w = s["omegas"].nodes()
    for iT in range(2):
        for Om in (0.0, 0.2):
            Gm, Gp = R.propagators(w, hcase["sigma"][:, :, iT], s["eps_i"], hcase["mu"][iT], hcase["Tlist"][iT], Om)
            J0 = np.zeros((len(w), 4, 3, 2, s["eps_i"].size), dtype=complex)
            for c0 in range(2):
                for c1 in range(2):
                    for c2 in range(2):
                        J0[:, c1 + 2 * c2, :, c0, :] = (Gm[:, c1 + 2 * c0, None, :] * s["v"][None, :, :]
                                                        * Gp[:, c0 + 2 * c2, None, :])
            LJ = oracle.apply_ladder_kernel(s, J0, hcase["sigma"][:, :, iT], hcase["mu"][iT], hcase["Tlist"][iT], Om,
                                            omega_acoustic=W_AC)
            assert np.max(np.abs(LJ)) <= 1e-12 * np.max(np.abs(J0))
            wrong = dict(s, R=np.abs(s["R"]))
            LJw = oracle.apply_ladder_kernel(wrong, J0, hcase["sigma"][:, :, iT], hcase["mu"][iT], hcase["Tlist"][iT],
                                             Om, omega_acoustic=W_AC)
            assert np.max(np.abs(LJw)) > 1e-3 * np.max(np.abs(J0))
    out = oracle.loop_ladder(s, hcase["sigma"], hcase["mu"], hcase["Tlist"], [0.0, 0.2], omega_acoustic=W_AC)
    assert np.linalg.norm(out["sigma_ladder"] - out["sigma_bubble"]) <= 1e-12 * np.linalg.norm(out["sigma_bubble"])
    assert out["converged"].all()


def test_holstein_density_vertex_ward_identity(oracle, hcase_nosym):
    # test/test_ladder_holstein.jl:28-45: with no symmetry the x slot of the vertex is not rotated,
    # and V = 1 there is the density vertex at q = 0. For Ω ≠ 0 the conserving ladder gives
    # χ^K_ρρ = 0, so the ratio of the dressed to the bare response measures the kernel's
    # discretisation error. The reference asserts convergence, a finite ratio and a non-zero bare
    # response (and logs the ratio); the bound on the ratio is this suite's own: a kernel that does
    # not conserve leaves it near 1 (here 4e-4 to 1.6e-2). GMRES at rtol 1e-8 takes 28-49
    # iterations on this case.
    c = hcase_nosym
    s = dict(c["setup"])
    v = np.zeros_like(s["v"])
    v[0, :] = 1.0
    s["v"] = v
    out = oracle.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], [0.1, 0.3], solver="gmres", rtol=1e-8, maxiter=200,
                             omega_acoustic=W_AC)
    assert out["converged"].all()
    bubble, ladder = out["sigma_bubble"][0, 0], out["sigma_ladder"][0, 0]
    assert np.all(bubble != 0)
    ratio = ladder / bubble
    assert np.all(np.isfinite(ratio))
    assert np.max(np.abs(ratio)) <= 0.05
    assert out["niter"].min() >= 10


def test_solvers_agree_and_vertex_equation(oracle, ccase):
    # test/test_ladder_pb.jl:11-57: GMRES and the fixed point agree to 10 rtol at Ω > 0; the stored
    # J satisfies J = J0 + L(J) to the solver tolerance; one fixed-point step stores J0 + L(J0).
    c = ccase
    s = c["setup"]
    rtol = 1e-6
    g = oracle.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], [0.1], solver="gmres", rtol=rtol, maxiter=60,
                           omega_acoustic=W_AC)
    fp = oracle.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], [0.1], solver="fixed_point", rtol=rtol, maxiter=200,
                            omega_acoustic=W_AC)
    assert g["converged"].all() and fp["converged"].all()
    assert np.linalg.norm(g["sigma_ladder"] - fp["sigma_ladder"]) <= 10 * rtol * np.linalg.norm(g["sigma_ladder"])
    assert np.linalg.norm(g["sigma_ladder"] - g["sigma_bubble"]) > 1e-2 * np.linalg.norm(g["sigma_bubble"])
    assert all(len(h["norms"]) == n + 1 for h, n in zip(g["history"].ravel(), g["niter"].ravel()))
    Omegas = [0.0, 0.1]
    one = oracle.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], Omegas, solver="fixed_point", maxiter=1,
                             store_vertex=True, omega_acoustic=W_AC)
    sol = oracle.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], Omegas, solver="gmres", rtol=1e-8, maxiter=60,
                             store_vertex=True, omega_acoustic=W_AC)
    w = s["omegas"].nodes()
    for iT in range(2):
        for iO, Om in enumerate(Omegas):
            Gm, Gp = R.propagators(w, c["sigma"][:, :, iT], s["eps_i"], c["mu"][iT], c["Tlist"][iT], Om)
            J0 = np.zeros((len(w), 4, 3, 2, s["eps_i"].size), dtype=complex)
            for c0 in range(2):
                for c1 in range(2):
                    for c2 in range(2):
                        J0[:, c1 + 2 * c2, :, c0, :] = (Gm[:, c1 + 2 * c0, None, :] * s["v"][None, :, :]
                                                        * Gp[:, c0 + 2 * c2, None, :])
            ap = lambda J: oracle.apply_ladder_kernel(s, J, c["sigma"][:, :, iT], c["mu"][iT], c["Tlist"][iT], Om,
                                                      omega_acoustic=W_AC)
            J1 = J0 + ap(J0)
            assert np.linalg.norm(one["J"][..., iO, iT] - J1) <= 1e-12 * np.linalg.norm(J1)
            J = sol["J"][..., iO, iT]
            assert np.linalg.norm(J - J0 - ap(J)) <= 10 * 1e-8 * np.linalg.norm(J0)


def test_ladder_argument_checks(oracle, ccase):
    # test/test_ladder_pb.jl:229-244 (the checks of the loop's arguments)
    c = ccase
    for kw in (dict(solver="newton"), dict(maxiter=0), dict(omega_acoustic=-1.0)):
        args = dict(solver="gmres", rtol=1e-2, maxiter=30, omega_acoustic=W_AC)
        args.update(kw)
        with pytest.raises(ArgumentError):
            oracle.loop_ladder(c["setup"], c["sigma"], c["mu"], c["Tlist"], [0.0], **args)
    with pytest.raises(ArgumentError):
        oracle.loop_ladder(c["setup"], c["sigma"], c["mu"], c["Tlist"], [], omega_acoustic=W_AC)


@pytest.mark.parametrize("tile", [None, 7])
def test_apply_sample_is_the_full_slice(oracle, ccase, tile):
    # the output-state range of one application (the bounded sample the full-size GPU parity tests
    # compare against) is bitwise the slice of the full application, with one chunk or several
    s = ccase["setup"]
    w = s["omegas"].nodes()
    nw, ni = len(w), s["eps_i"].size
    J = R.pseudorandom_complex(nw, 4, 3, 2, ni, seed=2.1)
    J[0] = 0
    J[-1] = 0
    args = (s, J, ccase["sigma"][:, :, 1], ccase["mu"][1], ccase["Tlist"][1], 0.09)
    full = oracle.apply_ladder_kernel(*args, omega_acoustic=W_AC, gpu_tile=tile)
    for i0, i1 in ((0, 2), (3, ni), (ni - 1, ni)):
        part = oracle.ladder_apply_sample(*args, i0, i1, omega_acoustic=W_AC, gpu_tile=tile)
        assert np.array_equal(part, full[..., i0:i1]), (i0, i1)


def test_chunk_operands_cover_the_contraction(oracle, ccase):
    # the CPU baseline times one chunk's C± += X± B̃ as a DGEMM: the chunks partition the outer
    # states in order, and the operands have the shapes of src/ladder.jl:283-290
    s = ccase["setup"]
    nw, ni = len(s["omegas"]), s["eps_i"].size
    chunks, ns = oracle.ladder_chunks(s, omega_acoustic=W_AC, gpu_tile=7)
    assert len(chunks) > 1 and chunks[0][0] == 0 and chunks[-1][1] == ni
    assert all(a[1] == b[0] for a, b in zip(chunks, chunks[1:]))
    J = R.pseudorandom_complex(nw, 4, 3, 2, ni, seed=0.4)
    for c in (0, len(chunks) - 1):
        Xp, Xm, Bt = oracle.ladder_chunk_operands(s, J, ccase["Tlist"][0], c, omega_acoustic=W_AC, gpu_tile=7)
        nk = ns * 3 * (chunks[c][1] - chunks[c][0])
        assert Xp.shape == Xm.shape == (16 * nw, nk) and Bt.shape == (nk, 6 * ni)
        assert np.all(np.isfinite(Xp @ Bt)) and np.linalg.norm(Bt) > 0 and not np.array_equal(Xp, Xm)
