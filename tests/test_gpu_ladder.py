"""GPU parity of the ladder path: the CUDA library through its C ABI against the oracle.

Tolerances: the FP64 paths (DIRECT_FP64 on the shift grid, GEMM_FP64 regrouped per mode) match the
oracle to 1e-10 relative in one application, σ and J, with equal iteration counts (the reference's
GPU gate, test/test_ladder_gpu.jl:122-126), and are bitwise reproducible run to run
(test/test_ladder_gpu.jl:129-131). The BF16x3 tensor-core path matches σ to 1e-4 relative.
"""
import numpy as np
import pytest

import refimpl as R
from epspectral_gb300 import ArgumentError, FrequencyGrid
from test_oracle_ladder import cubic_case, holstein_case

pytestmark = pytest.mark.gpu

W_AC = 1e-6


@pytest.fixture(scope="module")
def api():
    from epspectral_gb300 import api as A
    A.lib()
    return A


@pytest.fixture(scope="module")
def hc(oracle):
    return holstein_case(oracle, symmetry=False)


@pytest.fixture(scope="module")
def hsym(oracle):
    return holstein_case(oracle)


@pytest.fixture(scope="module")
def cc(oracle):
    return cubic_case(oracle)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def refined(setup, k):
    g = setup["omegas"]
    return dict(setup, omegas=FrequencyGrid(g.origin, g.unit / k, np.asarray(g.offsets) * k))


@pytest.mark.parametrize("case,Omega,k", [("hc", 0.2, 1), ("cc", 0.123, 1), ("cc", 0.123, 4)])
def test_apply_matches_oracle(api, oracle, request, case, Omega, k):
    c = request.getfixturevalue(case)
    s = refined(c["setup"], k)
    nw, ni = len(s["omegas"]), s["eps_i"].size
    J = R.pseudorandom_complex(nw, 4, 3, 2, ni, seed=1.3)
    J[0] = 0
    J[-1] = 0
    for iT in range(2):
        args = (J, c["sigma"][:, :, iT], c["mu"][iT], c["Tlist"][iT], Omega)
        ref = oracle.apply_ladder_kernel(s, *args, omega_acoustic=W_AC)
        # TF32 rounds both operands of the contraction to 11 significant bits (2^-12 relative)
        for path, tol in (("direct_fp64", 1e-10), ("gemm_fp64", 1e-10), ("gemm_bf16", 1e-4), ("gemm_tf32", 1e-3)):
            for tile in ((None, 7) if path == "direct_fp64" else (None,)):
                got = api.apply_ladder_kernel(s, *args, omega_acoustic=W_AC, path=path, gpu_tile=tile)
                assert rel(got, ref) <= tol, (path, tile, rel(got, ref))


def test_loop_matches_oracle(api, oracle, cc):
    c = cc
    s = c["setup"]
    Omegas = [0.0, 0.1]
    kw = dict(solver="gmres", rtol=1e-2, maxiter=30, store_vertex=True, omega_acoustic=W_AC)
    ref = oracle.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], Omegas, **kw)
    for path in ("direct_fp64", "gemm_fp64"):
        got = api.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], Omegas, path=path, **kw)
        assert np.array_equal(got["niter"], ref["niter"]) and got["converged"].all()
        assert rel(got["sigma_bubble"], ref["sigma_bubble"]) <= 1e-10
        assert rel(got["sigma_ladder"], ref["sigma_ladder"]) <= 1e-10
        assert rel(got["J"], ref["J"]) <= 1e-10
        assert np.linalg.norm(ref["sigma_ladder"] - ref["sigma_bubble"]) > 1e-2 * np.linalg.norm(ref["sigma_bubble"])
        again = api.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], Omegas, path=path, **kw)
        assert np.array_equal(again["J"], got["J"]) and np.array_equal(again["sigma_ladder"], got["sigma_ladder"])
        assert all(np.array_equal(a["norms"], b["norms"]) for a, b in zip(again["history"].ravel(), got["history"].ravel()))
    for path in ("gemm_bf16", "gemm_tf32"):  # the mixed-precision contract: σ to 1e-4 relative
        bf = api.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], Omegas, path=path, **kw)
        assert rel(bf["sigma_ladder"], ref["sigma_ladder"]) <= 1e-4, (path, rel(bf["sigma_ladder"], ref["sigma_ladder"]))
    # fixed point, streamed-size chunks, Ω > 0 (test/test_ladder_gpu.jl:134-139)
    fk = dict(solver="fixed_point", rtol=1e-6, maxiter=200, omega_acoustic=W_AC)
    fref = oracle.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], [0.1], **fk)
    fgot = api.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], [0.1], path="direct_fp64", gpu_tile=7, **fk)
    assert np.array_equal(fgot["niter"], fref["niter"]) and fgot["converged"].all()
    assert rel(fgot["sigma_ladder"], fref["sigma_ladder"]) <= 1e-10


def test_density_vertex_ward_identity_long_gmres(api, oracle, hc):
    # The Ward-identity case of the oracle tests (test/test_ladder_holstein.jl:28-45: no symmetry,
    # the density vertex V = 1 in the x slot, q = 0) on the FP64 paths. GMRES at rtol 1e-8 takes
    # 28-49 iterations here, so the device Arnoldi (multi-vector CGS2 passes, FP64 Givens) runs long
    # solves: iteration counts within one of the oracle's, the bare response to 1e-10, the dressed
    # one (which nearly cancels: 4e-4 to 1.6e-2 of the bare) to 1e-7 of the bare.
    c = hc
    s = dict(c["setup"])
    v = np.zeros_like(s["v"])
    v[0, :] = 1.0
    s["v"] = v
    Omegas = [0.1, 0.3]
    kw = dict(solver="gmres", rtol=1e-8, maxiter=200, omega_acoustic=W_AC)
    ref = oracle.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], Omegas, **kw)
    assert ref["niter"].min() >= 10
    nb = np.linalg.norm(ref["sigma_bubble"])
    for path in ("direct_fp64", "gemm_fp64"):
        got = api.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], Omegas, path=path, **kw)
        assert got["converged"].all(), path
        dn = np.abs(got["niter"].astype(np.int64) - ref["niter"].astype(np.int64)).max()
        assert dn <= 1, (path, got["niter"], ref["niter"])
        assert rel(got["sigma_bubble"], ref["sigma_bubble"]) <= 1e-10, path
        assert np.linalg.norm(got["sigma_ladder"] - ref["sigma_ladder"]) <= 1e-7 * nb, path
        ratio = got["sigma_ladder"][0, 0] / got["sigma_bubble"][0, 0]
        assert np.max(np.abs(ratio)) <= 0.05, (path, ratio)


def test_holstein_current_correction_vanishes(api, hsym):
    # test/test_ladder_holstein.jl:5-26 on the GPU paths; the tensor-core path keeps its vertices in
    # FP32, so there the correction vanishes to FP32 rounding (a surviving correction is ~1e-2)
    c = hsym
    for path, tol in (("direct_fp64", 1e-9), ("gemm_fp64", 1e-9), ("gemm_bf16", 1e-6), ("gemm_tf32", 1e-4)):
        out = api.loop_ladder(c["setup"], c["sigma"], c["mu"], c["Tlist"], [0.0, 0.2], path=path, omega_acoustic=W_AC)
        assert np.linalg.norm(out["sigma_ladder"] - out["sigma_bubble"]) <= tol * np.linalg.norm(out["sigma_bubble"])
        assert out["converged"].all()


def test_ladder_argument_checks(api, cc):
    c = cc
    s = c["setup"]
    for kw in (dict(solver="newton"), dict(maxiter=0)):
        with pytest.raises(ArgumentError):
            api.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], [0.0], omega_acoustic=W_AC, **kw)
    with pytest.raises(ArgumentError):
        api.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], [0.0], omega_acoustic=-1.0)
    with pytest.raises(ArgumentError):
        api.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], [], omega_acoustic=W_AC)
    with pytest.raises(ArgumentError):
        api.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], [0.0], gpu_tile=0, omega_acoustic=W_AC)


def test_batched_right_hand_sides_match_the_sequential_solves(api, oracle, cc):
    # 2 temperatures x 3 Ωs = 6 (T, Ω) pairs solved together as GMRES right-hand sides, in batches
    # of 4 (so one batch is partial), each from x0 = 0. Solved tightly (rtol 1e-6: the path's Krylov
    # vectors are FP32, so its residuals settle near 1e-7) the batched σ must equal the sequential
    # tensor-core run's to 2e-5 relative (the operator's BF16 rounding, met along other Krylov
    # paths) and the FP64 oracle's (solved to 1e-9) to 1e-4;
    # at the loop's usual rtol 1e-2 each pair's σ_ladder must agree with the sequential one to the
    # solver tolerance.
    c = cc
    s = c["setup"]
    Omegas = [0.0, 0.05, 0.1]
    plan = api.LadderPlan(s, path="gemm_bf16", omega_acoustic=W_AC)
    tight = dict(rtol=1e-6, maxiter=60)
    seq = plan.run(c["sigma"], c["mu"], c["Tlist"], Omegas, store_vertex=True, **tight)
    bat = plan.run(c["sigma"], c["mu"], c["Tlist"], Omegas, batch_rhs=4, store_vertex=True, **tight)
    assert bat["converged"].all() and seq["converged"].all()
    assert rel(bat["sigma_bubble"], seq["sigma_bubble"]) <= 1e-12
    assert rel(bat["sigma_ladder"], seq["sigma_ladder"]) <= 2e-5
    ref = oracle.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], Omegas, solver="gmres", omega_acoustic=W_AC,
                             rtol=1e-9, maxiter=60)
    assert rel(bat["sigma_ladder"], ref["sigma_ladder"]) <= 1e-4
    # the stored vertices: every pair's J equals the sequential solve's (both converged tightly)
    for iT in range(2):
        for iO in range(3):
            assert rel(bat["J"][..., iO, iT], seq["J"][..., iO, iT]) <= 1e-4
    loose_seq = plan.run(c["sigma"], c["mu"], c["Tlist"], Omegas, rtol=1e-2, maxiter=30)
    loose_bat = plan.run(c["sigma"], c["mu"], c["Tlist"], Omegas, rtol=1e-2, maxiter=30, batch_rhs=8)
    assert loose_bat["converged"].all()
    for iT in range(2):
        for iO in range(3):
            a, b = loose_bat["sigma_ladder"][:, :, iO, iT], loose_seq["sigma_ladder"][:, :, iO, iT]
            assert np.linalg.norm(a - b) <= 3e-2 * np.linalg.norm(b)
    with pytest.raises(ArgumentError):
        plan.run(c["sigma"], c["mu"], c["Tlist"], Omegas, solver="fixed_point", batch_rhs=4)
    plan.close()


def test_tf32_batched_right_hand_sides(api, oracle, cc):
    # the batched solves on the TF32 path: σ of every pair against the FP64 oracle to 1e-4
    # relative (rtol 1e-5: the operator's TF32 rounding is ~1e-4 per element, the Krylov vectors
    # FP32), and each pair against the sequential TF32 solve
    c = cc
    s = c["setup"]
    Omegas = [0.0, 0.05, 0.1]
    plan = api.LadderPlan(s, path="gemm_tf32", omega_acoustic=W_AC)
    kw = dict(rtol=1e-5, maxiter=60)
    seq = plan.run(c["sigma"], c["mu"], c["Tlist"], Omegas, **kw)
    bat = plan.run(c["sigma"], c["mu"], c["Tlist"], Omegas, batch_rhs=4, **kw)
    assert bat["converged"].all() and seq["converged"].all()
    ref = oracle.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], Omegas, solver="gmres", omega_acoustic=W_AC,
                             rtol=1e-9, maxiter=60)
    assert rel(bat["sigma_ladder"], ref["sigma_ladder"]) <= 1e-4, rel(bat["sigma_ladder"], ref["sigma_ladder"])
    assert rel(seq["sigma_ladder"], ref["sigma_ladder"]) <= 1e-4, rel(seq["sigma_ladder"], ref["sigma_ladder"])
    plan.close()


def test_tf32_is_a_ladder_path_only(api, cc):
    with pytest.raises(api.EpspError):
        api.Scgd0Plan(cc["setup"], path="gemm_tf32", omega_acoustic=W_AC)


def test_streamed_g2_gives_the_resident_ladder(api, cc):
    # the regrouped paths build G̃ from g2 streamed star by star (gpu_tile inner states per chunk):
    # bitwise the one-chunk result
    c = cc
    s = c["setup"]
    for path in ("gemm_fp64", "gemm_bf16", "gemm_tf32"):
        one = api.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], [0.1], path=path, omega_acoustic=W_AC)
        got = api.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], [0.1], path=path, gpu_tile=5, omega_acoustic=W_AC)
        assert np.array_equal(got["sigma_ladder"], one["sigma_ladder"]), path


def test_device_gather_gives_the_host_gather(api, cc):
    # A g2 in registered page-locked memory is gathered in star order by a kernel that reads it in
    # place; the test hook makes the set-ups gather it on the host and copy instead. The coupling
    # sums (scGD0) and G̃ (ladder) built either way are the same bits: FP64, FP32 and BF16 storage,
    # one chunk and chunks of 5 inner states, and a g2 whose address is one element past an aligned
    # one (the kernel then copies in element-sized words).
    from epspectral_gb300 import synthetic
    c = cc
    nw, ni = len(c["setup"]["omegas"]), c["setup"]["eps_i"].size
    J = R.pseudorandom_complex(nw, 4, 3, 2, ni, seed=0.61)
    J[0] = 0
    J[-1] = 0
    sig, mu, T = c["sigma"][:, :, 0], c["mu"][0], c["Tlist"][0]

    def shifted(a):
        buf = np.empty(a.size + 1, dtype=a.dtype)
        v = buf[1:].reshape(a.shape, order="F")
        v[...] = a
        return v

    def both_ways(s, tile):
        got = []
        for host in (False, True):
            ctx.g2_host_gather(host)
            sp = api.Scgd0Plan(s, path="gemm_fp64", gpu_tile=tile, omega_acoustic=W_AC, ctx=ctx)
            im = sp.imsigma(sig, mu, T)
            sp.close()
            lp = api.LadderPlan(s, path="gemm_tf32", gpu_tile=tile, omega_acoustic=W_AC, ctx=ctx)
            got.append((im, lp.apply(J, sig, mu, T, 0.07)))
            lp.close()
        return got

    g64 = np.array(c["setup"]["g2"], dtype=np.float64, order="F")
    g32 = g64.astype(np.float32, order="F")
    gbf = synthetic.float32_to_bf16_bits(g32)
    ctx = api.Context(0)
    try:
        for g2 in (g64, g32, gbf, shifted(g32), shifted(gbf)):
            s = dict(c["setup"], g2=g2)
            ctx.host_register(g2)
            try:
                for tile in (None, 5):
                    (im_d, ap_d), (im_h, ap_h) = both_ways(s, tile)
                    assert np.array_equal(im_d, im_h), (g2.dtype, tile)
                    assert np.array_equal(ap_d, ap_h), (g2.dtype, tile)
            finally:
                ctx.host_unregister(g2)
    finally:
        ctx.g2_host_gather(False)
        ctx.close()


@pytest.mark.parametrize("unit", [0.001, 0.0005])
def test_apply_on_fine_shift_grids(api, oracle, unit):
    # Fine grids make the shift window wide (nshift = 81 and 161 here, vertex windows of 4 x 198
    # and 4 x 358 nodes): the operand kernel then stages its window with 4 and 8 prefetch slots per
    # thread. One application against the oracle on both regrouped paths.
    from epspectral_gb300 import graded_frequency_grid, synthetic
    ws = graded_frequency_grid([(-0.2, 0.2, unit), (-0.8, 0.8, 10 * unit)])
    s = synthetic.cubic_t2g_setup(N=4, ws=ws, g2_dtype=np.float64, seed=3)
    nw, ni = len(ws), s["eps_i"].size
    sig = np.asfortranarray(np.full((nw, ni), complex(0.001, -0.02)))
    J = R.pseudorandom_complex(nw, 4, 3, 2, ni, seed=2.1)
    J[0] = 0
    J[-1] = 0
    T = 300 * synthetic.KELVIN
    ref = oracle.apply_ladder_kernel(s, J, sig, 0.0, T, 0.05, omega_acoustic=W_AC)
    for path, tol in (("gemm_fp64", 1e-10), ("gemm_bf16", 1e-4), ("gemm_tf32", 1e-3)):
        got = api.apply_ladder_kernel(s, J, sig, 0.0, T, 0.05, omega_acoustic=W_AC, path=path)
        assert np.all(np.isfinite(got)) and rel(got, ref) <= tol, (path, rel(got, ref))


@pytest.mark.parametrize("unit", [0.01, 0.001])
def test_every_contraction_tile_shape_matches_the_oracle(api, oracle, cc, unit):
    # the autotuner's candidates, each forced: BN 128 and 256 with K blocks of 64 (128-byte
    # swizzle), BN 256 with K blocks of 32 (64-byte swizzle, four stages), one and two splits
    from epspectral_gb300 import graded_frequency_grid, synthetic
    c = cc
    s = c["setup"] if unit == 0.01 else synthetic.cubic_t2g_setup(
        N=4, ws=graded_frequency_grid([(-0.2, 0.2, unit), (-0.8, 0.8, 10 * unit)]), g2_dtype=np.float64, seed=3)
    nw, ni = len(s["omegas"]), s["eps_i"].size
    sig = c["sigma"][:, :, 0] if unit == 0.01 else np.asfortranarray(np.full((nw, ni), complex(0.001, -0.02)))
    J = R.pseudorandom_complex(nw, 4, 3, 2, ni, seed=0.7)
    J[0] = 0
    J[-1] = 0
    T = c["Tlist"][0]
    ref = oracle.apply_ladder_kernel(s, J, sig, c["mu"][0], T, 0.07, omega_acoustic=W_AC)
    plan = api.LadderPlan(s, path="gemm_bf16", omega_acoustic=W_AC)
    assert plan.gemm_config()["bn"] in (128, 256)
    for bn, bk in ((128, 64), (256, 64), (256, 32)):
        for sp in (1, 2):
            plan.set_gemm_config(bn, sp, bk)
            got = plan.apply(J, sig, c["mu"][0], T, 0.07)
            assert np.all(np.isfinite(got)) and rel(got, ref) <= 1e-4, (bn, bk, sp, rel(got, ref))
            if (bn, bk) == (256, 32):
                # the persistent kernel (one CTA per SM over all tiles, two TMEM accumulators) runs
                # every tile's products in the same order: bitwise the same result
                plan.set_gemm_config(bn, sp, bk, persistent=True)
                assert plan.gemm_config()["persistent"]
                assert np.array_equal(plan.apply(J, sig, c["mu"][0], T, 0.07), got), (bn, bk, sp, "persistent")
                # CTA pairs (tcgen05 cta_group::2, 256-row tiles over two CTAs): bitwise the same
                plan.set_gemm_config(bn, sp, bk, pair=True)
                assert plan.gemm_config()["pair"]
                assert np.array_equal(plan.apply(J, sig, c["mu"][0], T, 0.07), got), (bn, bk, sp, "pair")
                # persistent CTA pairs (one cluster per two SMs over all tiles): bitwise the same
                plan.set_gemm_config(bn, sp, bk, persistent=True, pair=True)
                assert plan.gemm_config()["pair"] and plan.gemm_config()["persistent"]
                assert np.array_equal(plan.apply(J, sig, c["mu"][0], T, 0.07), got), (bn, bk, sp, "pair persistent")
    with pytest.raises(ArgumentError):
        plan.set_gemm_config(128, 1, 32)
    with pytest.raises(ArgumentError):
        plan.set_gemm_config(128, 1, 64, persistent=True)
    plan.close()
    # TF32: one product per K step of 8 (K boxes of 32 FP32 = 128 bytes), BN 128 (six stages) and
    # 256 (four), one and two splits, each also as the persistent kernel (bitwise the same)
    plan = api.LadderPlan(s, path="gemm_tf32", omega_acoustic=W_AC)
    assert plan.gemm_config()["bk"] == 32
    for bn, bk in ((128, 32), (256, 32)):
        for sp in (1, 2):
            plan.set_gemm_config(bn, sp, bk)
            got = plan.apply(J, sig, c["mu"][0], T, 0.07)
            assert np.all(np.isfinite(got)) and rel(got, ref) <= 1e-3, (bn, bk, sp, rel(got, ref))
            plan.set_gemm_config(bn, sp, bk, persistent=True)
            assert plan.gemm_config()["persistent"]
            assert np.array_equal(plan.apply(J, sig, c["mu"][0], T, 0.07), got), (bn, bk, sp, "persistent")
            if bn == 256:
                plan.set_gemm_config(bn, sp, bk, pair=True)
                assert plan.gemm_config()["pair"]
                assert np.array_equal(plan.apply(J, sig, c["mu"][0], T, 0.07), got), (bn, bk, sp, "pair")
                plan.set_gemm_config(bn, sp, bk, persistent=True, pair=True)
                assert plan.gemm_config()["pair"] and plan.gemm_config()["persistent"]
                assert np.array_equal(plan.apply(J, sig, c["mu"][0], T, 0.07), got), (bn, bk, sp, "pair persistent")
    with pytest.raises(ArgumentError):
        plan.set_gemm_config(256, 1, 64)
    with pytest.raises(ArgumentError):
        plan.set_gemm_config(128, 1, 16)
    with pytest.raises(ArgumentError):
        plan.set_gemm_config(128, 1, 32, pair=True)
    plan.close()


def test_bounded_wait_runs_out_and_the_plan_stays_usable(api, cc):
    # the one-CTA tensor-core kernel's producer skips K block 0 of every tile (a test hook): the MMA
    # thread's wait for that stage gives up after 4096 tries, the kernel records it, waits for its
    # own copies and products, frees its tensor memory and returns; the call reports EDEVICE_TIMEOUT,
    # and the same plan on the same context then applies the operator bitwise as before
    import time
    from epspectral_gb300 import abi
    c = cc
    s = c["setup"]
    nw, ni = len(s["omegas"]), s["eps_i"].size
    J = R.pseudorandom_complex(nw, 4, 3, 2, ni, seed=0.41)
    J[0] = 0
    J[-1] = 0
    args = (J, c["sigma"][:, :, 0], c["mu"][0], c["Tlist"][0], 0.07)
    plan = api.LadderPlan(s, path="gemm_tf32", omega_acoustic=W_AC)
    plan.set_gemm_config(128, 1, 32)  # the one-CTA kernel
    want = plan.apply(*args)
    plan.ctx.stall_gemm(0, 4096)
    try:
        t0 = time.perf_counter()
        with pytest.raises(api.EpspError) as err:
            plan.apply(*args)
        assert err.value.status == abi.EPSP_EDEVICE_TIMEOUT
        assert time.perf_counter() - t0 < 60
    finally:
        plan.ctx.stall_gemm()  # the context is shared with the other tests
    assert np.array_equal(plan.apply(*args), want)
    with pytest.raises(ArgumentError):
        plan.ctx.stall_gemm(-2, 0)
    with pytest.raises(ArgumentError):
        plan.ctx.stall_gemm(0, 8)
    plan.close()


def test_kept_g2_serves_the_next_set_up(api, cc):
    # epsp_ctx_keep_g2: the scGD0 plan's set-up streams g2 and the context keeps it; the ladder
    # plan's set-up of the same array reads the kept copy. Shown by the contract itself: g2 changed
    # in place between the two set-ups is not seen (the result is bitwise that of the old g2), and
    # with the copy freed a new set-up streams the changed array.
    c = cc
    s = dict(c["setup"])
    g2 = np.array(s["g2"], copy=True, order="F")
    s["g2"] = g2
    nw, ni = len(s["omegas"]), s["eps_i"].size
    J = R.pseudorandom_complex(nw, 4, 3, 2, ni, seed=0.53)
    J[0] = 0
    J[-1] = 0
    args = (J, c["sigma"][:, :, 0], c["mu"][0], c["Tlist"][0], 0.07)
    ref = api.LadderPlan(s, path="gemm_tf32", omega_acoustic=W_AC)
    want = ref.apply(*args)
    ctx = ref.ctx
    ref.close()
    ctx.keep_g2(True)
    try:
        api.Scgd0Plan(s, path="gemm_bf16", omega_acoustic=W_AC).close()  # streams g2, the context keeps it
        g2 *= 2  # in place: the same array, size and type
        lp = api.LadderPlan(s, path="gemm_tf32", omega_acoustic=W_AC)
        assert np.array_equal(lp.apply(*args), want)
        lp.close()
    finally:
        ctx.keep_g2(False)
    lp = api.LadderPlan(s, path="gemm_tf32", omega_acoustic=W_AC)
    assert not np.allclose(lp.apply(*args), want)
    lp.close()


def test_scgd0_sigma_stays_on_the_device_for_the_ladder(api, cc):
    # epsp_scgd0_run with sigma_out = NULL keeps Σ in the plan (epsp_scgd0_sigma_device); the ladder
    # reads it there (cudaMemcpyDefault): the same σ, bitwise, as from the downloaded Σ
    import ctypes as C
    c = cc
    s = c["setup"]
    # the fixture's own scGD0 settings (test_oracle_ladder.cubic_case): two iterations from η = 0.05
    occ = dict(Tlist=list(c["Tlist"]), nlist=[0.0, 0.0], nelec=1.0, spin_degeneracy=2.0)
    sp = api.Scgd0Plan(s, path="gemm_bf16", omega_acoustic=W_AC)
    p, n = C.c_void_p(), C.c_int64()
    assert api.lib().epsp_scgd0_sigma_device(sp.handle, C.byref(p), C.byref(n)) == 1  # EINVAL before a run
    kw = dict(eta_init=0.05, eta_min=[0.0, 0.03], tol=0.0, maxiter=2, mu_start=[-0.5, -0.5])
    host = sp.run(occ, **kw)
    dev = sp.run(occ, sigma_to_host=False, **kw)
    assert isinstance(dev["sigma"], api.DeviceSigma) and dev["sigma"].shape == host["sigma"].shape
    assert np.array_equal(dev["mu"], host["mu"]) and dev["niter"] == host["niter"]
    lp = api.LadderPlan(s, path="gemm_tf32", omega_acoustic=W_AC)
    a = lp.run(host["sigma"], host["mu"], c["Tlist"], [0.0, 0.1])
    b = lp.run(dev["sigma"], dev["mu"], c["Tlist"], [0.0, 0.1])
    assert np.array_equal(a["sigma_ladder"], b["sigma_ladder"]) and np.array_equal(a["sigma_bubble"], b["sigma_bubble"])
    bb = lp.run(dev["sigma"], dev["mu"], c["Tlist"], [0.0, 0.1], batch_rhs=4)
    ab = lp.run(host["sigma"], host["mu"], c["Tlist"], [0.0, 0.1], batch_rhs=4)
    assert np.array_equal(ab["sigma_ladder"], bb["sigma_ladder"])
    with pytest.raises(ValueError):
        lp.run(dev["sigma"], dev["mu"][:1], c["Tlist"][:1], [0.0])
    sp.run(occ, **kw)  # another run replaces the plan's Σ: the old handle is refused on the host
    with pytest.raises(ValueError):
        lp.run(dev["sigma"], dev["mu"], c["Tlist"], [0.0])
    lp.close()
    sp.close()
