"""GPU parity of the scGD0 path: the CUDA library through its C ABI against the oracle.

Tolerances: the plain FP64 paths (DIRECT_FP64, GEMM_FP64) match the oracle to 1e-10 relative in Σ
and μ (the reference's own GPU-vs-host gate, test/test_scgd0_gpu.jl:36-37) and are bitwise
reproducible run to run (test/test_scgd0_gpu.jl:38-40). The BF16x3 tensor-core path matches to
|ΔΣ| <= 1e-5 eV and |Δμ| <= 1e-5 eV.
"""
import numpy as np
import pytest

import refimpl as R
from epspectral_gb300 import ArgumentError, FrequencyGrid, graded_frequency_grid, synthetic

pytestmark = pytest.mark.gpu

W_AC = 1e-6


@pytest.fixture(scope="module")
def api():
    from epspectral_gb300 import api as A
    A.lib()
    return A


def occ(nlist=0.0, Tlist=(0.1,), typ="metal", nelec=1.0):
    return dict(Tlist=list(Tlist), nlist=[nlist] * len(Tlist), nelec=nelec, spin_degeneracy=2.0, type=typ)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def test_fan_migdal_sum_matches_oracle(api, oracle):
    # the case of test/test_scgd0_kernel.jl: per-pair ωq, an Inf coupling below ω_acoustic, a
    # random f -> i map, accumulation into a nonzero Im Σ, a graded grid.
    from test_oracle_scgd0 import per_pair_setup
    nm, ni, nf = 3, 13, 17
    g = FrequencyGrid.from_nodes(np.concatenate([np.arange(-1.0, -0.5999, 0.02), np.arange(-0.5, 0.5001, 0.1),
                                                 np.arange(0.6, 1.0001, 0.02)]))
    nw = len(g)
    Sin = 0.1 * R.pseudorandom(nw, ni, seed=7) + 1j * (-0.05 - 0.05 * np.abs(R.pseudorandom(nw, ni, seed=8)))
    g2 = np.abs(R.pseudorandom(nm, ni, nf, seed=9))
    wq = 0.05 + 0.2 * np.abs(R.pseudorandom(nm, ni, nf, seed=10))
    wq[1, 2, :] = 0.0
    g2[1, 2, :] = np.inf
    s = per_pair_setup(g, g2, wq, 0.8 * R.pseudorandom(nf, seed=11),
                       np.array([(5 * (f + 1)) % ni for f in range(nf)], dtype=np.int32), np.full(nf, 1.0 / nf))
    for tile in (None, 5):
        ref = oracle.imsigma(s, Sin, 0.07, 0.03, np.full((nw, ni), 0.5), omega_acoustic=1e-3, gpu_tile=tile)
        plan = api.Scgd0Plan(s, path="direct_fp64", gpu_tile=tile, omega_acoustic=1e-3)
        got = plan.imsigma(Sin, 0.07, 0.03, np.full((nw, ni), 0.5))
        assert np.all(np.isfinite(got))
        assert rel(got, ref) <= 1e-13


def test_dispersive_fan_migdal_fp32_matches_oracle(api, oracle):
    # the same per-pair-ωq case on the tensor-core plan, whose Fan-Migdal sum for dispersive modes
    # runs term by term in FP32 (float pairs where the value cancels): within 1e-5 relative of the
    # oracle's FP64 sum, the Inf coupling below ω_acoustic never read
    from test_oracle_scgd0 import per_pair_setup
    nm, ni, nf = 3, 13, 17
    g = FrequencyGrid.from_nodes(np.concatenate([np.arange(-1.0, -0.5999, 0.02), np.arange(-0.5, 0.5001, 0.1),
                                                 np.arange(0.6, 1.0001, 0.02)]))
    nw = len(g)
    Sin = 0.1 * R.pseudorandom(nw, ni, seed=7) + 1j * (-0.05 - 0.05 * np.abs(R.pseudorandom(nw, ni, seed=8)))
    g2 = np.abs(R.pseudorandom(nm, ni, nf, seed=9))
    wq = 0.05 + 0.2 * np.abs(R.pseudorandom(nm, ni, nf, seed=10))
    wq[1, 2, :] = 0.0
    g2[1, 2, :] = np.inf
    s = per_pair_setup(g, g2, wq, 0.8 * R.pseudorandom(nf, seed=11),
                       np.array([(5 * (f + 1)) % ni for f in range(nf)], dtype=np.int32), np.full(nf, 1.0 / nf))
    ref = oracle.imsigma(s, Sin, 0.07, 0.03, np.full((nw, ni), 0.5), omega_acoustic=1e-3)
    plan = api.Scgd0Plan(s, path="gemm_bf16", omega_acoustic=1e-3)
    got = plan.imsigma(Sin, 0.07, 0.03, np.full((nw, ni), 0.5))
    assert np.all(np.isfinite(got))
    assert rel(got, ref) <= 1e-5


def test_dispersive_loop_matches_oracle(api, oracle):
    # the small 3-band model with dispersive modes (±20 % over the zone): the tensor-core loop
    # (FP32 Fan-Migdal terms, BF16x3 Kramers-Kronig map) within |ΔΣ| <= 1e-5 eV, |Δμ| <= 1e-5 eV of the
    # oracle over three iterations with the μ update
    ws = graded_frequency_grid([(-0.3, 0.3, 0.01), (-1.5, 1.5, 0.05)])
    s = synthetic.with_dispersion(synthetic.cubic_t2g_setup(N=4, ws=ws, g2_dtype=np.float32, seed=5), 4, 0.2)
    o = occ(0.0, Tlist=(300 * synthetic.KELVIN, 600 * synthetic.KELVIN))
    kw = dict(eta_init=0.05, eta_min=[0.0, 0.03], tol=0.0, maxiter=3, mu_start=[-0.5, -0.5], omega_acoustic=W_AC)
    ref = oracle.loop_scgd0(s, o, **kw)
    got = api.loop_scgd0(s, o, path="gemm_bf16", **kw)
    assert np.max(np.abs(got["sigma"] - ref["sigma"])) <= 1e-5
    assert np.max(np.abs(got["mu"] - ref["mu"])) <= 1e-5
    direct = api.loop_scgd0(s, o, path="direct_fp64", **kw)
    assert rel(direct["sigma"], ref["sigma"]) <= 1e-10


@pytest.fixture(scope="module")
def holstein_gpu():
    ws = FrequencyGrid.from_nodes(np.arange(-200, 201) * 0.02)
    return synthetic.holstein_1d_setup(64, 1.0, 0.2, 0.2, ws)


@pytest.mark.parametrize("nlist", [0.0, -0.3])
def test_holstein_loop_matches_oracle(api, oracle, holstein_gpu, nlist):
    s = holstein_gpu
    kw = dict(eta_init=0.05, tol=1e-6, maxiter=30, mu_start=[0.0], omega_acoustic=W_AC)
    ref = oracle.loop_scgd0(s, occ(nlist), **kw)
    for path in ("direct_fp64", "gemm_fp64"):
        got = api.loop_scgd0(s, occ(nlist), path=path, **kw)
        assert got["niter"] == ref["niter"] and list(got["converged"]) == list(ref["converged"])
        assert rel(got["sigma"], ref["sigma"]) <= 1e-10
        assert abs(got["mu"][0] - ref["mu"][0]) <= 1e-10 * max(1.0, abs(ref["mu"][0]))
        again = api.loop_scgd0(s, occ(nlist), path=path, **kw)
        assert np.array_equal(again["sigma"], got["sigma"]) and np.array_equal(again["mu"], got["mu"])
    tiled = api.loop_scgd0(s, occ(nlist), path="direct_fp64", gpu_tile=7, **kw)
    assert rel(tiled["sigma"], ref["sigma"]) <= 1e-10
    bf = api.loop_scgd0(s, occ(nlist), path="gemm_bf16", **kw)
    assert np.max(np.abs(bf["sigma"] - ref["sigma"])) <= 1e-5
    assert abs(bf["mu"][0] - ref["mu"][0]) <= 1e-5


@pytest.fixture(scope="module")
def cubic_small():
    ws = graded_frequency_grid([(-0.3, 0.3, 0.01), (-1.5, 1.5, 0.05)])
    return synthetic.cubic_t2g_setup(N=4, ws=ws, g2_dtype=np.float32, seed=5)


def test_cubic_loop_matches_oracle(api, oracle, cubic_small):
    # two temperatures with their own η_min, multiplets, several modes, stars: three iterations
    # with the μ update, never converged (tol = 0), as test/test_scgd0_gpu.jl:9-11.
    s = cubic_small
    assert len(s["multiplets"]) > 0
    o = occ(0.0, Tlist=(300 * synthetic.KELVIN, 600 * synthetic.KELVIN))
    kw = dict(eta_init=0.05, eta_min=[0.0, 0.03], tol=0.0, maxiter=3, mu_start=[-0.5, -0.5], omega_acoustic=W_AC)
    ref = oracle.loop_scgd0(s, o, **kw)
    for path in ("direct_fp64", "gemm_fp64"):
        got = api.loop_scgd0(s, o, path=path, **kw)
        assert rel(got["sigma"], ref["sigma"]) <= 1e-10
        assert np.allclose(got["mu"], ref["mu"], rtol=1e-10, atol=1e-12)
        assert np.allclose(got["history"]["err"], ref["history"]["err"], rtol=1e-8)
        assert np.allclose(got["history"]["min_spectral_weight"], ref["history"]["min_spectral_weight"], rtol=1e-10)
    bf = api.loop_scgd0(s, o, path="gemm_bf16", **kw)
    assert np.max(np.abs(bf["sigma"] - ref["sigma"])) <= 1e-5
    assert np.max(np.abs(bf["mu"] - ref["mu"])) <= 1e-5
    gt = api.loop_scgd0(s, o, path="direct_fp64", gpu_tile=37, **kw)
    assert rel(gt["sigma"], ref["sigma"]) <= 1e-10


def test_errors_come_back_as_status(api, holstein_gpu, cubic_small):
    s = holstein_gpu
    with pytest.raises(ArgumentError, match="no chemical potential"):
        api.loop_scgd0(s, occ(1.5), eta_init=0.05, tol=1e-6, maxiter=5, mu_start=[0.0], omega_acoustic=W_AC)
    with pytest.raises(ArgumentError):
        api.loop_scgd0(s, occ(0.0), eta_init=0.05, tol=1e-6, maxiter=0, mu_start=[0.0], omega_acoustic=W_AC)
    with pytest.raises(ArgumentError):
        api.loop_scgd0(s, occ(0.0), eta_init=0.05, tol=1e-6, maxiter=2, mu_start=[0.0], eta_min=[0.0, 0.0],
                       omega_acoustic=W_AC)
    with pytest.raises(ArgumentError):
        api.loop_scgd0(s, occ(0.0), eta_init=0.05, tol=1e-6, maxiter=2, mu_start=[0.0],
                       sigma_init=np.zeros((401, 33, 2), complex), omega_acoustic=W_AC)
    # dispersive modes are refused by the FP64 recast path, accepted by the direct one and by the
    # tensor-core path (its FP32 term-by-term sum)
    disp = dict(s, omega_ph=np.asfortranarray(0.2 + 0.01 * np.arange(64.0)[None, :]))
    with pytest.raises(api.EpspError, match="dispersionless"):
        api.Scgd0Plan(disp, path="gemm_fp64", omega_acoustic=W_AC)
    api.Scgd0Plan(disp, path="direct_fp64", omega_acoustic=W_AC).close()
    api.Scgd0Plan(disp, path="gemm_bf16", omega_acoustic=W_AC).close()
    # a device allocation failure is reported, and the context stays usable
    ctx = api.Context(0)
    ctx.fail_next_alloc(1)
    with pytest.raises(api.EpspError, match="ENOMEM"):
        api.Scgd0Plan(s, path="direct_fp64", omega_acoustic=W_AC, ctx=ctx)
    r = api.loop_scgd0(s, occ(0.0), eta_init=0.05, tol=1e-6, maxiter=2, mu_start=[0.0], omega_acoustic=W_AC, ctx=ctx)
    assert r["niter"] == 2
    assert ctx.kernel_launches > 0


def test_temperatures_batched_in_one_launch_match_single_runs(api, oracle, cubic_small):
    # Four temperatures go through each iteration's launches together and freeze at different
    # iterations; every temperature's result must equal its own single-temperature run (bitwise on
    # the FP64 paths, whose Fan-Migdal sums still run per temperature; within 1e-6 eV on the
    # tensor-core path, whose stacked GEMM groups the K sums differently), and the oracle's
    # iteration history. The tensor-core path's iteration settles to ~1.2e-7 eV at 800 K (FP32
    # accumulation), so it runs to 5e-7 eV.
    s = cubic_small
    Ts = [150 * synthetic.KELVIN, 300 * synthetic.KELVIN, 450 * synthetic.KELVIN, 800 * synthetic.KELVIN]
    o = occ(0.0, Tlist=Ts)
    kw = dict(eta_init=0.05, tol=1e-7, maxiter=40, mu_start=[-0.5] * 4, omega_acoustic=W_AC)
    ref = oracle.loop_scgd0(s, o, **kw)
    assert len(set(ref["history"]["iter_frozen"])) > 1  # the temperatures freeze at different iterations
    for path in ("gemm_fp64", "gemm_bf16"):
        if path == "gemm_bf16":
            kw = dict(kw, tol=5e-7)
        got = api.loop_scgd0(s, o, path=path, **kw)
        assert list(got["converged"]) == [True] * 4
        for t in range(4):
            one = api.loop_scgd0(s, occ(0.0, Tlist=[Ts[t]]), path=path, **dict(kw, mu_start=[-0.5]))
            if path == "gemm_fp64":
                assert np.array_equal(got["sigma"][:, :, t], one["sigma"][:, :, 0])
                assert got["mu"][t] == one["mu"][0]
                assert got["history"]["iter_frozen"][t] == ref["history"]["iter_frozen"][t]
                assert rel(got["sigma"][:, :, t], ref["sigma"][:, :, t]) <= 1e-10
            else:
                assert np.max(np.abs(got["sigma"][:, :, t] - one["sigma"][:, :, 0])) <= 1e-6
                assert np.max(np.abs(got["sigma"][:, :, t] - ref["sigma"][:, :, t])) <= 1e-5


def test_streamed_g2_gives_the_resident_result(api, cubic_small):
    # gpu_tile streams g2 through the device in star-order chunks of that many inner states (the
    # caller's host g2 is never resident); the coupling sums run in the same order, so the GEMM
    # paths' results are bitwise those of one chunk. FP32 and BF16 storage.
    s = cubic_small
    o = occ(0.0, Tlist=(300 * synthetic.KELVIN,))
    kw = dict(eta_init=0.05, tol=0.0, maxiter=2, mu_start=[-0.5], omega_acoustic=W_AC)
    for g2 in (s["g2"], synthetic.float32_to_bf16_bits(s["g2"])):
        ss = dict(s, g2=np.asfortranarray(g2))
        for path in ("gemm_fp64", "gemm_bf16"):
            one = api.loop_scgd0(ss, o, path=path, **kw)
            for tile in (7, 100):
                got = api.loop_scgd0(ss, o, path=path, gpu_tile=tile, **kw)
                assert np.array_equal(got["sigma"], one["sigma"]) and np.array_equal(got["mu"], one["mu"]), (path, tile)
