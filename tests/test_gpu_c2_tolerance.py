"""The library at the full size of the 3-band benchmark model (16^3 k points: 495 outer / 12288 inner
states, 15 modes, graded 1251-node ωs, T = 300 K, one electron per cell).

* The mixed-precision paths against the FP64 path: scGD0 to 1e-6 eV on GEMM_BF16 from -iη_init, and
  the path the benchmark times -- scGD0 on GEMM_BF16 from the learned warm start with Σ kept on the
  device, then the ladder σ at Ω = 0.1 eV on GEMM_TF32 -- within the stated tolerances |ΔΣ| <= 1e-5
  eV, |Δμ| <= 1e-5 eV, relative σ <= 1e-4 (the network is trained on a few runs of the same model).
* The plain FP64 GPU paths against the oracle (the reference's loops restated in FP64 on the CPU)
  to 1e-10 relative, on bounded samples of outer states: the Fan-Migdal sum of both FP64 paths
  (src/scgd0_kernel.jl:59-86) and one ladder application of both (src/ladder.jl:245-296).
"""
import numpy as np
import pytest

import refimpl as R

pytestmark = pytest.mark.gpu

W_AC = 1e-4
# outer states sampled for the oracle comparisons (ranges [i0, i1))
IMSIGMA_SAMPLE = ((0, 4), (300, 302), (491, 495))
LADDER_SAMPLE = ((0, 2), (494, 495))


@pytest.fixture(scope="module")
def c2():
    from epspectral_gb300 import api, synthetic
    s = synthetic.cubic_t2g_setup(N=16, seed=0)
    T = 300 * synthetic.KELVIN
    occ = dict(Tlist=[T], nlist=[0.0], nelec=1.0, spin_degeneracy=2.0, type="metal")
    mu0 = synthetic.bare_mu(s, T, 1.0)
    ctx = api.Context(0)
    r64 = api.loop_scgd0(s, occ, eta_init=0.01, tol=1e-6, maxiter=50, mu_start=[mu0], omega_acoustic=W_AC,
                         path="gemm_fp64", ctx=ctx)
    assert r64["converged"][0]
    l64 = api.loop_ladder(s, r64["sigma"], r64["mu"], [T], [0.1], rtol=1e-2, maxiter=30, omega_acoustic=W_AC,
                          path="gemm_fp64", ctx=ctx)
    assert l64["converged"][0, 0]
    return dict(setup=s, T=T, occ=occ, mu0=mu0, ctx=ctx, r64=r64, l64=l64)


def _within(r, l, c2):
    r64, l64 = c2["r64"], c2["l64"]
    assert np.max(np.abs(r["sigma"] - r64["sigma"])) <= 1e-5
    assert abs(r["mu"][0] - r64["mu"][0]) <= 1e-5
    for key in ("sigma_bubble", "sigma_ladder"):
        a, b = l[key][:, :, 0, 0], l64[key][:, :, 0, 0]
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b), key


def test_bf16_path_within_stated_tolerance_of_fp64_at_full_size(c2):
    from epspectral_gb300 import api
    s, T = c2["setup"], c2["T"]
    r = api.loop_scgd0(s, c2["occ"], eta_init=0.01, tol=1e-6, maxiter=50, mu_start=[c2["mu0"]], omega_acoustic=W_AC,
                       path="gemm_bf16", ctx=c2["ctx"])
    assert r["converged"][0]
    l = api.loop_ladder(s, r["sigma"], r["mu"], [T], [0.1], rtol=1e-2, maxiter=30, omega_acoustic=W_AC,
                        path="gemm_bf16", ctx=c2["ctx"])
    assert l["converged"][0, 0]
    _within(r, l, c2)


def test_timed_path_within_stated_tolerance_of_fp64_at_full_size(c2):
    # the benchmark's step: warm-started BF16x3 scGD0, Σ handed to the TF32 ladder on the device
    from epspectral_gb300 import api
    from epspectral_gb300 import warmstart as W
    s, T, occ, ctx = c2["setup"], c2["T"], c2["occ"], c2["ctx"]
    runs = W.sample_runs(16, 11)
    X, Y, _ = W.generate_pairs(s, runs, ctx=ctx)
    ws = W.WarmStart(len(s["omegas"]), ctx=ctx)
    ws.fit(np.concatenate(X), np.concatenate(Y), epochs=20, batch=256, lr=1e-3)
    sp = api.Scgd0Plan(s, path="gemm_bf16", omega_acoustic=W_AC, ctx=ctx)
    lp = api.LadderPlan(s, path="gemm_tf32", omega_acoustic=W_AC, ctx=ctx)
    kw = dict(eta_init=0.01, tol=1e-6, maxiter=50, mu_start=[c2["mu0"]], warm=ws)
    r_dev = sp.run(occ, sigma_to_host=False, **kw)
    assert r_dev["converged"][0] and not r_dev["fallback"]
    l = lp.run(r_dev["sigma"], r_dev["mu"], [T], [0.1], solver="gmres", rtol=1e-2, maxiter=30)
    assert l["converged"][0, 0]
    r = sp.run(occ, **kw)  # the same run with Σ downloaded (deterministic: the same Σ)
    assert r["mu"][0] == r_dev["mu"][0]
    _within(r, l, c2)
    sp.close()
    lp.close()


@pytest.mark.parametrize("path", ["gemm_fp64", "direct_fp64"])
def test_fp64_fan_migdal_matches_oracle_on_samples_at_full_size(c2, oracle, path):
    from epspectral_gb300 import api
    s, T, ctx = c2["setup"], c2["T"], c2["ctx"]
    Sin = c2["r64"]["sigma"][:, :, 0]
    mu = c2["r64"]["mu"][0]
    got = api.Scgd0Plan(s, path=path, omega_acoustic=W_AC, ctx=ctx).imsigma(Sin, mu, T)
    for i0, i1 in IMSIGMA_SAMPLE:
        ref = oracle.imsigma_sample(s, Sin, mu, T, i0, i1, omega_acoustic=W_AC)[:, i0:i1]
        assert np.linalg.norm(ref) > 0
        assert np.linalg.norm(got[:, i0:i1] - ref) <= 1e-10 * np.linalg.norm(ref), (path, i0, i1)


@pytest.mark.parametrize("path", ["gemm_fp64", "direct_fp64"])
def test_fp64_ladder_application_matches_oracle_on_samples_at_full_size(c2, oracle, path):
    from epspectral_gb300 import api
    s, T, ctx = c2["setup"], c2["T"], c2["ctx"]
    nw, ni = len(s["omegas"]), s["eps_i"].size
    S = c2["r64"]["sigma"][:, :, 0]
    mu = c2["r64"]["mu"][0]
    J = R.pseudorandom_complex(nw, 4, 3, 2, ni, seed=0.37)
    J[0] = 0
    J[-1] = 0
    plan = api.LadderPlan(s, path=path, omega_acoustic=W_AC, ctx=ctx)
    got = plan.apply(J, S, mu, T, 0.1)
    plan.close()
    for i0, i1 in LADDER_SAMPLE:
        ref = oracle.ladder_apply_sample(s, J, S, mu, T, 0.1, i0, i1, omega_acoustic=W_AC)
        assert np.linalg.norm(ref) > 0
        assert np.linalg.norm(got[..., i0:i1] - ref) <= 1e-10 * np.linalg.norm(ref), (path, i0, i1)


def test_dispersive_fan_migdal_on_samples_at_full_size(c2, oracle):
    # the benchmark model with dispersive modes (±20 % over the zone): the tensor-core plan's FP32
    # term-by-term Fan-Migdal sum against the oracle's FP64 sum on bounded samples, |ΔImΣ| <= 1e-5 eV
    from epspectral_gb300 import api, synthetic
    s = synthetic.with_dispersion(c2["setup"], 16, 0.2)
    T, ctx = c2["T"], c2["ctx"]
    Sin = c2["r64"]["sigma"][:, :, 0]
    mu = c2["r64"]["mu"][0]
    plan = api.Scgd0Plan(s, path="gemm_bf16", omega_acoustic=W_AC, ctx=ctx)
    got = plan.imsigma(Sin, mu, T)
    plan.close()
    for i0, i1 in IMSIGMA_SAMPLE:
        ref = oracle.imsigma_sample(s, Sin, mu, T, i0, i1, omega_acoustic=W_AC)[:, i0:i1]
        assert np.linalg.norm(ref) > 0
        assert np.max(np.abs(got[:, i0:i1] - ref)) <= 1e-5, (i0, i1)
