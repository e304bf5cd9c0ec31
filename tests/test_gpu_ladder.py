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
        for path, tol in (("direct_fp64", 1e-10), ("gemm_fp64", 1e-10), ("gemm_bf16", 1e-4)):
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
    bf = api.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], Omegas, path="gemm_bf16", **kw)
    assert rel(bf["sigma_ladder"], ref["sigma_ladder"]) <= 1e-4
    # fixed point, streamed-size chunks, Ω > 0 (test/test_ladder_gpu.jl:134-139)
    fk = dict(solver="fixed_point", rtol=1e-6, maxiter=200, omega_acoustic=W_AC)
    fref = oracle.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], [0.1], **fk)
    fgot = api.loop_ladder(s, c["sigma"], c["mu"], c["Tlist"], [0.1], path="direct_fp64", gpu_tile=7, **fk)
    assert np.array_equal(fgot["niter"], fref["niter"]) and fgot["converged"].all()
    assert rel(fgot["sigma_ladder"], fref["sigma_ladder"]) <= 1e-10


def test_holstein_current_correction_vanishes(api, hsym):
    # test/test_ladder_holstein.jl:5-26 on the GPU paths
    c = hsym
    for path in ("direct_fp64", "gemm_fp64", "gemm_bf16"):
        out = api.loop_ladder(c["setup"], c["sigma"], c["mu"], c["Tlist"], [0.0, 0.2], path=path, omega_acoustic=W_AC)
        assert np.linalg.norm(out["sigma_ladder"] - out["sigma_bubble"]) <= 1e-9 * np.linalg.norm(out["sigma_bubble"])
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
