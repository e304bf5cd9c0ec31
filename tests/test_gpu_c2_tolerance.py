"""The mixed-precision path against the FP64 path at the full size of the 3-band benchmark model
(16^3 k points: 495 outer / 12288 inner states, 15 modes, graded 1251-node ωs, T = 300 K, one
electron per cell): scGD0 to 1e-6 eV from -iη_init (and from the learned warm start's fallback
path, the plain start) and the ladder σ at Ω = 0.1 eV. The stated tolerances: |ΔΣ| <= 1e-5 eV,
|Δμ| <= 1e-5 eV, relative σ error <= 1e-4. The FP64 path is itself checked against the oracle at
small sizes (test_gpu_scgd0.py, test_gpu_ladder.py).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bf16_path_within_stated_tolerance_of_fp64_at_full_size():
    from epspectral_gb300 import api, synthetic
    s = synthetic.cubic_t2g_setup(N=16, seed=0)
    T = 300 * synthetic.KELVIN
    occ = dict(Tlist=[T], nlist=[0.0], nelec=1.0, spin_degeneracy=2.0, type="metal")
    mu0 = synthetic.bare_mu(s, T, 1.0)
    res = {}
    for path in ("gemm_fp64", "gemm_bf16"):
        r = api.loop_scgd0(s, occ, eta_init=0.01, tol=1e-6, maxiter=50, mu_start=[mu0], omega_acoustic=1e-4, path=path)
        assert r["converged"][0], path
        l = api.loop_ladder(s, r["sigma"], r["mu"], [T], [0.1], rtol=1e-2, maxiter=30, omega_acoustic=1e-4,
                            path=path)
        assert l["converged"][0, 0], path
        res[path] = (r, l)
    (r64, l64), (r16, l16) = res["gemm_fp64"], res["gemm_bf16"]
    assert np.max(np.abs(r16["sigma"] - r64["sigma"])) <= 1e-5
    assert abs(r16["mu"][0] - r64["mu"][0]) <= 1e-5
    for key in ("sigma_bubble", "sigma_ladder"):
        a, b = l16[key][:, :, 0, 0], l64[key][:, :, 0, 0]
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b), key
