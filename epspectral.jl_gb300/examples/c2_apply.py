"""Example: the 3-band t2g model at 16^3 k points (the benchmark workload) through the Python API --
a short scGD0 run on the tensor-core path, then one ladder application at Ω = 0.1 eV on each
path, printing the device time of each. Also the target of the Nsight Compute captures.

    python epspectral.jl_gb300/examples/c2_apply.py [--path gemm_bf16|gemm_fp64] [--iters N]
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from epspectral_gb300 import api, synthetic  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--path", default="gemm_bf16")
    ap.add_argument("--iters", type=int, default=3)
    a = ap.parse_args()
    s = synthetic.cubic_t2g_setup(N=16, seed=0)
    T = 300 * synthetic.KELVIN
    occ = dict(Tlist=[T], nlist=[0.0], nelec=1.0, spin_degeneracy=2.0)
    mu0 = synthetic.bare_mu(s, T, 1.0)
    ctx = api.Context(0)
    plan = api.Scgd0Plan(s, path=a.path, omega_acoustic=1e-4, ctx=ctx)
    ctx.timer_begin()
    r = plan.run(occ, eta_init=0.01, tol=0.0, maxiter=a.iters, mu_start=[mu0])
    print(f"scGD0 {a.path}: {a.iters} iterations in {ctx.timer_end():.2f} ms, err {r['history']['err'][0]}")
    lp = api.LadderPlan(s, path=a.path, omega_acoustic=1e-4, ctx=ctx)
    nw, ni = len(s["omegas"]), s["eps_i"].size
    J = np.asfortranarray(np.full((nw, 4, 3, 2, ni), 1e-2 + 1e-2j))
    J[0] = 0
    J[-1] = 0
    ctx.timer_begin()
    LJ = lp.apply(J, r["sigma"][:, :, 0], r["mu"][0], T, 0.1)
    print(f"ladder apply {a.path}: {ctx.timer_end():.2f} ms (with host copies), |LJ| = {np.linalg.norm(LJ):.6e}")


if __name__ == "__main__":
    main()
