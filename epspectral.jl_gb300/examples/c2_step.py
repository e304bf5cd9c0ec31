"""Example: the benchmark step on the 3-band t2g model at 16^3 k points -- scGD0 to 1e-6 eV on the
tensor-core path (from a trained warm start when --warm names a saved network, e.g. the one
`bench.py --save-warm` writes), then the ladder σ(Ω) at Ω = 0.1 eV by GMRES (the contraction in
TF32, or --ladder-path gemm_bf16 for BF16x3) -- repeated --steps times, each part inside an NVTX
range ("scgd0", "ladder") so that Nsight Compute can select it. Σ stays on the device between the
two (the ladder reads the scGD0 plan's copy), as in bench.py's step.

    python epspectral.jl_gb300/examples/c2_step.py [--warm net.npz] [--steps N] [--ladder-path P]
"""
import argparse
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from epspectral_gb300 import api, synthetic  # noqa: E402
from epspectral_gb300 import warmstart as W  # noqa: E402


def nvtx():
    try:
        import torch
        return torch.cuda.nvtx.range_push, torch.cuda.nvtx.range_pop
    except Exception:  # no torch: no ranges
        return (lambda name: None), (lambda: None)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--warm", default=None)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--ladder-path", default="gemm_tf32", choices=("gemm_tf32", "gemm_bf16"))
    a = ap.parse_args()
    push, pop = nvtx()
    s = synthetic.cubic_t2g_setup(N=16, seed=0)
    T = 300 * synthetic.KELVIN
    occ = dict(Tlist=[T], nlist=[0.0], nelec=1.0, spin_degeneracy=2.0, type="metal")
    mu0 = synthetic.bare_mu(s, T, 1.0)
    ctx = api.Context(0)
    ws = W.WarmStart.load(a.warm, ctx=ctx) if a.warm else None
    sp = api.Scgd0Plan(s, path="gemm_bf16", omega_acoustic=1e-4, ctx=ctx)
    lp = api.LadderPlan(s, path=a.ladder_path, omega_acoustic=1e-4, ctx=ctx)
    for k in range(a.steps):
        push("scgd0")
        ctx.timer_begin()
        r = sp.run(occ, eta_init=0.01, tol=1e-6, maxiter=50, mu_start=[mu0], warm=ws, sigma_to_host=False)
        t_s = ctx.timer_end()
        pop()
        push("ladder")
        ctx.timer_begin()
        l = lp.run(r["sigma"], r["mu"], [T], [0.1], rtol=1e-2, maxiter=30)
        t_l = ctx.timer_end()
        pop()
        print(f"step {k}: scGD0 {r.get('iters_total', r['niter'])} iterations {t_s:.2f} ms, ladder "
              f"{int(l['niter'][0, 0])} GMRES iterations {t_l:.2f} ms, sigma_xx {l['sigma_ladder'][0, 0, 0, 0]:.6e}")


if __name__ == "__main__":
    main()
