"""Example: the large 3-band cubic t2g model -- 32^3 k points (2907 outer / 98304 inner states), 15
dispersionless modes, g2 stored as BF16 (8.6 GB, drawn in chunks from a seed), a graded grid of
4101 nodes (0.5 meV on ±0.4 eV, 2 meV on ±1.5 eV, 5 meV on ±4 eV, 20 meV on ±8 eV) -- on the
tensor-core path: plan set-up with g2 resident in host memory and streamed through the device in
chunks of --gpu-tile inner states, scGD0 of 8 temperatures (100-800 K) to 1e-6 eV in one batched
run, the FP64 recast path at one temperature for the error, and the ladder at a few Ωs (seconds per
Ω; the contraction in TF32, or --ladder-path gemm_bf16). Prints one JSON line.

    python epspectral.jl_gb300/examples/c5_large.py [--gpu-tile 8192] [--omegas 2] [--no-fp64] [--ladder-path P]
        [--fp64-ladder]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from epspectral_gb300 import api, graded_frequency_grid, synthetic  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--N", type=int, default=32)
    ap.add_argument("--gpu-tile", type=int, default=8192)
    ap.add_argument("--omegas", type=int, default=2)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--ladder-path", default="gemm_tf32", choices=("gemm_tf32", "gemm_bf16"))
    ap.add_argument("--fp64-ladder", action="store_true",
                    help="also the FP64 recast ladder at the first Omega on the FP64 Sigma (minutes), for the error")
    a = ap.parse_args()
    out = {}
    t0 = time.perf_counter()
    ws = graded_frequency_grid([(-0.4, 0.4, 0.0005), (-1.5, 1.5, 0.002), (-4.0, 4.0, 0.005), (-8.0, 8.0, 0.02)])
    s = synthetic.cubic_t2g_setup(N=a.N, ws=ws, g2_dtype="bf16", g2_chunk=2048, seed=0)
    out["model"] = dict(N=a.N, ni=int(s["eps_i"].size), nf=int(s["eps_f"].size), nw=len(ws),
                        nwa=len(s["omegas_spectral"]), g2_gb=s["g2"].nbytes / 1e9, g2_dtype="bf16",
                        build_s=time.perf_counter() - t0)
    print(json.dumps(out["model"]), flush=True)
    Ts = list(np.linspace(100.0, 800.0, 8) * synthetic.KELVIN)
    mus = [synthetic.bare_mu(s, T, 1.0) for T in Ts]
    occ = dict(Tlist=Ts, nlist=[0.0] * 8, nelec=1.0, spin_degeneracy=2.0, type="metal")
    ctx = api.Context(0)
    t0 = time.perf_counter()
    sp = api.Scgd0Plan(s, path="gemm_bf16", omega_acoustic=1e-4, gpu_tile=a.gpu_tile, ctx=ctx)
    out["scgd0_setup_streamed_s"] = time.perf_counter() - t0
    ctx.timer_begin()
    r = sp.run(occ, eta_init=0.01, tol=1e-6, maxiter=50, mu_start=mus)
    out["scgd0_8T_s"] = ctx.timer_end() / 1e3
    out["scgd0_8T_iters"] = int(r["niter"])
    out["scgd0_8T_frozen"] = [int(x) for x in r["history"]["iter_frozen"]]
    out["scgd0_converged"] = bool(r["converged"].all())
    sp.close()
    print(json.dumps({k: out[k] for k in ("scgd0_setup_streamed_s", "scgd0_8T_s", "scgd0_8T_iters")}), flush=True)
    T3 = Ts[2]  # 300 K
    o1 = dict(Tlist=[T3], nlist=[0.0], nelec=1.0, spin_degeneracy=2.0, type="metal")
    if not a.no_fp64:
        fp = api.Scgd0Plan(s, path="gemm_fp64", omega_acoustic=1e-4, ctx=ctx)
        ctx.timer_begin()
        r64 = fp.run(o1, eta_init=0.01, tol=1e-6, maxiter=50, mu_start=[mus[2]])
        out["fp64_scgd0_300K_s"] = ctx.timer_end() / 1e3
        out["fp64_scgd0_300K_iters"] = int(r64["niter"])
        fp.close()
        out["max_abs_dsigma_eV_300K"] = float(np.max(np.abs(r["sigma"][:, :, 2] - r64["sigma"][:, :, 0])))
        out["abs_dmu_eV_300K"] = float(abs(r["mu"][2] - r64["mu"][0]))
        print(json.dumps({k: out[k] for k in ("fp64_scgd0_300K_s", "max_abs_dsigma_eV_300K")}), flush=True)
    t0 = time.perf_counter()
    lp = api.LadderPlan(s, path=a.ladder_path, omega_acoustic=1e-4, gpu_tile=a.gpu_tile, ctx=ctx)
    out["ladder_path"] = a.ladder_path
    out["ladder_setup_streamed_s"] = time.perf_counter() - t0
    out["ladder_gemm_autotune"] = lp.gemm_config()
    Om = list(np.linspace(0.05, 0.1, a.omegas))
    ctx.profile("tc_ladder")
    ctx.timer_begin()
    l = lp.run(r["sigma"][:, :, 2:3], r["mu"][2:3], [T3], Om, rtol=1e-2, maxiter=30)
    out["ladder_s_per_omega"] = ctx.timer_end() / 1e3 / len(Om)
    ms, n = ctx.profile_read()
    ctx.profile(None)
    out["ladder_gmres_iters"] = [int(x) for x in l["niter"].ravel()]
    out["ladder_converged"] = bool(l["converged"].all())
    ni = int(s["eps_i"].size)
    # the contraction Z = Jr Bz: rows 16 nω (4 components x (c0, re/im) x nodes), columns 15 modes x 3ni,
    # depth 3ni (rows padded to 32 nodes are not counted)
    M, N, K = 16 * len(ws), 15 * 3 * ni, 3 * ni
    if n:
        out["tc_ladder_ms_per_launch"] = ms / n
        out["tc_ladder_useful_tflops"] = 2.0 * M * N * K / (ms / n / 1e3) / 1e12
    out["sigma_ladder_xx"] = float(l["sigma_ladder"][0, 0, 0, 0])
    lp.close()
    if a.fp64_ladder and not a.no_fp64:
        # the plain FP64 path end to end at the first Ω: FP64 Σ and μ (300 K), the recast ladder in FP64
        t0 = time.perf_counter()
        lp64 = api.LadderPlan(s, path="gemm_fp64", omega_acoustic=1e-4, gpu_tile=a.gpu_tile, ctx=ctx)
        out["fp64_ladder_setup_s"] = time.perf_counter() - t0
        ctx.timer_begin()
        l64 = lp64.run(r64["sigma"], r64["mu"], [T3], Om[:1], rtol=1e-2, maxiter=30)
        out["fp64_ladder_s"] = ctx.timer_end() / 1e3
        out["fp64_ladder_gmres_iters"] = int(l64["niter"][0, 0])
        lp64.close()
        a_, b_ = l["sigma_ladder"][:, :, 0, 0], l64["sigma_ladder"][:, :, 0, 0]
        out["rel_sigma_ladder_vs_fp64"] = float(np.linalg.norm(a_ - b_) / np.linalg.norm(b_))
        a_, b_ = l["sigma_bubble"][:, :, 0, 0], l64["sigma_bubble"][:, :, 0, 0]
        out["rel_sigma_bubble_vs_fp64"] = float(np.linalg.norm(a_ - b_) / np.linalg.norm(b_))
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
