"""Headline benchmark: the scGD0 iteration to tolerance plus the ladder conductivity at one probe
frequency, on the synthetic 3-band cubic t2g model (16^3 k points: 495 outer / 12288 inner states,
15 dispersionless modes in [10, 80] meV, log-normal FP32 g2 from a seed, graded 1251-node ωs, one
temperature 300 K).

One step = scGD0 to max|ΔΣ| < 1e-6 eV (maxiter 50) started from the learned warm start (the G0D0
iteration from Σ = -iη_init, η_init = 10 meV, then the network's Σ_init, on the device), then the
ladder σ(Ω) at Ω = 0.1 eV by GMRES (rtol 1e-2, maxiter 30), on the fast path (recast Fan-Migdal sum
and per-mode regrouped ladder on the tcgen05 tensor cores, BF16 split operands). `value` is the
device time of a step in seconds (CUDA events on the library's stream), inputs resident in HBM;
`e2e` is the same step through the public API from host arrays (plan set-up with the g2 upload,
results read back). Before the timed steps the warm-start network is trained on the GPU on pairs
the method generates (256 seeded runs of the same model with T in [100, 800] K, filling in
[0.5, 1.5] e/site, g2 scale in [0.5, 2]) and checked on 32 held-out runs. The plain FP64 GPU
paths are timed once beside it for the speed-up and the accuracy check.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun every rank runs an independent replica on its own GPU (the path has no exchange);
rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "epspectral.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "scGD0 s-to-tol & ladder s per Ω, mixed+warm vs plain FP64, |ΔΣ|≤1e-5 eV"
T_K = 300.0
ETA_INIT, TOL, MAXITER = 0.01, 1e-6, 50
OMEGA, L_RTOL, L_MAXITER = 0.1, 1e-2, 30
W_AC = 1e-4
# The ladder contraction's precision on the timed path: one TF32 product (operands rounded to TF32,
# FP32 accumulation); the BF16x3 path is timed beside it. scGD0 stays on BF16x3 split precision.
LADDER_PATH = "gemm_tf32"
# Iteration counts of this workload on the FP64 path (scGD0 iterations to tol; ladder operator
# applications per Ω: GMRES iterations plus one), as this script's FP64 leg measures them on a GB300.
# The reference arm cannot run the workload to the end on the CPU (hours) and runs without the GPU,
# so it scales its bounded samples by these counts; the GPU arm uses the counts of its own FP64 run
# and reports whether they still equal these.
FP64_SCGD0_ITERS = 12
FP64_LADDER_APPLIES = 2
# DRAM bytes (read + write) and tensor-pipe activity of one ladder-contraction launch of this
# workload (Z = Jr Bz, the TF32 persistent CTA-pair kernel), from one Nsight Compute
# capture of the same kernel on a GB300 (summarised with the other captures under profiles/)
TC_LADDER_TRAFFIC_BYTES = 1.643e9 + 1.786e9
TC_LADDER_TENSOR_PIPE_ACTIVE = 0.633
# learned warm start: training and held-out runs, epochs
WARM_TRAIN_RUNS, WARM_HELDOUT_RUNS, WARM_EPOCHS = 256, 32, 40


def workload():
    from epspectral_gb300 import synthetic
    s = synthetic.cubic_t2g_setup(N=16, seed=0)
    T = T_K * synthetic.KELVIN
    occ = dict(Tlist=[T], nlist=[0.0], nelec=1.0, spin_degeneracy=2.0, type="metal")
    mu0 = synthetic.bare_mu(s, T, 1.0)
    return s, T, occ, mu0


def bench_config(s, world) -> dict:
    """The workload, the same on both arms."""
    return dict(workload="3-band cubic t2g nk=16^3, 495 outer / 12288 inner states, 15 modes, graded "
                         "1251-node grid, T=300 K; scGD0 to 1e-6 eV + ladder at one Omega=0.1 eV",
                ni=int(s["eps_i"].size), nf=int(s["eps_f"].size), nw=len(s["omegas"]), nm=15,
                path=f"scgd0 gemm_bf16, ladder {LADDER_PATH}",
                warm_start=True, l2="flushed between steps (512 MB write)", parallelism=f"replicas x{world}")


def setup_bytes(s) -> int:
    n = 0
    for k, v in s.items():
        if isinstance(v, np.ndarray):
            n += v.nbytes
    return n


class _NvmlClocks:
    """Read-only NVML queries (SM clock, its maximum, power, clock-event reasons) through the driver's
    libnvidia-ml, for sampling at millisecond intervals; None where the library is absent."""

    # nvmlClocksEventReason* bits of the NVML API
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    @classmethod
    def open(cls, device: int):
        import ctypes
        try:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return None
        except (OSError, AttributeError):
            return None
        self = cls()
        self.ct, self.lib = ctypes, lib
        self.h = ctypes.c_void_p()
        bus = None
        try:
            import torch
            pr = torch.cuda.get_device_properties(device)
            bus = f"{pr.pci_domain_id:08X}:{pr.pci_bus_id:02X}:{pr.pci_device_id:02X}.0"
        except Exception:
            pass
        ok = bus is not None and lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(self.h)) == 0
        if not ok and lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(device), ctypes.byref(self.h)) != 0:
            lib.nvmlShutdown()
            return None
        self.reason_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
        v = ctypes.c_uint()
        self.max_mhz = float(v.value) if lib.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(v)) == 0 else None
        return self

    def sample(self):
        ct, lib = self.ct, self.lib
        mhz, mw, bits = ct.c_uint(), ct.c_uint(), ct.c_ulonglong()
        if lib.nvmlDeviceGetClockInfo(self.h, 1, ct.byref(mhz)) != 0:
            return None
        lib.nvmlDeviceGetPowerUsage(self.h, ct.byref(mw))
        self.reason_fn(self.h, ct.byref(bits))
        return float(mhz.value), mw.value / 1e3, [n for b, n in self.REASONS.items() if bits.value & b]

    def close(self):
        self.lib.nvmlShutdown()


class ClockSampler:
    """SM clock, power and clock-event reasons sampled while the timed region runs: NVML every 2 ms
    (the timed region lasts a fraction of a second), else nvidia-smi every 100 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.nvml = None
        self.lines = []
        self.samples = []
        self.stop = threading.Event()

    def __enter__(self):
        self.nvml = _NvmlClocks.open(self.device)
        if self.nvml is not None:
            self.t = threading.Thread(target=self._poll, daemon=True)
            self.t.start()
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _poll(self):
        while not self.stop.is_set():
            x = self.nvml.sample()
            if x is not None:
                self.samples.append(x)
            self.stop.wait(0.002)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.nvml is not None:
            self.stop.set()
            self.t.join(timeout=5)
            self.nvml.close()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.nvml is not None:
            sm = [x[0] for x in self.samples]
            reasons = sorted({r for x in self.samples for r in x[2]})
            return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": self.nvml.max_mhz,
                    "sm_min_mhz": float(min(sm)) if sm else None, "reasons": reasons, "samples": len(sm),
                    "power_w_median": float(np.median([x[1] for x in self.samples])) if sm else None,
                    "source": "NVML every 2 ms"}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                mx = float(p[1])
            except ValueError:
                continue
            for nm, v in zip(names, p[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvidia-smi every 100 ms"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["bf16_tflops"]), float(p["bf16_tflops_sustained"]), float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, 1700.0, 6800.0, "fallback"


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def flush_l2(device: int, nbytes=512 << 20):
    """Overwrite a buffer larger than L2 (129 MB) between timed steps."""
    import torch
    b = torch.empty(nbytes // 4, dtype=torch.float32, device=f"cuda:{device}")
    b.fill_(1.0)
    torch.cuda.synchronize()
    del b


def train_warm_start(s, ctx):
    """Trains the warm start on the GPU on pairs from the method itself and measures it on held-out
    runs (plain iterations from the pair generation, warm-started iterations on the device)."""
    from epspectral_gb300 import api
    from epspectral_gb300 import warmstart as W
    t0 = time.perf_counter()
    runs_tr = W.sample_runs(WARM_TRAIN_RUNS, 11)
    runs_te = W.sample_runs(WARM_HELDOUT_RUNS, 12, group=4)
    Xtr, Ytr, _ = W.generate_pairs(s, runs_tr, ctx=ctx)
    Xte, Yte, rte = W.generate_pairs(s, runs_te, ctx=ctx)
    t_gen = time.perf_counter() - t0
    nw = len(s["omegas"])
    ws = W.WarmStart(nw, ctx=ctx)
    t0 = time.perf_counter()
    hist = ws.fit(np.concatenate(Xtr), np.concatenate(Ytr), epochs=WARM_EPOCHS, batch=256, lr=1e-3)
    t_fit = time.perf_counter() - t0
    del Xtr, Ytr
    plain, warm, dsig, fallbacks = [], [], [], 0
    plan, plan_scale = None, None
    for run, rec, X, Y in zip(runs_te, rte, Xte, Yte):
        if plan is None or run["scale"] != plan_scale:
            if plan is not None:
                plan.close()
            ss = dict(s)
            ss["g2"] = np.asfortranarray(s["g2"] * np.float32(run["scale"]))
            plan, plan_scale = api.Scgd0Plan(ss, path="gemm_bf16", omega_acoustic=W_AC, ctx=ctx), run["scale"]
        occ = dict(Tlist=[rec["T"]], nlist=[0.0], nelec=run["filling"], spin_degeneracy=2.0, type="metal")
        r = plan.run(occ, eta_init=ETA_INIT, tol=TOL, maxiter=MAXITER, mu_start=[rec["mu0"]], warm=ws,
                     coupling_scale=run["scale"])
        fallbacks += int(r["fallback"])
        S_plain = (X[:, :nw] + Y[:, :nw] + 1j * (X[:, nw:2 * nw] + Y[:, nw:])).T
        dsig.append(float(np.max(np.abs(r["sigma"][:, :, 0] - S_plain))))
        plain.append(rec["niter"])
        warm.append(r["iters_total"])
    plan.close()
    info = dict(train_runs=WARM_TRAIN_RUNS, heldout_runs=WARM_HELDOUT_RUNS, epochs=WARM_EPOCHS,
                network=f"MLP {'-'.join(map(str, ws.dims))}, SiLU, BF16 weights / FP32 accumulate, Adam",
                pair_generation_s=t_gen, train_s=t_fit, train_device_s=ws.train_device_s,
                final_loss=float(hist[-1]), first_loss=float(hist[0]),
                heldout_plain_iters_mean=float(np.mean(plain)), heldout_warm_iters_mean=float(np.mean(warm)),
                heldout_fallbacks=fallbacks, heldout_max_abs_dsigma_vs_plain_eV=float(np.max(dsig)))
    return ws, info


def run_ours(args, world, rank, local):
    from epspectral_gb300 import api, synthetic
    s, T, occ, mu0 = workload()
    ctx = api.Context(local)
    ws, warm_info = train_warm_start(s, ctx)
    if args.save_warm:
        ws.save(args.save_warm)
    sp = api.Scgd0Plan(s, path="gemm_bf16", omega_acoustic=W_AC, ctx=ctx)
    lp = api.LadderPlan(s, path=LADDER_PATH, omega_acoustic=W_AC, ctx=ctx)
    nw, ni = len(s["omegas"]), s["eps_i"].size

    def step():
        # Σ stays on the device between the two loops (the ladder reads the scGD0 plan's own copy);
        # μ, the convergence flags and the history come back to the host
        ctx.timer_begin()
        r = sp.run(occ, eta_init=ETA_INIT, tol=TOL, maxiter=MAXITER, mu_start=[mu0], warm=ws, sigma_to_host=False)
        t_s = ctx.timer_end() / 1e3
        ctx.timer_begin()
        l = lp.run(r["sigma"], r["mu"], [T], [OMEGA], solver="gmres", rtol=L_RTOL, maxiter=L_MAXITER)
        t_l = ctx.timer_end() / 1e3
        return r, l, t_s, t_l

    for _ in range(args.warmup):
        r, l, _, _ = step()
    flush_l2(local)
    launches0 = ctx.kernel_launches
    ctx.profile("tc_ladder")
    times, ts, tl = [], [], []
    barrier(world)
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            r, l, t_s, t_l = step()
            ts.append(t_s)
            tl.append(t_l)
            times.append(t_s + t_l)
            if k + 1 < args.steps:
                flush_l2(local)
    barrier(world)
    prof_ms, prof_n = ctx.profile_read()
    ctx.profile(None)
    launches = ctx.kernel_launches - launches0
    total = max_over_ranks(float(np.sum(times)), world)
    value = total / (args.steps * world)
    out = dict(metric=METRIC, value=value, unit="s", n_gpus=world, steps=args.steps, warmup=args.warmup,
               ms_per_step=1e3 * total / args.steps, higher_is_better=False,
               scaling="weak", vs_baseline=None,
               dtype="scGD0: bf16x3 GEMMs; ladder: tf32 contraction, bf16x3 Kramers-Kronig product (fp32 accumulate); "
                     "fp64 reductions",
               data="synthetic (seeded 3-band t2g model, log-normal g2)",
               config=bench_config(s, world))
    if rank != 0:
        return
    out["scgd0_s_to_tol"] = float(np.median(ts))
    out["e2e_cold_note"] = "e2e_cold: the same public-API calls in a fresh process (empty autotune cache, first launches)"
    out["scgd0_iters"] = int(r["iters_total"])
    out["scgd0_warm_fallback"] = bool(r["fallback"])
    # the same run with Σ downloaded, for the accuracy figures below
    r = sp.run(occ, eta_init=ETA_INIT, tol=TOL, maxiter=MAXITER, mu_start=[mu0], warm=ws)
    ctx.timer_begin()
    r_cold = sp.run(occ, eta_init=ETA_INIT, tol=TOL, maxiter=MAXITER, mu_start=[mu0])
    out["scgd0_s_to_tol_without_warm_start"] = ctx.timer_end() / 1e3
    out["scgd0_iters_without_warm_start"] = int(r_cold["niter"])
    out["warm_start"] = warm_info
    # what the warm start costs and when it pays: pair generation plus training, against the device
    # time it saves per scGD0 run on this workload
    saved = out["scgd0_s_to_tol_without_warm_start"] - out["scgd0_s_to_tol"]
    cost = warm_info["pair_generation_s"] + warm_info["train_s"]
    out["warm_start_cost"] = dict(pair_generation_plus_train_s=cost, saved_s_per_scgd0_run=saved,
                                  break_even_runs=(cost / saved) if saved > 0 else None,
                                  note="the 5x target against plain FP64 is met by precision alone; the warm start "
                                       "pays only for a model family run many times")
    out["ladder_s_per_omega"] = float(np.median(tl))
    out["ladder_gemm_autotune"] = lp.gemm_config()
    out["ladder_gmres_iters"] = int(l["niter"][0, 0])
    out["gpu_launches"] = int(launches)
    # roofline of the dominant kernel: the ladder's tensor-core contraction Z = Jr Bz (rows: 16 per
    # node; columns: 15 modes x 3ni; K: 3ni pairs), useful work without the node padding
    M, N, K = 16 * nw, 15 * 3 * ni, 3 * ni
    if prof_n:
        avg_s = prof_ms / prof_n / 1e3
        flops = 2.0 * M * N * K
        burst, sust, hbm, src = peaks()
        achieved = flops / avg_s / 1e12
        tf32 = measure_tf32_peak(local)
        out["roofline"] = dict(kernel=f"tc_gemm {LADDER_PATH[5:]} (ladder contraction)", bound="tensor",
                               achieved=achieved, peak=burst, unit="TFLOP/s", frac=achieved / burst,
                               traffic=TC_LADDER_TRAFFIC_BYTES,
                               traffic_source="ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch "
                                              "(the contraction's capture under profiles/)",
                               peak_source=f"{src} bf16 burst (cuBLAS, MEASURED_PEAKS.json)", launches=prof_n,
                               avg_ms=1e3 * avg_s, flops_per_launch=flops,
                               tf32_peak=tf32, frac_of_tf32_peak=(achieved / tf32) if tf32 else None,
                               tf32_peak_source="cuBLAS TF32 GEMM 8192^3 through torch, best of 10, this run",
                               tensor_pipe_active_ncu=TC_LADDER_TENSOR_PIPE_ACTIVE,
                               tensor_pipe_source="ncu sm__pipe_tensor_cycles_active of one launch "
                                                  "(the contraction's capture under profiles/)")
    out["clocks"] = clk.summary()
    # end to end through the public API from host arrays, g2 in page-locked host memory (registered
    # before the timed region, as a caller keeps a large input pinned; pageable if that fails)
    t0 = time.perf_counter()
    pinned = register_g2(ctx, s)
    t_reg = time.perf_counter() - t0
    try:  # three full sequences (each streams g2 afresh), their mean reported
        e2e_samples = [e2e_calls(s, ws, ctx, T, occ, mu0) for _ in range(3)]
    finally:
        if pinned is True:
            ctx.host_unregister(s["g2"])
    e2e = float(np.mean(e2e_samples))
    # both set-ups' arrays, g2 once (the context keeps it for the second), Σ to the ladder
    how = (f"page-locked with epsp_host_register before the timed region ({t_reg:.3f} s), read in place by the "
           f"set-up's gather kernel" if pinned is True else f"pageable (registration failed: {pinned}), gathered on "
           f"the host")
    out["e2e"] = dict(value=e2e, unit="s", h2d_bytes_per_step=2 * setup_bytes(s) - s["g2"].nbytes + 16 * nw * ni,
                      d2h_bytes_per_step=16 * nw * ni + 8 * 9 * 2, samples=e2e_samples,
                      note=f"mean of {len(e2e_samples)} sequences; g2 ({s['g2'].nbytes / 1e6:.0f} MB) {how}")
    out["e2e_cold"] = e2e_cold(ws)
    # plain FP64 GPU paths, timed once
    plain = {}
    fp = api.Scgd0Plan(s, path="gemm_fp64", omega_acoustic=W_AC, ctx=ctx)
    ctx.timer_begin()
    r64 = fp.run(occ, eta_init=ETA_INIT, tol=TOL, maxiter=MAXITER, mu_start=[mu0])
    plain["recast_fp64_scgd0_s_to_tol"] = ctx.timer_end() / 1e3
    plain["fp64_scgd0_iters"] = int(r64["niter"])
    fp.close()
    lp64 = api.LadderPlan(s, path="gemm_fp64", omega_acoustic=W_AC, ctx=ctx)
    ctx.timer_begin()
    l64 = lp64.run(r64["sigma"], r64["mu"], [T], [OMEGA], rtol=L_RTOL, maxiter=L_MAXITER)
    plain["recast_fp64_ladder_s_per_omega"] = ctx.timer_end() / 1e3
    plain["fp64_ladder_gmres_iters"] = int(l64["niter"][0, 0])
    plain["counts_equal_reference_arm_constants"] = (plain["fp64_scgd0_iters"] == FP64_SCGD0_ITERS and
                                                     plain["fp64_ladder_gmres_iters"] + 1 == FP64_LADDER_APPLIES)
    lp64.close()
    # the BF16x3 ladder on the same Σ as the timed TF32 one (median of 5 runs)
    lpb = api.LadderPlan(s, path="gemm_bf16", omega_acoustic=W_AC, ctx=ctx)
    tb = []
    for _ in range(6):
        ctx.timer_begin()
        lb = lpb.run(r["sigma"], r["mu"], [T], [OMEGA], rtol=L_RTOL, maxiter=L_MAXITER)
        tb.append(ctx.timer_end() / 1e3)
    out["ladder_bf16x3"] = dict(s_per_omega=float(np.median(tb[1:])), gemm=lpb.gemm_config(),
                                rel_sigma_vs_timed_path=float(np.linalg.norm(lb["sigma_ladder"] - l["sigma_ladder"]) /
                                                              np.linalg.norm(lb["sigma_ladder"])))
    lpb.close()
    # the reference's algorithm (term by term, FP64) costs the same per iteration with or without
    # dispersion: one iteration is timed on the dispersive variant of the model, where it is also the
    # check of the tensor-core path's FP32 term-by-term sum
    sd = synthetic.with_dispersion(s, 16, 0.2)
    dp = api.Scgd0Plan(sd, path="direct_fp64", omega_acoustic=W_AC, ctx=ctx)
    ctx.timer_begin()
    d1 = dp.run(occ, eta_init=ETA_INIT, tol=0.0, maxiter=1, mu_start=[mu0])
    it_direct = ctx.timer_end() / 1e3
    dp.close()
    plain["direct_fp64_scgd0_s_per_iter"] = it_direct
    plain["direct_fp64_scgd0_s_to_tol"] = it_direct * plain["fp64_scgd0_iters"]
    plain["direct_fp64_scgd0_note"] = ("one iteration timed (dispersive variant, the same work per iteration), times "
                                       "the FP64 iteration count")
    out["dispersive"] = dispersive_leg(sd, ctx, occ, mu0, d1, it_direct)
    out["plain_fp64"] = plain
    fast = out["scgd0_s_to_tol"] + out["ladder_s_per_omega"]
    out["speedup_vs_recast_fp64"] = (plain["recast_fp64_scgd0_s_to_tol"] + plain["recast_fp64_ladder_s_per_omega"]) / fast
    out["speedup_scgd0_vs_direct_fp64"] = plain["direct_fp64_scgd0_s_to_tol"] / out["scgd0_s_to_tol"]
    out["accuracy_vs_fp64"] = dict(
        max_abs_dsigma_eV=float(np.max(np.abs(r["sigma"] - r64["sigma"]))),
        max_abs_dsigma_without_warm_start_eV=float(np.max(np.abs(r_cold["sigma"] - r64["sigma"]))),
        abs_dmu_eV=float(abs(r["mu"][0] - r64["mu"][0])),
        rel_sigma_ladder=float(np.linalg.norm(l["sigma_ladder"] - l64["sigma_ladder"]) / np.linalg.norm(l64["sigma_ladder"])))
    out["gmres_tight"] = gmres_tight(s, ctx, T, r, r64)
    out["batched_c3"] = batched_c3(s, ctx, ws)
    if not args.no_c5:
        sp.close()
        lp.close()
        try:
            out["large_c5"] = large_c5(ctx)
        except Exception as e:  # reported in the line, the rest of which stands
            out["large_c5"] = dict(error=f"{type(e).__name__}: {e}")
    flush_l2(local)
    out["cpu_baseline"] = cpu_baseline(s, T, r64, plain["fp64_scgd0_iters"], plain["fp64_ladder_gmres_iters"])
    print(json.dumps(out), flush=True)


def measure_tf32_peak(device: int):
    """cuBLAS FP32 GEMM with TF32 tensor cores (torch, 8192^3, best of 10 by CUDA events), TFLOP/s:
    the library-measured denominator for a TF32 kernel, as MEASURED_PEAKS.json's bf16 figure is for
    BF16. None where torch cannot run it."""
    try:
        import torch
        prev = torch.get_float32_matmul_precision()
        torch.set_float32_matmul_precision("high")
        n = 8192
        dev = f"cuda:{device}"
        a = torch.randn(n, n, device=dev)
        b = torch.randn(n, n, device=dev)
        c = a @ b
        best = None
        for _ in range(10):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b, out=c)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        torch.set_float32_matmul_precision(prev)
        del a, b, c
        torch.cuda.empty_cache()
        return 2.0 * n ** 3 / (best / 1e3) / 1e12
    except Exception:
        return None


def register_g2(ctx, s):
    """Page-lock the model's g2 (epsp_host_register): True, or the error's text when it fails (the
    set-ups then gather the pageable array on the host)."""
    from epspectral_gb300 import api
    try:
        ctx.host_register(s["g2"])
        return True
    except api.EpspError as e:
        return str(e)


def e2e_calls(s, ws, ctx, T, occ, mu0):
    """The end-to-end sequence through the public API from host arrays: the scGD0 plan's set-up (g2
    upload), scGD0 from the warm start, Σ back to the host, the ladder's set-up and σ(Ω). The context
    keeps the g2 the first set-up streams (epsp_ctx_keep_g2, switched on afresh here, so the first
    set-up does stream it) for the ladder's set-up of the same array. Seconds."""
    from epspectral_gb300 import api
    ctx.keep_g2(False)
    t0 = time.perf_counter()
    ctx.keep_g2(True)
    sp_e = api.Scgd0Plan(s, path="gemm_bf16", omega_acoustic=W_AC, ctx=ctx)
    r_e = sp_e.run(occ, eta_init=ETA_INIT, tol=TOL, maxiter=MAXITER, mu_start=[mu0], warm=ws)
    sp_e.close()
    api.loop_ladder(s, r_e["sigma"], r_e["mu"], [T], [OMEGA], rtol=L_RTOL, maxiter=L_MAXITER, omega_acoustic=W_AC,
                    path=LADDER_PATH, ctx=ctx)
    t = time.perf_counter() - t0
    ctx.keep_g2(False)
    return t


def e2e_cold(ws) -> dict:
    """The e2e sequence in a fresh process (its library load, CUDA context and empty autotune cache
    are not timed; the first plan's tuning and first launches are), with the network trained here."""
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "warm.npz")
        ws.save(path)
        r = subprocess.run([sys.executable, os.path.abspath(__file__), "--e2e-cold", path], capture_output=True,
                           text=True, timeout=600)
    try:
        line = [x for x in r.stdout.splitlines() if x.startswith("{")][-1]
        return json.loads(line)
    except (IndexError, ValueError):
        return dict(value=None, error=(r.stderr or r.stdout)[-300:])


def run_e2e_cold(path: str, local: int):
    from epspectral_gb300 import api
    from epspectral_gb300 import warmstart as W
    s, T, occ, mu0 = workload()
    ctx = api.Context(local)
    ws = W.WarmStart.load(path, ctx=ctx)
    pinned = register_g2(ctx, s)
    try:
        t = e2e_calls(s, ws, ctx, T, occ, mu0)
    finally:
        if pinned is True:
            ctx.host_unregister(s["g2"])
    print(json.dumps(dict(value=t, unit="s", note="fresh process: plan set-ups incl. the autotuner, first launches")),
          flush=True)


def dispersive_leg(sd, ctx, occ, mu0, d1, it_direct) -> dict:
    """The same model with dispersive modes (±20 % over the zone): scGD0 to tol on the tensor-core
    path (the Fan-Migdal sum term by term in FP32, fm_disp_f32_kernel) and its first iteration
    against the direct FP64 path's (d1, timed it_direct seconds)."""
    from epspectral_gb300 import api
    sp = api.Scgd0Plan(sd, path="gemm_bf16", omega_acoustic=W_AC, ctx=ctx)
    r1 = sp.run(occ, eta_init=ETA_INIT, tol=0.0, maxiter=1, mu_start=[mu0])
    ctx.timer_begin()
    sp.run(occ, eta_init=ETA_INIT, tol=0.0, maxiter=1, mu_start=[mu0])
    t1 = ctx.timer_end() / 1e3
    ctx.timer_begin()
    r = sp.run(occ, eta_init=ETA_INIT, tol=TOL, maxiter=MAXITER, mu_start=[mu0])
    t = ctx.timer_end() / 1e3
    sp.close()
    return dict(model="3-band t2g nk=16^3, modes w_nu (1 + 0.2 (cos 2pi q1/N + cos 2pi q2/N + cos 2pi q3/N) / 3)",
                scgd0_s_to_tol=t, scgd0_iters=int(r["niter"]), converged=bool(r["converged"][0]),
                s_per_iter=t1, direct_fp64_s_per_iter=it_direct, speedup_per_iter=it_direct / t1,
                first_iteration_max_abs_dsigma_vs_direct_fp64_eV=float(np.max(np.abs(r1["sigma"] - d1["sigma"]))),
                first_iteration_abs_dmu_eV=float(abs(r1["mu"][0] - d1["mu"][0])))


def gmres_tight(s, ctx, T, r, r64, rtol=1e-10) -> dict:
    """The ladder solve at Ω = 0.1 eV to a tight tolerance, so that GMRES runs several Arnoldi steps
    (8 on this model at 1e-10): the timed path (TF32 contraction, FP32 vertices, the Arnoldi step
    on the device) on its scGD0 Σ against the plain FP64 path on the FP64 Σ. Device seconds."""
    from epspectral_gb300 import api
    lp = api.LadderPlan(s, path=LADDER_PATH, omega_acoustic=W_AC, ctx=ctx)
    lp.run(r["sigma"], r["mu"], [T], [OMEGA], rtol=rtol, maxiter=60)  # warm-up (Krylov vectors allocated)
    ctx.timer_begin()
    lt = lp.run(r["sigma"], r["mu"], [T], [OMEGA], rtol=rtol, maxiter=60)
    t_tc = ctx.timer_end() / 1e3
    lp.close()
    lp64 = api.LadderPlan(s, path="gemm_fp64", omega_acoustic=W_AC, ctx=ctx)
    ctx.timer_begin()
    l64 = lp64.run(r64["sigma"], r64["mu"], [T], [OMEGA], rtol=rtol, maxiter=60)
    t_64 = ctx.timer_end() / 1e3
    lp64.close()
    n_tc, n_64 = int(lt["niter"][0, 0]), int(l64["niter"][0, 0])
    return dict(rtol=rtol, niter=n_tc, s=t_tc, s_per_iter=t_tc / max(1, n_tc), converged=bool(lt["converged"][0, 0]),
                fp64_niter=n_64, fp64_s=t_64, fp64_s_per_iter=t_64 / max(1, n_64),
                rel_sigma_vs_fp64=float(np.linalg.norm(lt["sigma_ladder"] - l64["sigma_ladder"]) /
                                        np.linalg.norm(l64["sigma_ladder"])))


def batched_c3(s, ctx, ws) -> dict:
    """The same model batched (8 temperatures 100-800 K, ladder at 32 Ωs on [0, 0.5] eV): scGD0 of
    all temperatures in one run (one launch per kernel per iteration, learned warm start) against
    the temperatures one by one, and the 256 (T, Ω) pairs as GMRES right-hand sides (batches of 8,
    each from x0 = 0) against the reference's sequential order with warm starts. Device seconds."""
    from epspectral_gb300 import api, synthetic
    Ts = list(np.linspace(100.0, 800.0, 8) * synthetic.KELVIN)
    Om = list(np.linspace(0.0, 0.5, 32))
    mus = [synthetic.bare_mu(s, t, 1.0) for t in Ts]
    occ8 = dict(Tlist=Ts, nlist=[0.0] * 8, nelec=1.0, spin_degeneracy=2.0, type="metal")
    sp = api.Scgd0Plan(s, path="gemm_bf16", omega_acoustic=W_AC, ctx=ctx)
    sp.run(occ8, eta_init=ETA_INIT, tol=TOL, maxiter=MAXITER, mu_start=mus, warm=ws)  # warm-up
    ctx.timer_begin()
    r8 = sp.run(occ8, eta_init=ETA_INIT, tol=TOL, maxiter=MAXITER, mu_start=mus, warm=ws)
    t_batched = ctx.timer_end() / 1e3
    t_single, it_single = 0.0, []
    for t, m in zip(Ts, mus):
        o1 = dict(Tlist=[t], nlist=[0.0], nelec=1.0, spin_degeneracy=2.0, type="metal")
        ctx.timer_begin()
        r1 = sp.run(o1, eta_init=ETA_INIT, tol=TOL, maxiter=MAXITER, mu_start=[m], warm=ws)
        t_single += ctx.timer_end() / 1e3
        it_single.append(int(r1["iters_total"]))
    sp.close()
    lp = api.LadderPlan(s, path=LADDER_PATH, omega_acoustic=W_AC, ctx=ctx)
    ctx.timer_begin()
    lb = lp.run(r8["sigma"], r8["mu"], Ts, Om, rtol=L_RTOL, maxiter=L_MAXITER, batch_rhs=8)
    t_lb = ctx.timer_end() / 1e3
    ctx.timer_begin()
    ls = lp.run(r8["sigma"], r8["mu"], Ts, Om, rtol=L_RTOL, maxiter=L_MAXITER)
    t_ls = ctx.timer_end() / 1e3
    lp.close()
    rel = float(np.max(np.abs(lb["sigma_ladder"] - ls["sigma_ladder"])) / np.max(np.abs(ls["sigma_ladder"])))
    # errors against the plain FP64 path: Σ and μ per temperature (all 8), σ per (T, Ω) on the FP64
    # ladder's subset (every T at Ω = 0 and 0.5 eV: 16 of the 256 pairs, ~2 s each in FP64)
    fp = api.Scgd0Plan(s, path="gemm_fp64", omega_acoustic=W_AC, ctx=ctx)
    r64 = fp.run(occ8, eta_init=ETA_INIT, tol=TOL, maxiter=MAXITER, mu_start=mus)
    fp.close()
    dsig_T = [float(np.max(np.abs(r8["sigma"][:, :, k] - r64["sigma"][:, :, k]))) for k in range(8)]
    dmu_T = [float(abs(r8["mu"][k] - r64["mu"][k])) for k in range(8)]
    sub = [0, len(Om) - 1]
    # σ: the mixed path against FP64 on the same Ω chain (the same warm starts, so the difference is
    # the precision's, not the solver tolerance's), each on its own scGD0 Σ
    oms = [Om[j] for j in sub]
    lp64 = api.LadderPlan(s, path="gemm_fp64", omega_acoustic=W_AC, ctx=ctx)
    l64 = lp64.run(r64["sigma"], r64["mu"], Ts, oms, rtol=L_RTOL, maxiter=L_MAXITER)
    lp64.close()
    lp = api.LadderPlan(s, path=LADDER_PATH, omega_acoustic=W_AC, ctx=ctx)
    lm = lp.run(r8["sigma"], r8["mu"], Ts, oms, rtol=L_RTOL, maxiter=L_MAXITER)
    lp.close()
    rel_m = [[float(np.linalg.norm(lm["sigma_ladder"][:, :, n, k] - l64["sigma_ladder"][:, :, n, k]) /
                    np.linalg.norm(l64["sigma_ladder"][:, :, n, k])) for n in range(len(oms))] for k in range(8)]
    err = dict(scgd0_max_abs_dsigma_eV_per_T=dsig_T, scgd0_abs_dmu_eV_per_T=dmu_T,
               ladder_pairs_checked=f"8 T x Omega in {{{oms[0]:g}, {oms[1]:g}}} eV, both paths on that Omega chain",
               ladder_rel_sigma_per_T_Omega=rel_m, max_abs_dsigma_eV=max(dsig_T),
               max_rel_sigma=max(max(x) for x in rel_m),
               niter_equal=bool(np.array_equal(lm["niter"], l64["niter"])))
    return dict(workload="8 T (100-800 K) x 32 Omega (0-0.5 eV), same model", errors_vs_fp64=err,
                scgd0_8T_batched_s=t_batched, scgd0_8T_iters=int(r8["iters_total"]),
                scgd0_8T_one_by_one_s=t_single, scgd0_one_by_one_iters=it_single,
                ladder_256_pairs_batched_s=t_lb, ladder_batched_s_per_omega=t_lb / 256,
                ladder_256_pairs_sequential_s=t_ls, ladder_sequential_s_per_omega=t_ls / 256,
                ladder_batched_vs_sequential_max_rel_dsigma=rel,
                ladder_converged=bool(lb["converged"].all() and ls["converged"].all()))


def large_c5(ctx) -> dict:
    """The large model (32^3 k: 2907 outer / 98304 inner states, 15 modes, g2 as BF16 8.6 GB held in
    host memory and streamed through the device in 8192-state chunks, graded grid of 4101 nodes,
    8 temperatures 100-800 K, Ωs on [0, 0.5] eV), bounded to about a minute: scGD0 of the 8
    temperatures in one run from -iη_init and from a warm start trained on 16 seeded runs of this
    model (T and filling varied, coupling scale 1), the plain FP64 recast path at 100 K and 800 K for
    the error, and the ladder at 4 of the 64 Ωs at 300 K (TF32, the bench's path; BF16x3 on the same
    Σ for the spread between the two precisions: the FP64 ladder at this size, ~2.4e14 flop per
    application on the FP64 unit, is outside the bench's time). Device seconds."""
    from epspectral_gb300 import api, graded_frequency_grid, synthetic
    from epspectral_gb300 import warmstart as W
    tile = 8192
    t0 = time.perf_counter()
    grid = graded_frequency_grid([(-0.4, 0.4, 0.0005), (-1.5, 1.5, 0.002), (-4.0, 4.0, 0.005), (-8.0, 8.0, 0.02)])
    s = synthetic.cubic_t2g_setup(N=32, ws=grid, g2_dtype="bf16", g2_chunk=2048, seed=0)
    nw, ni = len(s["omegas"]), int(s["eps_i"].size)
    out = dict(workload="3-band t2g nk=32^3, 2907 outer / 98304 inner states, 15 modes, g2 BF16 in host memory "
                        "streamed in 8192-state chunks, graded 4101-node grid; 8 T (100-800 K); ladder at 4 of 64 "
                        "Omegas on [0, 0.5] eV at 300 K",
               ni=ni, nf=int(s["eps_f"].size), nw=nw, g2_gb=s["g2"].nbytes / 1e9, model_build_s=time.perf_counter() - t0)
    Ts = list(np.linspace(100.0, 800.0, 8) * synthetic.KELVIN)
    mus = [synthetic.bare_mu(s, t, 1.0) for t in Ts]
    occ8 = dict(Tlist=Ts, nlist=[0.0] * 8, nelec=1.0, spin_degeneracy=2.0, type="metal")
    # the warm start: pairs from 16 runs of this model, then the network trained on the GPU
    t0 = time.perf_counter()
    X, Y, recs = W.generate_pairs(s, W.sample_runs(16, 31, scale_range=(1.0, 1.0)), gpu_tile=tile, ctx=ctx)
    t_gen = time.perf_counter() - t0
    ws = W.WarmStart(nw, ctx=ctx)
    t0 = time.perf_counter()
    hist = ws.fit(np.concatenate(X), np.concatenate(Y), epochs=20, batch=256, lr=1e-3)
    t_fit = time.perf_counter() - t0
    del X, Y
    out["warm_start"] = dict(train_runs=16, epochs=20, rows=16 * ni, pair_generation_s=t_gen, train_s=t_fit,
                             train_device_s=ws.train_device_s,
                             first_loss=float(hist[0]), final_loss=float(hist[-1]),
                             train_runs_plain_iters_mean=float(np.mean([r["niter"] for r in recs])))
    t0 = time.perf_counter()
    sp = api.Scgd0Plan(s, path="gemm_bf16", omega_acoustic=W_AC, gpu_tile=tile, ctx=ctx)
    out["scgd0_setup_s"] = time.perf_counter() - t0
    kw = dict(eta_init=ETA_INIT, tol=TOL, maxiter=MAXITER, mu_start=mus)
    sp.run(occ8, **kw)  # first run: graph capture, first launches
    ctx.timer_begin()
    r_plain = sp.run(occ8, **kw)
    out["scgd0_8T_s"] = ctx.timer_end() / 1e3
    out["scgd0_8T_iters"] = int(r_plain["niter"])
    ctx.timer_begin()
    r_warm = sp.run(occ8, warm=ws, **kw)
    out["scgd0_8T_warm_s"] = ctx.timer_end() / 1e3
    out["scgd0_8T_warm_iters"] = int(r_warm["iters_total"])
    out["scgd0_8T_warm_fallback"] = bool(r_warm["fallback"])
    out["scgd0_converged"] = bool(r_plain["converged"].all() and r_warm["converged"].all())
    sp.close()
    # the plain FP64 recast path at the two ends of the temperature range, for the error
    pick = [0, 7]
    fp = api.Scgd0Plan(s, path="gemm_fp64", omega_acoustic=W_AC, gpu_tile=tile, ctx=ctx)
    occ2 = dict(Tlist=[Ts[k] for k in pick], nlist=[0.0, 0.0], nelec=1.0, spin_degeneracy=2.0, type="metal")
    ctx.timer_begin()
    r64 = fp.run(occ2, eta_init=ETA_INIT, tol=TOL, maxiter=MAXITER, mu_start=[mus[k] for k in pick])
    out["fp64_scgd0_2T_s"] = ctx.timer_end() / 1e3
    out["fp64_scgd0_2T_iters"] = int(r64["niter"])
    fp.close()
    err = {}
    for name, r in (("plain", r_plain), ("warm", r_warm)):
        err[f"{name}_max_abs_dsigma_eV"] = [float(np.max(np.abs(r["sigma"][:, :, k] - r64["sigma"][:, :, n])))
                                            for n, k in enumerate(pick)]
        err[f"{name}_abs_dmu_eV"] = [float(abs(r["mu"][k] - r64["mu"][n])) for n, k in enumerate(pick)]
    err["temperatures_K"] = [float(np.linspace(100.0, 800.0, 8)[k]) for k in pick]
    out["errors_vs_fp64"] = err
    # the ladder at 4 of the 64 Ωs, 300 K, on the warm-started Σ
    Om = list(np.linspace(0.0, 0.5, 64)[[0, 21, 42, 63]])
    S3, mu3 = r_warm["sigma"][:, :, 2:3], r_warm["mu"][2:3]
    lad = {}
    for path in (LADDER_PATH, "gemm_bf16"):
        t0 = time.perf_counter()
        lp = api.LadderPlan(s, path=path, omega_acoustic=W_AC, gpu_tile=tile, ctx=ctx)
        setup_s = time.perf_counter() - t0
        ctx.timer_begin()
        l = lp.run(S3, mu3, [Ts[2]], Om, rtol=L_RTOL, maxiter=L_MAXITER)
        lad[path] = dict(s_per_omega=ctx.timer_end() / 1e3 / len(Om), setup_s=setup_s, gemm=lp.gemm_config(),
                         gmres_iters=[int(x) for x in l["niter"].ravel()], converged=bool(l["converged"].all()),
                         sigma=l["sigma_ladder"])
        lp.close()
    a, b = lad[LADDER_PATH].pop("sigma"), lad["gemm_bf16"].pop("sigma")
    rel = [float(np.linalg.norm(a[:, :, n, 0] - b[:, :, n, 0]) / np.linalg.norm(b[:, :, n, 0])) for n in range(len(Om))]
    out["ladder"] = dict(T_K=300.0, omegas_eV=[float(x) for x in Om], tf32=lad[LADDER_PATH], bf16x3=lad["gemm_bf16"],
                         rel_sigma_tf32_vs_bf16x3=rel)
    return out


def _blas_name() -> str:
    try:
        cfg = np.show_config(mode="dicts")
        return str(cfg["Build Dependencies"]["blas"]["name"])
    except Exception:
        return "numpy's BLAS"


def cpu_samples(s, T, sigma, mu):
    """Timed bounded samples of the reference's CPU algorithm, on every host core: the Fan-Migdal sum
    (the oracle's C++ FP64 restatement, OpenMP over (i, ω)) of one outer state per core, and the
    first chunk of one ladder application (src/ladder.jl:254-290): its coupling B, B̃ and shifted
    vertices X± built by the oracle, then C± += X± B̃ for all 6 ni output columns as two DGEMMs in
    numpy's BLAS, as the reference's mul! runs them. Both parts are linear in what they sample (outer
    states of the sum; K rows, i.e. the chunk's outer states, of the contraction), so the full cost is
    the sample's time scaled by the sampled fraction's inverse."""
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    ni = s["eps_i"].size
    nw = len(s["omegas"])
    sin = np.asfortranarray(sigma[:, :, 0])
    nsel = min(max(threads, 16), ni)
    t0 = time.perf_counter()
    O.imsigma_sample(s, sin, mu, T, 0, nsel, omega_acoustic=W_AC)
    t_fm_sample = time.perf_counter() - t0
    J = np.asfortranarray(np.full((nw, 4, 3, 2, ni), 1e-3 + 1e-3j))
    chunks, _ = O.ladder_chunks(s, omega_acoustic=W_AC)
    i_lo, i_hi = chunks[0]
    t0 = time.perf_counter()
    Xp, Xm, Bt = O.ladder_chunk_operands(s, J, T, 0, omega_acoustic=W_AC)
    t_ops = time.perf_counter() - t0
    t0 = time.perf_counter()
    Cp = Xp @ Bt
    Cm = Xm @ Bt
    t_gemm = time.perf_counter() - t0
    flops = 2.0 * 2 * Xp.shape[0] * Xp.shape[1] * Bt.shape[1]
    del Xp, Xm, Bt, Cp, Cm
    frac_fm = nsel / ni
    frac_l = (i_hi - i_lo) / ni
    info = dict(extrapolated=True, threads=threads,
                scgd0_sampled_fraction=frac_fm, scgd0_sample_s=t_fm_sample,
                scgd0_sample=f"Fan-Migdal sum of {nsel} of {ni} outer states (oracle, C++ FP64, {threads} threads)",
                ladder_sampled_fraction=frac_l, ladder_sample_s=t_ops + t_gemm,
                ladder_sample_operands_s=t_ops, ladder_sample_dgemm_s=t_gemm,
                ladder_sample_dgemm_gflops=flops / t_gemm / 1e9,
                ladder_sample=f"chunk 1 of {len(chunks)} (outer states {i_lo}-{i_hi - 1}): B, B~, X+- by the "
                              f"oracle, C+- += X+- B~ as two DGEMMs of {flops / 2e9 / 2:.0f} GFLOP each in numpy "
                              f"({_blas_name()})")
    return t_fm_sample / frac_fm, (t_ops + t_gemm) / frac_l, threads, info


def cpu_baseline(s, T, r64, n_it, n_gm):
    t_it, t_ap, thr, info = cpu_samples(s, T, r64["sigma"], r64["mu"][0])
    applies = n_gm + 1
    value = t_it * n_it + t_ap * applies
    return dict(value=value, unit="s", cores=thr, kind="port",
                sample=f"{info['scgd0_sample']}; {info['ladder_sample']}; step = {n_it} scGD0 iterations + "
                       f"{applies} ladder applications (this run's FP64 counts), each scaled from its sample",
                scgd0_s_per_iter=t_it, ladder_s_per_apply=t_ap, **info)


def run_reference(args, world, rank, local):
    if rank != 0:
        return
    s, T, occ, mu0 = workload()
    nw, ni = len(s["omegas"]), s["eps_i"].size
    # The Fan-Migdal sum costs the same for any Σ (same terms, no data-dependent branch but the
    # ω_acoustic cut), so the sample runs on Σ = -iη_init.
    sigma = np.asfortranarray(np.full((nw, ni, 1), complex(0.0, -ETA_INIT)))
    n_it, n_ap = FP64_SCGD0_ITERS, FP64_LADDER_APPLIES
    vals, info = [], {}
    for k in range(args.warmup + args.steps):
        t_it, t_ap, thr, info = cpu_samples(s, T, sigma, mu0)
        if k >= args.warmup:
            vals.append(t_it * n_it + t_ap * n_ap)
    v = float(np.median(vals))
    out = dict(metric=METRIC, value=v, unit="s", n_gpus=world, steps=args.steps, warmup=args.warmup,
               ms_per_step=1e3 * v, higher_is_better=False, scaling="weak", vs_baseline=None, dtype="fp64",
               data="synthetic (seeded 3-band t2g model, log-normal g2)", impl="reference",
               config=bench_config(s, world),
               cpu_baseline=dict(value=v, unit="s", cores=thr, kind="port",
                                 sample=f"{info['scgd0_sample']}; {info['ladder_sample']}; step = {n_it} scGD0 "
                                        f"iterations + {n_ap} ladder applications (the FP64 path's counts on this "
                                        f"workload), each scaled from its sample", **info),
               e2e=dict(value=v, unit="s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--save-warm", default=None, help="write the trained warm-start network to this .npz")
    ap.add_argument("--no-c5", action="store_true", help="leave out the large-model leg (about a minute)")
    ap.add_argument("--e2e-cold", default=None, help=argparse.SUPPRESS)  # internal: the cold e2e leg's process
    args = ap.parse_args()
    if args.e2e_cold:
        run_e2e_cold(args.e2e_cold, int(os.environ.get("LOCAL_RANK", "0")))
        return
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, local)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
