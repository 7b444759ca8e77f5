"""Benchmark: forward+adjoint groundwater solves per second at 1M cells.

Workload (one "step"): a batch of B independent realizations of the 1M-cell
problem -- regulargrid3d 200x200x25 nodes over 100x100x10 m, fully 3-D Matern
(nu=1) logK with correlation length 20 m, sigma 2, mean -9 (seeded synthetic
fields; no dataset is involved), Qs = 1e-4 m^3/s in cell 0, Dirichlet h = 0 in
the last cell -- each solved to 1e-10 relative residual, then differentiated:
J = sum of squared heads at 100 seeded observation cells, gradient dJ/dlogK over
all cells. Default precision: FP32 V-cycle/CG inside FP64 iterative refinement.

  value : solves/s with inputs resident in HBM (CUDA events on the solver's stream)
  e2e   : solves/s through the C ABI with page-locked host buffers, copies included
  plain_fp64_gpu : the same forward+adjoint, one realization per call, all FP64

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--batch B] [--impl ours|reference]
Under torchrun each rank runs its own batch (replicas, weak scaling).
"""
import argparse
import gc
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GRID = (200, 200, 25)
MINS = (0.0, 0.0, 0.0)
MAXS = (100.0, 100.0, 10.0)
ELL, SIGMA, MU = 20.0, 2.0, -9.0
NOBS = 100
RELTOL = 1e-10
WORKLOAD = "gw_steady_fwd_adj_200x200x25_matern3d_l20_s2"
METRIC = "forward+adjoint solves/sec at 1M cells vs plain FP64 GPU, at 1e-8 rel head err"

# algorithmic bytes per cell of each kernel (vector/coefficient element size T):
# reads and writes of every array the kernel touches once per cell
def _coef(T):
    """Bytes of one stored operator coefficient: FP64 levels keep FP64, the FP32 V-cycle bf16."""
    return 2 if T == 4 else 8


BYTES_PER_CELL = {
    "k_cheb_step": lambda T: 5 * T + 4 * _coef(T),    # xin, b, d, cx, cy, cz, leak in; xout, d out
    "k_cheb_step0": lambda T: 4 * T + 4 * _coef(T),   # first step after prolongation: d is not read
    "k_prolong_add": lambda T: 2 * T + T / 8 + 1,     # x, e/8, dir in; x out
    "k_cheb_first": lambda T: 3 * T + 4 * _coef(T),   # b, cx, cy, cz, leak in; x, d out
    "k_cheb_first2": lambda T: 4 * T + 4 * _coef(T),  # b, idg, cx, cy, cz, leak in; xout, d out
    # per coarse cell: 8 fine cells x (x, b, 4 coeffs) + bc out
    "k_restrict": lambda T: 17 * T + 32 * _coef(T),
    "k_pm_restrict": lambda T: 17 * T + 32 * _coef(T),
    "k_spmv_pq": lambda T: 6 * T,              # p, 4 coeffs in; q out (FP64 CG)
    "k_update_xr": lambda T: 6 * T,            # x, p, r, q in; x, r out
    "k_update_p": lambda T: 3 * T,             # z, p in; p out
    "k_cg_start": lambda T: 7 * T,             # x, b, 4 coeffs in; r out
    "k_df_spmv_pq": lambda T: 48,              # p (2 floats), 4 double-float coeffs in; q out
    "k_df_update_xr": lambda T: 52,            # x (f64), p, r, q (2 floats each) in; x, r, r32 out
    "k_df_update_p": lambda T: 20,             # z, p in; p out
    "k_df_residual": lambda T: 56,             # x64, b64, 4 FP64 coeffs in; r64 out
    "k_df_begin": lambda T: 20,                # r64 in; r (2 floats), r32 out
    "k_grad_logk": lambda T: 32,               # logK, h, lambda in; g out
    # plane-marching smoothers (Chebyshev degree 2): each value is read from HBM once
    "k_pm_first2": lambda T: 3 * T + 4 * _coef(T),   # b, idg, cx, cy, cz, leak in; x out (no direction)
    "k_pm_step": lambda T: 4 * T + 4 * _coef(T),     # x, b, d, cx, cy, cz, leak in; x out (last step)
    "k_pm_prolong_step": lambda T: 4 * T + T / 8 + 1 + 4 * _coef(T),  # x, e/8, dir, b, 4 coeffs in; x, d out
    "k_df_residual0": lambda T: 17,            # b, dir in; r out
    "k_pm_df_flux": lambda T: 48,              # plane-marching form of k_df_spmv_pq (each face flux once)
}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            import torch
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            dist.init_process_group(backend=backend)
        return dist, dist.get_rank(), ws
    return None, 0, 1


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    dev = "cuda" if torch.cuda.is_available() and dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(batch_per_rank, steps, world_size, t_max):
    """Whole-job solves/s: every rank solves its own batch each step (replicas, no exchange);
    t_max is the slowest rank's timed region."""
    return batch_per_rank * steps * world_size / t_max


def make_workload(pkg, B, seed0, grid=GRID, mins=MINS, maxs=MAXS):
    """B seeded realizations (logK concatenated in cell order), shared Qs/Dirichlet/obs layout.
    Each rank passes its own seed0, so replicas solve different realizations."""
    N = grid[0] * grid[1] * grid[2]
    logK = np.concatenate([pkg.fields.volume_logk(grid, mins, maxs, ELL, SIGMA, MU, seed0 + p) for p in range(B)])
    Qs = np.zeros(B * N)
    Qs[np.arange(B) * N] = 1e-4
    dh = np.zeros(B * N)
    rng = np.random.default_rng(seed0 + 7919)
    obs = [rng.choice(N, min(NOBS, N), replace=False) for _ in range(B)]
    return N, logK, dh, Qs, obs


class ClockSampler:
    """nvidia-smi samples (SM clock, max clock, throttle reasons) during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.rows = []
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) < 9:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def flush_l2(torch, buf):
    buf.add_(1.0)  # 512 MiB write > 129 MB L2


def run_ours(args, dist, rank, ws):
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    ge._load_build_module().build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    B = args.batch
    N, logK, dh, Qs, obs = make_workload(pkg, B, seed0=1000 * rank)
    prec = args.precision
    tuned, tune_ms, tune_s = {}, None, None
    if args.autotune:
        # smoother degree and launch shapes chosen by the library's autotuner on this workload
        t0 = time.perf_counter()
        tuned, tune_ms = pkg.autotune_batch([GRID] * B, [MINS] * B, [MAXS] * B, [[N - 1]] * B, logK, dh, Qs, obs,
                                            repeats=2, reltol=RELTOL, precision=prec)
        tune_s = time.perf_counter() - t0
    opts = dict(tuned)
    if args.streams > 0:
        opts["streams"] = args.streams
    batch = pkg.GroundwaterBatch([GRID] * B, [MINS] * B, [MAXS] * B, [[N - 1]] * B, reltol=RELTOL, precision=prec,
                                 use_graphs=0 if args.no_graphs else 1, **opts)
    d_logK = torch.tensor(logK, device=dev)
    d_dh = torch.tensor(dh, device=dev)
    d_Qs = torch.tensor(Qs, device=dev)
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float64, device=dev)

    import warnings
    warnings.simplefilter("error", RuntimeWarning)  # a solve that misses reltol must not be timed silently

    def step_dev():
        return batch.solve_grad_logk(d_logK, d_dh, d_Qs, obs)

    for _ in range(args.warmup):
        step_dev()
    torch.cuda.synchronize()
    # ---- value: device-resident inputs, CUDA events per step, L2 flushed between steps
    clocks = ClockSampler(local)
    clocks.start()
    _barrier(dist)
    torch.cuda.synchronize()
    gc.collect()
    gc.disable()  # no garbage-collection pass inside the timed steps (re-enabled below)
    launches0 = batch.launch_count
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.steps):
        flush_l2(torch, flush)
        ev[k][0].record()
        h, g = step_dev()
        ev[k][1].record()
    torch.cuda.synchronize()
    gc.enable()
    _barrier(dist)
    clk = clocks.stop()
    launches = batch.launch_count - launches0
    t_dev = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    t_dev = _max_over_ranks(dist, t_dev)
    stats = batch.stats
    if args.main_only:
        if rank == 0:
            return {"metric": METRIC, "value": round(replica_throughput(B, args.steps, ws, t_dev), 3), "unit": "solves/s",
                    "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "gpu_launches": int(launches),
                    "note": "--main-only: timed region only (no e2e, roofline, baselines)"}
        return None
    # ---- e2e: page-locked host buffers through the C ABI, copies inside the timed region
    h_logK = torch.from_numpy(logK).pin_memory()
    h_dh = torch.from_numpy(dh).pin_memory()
    h_Qs = torch.from_numpy(Qs).pin_memory()
    h_h = torch.empty(B * N, dtype=torch.float64).pin_memory()
    h_g = torch.empty(B * N, dtype=torch.float64).pin_memory()
    for _ in range(args.warmup):  # the host-buffer path's own warm-up (its copy stream, first touches)
        batch.solve_grad_logk(h_logK.numpy(), h_dh.numpy(), h_Qs.numpy(), obs, out=(h_h.numpy(), h_g.numpy()))
    _barrier(dist)
    torch.cuda.synchronize()
    # wall-clock region: no Python garbage-collection pass inside it (as timeit does); a full pass
    # over this process's heap takes tens of milliseconds, longer than the host's part of a step
    gc.collect()
    gc.disable()
    t0 = time.perf_counter()
    e2e_steps = []
    for k in range(args.steps):
        t1 = time.perf_counter()
        h_e2e, g_e2e = batch.solve_grad_logk(h_logK.numpy(), h_dh.numpy(), h_Qs.numpy(), obs,
                                             out=(h_h.numpy(), h_g.numpy()))
        e2e_steps.append(time.perf_counter() - t1)  # each call returns with its outputs in host memory
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t0
    gc.enable()
    t_e2e = _max_over_ranks(dist, t_wall)
    # ---- roofline of the dominant kernel (profiling pass on identical realizations so every
    # scheduled cell is active in every launch)
    rep = profile_pass(pkg, torch, dev, B, N, prec, args, tuned)
    # ---- plain FP64 single-realization GPU solve (the metric's denominator)
    plain = plain_fp64(pkg, torch, dev, N, logK[:N], dh[:N], Qs[:N], obs[0], args)
    # ---- accuracy of the timed configuration against FP64 (spot check on realization 0)
    if rank != 0:
        return None
    solves = B * args.steps * ws
    value = replica_throughput(B, args.steps, ws, t_dev)
    out = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": "solves/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(1e3 * t_dev / args.steps, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 V-cycle + double-float CG (f32 ops), f64 residual" if prec == "mixed" else "f64",
        "data": "synthetic (seeded Matern logK fields)",
        "config": {"workload": WORKLOAD, "cells": N, "batch_per_gpu": B, "precision": prec, "reltol": RELTOL,
                   "l2": "flushed between timed steps (512 MiB write); batch working set > L2",
                   "parallelism": "replicas" if ws > 1 else "single",
                   "autotuned": tuned or None,
                   "autotune_seconds": round(tune_s, 2) if tune_s else None},
        "e2e": {"value": round(solves / t_e2e, 3), "unit": "solves/s",
                "h2d_bytes_per_step": int(3 * 8 * B * N), "d2h_bytes_per_step": int(2 * 8 * B * N),
                "step_ms": [round(1e3 * t, 2) for t in e2e_steps]},
        "gpu_launches": int(launches),
        "clocks": clk,
        "iterations_last_adjoint": stats["iterations"],
        "plain_fp64_gpu": plain,
        "speedup_vs_plain_fp64": round(value / plain["value"], 3) if plain["value"] else None,
        "roofline": rep,
    }
    out["accuracy"] = accuracy_check(pkg, torch, dev, N, logK[:N], dh[:N], Qs[:N], obs[0], h[:N], g[:N])
    out["accuracy"].update(oracle_accuracy(pkg, N, logK[:N], dh[:N], Qs[:N], obs[0], h[:N], g[:N]))
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(pkg, N, logK[:N], dh[:N], Qs[:N], obs[0], args.cpu_steps)
    return out


def profile_pass(pkg, torch, dev, B, N, prec, args, tuned=None):
    import json as _json
    peaks = {}
    try:
        peaks = _json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    src = "measured" if "hbm_gbs" in peaks else "fallback"
    lk = pkg.fields.volume_logk(GRID, MINS, MAXS, ELL, SIGMA, MU, 4242)
    logK = np.tile(lk, B)
    Qs = np.zeros(B * N)
    Qs[np.arange(B) * N] = 1e-4
    dh = np.zeros(B * N)
    obs = [np.arange(0, N, N // NOBS)[:NOBS]] * B
    # per-kernel events need a saturated stream: convergence is read back every 4
    # iterations here so the host stays ahead of the GPU (graphs are off while profiling);
    # the launch shapes are the timed run's
    # one stream: with the batch split into concurrent parts, a kernel's events would also span
    # the other parts' kernels running beside it, so each kernel is timed alone here
    opts = dict(tuned or {})
    opts["streams"] = 1
    b = pkg.GroundwaterBatch([GRID] * B, [MINS] * B, [MAXS] * B, [[N - 1]] * B, reltol=RELTOL, precision=prec,
                             check_every=4, **opts)
    d = [torch.tensor(x, device=dev) for x in (logK, dh, Qs)]
    b.solve_grad_logk(*d, obs)
    b.profile(True)
    for _ in range(max(1, min(args.steps, 3))):
        b.solve_grad_logk(*d, obs)
    rep = b.profile_report()
    b.profile(False)
    total = sum(v[1] for v in rep.values())
    top = sorted(rep.items(), key=lambda kv: -kv[1][1])
    # the dominant kernel with an algorithmic byte count (the fused tail is compute-bound)
    name, (cnt, ms, cells) = next((kv for kv in top if kv[0].split("<")[0] in BYTES_PER_CELL), top[0])
    base = name.split("<")[0]
    T = 4 if "<f32>" in name else 8
    bpc = BYTES_PER_CELL.get(base)
    achieved = (bpc(T) * cells / (ms / 1e3) / 1e9) if bpc else None
    traffic = None
    try:
        meas = _json.load(open(os.path.join(ROOT, "profiles", "dram_bytes_per_cell.json")))
        if base in meas.get("kernels", {}):
            traffic = int(meas["kernels"][base] * cells / cnt)
    except (OSError, ValueError):
        pass
    return {
        "bound": "hbm",
        "kernel": name,
        "achieved": round(achieved, 1) if achieved else None,
        "peak": peak,
        "unit": "GB/s",
        "frac": round(achieved / peak, 4) if achieved else None,
        "peak_source": src,
        "traffic": traffic,
        "traffic_source": "profiles/dram_bytes_per_cell.json (ncu dram__bytes_read+write per cell x cells per launch)",
        "bytes_per_launch": int(bpc(T) * cells / cnt) if bpc else None,
        "avg_launch_us": round(1e3 * ms / cnt, 3),
        "share": round(ms / total, 4) if total else None,
        "top": [{"kernel": k, "launches": v[0], "ms": round(v[1], 3),
                 "GBps": round(BYTES_PER_CELL[k.split("<")[0]](4 if "<f32>" in k else 8) * v[2] / (v[1] / 1e3) / 1e9, 1)
                 if k.split("<")[0] in BYTES_PER_CELL and v[1] > 0 else None} for k, v in top[:8]],
        "measured": "per-kernel CUDA events on the solver stream over %d forward+adjoint steps of a profiling pass: the "
                    "timed run's launch shapes and batch size, the batch on one stream (each kernel alone), %d identical "
                    "realizations of a different seed (every scheduled cell active in every launch), convergence read "
                    "every 4 iterations with graphs off" % (max(1, min(args.steps, 3)), B),
        "profile_options": {k: v for k, v in opts.items()},
    }


def plain_fp64(pkg, torch, dev, N, logK, dh, Qs, obs, args):
    P = pkg.GroundwaterProblem.regular3d(MINS, MAXS, GRID, [N - 1], reltol=RELTOL, precision="fp64")
    d = [torch.tensor(x, device=dev) for x in (logK, dh, Qs)]
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float64, device=dev)
    for _ in range(max(2, args.warmup)):
        P.solve_grad_logk(*d, obs)
    torch.cuda.synchronize()
    n = max(3, args.steps)
    tot = 0.0
    for _ in range(n):
        flush_l2(torch, flush)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        P.solve_grad_logk(*d, obs)
        b.record()
        torch.cuda.synchronize()
        tot += a.elapsed_time(b) / 1e3
    return {"value": round(n / tot, 3), "unit": "solves/s", "ms_per_solve": round(1e3 * tot / n, 3),
            "iterations_last_adjoint": P.stats["iterations"]}


def accuracy_check(pkg, torch, dev, N, logK, dh, Qs, obs, h, g):
    """Relative errors of the timed configuration's realization 0 against an FP64 GPU solve at 1e-13."""
    P = pkg.GroundwaterProblem.regular3d(MINS, MAXS, GRID, [N - 1], reltol=1e-13, precision="fp64")
    h64, g64 = P.solve_grad_logk(logK, dh, Qs, obs)
    h = h.cpu().numpy() if hasattr(h, "cpu") else h
    g = g.cpu().numpy() if hasattr(g, "cpu") else g
    return {"rel_head_err_vs_fp64_1e-13": float(np.linalg.norm(h - h64) / np.linalg.norm(h64)),
            "rel_grad_err_vs_fp64_1e-13": float(np.linalg.norm(g - g64) / np.linalg.norm(g64))}


def oracle_accuracy(pkg, N, logK, dh, Qs, obs, h, g):
    """Relative L2 errors of the timed run's realization 0 (head, dJ/dlogK) against the oracle
    (the C restatement of the reference's solve and rrule) solved to reltol 1e-14 on the host."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    orc.build()
    orc.set_threads(os.cpu_count() or 1)
    _, nb, aol, _ = pkg.regulargrid3d(MINS, MAXS, GRID)
    O = orc.Problem(N, nb, aol, [N - 1])
    h_or = O.steady(orc.logk_to_faces(nb, logK), dh, Qs, reltol=1e-14)
    delta = np.zeros(N)
    np.add.at(delta, obs, 2 * h_or[obs])
    dKs, _, _ = O.adjoint(dh, delta, reltol=1e-14)
    g_or = orc.logk_to_faces_vjp(nb, logK, dKs)
    h = h.cpu().numpy() if hasattr(h, "cpu") else h
    g = g.cpu().numpy() if hasattr(g, "cpu") else g
    return {"rel_head_err_vs_oracle_1e-14": float(np.linalg.norm(h - h_or) / np.linalg.norm(h_or)),
            "rel_grad_err_vs_oracle_1e-14": float(np.linalg.norm(g - g_or) / np.linalg.norm(g_or))}


def cpu_oracle_step(orc, nb, aol, N, logK, dh, Qs, obs):
    Ks = orc.logk_to_faces(nb, logK)
    P = orc.Problem(N, nb, aol, [N - 1])
    h = P.steady(Ks, dh, Qs, reltol=RELTOL)
    delta = np.zeros(N)
    delta[obs] = 2 * h[obs]
    dKs, _, _ = P.adjoint(dh, delta, reltol=RELTOL)
    return orc.logk_to_faces_vjp(nb, logK, dKs)


def cpu_baseline(pkg, N, logK, dh, Qs, obs, steps):
    """The oracle (C restatement of the reference's Ruge-Stueben AMG + CG path, FP64) on all host cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    orc.build()
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    _, nb, aol, _ = pkg.regulargrid3d(MINS, MAXS, GRID)
    cpu_oracle_step(orc, nb, aol, N, logK, dh, Qs, obs)
    t0 = time.perf_counter()
    for _ in range(steps):
        cpu_oracle_step(orc, nb, aol, N, logK, dh, Qs, obs)
    dt = time.perf_counter() - t0
    return {"value": round(steps / dt, 4), "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": "%d forward+adjoint solve(s) of one 1M-cell realization (RS-AMG-preconditioned CG, FP64, "
                      "reltol 1e-10), after one untimed warm-up solve" % steps}


def run_reference(args, dist, rank, ws):
    """Reference arm: the reference's CPU path for this workload, i.e. the oracle port (the Julia
    reference cannot run here), on all host cores; rank 0 only."""
    if rank != 0:
        return None
    import __graft_entry__ as ge
    pkg = ge.load_package()
    N, logK, dh, Qs, obs = make_workload(pkg, 1, seed0=0)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    orc.build()
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    _, nb, aol, _ = pkg.regulargrid3d(MINS, MAXS, GRID)
    for _ in range(args.warmup):
        cpu_oracle_step(orc, nb, aol, N, logK, dh, Qs, obs[0])
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_oracle_step(orc, nb, aol, N, logK, dh, Qs, obs[0])
    dt = time.perf_counter() - t0
    v = args.steps / dt
    return {
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "solves/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * dt / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Matern logK fields)",
        "config": {"workload": WORKLOAD, "cells": N, "batch_per_gpu": 1, "precision": "fp64", "reltol": RELTOL},
        "cpu_baseline": {"value": round(v, 4), "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": "one forward+adjoint solve of one 1M-cell realization per step"},
        "e2e": {"value": round(v, 4), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the Julia reference needs Julia + its package depot, absent on this machine; the timed CPU path is "
                "the C restatement of its Ruge-Stueben AMG + CG solve and rrule",
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=32,
                    help="1M-cell realizations per GPU per step (the headline batch: 32, about 6 GB on the device)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--autotune", type=int, default=1,
                    help="1: choose smoother degree and launch shapes with the library's autotuner before timing")
    ap.add_argument("--no-graphs", action="store_true",
                    help="launch the CG loop from the host (ncu cannot profile kernels inside conditional graphs)")
    ap.add_argument("--main-only", action="store_true", help="only the timed region (for profiling runs)")
    ap.add_argument("--streams", type=int, default=0,
                    help="split the batch into this many concurrent parts (0: the autotuner's choice)")
    ap.add_argument("--workload", default="steady_1m", choices=["steady_1m", "steady_100k", "uneven_batch", "transient", "general_1m",
                                                                "richards", "dfn", "cholesky"],
                    help="steady_1m is the headline; the others are the remaining configurations (bench_workloads.py)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    dist, rank, ws = _dist()
    if args.workload != "steady_1m" and args.impl == "ours":
        import bench_workloads
        if args.batch == 32:
            args.batch = 0  # the workload's own default batch
        out = bench_workloads.run(args.workload, args, dist, rank, ws)
    else:
        out = run_reference(args, dist, rank, ws) if args.impl == "reference" else run_ours(args, dist, rank, ws)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
