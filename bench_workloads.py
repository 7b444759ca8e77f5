"""Secondary benchmark workloads: the other configurations of the groundwater path, timed
with the same harness as bench.py's headline (CUDA events on the solver stream, W warm-up
steps, L2 flushed between steps, a plain FP64 GPU run of the same workload beside it).

    python bench.py --workload steady_100k     # 100x100x10, layered Matern (l=50, s=1), J at 100 cells
    python bench.py --workload uneven_batch    # 256 realizations of 4 grid sizes (~73M cells), random
                                               # l, sigma, 1-4 injection and 1-4 Dirichlet cells
    python bench.py --workload transient       # 200x200x20, 100 backward-Euler steps of 3600 s,
                                               # Dirichlet x = max face, J = sum_t sum_50obs h^2
    python bench.py --workload general_1m      # the 1M-cell grid as a shuffled face list: CSR path
    python bench.py --workload richards        # steady Richards, 100x100x20 unsaturated column, rrule

All inputs are seeded synthetic data. One "solve" is a forward + adjoint (for the transient
workload: the whole 100-step forward run and its adjoint).
"""
import os
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))


def _events(torch, fn, steps, warmup, flush):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for k in range(steps):
        flush.add_(1.0)
        ev[k][0].record()
        fn()
        ev[k][1].record()
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / 1e3


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# ---------------------------------------------------------------- steady, 100k cells
def steady_100k(pkg, torch, dev, args):
    grid, mins, maxs = (100, 100, 10), (0.0, 0.0, 0.0), (50.0, 50.0, 5.0)
    N = 100 * 100 * 10
    B = args.batch if args.batch else 64
    logK = np.concatenate([pkg.fields.layered_logk(grid, mins, maxs, 50.0, 1.0, -9.0, 5000 + p) for p in range(B)])
    Qs = np.zeros(B * N)
    Qs[np.arange(B) * N] = 1e-4
    dh = np.zeros(B * N)
    rng = np.random.default_rng(17)
    obs = [rng.choice(N, 100, replace=False) for _ in range(B)]

    def make(prec, tol):
        return pkg.GroundwaterBatch([grid] * B, [mins] * B, [maxs] * B, [[N - 1]] * B, reltol=tol, precision=prec)

    d = [torch.tensor(x, device=dev) for x in (logK, dh, Qs)]
    res = {"workload": "gw_steady_fwd_adj_100x100x10_layered_l50_s1", "cells": N, "batch_per_gpu": B,
           "problems": B}
    return res, make, d, obs, B, [(grid, mins, maxs, [N - 1], slice(0, N))]


# ---------------------------------------------------------------- uneven batch
def uneven_batch(pkg, torch, dev, args):
    sizes = [(50, 50, 5), (100, 100, 10), (150, 150, 10), (200, 200, 20)]
    B = args.batch if args.batch else 256
    rng = np.random.default_rng(33)
    grids, mins, maxs, dns, Q, ells, sigs, obs = [], [], [], [], [], [], [], []
    for p in range(B):
        g = sizes[rng.integers(4)]
        mx = tuple(0.5 * (n - 1) for n in g)
        N = int(np.prod(g))
        ells.append(rng.uniform(0.5, 2.0) * mx[0])
        sigs.append(rng.uniform(0.5, 2.0))
        cells = rng.choice(N, 8, replace=False)
        ninj, ndir = 1 + rng.integers(4), 1 + rng.integers(4)
        q = np.zeros(N)
        q[cells[:ninj]] = rng.uniform(1e-5, 1e-3, ninj)
        grids.append(g), mins.append((0.0, 0.0, 0.0)), maxs.append(mx)
        dns.append(np.sort(cells[4:4 + ndir]))
        Q.append(q)
        obs.append(rng.choice(N, 100, replace=False))
    # the fields: the library's Matern sampler (dpf_batch_sample_logk) on the GPU, seeds 9000 + p
    sampler = pkg.GroundwaterBatch(grids, mins, maxs, dns, precision="mixed")
    logK = sampler.sample_logk(9000 + np.arange(B), ells, sigs, -9.0, nmodes=512, out="cuda")
    sampler.close()
    Qs = torch.tensor(np.concatenate(Q), device=dev)
    dh = torch.zeros_like(Qs)

    def make(prec, tol):
        return pkg.GroundwaterBatch(grids, mins, maxs, dns, reltol=tol, precision=prec)

    cells = int(sum(np.prod(g) for g in grids))
    res = {"workload": "gw_steady_fwd_adj_uneven_batch_256", "cells": cells, "batch_per_gpu": B, "problems": B,
           "sizes": "uniform over 50x50x5, 100x100x10, 150x150x10, 200x200x20 (0.5 m spacing)",
           "fields": "drawn on the GPU by the library's Matern sampler (dpf_batch_sample_logk, 512 modes)"}
    off = np.concatenate([[0], np.cumsum([np.prod(g) for g in grids])]).astype(np.int64)
    # checked members: the first problem of each grid size (the 200x200x20 one included)
    firsts = sorted({tuple(g): p for p, g in reversed(list(enumerate(grids)))}.values())
    check = [(grids[p], mins[p], maxs[p], dns[p], slice(off[p], off[p + 1])) for p in firsts]
    return res, make, [logK, dh, Qs], obs, B, check


def run_steady(name, args, dist, rank, ws, METRIC_NAME):
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    ge._load_build_module().build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    cfg, make, d, obs, B, check = (steady_100k if name == "steady_100k" else uneven_batch)(pkg, torch, dev, args)
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float64, device=dev)
    import warnings
    warnings.simplefilter("error", RuntimeWarning)
    mixed = make(args.precision, 1e-10)
    t = _events(torch, lambda: mixed.solve_grad_logk(*d, obs), args.steps, args.warmup, flush)
    h, g = mixed.solve_grad_logk(*d, obs)
    # e2e: page-locked host buffers in and out
    hosts = [x.cpu().pin_memory() for x in d]
    hh = torch.empty(mixed.N, dtype=torch.float64).pin_memory()
    hg = torch.empty(mixed.N, dtype=torch.float64).pin_memory()
    for _ in range(args.warmup):  # the host-buffer path's own warm-up
        mixed.solve_grad_logk(*[x.numpy() for x in hosts], obs, out=(hh.numpy(), hg.numpy()))
    torch.cuda.synchronize()
    import gc
    gc.collect()
    gc.disable()  # no garbage-collection pass inside the wall-clock region
    t0 = time.perf_counter()
    for _ in range(args.steps):
        mixed.solve_grad_logk(*[x.numpy() for x in hosts], obs, out=(hh.numpy(), hg.numpy()))
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    gc.enable()
    # plain FP64 GPU and accuracy against an FP64 solve at 1e-13
    plain = make("fp64", 1e-10)
    t64 = _events(torch, lambda: plain.solve_grad_logk(*d, obs), max(1, args.steps // 2), 1, flush)
    ref = make("fp64", 1e-13)
    warnings.simplefilter("ignore", RuntimeWarning)
    h64, g64 = ref.solve_grad_logk(*d, obs)
    h, g, h64, g64 = (x.cpu().numpy() for x in (h, g, h64, g64))
    errs = [(_rel(h[s], h64[s]), _rel(g[s], g64[s])) for (_, _, _, _, s) in check]
    solves = B * args.steps
    out = {
        "metric": METRIC_NAME, "value": round(solves / t, 3), "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * t / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 V-cycle + double-float CG (f32 ops), f64 residual",
        "data": "synthetic (seeded Matern logK fields)", "config": dict(cfg, precision=args.precision, reltol=1e-10,
                                                                      l2="flushed between timed steps"),
        "e2e": {"value": round(solves / t_e2e, 3), "unit": "solves/s",
                "h2d_bytes_per_step": int(3 * 8 * mixed.N), "d2h_bytes_per_step": int(2 * 8 * mixed.N)},
        "plain_fp64_gpu": {"value": round(B * max(1, args.steps // 2) / t64, 3), "unit": "solves/s"},
        "accuracy": {"max_rel_head_err_vs_fp64_1e-13": max(e[0] for e in errs),
                     "max_rel_grad_err_vs_fp64_1e-13": max(e[1] for e in errs), "problems_checked": len(errs)},
        "iterations_last_adjoint": mixed.stats["iterations"],
    }
    out["speedup_vs_plain_fp64"] = round(out["value"] / out["plain_fp64_gpu"]["value"], 3)
    if name == "uneven_batch":
        # the checked members against the oracle (reltol 1e-14 on the host)
        import sys
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc
        orc.build()
        orc.set_threads(os.cpu_count() or 1)
        oe = []
        for grid, mn, mx, dn, s in check:
            p = int(np.searchsorted(mixed.cell_offsets, s.start))  # the member's problem index
            n = s.stop - s.start
            _, nb, aol, _ = pkg.regulargrid3d(mn, mx, grid)
            lk = d[0][s].cpu().numpy()
            O = orc.Problem(n, nb, aol, np.asarray(dn, np.int64))
            ho = O.steady(orc.logk_to_faces(nb, lk), np.zeros(n), d[2][s].cpu().numpy(), reltol=1e-14)
            delta = np.zeros(n)
            np.add.at(delta, obs[p], 2 * ho[obs[p]])
            dKs, _, _ = O.adjoint(np.zeros(n), delta, reltol=1e-14)
            oe.append((_rel(h[s], ho), _rel(g[s], orc.logk_to_faces_vjp(nb, lk, dKs))))
        out["accuracy"]["max_rel_head_err_vs_oracle_1e-14"] = max(e[0] for e in oe)
        out["accuracy"]["max_rel_grad_err_vs_oracle_1e-14"] = max(e[1] for e in oe)
        out["accuracy"]["oracle_grids"] = [list(c[0]) for c in check]
    if name == "steady_100k" and not args.no_cpu_baseline:
        # the oracle on realization 0: parity and the CPU rate at this size
        import sys
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc
        orc.build()
        orc.set_threads(os.cpu_count() or 1)
        grid, mn, mx, dn, s = check[0]
        _, nb, aol, _ = pkg.regulargrid3d(mn, mx, grid)
        lk = d[0][s].cpu().numpy()
        t0 = time.perf_counter()
        O = orc.Problem(s.stop - s.start, nb, aol, np.asarray(dn, np.int64))
        ho = O.steady(orc.logk_to_faces(nb, lk), np.zeros(s.stop - s.start), d[2][s].cpu().numpy(), reltol=1e-14)
        delta = np.zeros(s.stop - s.start)
        np.add.at(delta, obs[0], 2 * ho[obs[0]])
        dKs, _, _ = O.adjoint(np.zeros(s.stop - s.start), delta, reltol=1e-14)
        go = orc.logk_to_faces_vjp(nb, lk, dKs)
        tc = time.perf_counter() - t0
        out["accuracy"]["rel_head_err_vs_oracle"] = _rel(h[s], ho)
        out["accuracy"]["rel_grad_err_vs_oracle"] = _rel(g[s], go)
        out["cpu_baseline"] = {"value": round(1.0 / tc, 4), "unit": "solves/s", "cores": os.cpu_count() or 1,
                               "kind": "port", "sample": "one forward+adjoint of realization 0 (oracle, reltol 1e-14)"}
    return out


# ---------------------------------------------------------------- transient
def run_transient(args, dist, rank, ws, METRIC_NAME):
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    ge._load_build_module().build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    grid, mins, maxs = (200, 200, 20), (0.0, 0.0, 0.0), (100.0, 100.0, 10.0)
    nx, ny, nz = grid
    N = nx * ny * nz
    lk = pkg.fields.volume_logk(grid, mins, maxs, 30.0, 1.5, -9.0, 777)
    rng = np.random.default_rng(55)
    dn = np.arange((nx - 1) * ny * nz, N)  # the x = max face
    free = np.arange(0, (nx - 1) * ny * nz)
    Qs = np.zeros(N)
    Qs[rng.choice(free, 4, replace=False)] = 1e-3
    obs = rng.choice(free, 50, replace=False)
    Ss = np.full(N, 1e-5)
    dt, nsteps, ck = 3600.0, 100, 10
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float64, device=dev)
    import warnings
    warnings.simplefilter("error", RuntimeWarning)

    def make(prec, tol):
        return pkg.GroundwaterProblem.regular3d(mins, maxs, grid, dn, reltol=tol, precision=prec)

    d_lk = torch.tensor(lk, device=dev)
    d = {k: torch.tensor(v, device=dev) for k, v in (("dh", np.zeros(N)), ("Q", Qs), ("S", Ss), ("h0", np.zeros(N)))}
    w = torch.ones(50, dtype=torch.float64, device=dev)

    def run(P):
        Ks = P.logk_to_faces(d_lk)
        P.transient_forward(Ks, d["dh"], d["Q"], d["S"], dt, nsteps, d["h0"], checkpoint_every=ck)
        return P.transient_adjoint(obs, weights=w)

    # every step to reltol 1e-11: at 1e-10 per step the states drift 3e-8 from the oracle's over
    # a few steps, above the 1e-8 head bar
    mixed = make(args.precision, 1e-11)
    steps = max(1, args.steps // 2)
    t = _events(torch, lambda: run(mixed), steps, max(1, args.warmup - 1), flush)
    dK = run(mixed)[0]
    plain = make("fp64", 1e-11)
    t64 = _events(torch, lambda: run(plain), 1, 1, flush)
    warnings.simplefilter("ignore", RuntimeWarning)
    dK64 = run(make("fp64", 1e-13))[0]
    acc = {"rel_dKs_err_vs_fp64_1e-13": _rel(dK.cpu().numpy(), dK64.cpu().numpy())}
    acc.update(_transient_vs_oracle(pkg, torch, mixed, lk, dn, Qs, Ss, dt, obs, vol=maxs, grid=grid, mins=mins))
    return {
        "metric": METRIC_NAME, "value": round(steps / t, 4), "unit": "runs/s", "n_gpus": ws, "steps": steps,
        "warmup": max(1, args.warmup - 1), "ms_per_step": round(1e3 * t / steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 V-cycle + double-float CG (f32 ops), f64 residual",
        "data": "synthetic (seeded Matern logK field)",
        "config": {"workload": "gw_transient_fwd_adj_200x200x20_100steps_ckpt10", "cells": N, "steps": nsteps,
                   "dt": dt, "checkpoint_every": ck, "dirichlet": "x = max face (4000 cells)", "obs": 50,
                   "precision": args.precision, "reltol": 1e-11},
        "plain_fp64_gpu": {"value": round(1.0 / t64, 4), "unit": "runs/s"},
        "speedup_vs_plain_fp64": round(t64 / (t / steps), 3),
        "accuracy": acc,
    }


def _transient_vs_oracle(pkg, torch, P, lk, dn, Qs, Ss, dt, obs, vol, grid, mins, nsteps=10, ck=5):
    """The first `nsteps` steps of the timed configuration (checkpoint every `ck`) on the timed
    handle against the oracle's backward Euler and its discrete adjoint (reltol 1e-14)."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    orc.build()
    orc.set_threads(os.cpu_count() or 1)
    N = int(np.prod(grid))
    _, nb, aol, V = pkg.regulargrid3d(mins, vol, grid)
    Ks = orc.logk_to_faces(nb, lk)
    dh = np.zeros(N)
    O = orc.Problem(N, nb, aol, dn)
    st_or = O.transient(Ks, dh, Qs, Ss, V, dt, nsteps, np.zeros(O.nfree), reltol=1e-14)
    dK_or = O.transient_adjoint(dh, obs, reltol=1e-14)[0]
    _, st = P.transient_forward(Ks, dh, Qs, Ss, dt, nsteps, np.zeros(N), checkpoint_every=ck, return_states=True)
    dK = P.transient_adjoint(obs)[0]
    isf, _, _ = pkg.getfreenodes(N, dn)
    return {"rel_state_err_vs_oracle_1e-14": _rel(st[:, isf], st_or), "rel_dKs_err_vs_oracle_1e-14": _rel(dK, dK_or),
            "oracle_steps": nsteps, "oracle_checkpoint_every": ck}


# ---------------------------------------------------------------- general (CSR) path, 1M cells
def run_general(args, dist, rank, ws, METRIC_NAME):
    """The 1M-cell grid given as a shuffled face list, so the library takes its CSR path
    (graph aggregation AMG), solved beside the structured path on the same inputs."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    ge._load_build_module().build()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    grid, mins, maxs = (200, 200, 25), (0.0, 0.0, 0.0), (100.0, 100.0, 10.0)
    N = 200 * 200 * 25
    _, nb, aol, _ = pkg.regulargrid3d(mins, maxs, grid)
    perm = np.random.default_rng(8).permutation(len(aol))
    nbs, aols = np.ascontiguousarray(np.asarray(nb)[perm]), np.ascontiguousarray(np.asarray(aol)[perm])
    lk = pkg.fields.volume_logk(grid, mins, maxs, 20.0, 2.0, -9.0, 4)
    Qs = np.zeros(N)
    Qs[0] = 1e-4
    obs = np.random.default_rng(9).choice(N, 100, replace=False)
    d = [torch.tensor(x, device=dev) for x in (lk, np.zeros(N), Qs)]
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float64, device=dev)
    import warnings
    warnings.simplefilter("error", RuntimeWarning)
    t0 = time.perf_counter()
    G = pkg.GroundwaterProblem(nbs, aols, [N - 1], N=N, reltol=1e-10, precision=args.precision)
    setup_s = time.perf_counter() - t0
    assert not G.structured
    steps = max(1, args.steps // 2)
    t = _events(torch, lambda: G.solve_grad_logk(*d, obs), steps, 2, flush)
    h, g = G.solve_grad_logk(*d, obs)
    G64 = pkg.GroundwaterProblem(nbs, aols, [N - 1], N=N, reltol=1e-10, precision="fp64")
    t64 = _events(torch, lambda: G64.solve_grad_logk(*d, obs), 1, 1, flush)
    S = pkg.GroundwaterProblem.regular3d(mins, maxs, grid, [N - 1], reltol=1e-13, precision="fp64")
    warnings.simplefilter("ignore", RuntimeWarning)
    hs, gs = S.solve_grad_logk(*d, obs)
    return {
        "metric": METRIC_NAME, "value": round(steps / t, 3), "unit": "solves/s", "n_gpus": ws, "steps": steps,
        "warmup": 2, "ms_per_step": round(1e3 * t / steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 V-cycle + double-float CG (f32 ops), f64 residual",
        "data": "synthetic (seeded Matern logK field)",
        "config": {"workload": "gw_steady_fwd_adj_general_csr_1M", "cells": N, "faces": int(len(aol)),
                   "path": "CSR (face list shuffled, not recognised as a regular grid)",
                   "setup_seconds": round(setup_s, 2), "precision": args.precision, "reltol": 1e-10},
        "plain_fp64_gpu": {"value": round(1.0 / t64, 3), "unit": "solves/s"},
        "speedup_vs_plain_fp64": round(t64 / (t / steps), 3),
        "accuracy": {"rel_head_err_vs_structured_fp64_1e-13": _rel(h.cpu().numpy(), hs.cpu().numpy()),
                     "rel_grad_err_vs_structured_fp64_1e-13": _rel(g.cpu().numpy(), gs.cpu().numpy())},
        "iterations_last_adjoint": G.stats["iterations"],
    }


def run_richards(args, dist, rank, ws, METRIC_NAME):
    """The steady Richards equation and its rrule (DPFEHM src/richards.jl:148-190) on a
    100x100x20 grid over 50x50x10 m: a Dirichlet top layer at psi = -2 m (an unsaturated zone above
    the water table), a 1e-6 m^3/s source at depth (as in examples/richards_steadystate_3d),
    Matern(l = 15 m, sigma = 1) logK, van Genuchten alpha ~ 0.375 and N ~ 1.25 per face;
    J = sum psi^2 at 100 cells. One "solve" is the forward solve and its pullback."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    ge._load_build_module().build()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    grid, mins, maxs = (100, 100, 20), (0.0, 0.0, 0.0), (50.0, 50.0, 10.0)
    coords, nb, aol, _ = pkg.regulargrid3d(mins, maxs, grid)
    N, F = coords.shape[1], len(aol)
    lk = pkg.fields.volume_logk(grid, mins, maxs, 15.0, 1.0, -9.0, 21)
    Ks = np.exp(0.5 * (lk[nb[:, 0]] + lk[nb[:, 1]]))
    z = coords[2]
    dn = np.nonzero(np.isclose(z, maxs[2]))[0]
    dpsi = np.zeros(N)
    dpsi[dn] = -2.0
    Qs = np.zeros(N)
    Qs[0] = 1e-6
    rng = np.random.default_rng(22)
    alphas = 0.375 * np.exp(0.1 * rng.standard_normal(F))
    Ns = 1.25 + 0.05 * rng.uniform(0, 1, F)
    obs = rng.choice(np.setdiff1d(np.arange(N), dn), 100, replace=False)
    delta = np.zeros(N)
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float64, device=dev)
    d = {k: torch.tensor(v, device=dev) for k, v in (("Ks", Ks), ("dpsi", dpsi), ("z", z), ("al", alphas),
                                                   ("N", Ns), ("Q", Qs), ("psi0", np.full(N, -2.0)))}
    import warnings
    warnings.simplefilter("error", RuntimeWarning)

    def make(prec):
        return pkg.GroundwaterProblem(nb, aol, dn, N=N, general=True, reltol=1e-10, precision=prec)

    def step(P):
        psi = P.richards_steady(d["psi0"], d["Ks"], d["dpsi"], d["z"], d["al"], d["N"], d["Q"], 1e-10, 300)
        dl = torch.zeros(N, dtype=torch.float64, device=dev)
        dl[obs] = 2 * psi[obs]
        return psi, P.richards_adjoint(dl, 1e-8, 300)

    P = make(args.precision)
    steps = max(1, args.steps // 2)
    t = _events(torch, lambda: step(P), steps, 1, flush)
    psi, grads = step(P)
    st = P.richards_stats
    P64 = make("fp64")
    t64 = _events(torch, lambda: step(P64), 1, 1, flush)
    psi64, g64 = step(P64)
    return {
        "metric": METRIC_NAME, "value": round(steps / t, 3), "unit": "solves/s", "n_gpus": ws, "steps": steps,
        "warmup": 1, "ms_per_step": round(1e3 * t / steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 residuals and kr; inner CG: f32 V-cycle + double-float CG" if args.precision == "mixed" else "f64",
        "data": "synthetic (seeded Matern logK field, seeded van Genuchten parameters)",
        "config": {"workload": "richards_steady_fwd_adj_100x100x20_unsaturated", "cells": N, "faces": F,
                   "dirichlet": "top layer, psi = -2 m", "precision": args.precision, "tol": 1e-10,
                   "path": "CSR (dpf_create_general)"},
        "picard_iterations": st["iterations"], "adjoint_gmres_iterations": st["adjoint_iterations"],
        "unsaturated_fraction": float((psi < 0).double().mean()),
        "plain_fp64_gpu": {"value": round(1.0 / t64, 3), "unit": "solves/s"},
        "speedup_vs_plain_fp64": round(t64 / (t / steps), 3),
        "accuracy": {"rel_psi_err_vs_fp64": _rel(psi.cpu().numpy(), psi64.cpu().numpy()),
                     "rel_dKs_err_vs_fp64": _rel(grads[0].cpu().numpy(), g64[0].cpu().numpy())},
    }


def run_cholesky(args, dist, rank, ws, METRIC_NAME):
    """The direct solver (linear_solver = cholesky_solver, DPFEHM src/groundwater.jl:56-60): a
    banded Cholesky factorisation of the FP64 operator on the GPU, for the grid classes the
    reference's own Cholesky-versus-CG comparison covers (examples/fracture_network_solver_scaling/
    porous_media_comparison.jl: unit conductivity, Dirichlet h = 1 and 0 on the x = min and x = max
    faces). Here: a 2-D grid of 500 x 500 cells and a 3-D grid of 48^3, each with a Matern
    (l = 20 cells, sigma = 1) logK. One "solve" is a forward solve (factorisation included) and its
    adjoint; the same on the AMG-preconditioned CG in FP64 for comparison; heads against the
    oracle (its CG to 1e-14) on the host."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    ge._load_build_module().build()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    import warnings
    warnings.simplefilter("error", RuntimeWarning)
    cases = []
    for grid in ((500, 500, 1), (48, 48, 48)):
        mins = (0.0, 0.0, 0.0)
        maxs = tuple(float(n - 1) for n in grid)
        coords, nb, aol, vol = pkg.regulargrid3d(mins, maxs, grid)
        N = coords.shape[1]
        lk = pkg.fields.volume_logk(grid, mins, maxs, 20.0, 1.0, -9.0, 31)
        Ks = np.exp(0.5 * (lk[nb[:, 0]] + lk[nb[:, 1]]))
        x = coords[0]
        dn = np.nonzero((x == mins[0]) | (x == maxs[0]))[0]
        dh = np.where(x == mins[0], 1.0, 0.0)
        Qs = np.zeros(N)
        rng = np.random.default_rng(32)
        delta = np.zeros(N)
        delta[rng.choice(np.setdiff1d(np.arange(N), dn), 100, replace=False)] = 1.0
        row = {"grid": list(grid), "cells": N, "band": int(grid[1] * grid[2]) if grid[2] > 1 else int(grid[1])}
        for solver, prec, tol in (("cholesky", "fp64", 1e-10), ("cg", "fp64", 1e-10)):
            P = pkg.GroundwaterProblem(nb, aol, dn, N=N, solver=solver, precision=prec, reltol=tol)
            P.forward(Ks, dh, Qs)  # warm-up (and the band set-up)
            P.adjoint(delta)
            torch.cuda.synchronize()
            reps = 2
            t0 = time.perf_counter()
            for _ in range(reps):
                h = P.forward(Ks, dh, Qs)
                g = P.adjoint(delta)
            torch.cuda.synchronize()
            row[solver + "_ms_per_solve"] = round(1e3 * (time.perf_counter() - t0) / reps, 2)
            row[solver + "_relres"] = P.stats["relres"]
            row[solver + "_iterations"] = P.stats["iterations"]
            row[solver + "_h"] = np.asarray(h)
        cases.append((grid, nb, aol, dn, Ks, dh, Qs, row))
    import sys
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    orc.build()
    orc.set_threads(os.cpu_count() or 1)
    out_rows = []
    for grid, nb, aol, dn, Ks, dh, Qs, row in cases:
        O = orc.Problem(row["cells"], nb, aol, np.asarray(dn, np.int64))
        t0 = time.perf_counter()
        ho = O.steady(Ks, dh, Qs, reltol=1e-14)
        row["oracle_forward_s"] = round(time.perf_counter() - t0, 3)
        row["rel_head_err_vs_oracle"] = _rel(row.pop("cholesky_h"), ho)
        row["cg_rel_head_err_vs_oracle"] = _rel(row.pop("cg_h"), ho)
        out_rows.append(row)
    t_main = out_rows[0]["cholesky_ms_per_solve"] / 1e3
    return {
        "metric": METRIC_NAME, "value": round(1.0 / t_main, 3), "unit": "solves/s", "n_gpus": ws, "steps": 2,
        "warmup": 1, "ms_per_step": out_rows[0]["cholesky_ms_per_solve"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Matern logK fields)",
        "config": {"workload": "gw_steady_fwd_adj_direct_cholesky", "precision": "fp64", "solver": "cholesky",
                   "value_case": "2-D 500 x 500", "cases": out_rows},
    }


def run_dfn(args, dist, rank, ws, METRIC_NAME):
    """A synthetic fracture network mesh (grid.fracture_network: 3000 square fractures with power-law
    sizes from 4 to 50 m in a 100 m cube, cells of 0.25 m, about 5M cells after keeping the largest
    connected component; degrees 2-9) through dpf_create, so the CSR path solves it: h = 1 within
    5 m of x = 0, h = 0 within 5 m of x = 100, two 1e-6 m^3/s injections, one log-conductivity per
    fracture (N(-9, 1)), J = sum of h^2 at 100 cells. Host setup (topology, aggregation hierarchy)
    is timed separately from the solves."""
    import sys
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    ge._load_build_module().build()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    t0 = time.perf_counter()
    c, vol, nb, areas, lengths, fr = pkg.grid.fracture_network(3000, 100.0, 0.25, 3, smin=4.0)
    gen_s = time.perf_counter() - t0
    N, F = c.shape[1], len(nb)
    aol = areas / lengths
    rng = np.random.default_rng(4)
    logK = rng.normal(-9.0, 1.0, fr.max() + 1)[fr]
    x = c[0]
    dn = np.nonzero((x < 5.0) | (x > 95.0))[0]
    dh = np.zeros(N)
    dh[x < 5.0] = 1.0
    Qs = np.zeros(N)
    Qs[rng.choice(np.nonzero((x > 30) & (x < 70))[0], 2, replace=False)] = 1e-6
    obs = rng.choice(np.setdiff1d(np.arange(N), dn), 100, replace=False)
    d = [torch.tensor(v, device=dev) for v in (logK, dh, Qs)]
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float64, device=dev)
    import warnings
    warnings.simplefilter("error", RuntimeWarning)
    t0 = time.perf_counter()
    # coarse-correction scale 2.0: on this mesh 87 CG iterations against 108 with the general
    # path's default 3.5 (tuned on grids given as face lists)
    G = pkg.GroundwaterProblem(nb, aol, dn, N=N, volumes=vol, reltol=1e-10, precision=args.precision,
                               coarse_scale=2.0)
    setup_s = time.perf_counter() - t0
    assert not G.structured
    steps = max(1, args.steps // 2)
    t = _events(torch, lambda: G.solve_grad_logk(*d, obs), steps, 2, flush)
    h, g = G.solve_grad_logk(*d, obs)
    iters = G.stats["iterations"]
    # per-kernel CUDA events over one more forward + adjoint: the dominant kernel against the roofline
    G.profile(True)
    G.solve_grad_logk(*d, obs)
    rep = G.profile_report()
    G.profile(False)
    total = sum(v[1] for v in rep.values())
    top = sorted(rep.items(), key=lambda kv: -kv[1][1])
    name, (cnt, ms, cells) = top[0]
    nnz = 2 * int(np.sum(~(np.isin(nb[:, 0], dn) | np.isin(nb[:, 1], dn))))  # couplings between free cells
    # algorithmic bytes per launch of the finest level's kernels (every array element once):
    # Chebyshev step: column index and FP32 value per coupling (8 B), row pointer, x in, b, d in,
    # leak, d out, x out per row (28 B; the first step after prolongation reads no d: 24 B);
    # double-float product: index and double-float value per coupling (12 B), row pointer, p, leak,
    # q per row (28 B); x/r update: 52 B per row
    level_bytes = {"kg_cheb_step": 8 * nnz + 28 * N, "kg_cheb_step0": 8 * nnz + 24 * N,
                   "kg_cheb_first2": 8 * nnz + 24 * N, "kg_df_spmv_pq": 12 * nnz + 28 * N,
                   "kg_df_update_xr": 52 * N}
    known = [(k, v) for k, v in top if k.endswith("<f32>/L0") and k.split("<")[0] in level_bytes]
    name, sp = known[0] if known else (None, None)
    peaks = {}
    try:
        import json as _json
        peaks = _json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    roof = None
    if sp:
        bpl = level_bytes[name.split("<")[0]]
        ach = bpl * sp[0] / (sp[1] / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": name, "achieved": round(ach, 1), "peak": peak,
                "unit": "GB/s", "frac": round(ach / peak, 4),
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback", "traffic": None,
                "bytes_per_launch": int(bpl), "avg_launch_us": round(1e3 * sp[1] / sp[0], 3),
                "share": round(sp[1] / total, 4) if total else None,
                "measured": "per-kernel CUDA events on the solver stream over one forward+adjoint of this workload"}
    G64 = pkg.GroundwaterProblem(nb, aol, dn, N=N, volumes=vol, reltol=1e-10, precision="fp64", coarse_scale=2.0)
    t64 = _events(torch, lambda: G64.solve_grad_logk(*d, obs), 1, 1, flush)
    h, g = h.cpu().numpy(), g.cpu().numpy()
    # the oracle: timed at the run's reltol (the CPU baseline), then at 1e-13 for the errors
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    orc.build()
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    Ks = orc.logk_to_faces(nb, logK)

    def oracle_step(tol):
        O = orc.Problem(N, nb, aol, dn)
        ho = O.steady(Ks, dh, Qs, reltol=tol)
        delta = np.zeros(N)
        np.add.at(delta, obs, 2 * ho[obs])
        dKs, _, _ = O.adjoint(dh, delta, reltol=tol)
        return ho, orc.logk_to_faces_vjp(nb, logK, dKs)

    t0 = time.perf_counter()
    oracle_step(1e-10)
    tc = time.perf_counter() - t0
    ho, go = oracle_step(1e-13)
    return {
        "metric": METRIC_NAME, "value": round(steps / t, 3), "unit": "solves/s", "n_gpus": ws, "steps": steps,
        "warmup": 2, "ms_per_step": round(1e3 * t / steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 V-cycle + double-float CG (f32 ops), f64 residual"
        if args.precision == "mixed" else "f64",
        "data": "synthetic (seeded fracture network, one log-conductivity per fracture)",
        "config": {"workload": "gw_steady_fwd_adj_dfn_5M", "cells": N, "faces": F,
                   "fractures": int(len(np.unique(fr))), "max_degree": int(np.bincount(nb.ravel()).max()),
                   "dirichlet_cells": int(len(dn)), "path": "CSR (dpf_create on a face list)",
                   "generate_seconds": round(gen_s, 2), "setup_seconds": round(setup_s, 2), "coarse_scale": 2.0,
                   "precision": args.precision, "reltol": 1e-10},
        "iterations_last_adjoint": iters,
        "plain_fp64_gpu": {"value": round(1.0 / t64, 3), "unit": "solves/s"},
        "speedup_vs_plain_fp64": round(t64 / (t / steps), 3),
        "roofline": roof,
        "top": [{"kernel": k, "launches": v[0], "ms": round(v[1], 3)} for k, v in top[:8]],
        "accuracy": {"rel_head_err_vs_oracle_1e-13": _rel(h, ho), "rel_grad_err_vs_oracle_1e-13": _rel(g, go)},
        "cpu_baseline": {"value": round(1.0 / tc, 4), "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": "one forward+adjoint of this workload (oracle: Ruge-Stueben AMG + CG, FP64, "
                                   "reltol 1e-10, setup included)"},
    }


def run(name, args, dist, rank, ws):
    if rank != 0:
        return None
    if name == "dfn":
        return run_dfn(args, dist, rank, ws, "forward+adjoint solves/sec, 5M-cell fracture network, CSR path")
    if name == "cholesky":
        return run_cholesky(args, dist, rank, ws, "forward+adjoint solves/sec, direct (banded Cholesky) solver")
    if name == "richards":
        return run_richards(args, dist, rank, ws, "Richards steady forward+adjoint solves/sec, 200k cells")
    if name == "general_1m":
        return run_general(args, dist, rank, ws, "forward+adjoint solves/sec at 1M cells, general (CSR) path")
    if name == "transient":
        return run_transient(args, dist, rank, ws, "transient forward+adjoint runs/sec, 800k cells x 100 BE steps")
    metric = ("forward+adjoint solves/sec at 100k cells" if name == "steady_100k"
              else "forward+adjoint solves/sec, uneven batch of 256 grids")
    return run_steady(name, args, dist, rank, ws, metric)
