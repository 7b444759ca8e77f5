"""Batched solves (uneven grids, one set of launches) against the oracle, and the
CUDA-graph and host-driven CG loops against each other."""
import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu


def _problem(pkg, ns, seed):
    mins = (0.0, 0.0, 0.0)
    maxs = tuple(0.5 * (n - 1) for n in ns)
    logK = pkg.fields.volume_logk(ns, mins, maxs, 0.5 * maxs[0] + 1.0, 1.0 + 0.5 * (seed % 3), -9.0, seed)
    N = int(np.prod(ns))
    rng = np.random.default_rng(seed)
    Qs = np.zeros(N)
    q = rng.choice(N, 1 + seed % 4, replace=False)
    Qs[q] = rng.uniform(1e-5, 1e-3, len(q))
    dn = np.sort(rng.choice(np.setdiff1d(np.arange(N), q), 1 + (seed + 1) % 4, replace=False))
    dh = np.zeros(N)
    obs = rng.choice(N, 10, replace=False)
    return dict(ns=ns, mins=mins, maxs=maxs, logK=logK, N=N, Qs=Qs, dn=dn, dh=dh, obs=obs)


def _oracle(orc, pkg, c):
    _, nb, aol, _ = pkg.regulargrid3d(c["mins"], c["maxs"], c["ns"])
    O = orc.Problem(c["N"], nb, aol, c["dn"])
    h = O.steady(orc.logk_to_faces(nb, c["logK"]), c["dh"], c["Qs"], reltol=1e-14)
    delta = np.zeros(c["N"])
    np.add.at(delta, c["obs"], 2 * h[c["obs"]])
    dKs, _, _ = O.adjoint(c["dh"], delta, reltol=1e-14)
    return h, orc.logk_to_faces_vjp(nb, c["logK"], dKs)


@pytest.mark.parametrize("precision,plane", [("fp64", 1), ("mixed", 1), ("mixed", 2)])
def test_uneven_batch_vs_oracle(gpu_lib, orc, precision, plane):
    """plane=2 forces the plane-marching smoothers at these small sizes (by default a handle this
    small runs the grid-stride ones)."""
    pkg = gpu_lib
    shapes = [(20, 16, 5), (9, 9, 9), (40, 30, 6), (3, 4, 2), (25, 25, 4), (17, 5, 11)]
    probs = [_problem(pkg, ns, 11 + k) for k, ns in enumerate(shapes)]
    B = pkg.GroundwaterBatch([p["ns"] for p in probs], [p["mins"] for p in probs], [p["maxs"] for p in probs],
                             [p["dn"] for p in probs], reltol=1e-11, precision=precision, plane=plane)
    assert B.nprob == len(probs)
    cat = lambda k: np.concatenate([p[k] for p in probs])
    h, g = B.solve_grad_logk(cat("logK"), cat("dh"), cat("Qs"), [p["obs"] for p in probs])
    for k, p in enumerate(probs):
        a, b = B.cell_offsets[k], B.cell_offsets[k + 1]
        h_or, g_or = _oracle(orc, pkg, p)
        assert rel(h[a:b], h_or) < 1e-8, k
        assert rel(g[a:b], g_or) < 1e-6, k


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_and_host_loops_agree(gpu_lib, precision):
    pkg = gpu_lib
    c = _problem(pkg, (30, 24, 10), 5)
    res = []
    for graphs in (1, 0):
        P = pkg.GroundwaterProblem.regular3d(c["mins"], c["maxs"], c["ns"], c["dn"], reltol=1e-11,
                                              precision=precision, use_graphs=graphs, check_every=3)
        res.append((P.solve_grad_logk(c["logK"], c["dh"], c["Qs"], c["obs"]), P.stats))
    (h1, g1), s1 = res[0]
    (h2, g2), s2 = res[1]
    assert s1["iterations"] == s2["iterations"]
    assert rel(h1, h2) < 1e-12 and rel(g1, g2) < 1e-10


def test_batch_of_identical_problems_is_uniform(gpu_lib):
    pkg = gpu_lib
    c = _problem(pkg, (16, 16, 8), 3)
    nb = 5
    B = pkg.GroundwaterBatch([c["ns"]] * nb, [c["mins"]] * nb, [c["maxs"]] * nb, [c["dn"]] * nb, reltol=1e-11,
                             precision="mixed")
    h, g = B.solve_grad_logk(np.tile(c["logK"], nb), np.tile(c["dh"], nb), np.tile(c["Qs"], nb), [c["obs"]] * nb)
    N = c["N"]
    for k in range(1, nb):
        assert np.array_equal(h[k * N:(k + 1) * N], h[:N])
        assert np.array_equal(g[k * N:(k + 1) * N], g[:N])


def test_profile_report_and_launch_count(gpu_lib):
    pkg = gpu_lib
    c = _problem(pkg, (20, 20, 6), 9)
    P = pkg.GroundwaterProblem.regular3d(c["mins"], c["maxs"], c["ns"], c["dn"], precision="mixed")
    n0 = P.launch_count
    P.profile(True)
    P.solve_grad_logk(c["logK"], c["dh"], c["Qs"], c["obs"])
    rep = P.profile_report()
    P.profile(False)
    assert P.launch_count > n0
    assert any(k.startswith(("k_pm_post2<f32>/L0", "k_pm_step<f32>/L0", "k_cheb_step<f32>/L0")) for k in rep)
    assert all(v[0] > 0 and v[1] >= 0 for v in rep.values())
    assert sum(v[0] for v in rep.values()) == P.launch_count - n0


def test_fused_and_separate_plane_passes_agree(gpu_lib, orc):
    """The fused plane passes (pre-smoothing + restriction, prolongation + post-smoothing in one
    pass each) give the separate passes' solve to rounding and the oracle's, on an uneven batch
    whose problems reach the fused small-level tail at different levels (so a level is
    smoothed by per-level kernels for some problems and inside the tail for others)."""
    pkg = gpu_lib
    shapes = [(50, 50, 5), (66, 60, 10), (31, 29, 7), (24, 20, 8), (9, 9, 9)]
    probs = [_problem(pkg, ns, 141 + k) for k, ns in enumerate(shapes)]
    cat = lambda k: np.concatenate([p[k] for p in probs])
    out = {}
    for fuse in (1, -1):
        B = pkg.GroundwaterBatch([p["ns"] for p in probs], [p["mins"] for p in probs], [p["maxs"] for p in probs],
                                 [p["dn"] for p in probs], reltol=1e-11, precision="mixed", fuse=fuse, plane=2)
        out[fuse] = B.solve_grad_logk(cat("logK"), cat("dh"), cat("Qs"), [p["obs"] for p in probs])
    assert rel(out[1][0], out[-1][0]) < 1e-9 and rel(out[1][1], out[-1][1]) < 1e-7
    off = np.cumsum([0] + [p["N"] for p in probs])
    for k, p in enumerate(probs):
        h_or, g_or = _oracle(orc, pkg, p)
        assert rel(out[1][0][off[k]:off[k + 1]], h_or) < 1e-8, k
        assert rel(out[1][1][off[k]:off[k + 1]], g_or) < 1e-6, k


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_plane_and_grid_stride_smoothers_agree(gpu_lib, precision):
    """The plane-marching smoothers (shared-memory staged, prolongation fused) and the
    grid-stride kernels apply the same arithmetic; solves agree to rounding of the r.z sums."""
    pkg = gpu_lib
    shapes = [(20, 16, 5), (9, 9, 9), (40, 30, 6), (3, 4, 2), (25, 25, 4), (17, 5, 11), (12, 3, 70), (8, 40, 1)]
    probs = [_problem(pkg, ns, 31 + k) for k, ns in enumerate(shapes)]
    cat = lambda k: np.concatenate([p[k] for p in probs])
    out = {}
    for plane in (2, -1):  # 2: the plane kernels also at these small sizes
        for tail in (4096, -1):
            B = pkg.GroundwaterBatch([p["ns"] for p in probs], [p["mins"] for p in probs],
                                     [p["maxs"] for p in probs], [p["dn"] for p in probs], reltol=1e-12,
                                     precision=precision, plane=plane, tail_cells=tail,
                                     df_plane_cells=256 if plane > 0 else -1)
            out[(plane, tail)] = B.solve_grad_logk(cat("logK"), cat("dh"), cat("Qs"), [p["obs"] for p in probs])
    h0, g0 = out[(-1, -1)]
    for key, (h, g) in out.items():
        assert rel(h, h0) < 1e-11, key
        assert rel(g, g0) < 1e-9, key


@pytest.mark.parametrize("streams", [1, 3])
def test_host_buffers_match_device_buffers(gpu_lib, streams):
    """Host (page-locked) inputs and outputs give the device-resident results bit for bit, also
    when the batch runs as concurrent parts whose host inputs are copied part after part and
    whose heads are copied out during the adjoint solve."""
    import torch
    pkg = gpu_lib
    shapes = [(20, 16, 5), (9, 9, 9), (40, 30, 6), (12, 3, 70)]
    probs = [_problem(pkg, ns, 51 + k) for k, ns in enumerate(shapes)]
    cat = lambda k: np.concatenate([p[k] for p in probs])
    B = pkg.GroundwaterBatch([p["ns"] for p in probs], [p["mins"] for p in probs], [p["maxs"] for p in probs],
                             [p["dn"] for p in probs], reltol=1e-11, precision="mixed", streams=streams)
    obs = [p["obs"] for p in probs]
    dev = [torch.tensor(cat(k), device="cuda") for k in ("logK", "dh", "Qs")]
    hd, gd = B.solve_grad_logk(*dev, obs)
    hd, gd = hd.cpu().numpy(), gd.cpu().numpy()
    host = [torch.from_numpy(cat(k)).pin_memory() for k in ("logK", "dh", "Qs")]
    outs = [torch.full((B.N,), np.nan, dtype=torch.float64).pin_memory() for _ in range(2)]
    for _ in range(2):  # twice: the second call reuses the copy stream and the staged inputs
        h, g = B.solve_grad_logk(*[x.numpy() for x in host], obs, out=tuple(x.numpy() for x in outs))
        assert np.array_equal(h, hd) and np.array_equal(g, gd)
    # pageable host arrays as well
    h, g = B.solve_grad_logk(cat("logK"), cat("dh"), cat("Qs"), obs)
    assert np.array_equal(h, hd) and np.array_equal(g, gd)
    B.close()


def test_caller_output_buffers(gpu_lib):
    """solve_grad_logk(out=(h, g)) fills the caller's host buffers with the same values."""
    pkg = gpu_lib
    c = _problem(pkg, (14, 12, 5), 21)
    B = pkg.GroundwaterBatch([c["ns"]], [c["mins"]], [c["maxs"]], [c["dn"]], reltol=1e-11, precision="mixed")
    h0, g0 = B.solve_grad_logk(c["logK"], c["dh"], c["Qs"], [c["obs"]])
    hb, gb = np.full(c["N"], np.nan), np.full(c["N"], np.nan)
    h1, g1 = B.solve_grad_logk(c["logK"], c["dh"], c["Qs"], [c["obs"]], out=(hb, gb))
    assert h1 is hb and g1 is gb
    assert np.array_equal(hb, h0) and np.array_equal(gb, g0)
    with pytest.raises(ValueError):
        B.solve_grad_logk(c["logK"], c["dh"], c["Qs"], [c["obs"]], out=(np.zeros(c["N"], np.float32), gb))


def test_autotune_batch(gpu_lib):
    """The autotuner returns options from its candidate sets that give the same solution."""
    pkg = gpu_lib
    shapes = [(20, 16, 5), (9, 9, 9), (40, 30, 6)]
    probs = [_problem(pkg, ns, 41 + k) for k, ns in enumerate(shapes)]
    cat = lambda k: np.concatenate([p[k] for p in probs])
    args = ([p["ns"] for p in probs], [p["mins"] for p in probs], [p["maxs"] for p in probs],
            [p["dn"] for p in probs])
    tuned, ms = pkg.autotune_batch(*args, cat("logK"), cat("dh"), cat("Qs"), [p["obs"] for p in probs],
                                   repeats=1, reltol=1e-11, precision="mixed")
    assert ms > 0
    assert tuned["cheb_degree"] in (1, 2, 3) and tuned["plane_cells"] in (512, 768, 1024)
    assert tuned["plane_blocks_per_sm"] in (1, 2, 3) and tuned["tail_cells"] in (-1, 1024, 4096, 16384)
    assert tuned["blocks_per_sm"] in (8, 16, 24) and tuned["df_plane_cells"] in (-1, 256)
    assert tuned["tail_cluster"] in (1, 8)
    B0 = pkg.GroundwaterBatch(*args, reltol=1e-11, precision="mixed")
    B1 = pkg.GroundwaterBatch(*args, reltol=1e-11, precision="mixed", **tuned)
    h0, g0 = B0.solve_grad_logk(cat("logK"), cat("dh"), cat("Qs"), [p["obs"] for p in probs])
    h1, g1 = B1.solve_grad_logk(cat("logK"), cat("dh"), cat("Qs"), [p["obs"] for p in probs])
    assert rel(h1, h0) < 1e-9 and rel(g1, g0) < 1e-7


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cluster_tail_agrees(gpu_lib, precision):
    """The fused small-level tail run by a thread-block cluster per problem (levels from 1
    down) gives the per-level kernels' solution."""
    pkg = gpu_lib
    shapes = [(20, 16, 5), (9, 9, 9), (40, 30, 6), (3, 4, 2), (17, 5, 11)]
    probs = [_problem(pkg, ns, 61 + k) for k, ns in enumerate(shapes)]
    cat = lambda k: np.concatenate([p[k] for p in probs])
    res = []
    for tail, cl in ((-1, 1), (20000, 8), (20000, 1), (4096, 16)):
        B = pkg.GroundwaterBatch([p["ns"] for p in probs], [p["mins"] for p in probs], [p["maxs"] for p in probs],
                                 [p["dn"] for p in probs], reltol=1e-12, precision=precision, tail_cells=tail,
                                 tail_cluster=cl)
        res.append(B.solve_grad_logk(cat("logK"), cat("dh"), cat("Qs"), [p["obs"] for p in probs]))
    for h, g in res[1:]:
        assert rel(h, res[0][0]) < 1e-11 and rel(g, res[0][1]) < 1e-9


def test_batch_split_into_concurrent_parts(gpu_lib, orc):
    """streams = k splits a batch into k parts of consecutive problems (sizes differing by one
    when k does not divide the batch), each on its own stream and host thread. Every part is a
    smaller batch of the same solver, whose per-problem reductions run over a different number
    of blocks, so the results equal the single-stream ones to rounding and the oracle's to the
    usual tolerances. Entry points other than the batched solve are refused on a split handle."""
    pkg = gpu_lib
    shapes = [(20, 16, 5), (9, 9, 9), (40, 30, 6), (17, 5, 11), (24, 20, 8)]
    probs = [_problem(pkg, ns, 81 + k) for k, ns in enumerate(shapes)]
    cat = lambda k: np.concatenate([p[k] for p in probs])
    args = ([p["ns"] for p in probs], [p["mins"] for p in probs], [p["maxs"] for p in probs],
            [p["dn"] for p in probs])
    res = {}
    for streams in (1, 2, 3, 4):
        B = pkg.GroundwaterBatch(*args, reltol=1e-12, precision="mixed", streams=streams, plane=2)
        for _ in range(2):  # the first solve of fresh parts, then a repeat on the same handles
            res[streams] = B.solve_grad_logk(cat("logK"), cat("dh"), cat("Qs"), [p["obs"] for p in probs])
        assert list(B.cell_offsets) == list(np.cumsum([0] + [p["N"] for p in probs]))
        if streams > 1:
            with pytest.raises(pkg.DPFError) as e:
                B.forward_logk(cat("logK"), cat("dh"), cat("Qs"))
            assert e.value.code == pkg._lib.DPF_UNSUPPORTED
        else:
            B.forward_logk(cat("logK"), cat("dh"), cat("Qs"))
        B.close()
    h1, g1 = res[1]
    for s in (2, 3, 4):
        assert rel(res[s][0], h1) < 1e-11 and rel(res[s][1], g1) < 1e-9, s
    for k, p in enumerate(probs):
        a, b = int(np.sum([q["N"] for q in probs[:k]])), int(np.sum([q["N"] for q in probs[:k + 1]]))
        h_or, g_or = _oracle(orc, pkg, p)
        assert rel(res[4][0][a:b], h_or) < 1e-8 and rel(res[4][1][a:b], g_or) < 1e-6, k


def test_set_stream(gpu_lib):
    """Work issued on a caller's stream gives the default stream's results."""
    import torch
    pkg = gpu_lib
    c = _problem(pkg, (18, 14, 6), 31)
    P = pkg.GroundwaterProblem.regular3d(c["mins"], c["maxs"], c["ns"], c["dn"], reltol=1e-11, precision="mixed")
    h0, g0 = P.solve_grad_logk(c["logK"], c["dh"], c["Qs"], c["obs"])
    s = torch.cuda.Stream()
    P.set_stream(s)
    h1, g1 = P.solve_grad_logk(c["logK"], c["dh"], c["Qs"], c["obs"])
    P.set_stream(None)
    assert np.array_equal(h0, h1) and np.array_equal(g0, g1)
