"""Parity with the oracle at the full sizes of the benchmark configurations, through the C ABI.

  * the 1M-cell steady forward + adjoint (200x200x25 nodes over 100x100x10 m, 3-D Matern logK with
    correlation length 20 m, sigma 2, mean -9; Qs = 1e-4 in cell 0; Dirichlet h = 0 in the last
    cell; J = sum of h^2 at 100 seeded cells; gradient d/dlogK), in mixed precision and in FP64,
    on the benchmark's realization 0;
  * an uneven batch holding one grid of each size of the 256-grid configuration (50x50x5,
    100x100x10, 150x150x10, 200x200x20), its random correlation lengths, sigmas, 1-4 injection
    and 1-4 Dirichlet cells, mixed precision; every member against the oracle;
  * the 800k-cell transient run (200x200x20 over 100x100x10 m, Ss = 1e-5, dt = 3600 s, Dirichlet
    h = 0 on the x = max face, 1e-3 at 4 seeded cells, Matern l = 30 m, sigma 1.5; J = sum over
    steps of h^2 at 50 cells) on its full grid, cut from 100 to 12 steps with a checkpoint every
    5 steps (so the last segment is partial) to keep the oracle's 24 solves within a minute.

The oracle solves to reltol 1e-14; the GPU to the configurations' 1e-10, except the transient run,
whose every step is solved to 1e-11: the states of 12 steps at 1e-10 per step were 2.8e-8 from the
oracle's (both precisions alike), above the 1e-8 head bar. Tolerances (relative L2): heads 1e-8,
gradients 1e-6.
"""
import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu
HEAD_TOL = 1e-8
GRAD_TOL = 1e-6


def _oracle_steady_grad(orc, pkg, grid, mins, maxs, logK, dn, Qs, obs):
    """Oracle head and dJ/dlogK for J = sum h[obs]^2 (geometric face means)."""
    _, nb, aol, _ = pkg.regulargrid3d(mins, maxs, grid)
    N = int(np.prod(grid))
    O = orc.Problem(N, nb, aol, np.asarray(dn, np.int64))
    dh = np.zeros(N)
    h = O.steady(orc.logk_to_faces(nb, logK), dh, Qs, reltol=1e-14)
    delta = np.zeros(N)
    np.add.at(delta, obs, 2 * h[obs])
    dKs, _, _ = O.adjoint(dh, delta, reltol=1e-14)
    return h, orc.logk_to_faces_vjp(nb, logK, dKs)


@pytest.fixture(scope="module")
def config_1m(gpu_lib, orc):
    """The benchmark's realization 0 and its oracle solution (computed once for both precisions)."""
    import os
    pkg = gpu_lib
    orc.set_threads(os.cpu_count() or 1)
    grid, mins, maxs = (200, 200, 25), (0.0, 0.0, 0.0), (100.0, 100.0, 10.0)
    N = 200 * 200 * 25
    logK = pkg.fields.volume_logk(grid, mins, maxs, 20.0, 2.0, -9.0, 0)
    Qs = np.zeros(N)
    Qs[0] = 1e-4
    obs = np.random.default_rng(7919).choice(N, 100, replace=False)
    h_or, g_or = _oracle_steady_grad(orc, pkg, grid, mins, maxs, logK, [N - 1], Qs, obs)
    return dict(grid=grid, mins=mins, maxs=maxs, N=N, logK=logK, Qs=Qs, obs=obs, h=h_or, g=g_or)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_1m_cells_forward_adjoint_vs_oracle(gpu_lib, config_1m, precision):
    pkg, c = gpu_lib, config_1m
    P = pkg.GroundwaterProblem.regular3d(c["mins"], c["maxs"], c["grid"], [c["N"] - 1], reltol=1e-10,
                                          precision=precision)
    h, g = P.solve_grad_logk(c["logK"], np.zeros(c["N"]), c["Qs"], c["obs"])
    assert rel(h, c["h"]) < HEAD_TOL
    assert rel(g, c["g"]) < GRAD_TOL
    assert h[c["N"] - 1] == 0.0
    assert P.stats["iterations"] < 60


def test_1m_cells_batch_of_the_benchmark_vs_oracle(gpu_lib, config_1m):
    """Realization 0 inside a batch of 4 (the benchmark's form), mixed precision."""
    pkg, c = gpu_lib, config_1m
    N, B = c["N"], 4
    lks = [c["logK"]] + [pkg.fields.volume_logk(c["grid"], c["mins"], c["maxs"], 20.0, 2.0, -9.0, p)
                         for p in range(1, B)]
    rng = np.random.default_rng(3)
    obs = [c["obs"]] + [rng.choice(N, 100, replace=False) for _ in range(1, B)]
    Bt = pkg.GroundwaterBatch([c["grid"]] * B, [c["mins"]] * B, [c["maxs"]] * B, [[N - 1]] * B, reltol=1e-10,
                              precision="mixed")
    h, g = Bt.solve_grad_logk(np.concatenate(lks), np.zeros(B * N), np.tile(c["Qs"], B), obs)
    assert rel(h[:N], c["h"]) < HEAD_TOL
    assert rel(g[:N], c["g"]) < GRAD_TOL


def _uneven_members(pkg, seed=33):
    sizes = [(50, 50, 5), (100, 100, 10), (150, 150, 10), (200, 200, 20)]
    rng = np.random.default_rng(seed)
    out = []
    for p, g in enumerate(sizes):
        mx = tuple(0.5 * (n - 1) for n in g)
        N = int(np.prod(g))
        ell = rng.uniform(0.5, 2.0) * mx[0]
        sig = rng.uniform(0.5, 2.0)
        logK = pkg.fields.volume_logk(g, (0.0, 0.0, 0.0), mx, ell, sig, -9.0, 9100 + p)
        cells = rng.choice(N, 8, replace=False)
        ninj, ndir = 1 + rng.integers(4), 1 + rng.integers(4)
        Qs = np.zeros(N)
        Qs[cells[:ninj]] = rng.uniform(1e-5, 1e-3, ninj)
        out.append(dict(grid=g, mins=(0.0, 0.0, 0.0), maxs=mx, N=N, logK=logK, Qs=Qs,
                        dn=np.sort(cells[4:4 + ndir]), obs=rng.choice(N, 100, replace=False)))
    return out


def test_uneven_batch_with_the_largest_grid_vs_oracle(gpu_lib, orc):
    pkg = gpu_lib
    ms = _uneven_members(pkg)
    B = pkg.GroundwaterBatch([m["grid"] for m in ms], [m["mins"] for m in ms], [m["maxs"] for m in ms],
                             [m["dn"] for m in ms], reltol=1e-10, precision="mixed")
    cat = lambda k: np.concatenate([m[k] for m in ms])
    h, g = B.solve_grad_logk(cat("logK"), np.zeros(B.N), cat("Qs"), [m["obs"] for m in ms])
    for k, m in enumerate(ms):
        a, b = B.cell_offsets[k], B.cell_offsets[k + 1]
        h_or, g_or = _oracle_steady_grad(orc, pkg, m["grid"], m["mins"], m["maxs"], m["logK"], m["dn"], m["Qs"],
                                         m["obs"])
        assert rel(h[a:b], h_or) < HEAD_TOL, m["grid"]
        assert rel(g[a:b], g_or) < GRAD_TOL, m["grid"]
        assert np.array_equal(h[a:b][m["dn"]], np.zeros(len(m["dn"])))


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_transient_800k_cells_vs_oracle(gpu_lib, orc, precision):
    import os
    pkg = gpu_lib
    orc.set_threads(os.cpu_count() or 1)
    grid, mins, maxs = (200, 200, 20), (0.0, 0.0, 0.0), (100.0, 100.0, 10.0)
    nx, ny, nz = grid
    N = nx * ny * nz
    _, nb, aol, vol = pkg.regulargrid3d(mins, maxs, grid)
    lk = pkg.fields.volume_logk(grid, mins, maxs, 30.0, 1.5, -9.0, 777)
    rng = np.random.default_rng(55)
    dn = np.arange((nx - 1) * ny * nz, N)  # the x = max face (4000 cells)
    free = np.arange(0, (nx - 1) * ny * nz)
    Qs = np.zeros(N)
    Qs[rng.choice(free, 4, replace=False)] = 1e-3
    obs = rng.choice(free, 50, replace=False)
    Ss = np.full(N, 1e-5)
    dt, nsteps, ck = 3600.0, 12, 5
    dh = np.zeros(N)
    Ks = orc.logk_to_faces(nb, lk)
    O = orc.Problem(N, nb, aol, dn)
    st_or = O.transient(Ks, dh, Qs, Ss, vol, dt, nsteps, np.zeros(O.nfree), reltol=1e-14)
    dK_or, ddh_or, dQ_or, dh0_or = O.transient_adjoint(dh, obs, reltol=1e-14)
    P = pkg.GroundwaterProblem.regular3d(mins, maxs, grid, dn, reltol=1e-11, precision=precision)
    hT, states = P.transient_forward(Ks, dh, Qs, Ss, dt, nsteps, np.zeros(N), checkpoint_every=ck,
                                     return_states=True)
    isf, _, _ = pkg.getfreenodes(N, dn)
    assert rel(states[:, isf], st_or) < HEAD_TOL
    assert np.array_equal(states[:, ~isf], np.zeros((nsteps, len(dn))))
    dK, ddh, dQ, dh0 = P.transient_adjoint(obs)
    assert rel(dK, dK_or) < GRAD_TOL
    assert rel(ddh, ddh_or) < GRAD_TOL
    assert rel(dQ, dQ_or) < GRAD_TOL
    assert rel(dh0[isf], dh0_or) < GRAD_TOL
