"""The direct solver (options solver="cholesky", the reference's cholesky_solver,
src/groundwater.jl:56-60): a banded Cholesky factorisation of the FP64 operator on the GPU,
checked against the oracle (its CG solved to 1e-14) on regular grids, unstructured meshes,
batches, adjoints and transient runs; a band too wide for the device falls back to the CG
solve. Tolerances: heads 1e-11, tangents 1e-9 (a direct solve of the 48-bit-rounded operator of
the mixed handles; the oracle's own CG stops at 1e-14)."""
import numpy as np
import pytest

from helpers import rel, steady_case
from test_gpu_general import random_mesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ns", [(60, 40, 1), (12, 10, 8), (1, 30, 20), (7, 1, 1), (40, 3, 5)])
def test_regular_grid_vs_oracle(gpu_lib, orc, ns):
    pkg = gpu_lib
    c = steady_case(pkg, ns, sigma=1.5, seed=sum(ns), ndir=2, nq=3)
    rng = np.random.default_rng(5)
    delta = rng.standard_normal(c["N"])
    O = orc.Problem(c["N"], c["nb"], c["aol"], c["dn"])
    h_or = O.steady(c["Ks"], c["dh"], c["Qs"], reltol=1e-14)
    dKs_or, ddh_or, dQs_or = O.adjoint(c["dh"], delta, reltol=1e-14)
    h, back = pkg.rrule_groundwater_steadystate(c["Ks"], c["nb"], c["aol"], c["dn"], c["dh"], c["Qs"],
                                                linear_solver=pkg.cholesky_solver)
    assert back.problem.structured
    st = back.problem.stats
    assert st["iterations"] == 0 and st["outer"] == 0 and st["relres"] < 1e-12, st
    assert rel(h, h_or) < 1e-11
    assert np.array_equal(h[c["dn"]], c["dh"][c["dn"]])
    _, dKs, _, _, _, ddh, dQs = back(delta)
    assert back.problem.stats["iterations"] == 0
    assert rel(dKs, dKs_or) < 1e-9 and rel(ddh, ddh_or) < 1e-9 and rel(dQs, dQs_or) < 1e-9


@pytest.mark.parametrize("n,ndir", [(500, 1), (3000, 4)])
def test_unstructured_mesh_vs_oracle(gpu_lib, orc, n, ndir):
    """Reverse Cuthill-McKee band of a k-nearest-neighbour mesh (duplicated couplings of a pair of
    cells are summed into one band entry)."""
    pkg = gpu_lib
    pts, nb, aol = random_mesh(n, seed=n + 7)
    nb = np.concatenate([nb, nb[:5]])  # five faces listed twice
    aol = np.concatenate([aol, aol[:5]])
    rng = np.random.default_rng(n)
    logK = -9.0 + rng.standard_normal(n)
    Ks = np.exp(0.5 * (logK[nb[:, 0]] + logK[nb[:, 1]]))
    dn = rng.choice(n, ndir, replace=False)
    dh = np.zeros(n)
    dh[dn] = rng.uniform(0, 1, ndir)
    Qs = np.zeros(n)
    Qs[rng.choice(np.setdiff1d(np.arange(n), dn), 3, replace=False)] = [1e-4, 5e-5, -2e-5]
    delta = rng.standard_normal(n)
    P = pkg.GroundwaterProblem(nb, aol, dn, N=n, solver="cholesky", precision="fp64")
    assert not P.structured
    h = P.forward(Ks, dh, Qs)
    assert P.stats["iterations"] == 0 and P.stats["relres"] < 1e-12, P.stats
    dKs, ddh, dQs = P.adjoint(delta)
    O = orc.Problem(n, nb, aol, dn)
    h_or = O.steady(Ks, dh, Qs, reltol=1e-14)
    dKs_or, ddh_or, dQs_or = O.adjoint(dh, delta, reltol=1e-14)
    assert rel(h, h_or) < 1e-11
    assert rel(dKs, dKs_or) < 1e-9 and rel(ddh, ddh_or) < 1e-9 and rel(dQs, dQs_or) < 1e-9


def test_batch_solve_grad_logk(gpu_lib, orc):
    """A batch of regular grids: one band over all problems (each in its own rows)."""
    pkg = gpu_lib
    grids = [(20, 16, 1), (9, 9, 9), (30, 4, 6)]
    cases = [steady_case(pkg, g, sigma=1.0, seed=41 + k, ndir=1, nq=2) for k, g in enumerate(grids)]
    B = pkg.GroundwaterBatch(grids, [c["mins"] for c in cases], [c["maxs"] for c in cases],
                             [c["dn"] for c in cases], solver="cholesky", precision="fp64")
    cat = lambda k: np.concatenate([c[k] for c in cases])
    obs = [np.arange(0, c["N"], 7) for c in cases]
    h, g = B.solve_grad_logk(cat("logK"), cat("dh"), cat("Qs"), obs)
    h, g = np.asarray(h), np.asarray(g)
    assert B.stats["iterations"] == 0
    off = B.cell_offsets
    for k, c in enumerate(cases):
        O = orc.Problem(c["N"], c["nb"], c["aol"], c["dn"])
        ho = O.steady(orc.logk_to_faces(c["nb"], c["logK"]), c["dh"], c["Qs"], reltol=1e-14)
        d = np.zeros(c["N"])
        np.add.at(d, obs[k], 2 * ho[obs[k]])
        dK, _, _ = O.adjoint(c["dh"], d, reltol=1e-14)
        assert rel(h[off[k]:off[k + 1]], ho) < 1e-11, k
        assert rel(g[off[k]:off[k + 1]], orc.logk_to_faces_vjp(c["nb"], c["logK"], dK)) < 1e-9, k


def test_transient_direct_matches_iterative(gpu_lib):
    """Backward Euler with the factor of (D / dt + A), computed once per run, against the CG run."""
    pkg = gpu_lib
    c = steady_case(pkg, (24, 20, 1), sigma=1.5, seed=3, ndir=1, nq=3)
    N = c["N"]
    dn = np.arange(N - 20, N)
    dh = np.zeros(N)
    Ss = np.full(N, 1e-5)
    obs = np.arange(0, N - 20, 11)
    out = []
    for solver in ("cholesky", "cg"):
        P = pkg.GroundwaterProblem(c["nb"], c["aol"], dn, N=N, volumes=c["vol"], reltol=1e-13, precision="fp64",
                                   solver=solver)
        hT = P.transient_forward(c["Ks"], dh, c["Qs"], Ss, 3600.0, 10, np.zeros(N), checkpoint_every=5)
        out.append((np.asarray(hT),) + tuple(np.asarray(v) for v in P.transient_adjoint(obs)))
    for a, b in zip(out[0], out[1]):
        assert rel(a, b) < 1e-9


def test_wide_band_falls_back_to_cg(gpu_lib):
    """200 x 200 x 25 cells: a band of 5000 and 2.5e13 multiply-adds, above the direct solver's
    limit, so the solve runs the CG (to the floor, through the cholesky selector) instead."""
    pkg = gpu_lib
    ns = (200, 200, 25)
    c = steady_case(pkg, ns, sigma=1.0, seed=2, ndir=1, nq=1)
    h = pkg.groundwater_steadystate(c["Ks"], c["nb"], c["aol"], c["dn"], c["dh"], c["Qs"],
                                    linear_solver=pkg.cholesky_solver)
    P = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"], solver="cholesky", precision="mixed",
                               reltol=1e-10)
    h2 = P.forward(c["Ks"], c["dh"], c["Qs"])
    assert P.stats["iterations"] > 0
    assert rel(h2, h) < 1e-8
