"""Parity of the GPU steady solve and its adjoint with the oracle, through the C ABI.

Tolerances (the path is FP64 / mixed precision floating point):
  heads    relative L2 error <= 1e-8   (reltol 1e-10 or tighter)
  gradient relative L2 error <= 1e-6
"""
import os

import numpy as np
import pytest

from helpers import rel, steady_case

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
HEAD_TOL = 1e-8
GRAD_TOL = 1e-6


def _oracle_steady(orc, c, delta=None):
    P = orc.Problem(c["N"], c["nb"], c["aol"], c["dn"])
    h = P.steady(c["Ks"], c["dh"], c["Qs"], reltol=1e-14)
    out = {"h": h}
    if delta is not None:
        out["dKs"], out["ddh"], out["dQs"] = P.adjoint(c["dh"], delta, reltol=1e-14)
    return out


@pytest.mark.parametrize("name", ["steady_regular3d.npz", "steady_harmonic_multidir.npz"])
def test_golden_steady(gpu_lib, name):
    pkg = gpu_lib
    g = dict(np.load(os.path.join(GOLD, name)))
    N = int(np.prod(g["ns"]))
    h, back = pkg.rrule_groundwater_steadystate(g["Ks"], g["nb"], g["aol"], g["dn"], g["dh"], g["Qs"], reltol=1e-13)
    assert back.problem.structured
    assert rel(h, g["h"]) < HEAD_TOL
    assert np.array_equal(h[g["dn"]], g["dh"][g["dn"]])
    _, dKs, _, _, _, ddh, dQs = back(g["delta"])
    assert rel(dKs, g["dKs"]) < GRAD_TOL
    assert rel(ddh, g["ddh"]) < GRAD_TOL
    assert rel(dQs, g["dQs"]) < GRAD_TOL
    assert h.shape == (N,)


def test_golden_twophase_pressure(gpu_lib):
    """solvepressure and its rrule (src/twophase.jl:48-82) against the literal restatement."""
    pkg = gpu_lib
    g = dict(np.load(os.path.join(GOLD, "twophase_pressure.npz")))
    h0 = pkg.solvepressure(g["Ks"], g["nb"], g["aol"], g["dn"], g["dh"], g["Qs"])
    assert rel(h0, g["h"]) < HEAD_TOL
    h, back = pkg.rrule_solvepressure(g["Ks"], g["nb"], g["aol"], g["dn"], g["dh"], g["Qs"])
    assert rel(h, g["h"]) < HEAD_TOL
    assert np.array_equal(h[g["dn"]], g["dh"][g["dn"]])
    _, dKs, _, _, _, ddh, dQs = back(g["delta"])
    assert rel(dKs, g["dKs"]) < GRAD_TOL
    assert rel(ddh, g["ddh"]) < GRAD_TOL
    assert rel(dQs, g["dQs"]) < GRAD_TOL


def test_cholesky_solver_selector(gpu_lib):
    """linear_solver=cholesky_solver solves to the FP64 rounding floor (direct-solve accuracy),
    ends there with status OK (RuntimeWarnings are errors in the GPU tests) and needs only a
    few rounds to get there."""
    pkg = gpu_lib
    g = dict(np.load(os.path.join(GOLD, "steady_harmonic_multidir.npz")))
    h = pkg.groundwater_steadystate(g["Ks"], g["nb"], g["aol"], g["dn"], g["dh"], g["Qs"],
                                    linear_solver=pkg.cholesky_solver)
    assert rel(h, g["h"]) < 1e-12
    h1, back = pkg.rrule_groundwater_steadystate(g["Ks"], g["nb"], g["aol"], g["dn"], g["dh"], g["Qs"],
                                                 linear_solver=pkg.cholesky_solver)
    st = back.problem.stats
    assert rel(h1, g["h"]) < 1e-12
    assert st["relres"] < 1e-11 and st["outer"] <= 6 and st["iterations"] <= 120, st
    h2 = pkg.groundwater_steadystate(g["Ks"], g["nb"], g["aol"], g["dn"], g["dh"], g["Qs"],
                                     linear_solver=pkg.amg_solver, reltol=1e-10)
    assert rel(h2, g["h"]) < HEAD_TOL
    with pytest.raises(ValueError):
        pkg.groundwater_steadystate(g["Ks"], g["nb"], g["aol"], g["dn"], g["dh"], g["Qs"], linear_solver="lu")


@pytest.mark.parametrize("ns", [(12, 10, 6), (9, 7, 5), (16, 1, 9), (33, 17, 1), (5, 5, 5), (3, 2, 2), (64, 3, 2)])
def test_steady_shapes_vs_oracle(gpu_lib, orc, ns):
    c = steady_case(gpu_lib, ns, sigma=1.5, seed=sum(ns), ndir=2, nq=3)
    rng = np.random.default_rng(7)
    delta = rng.standard_normal(c["N"])
    ref = _oracle_steady(orc, c, delta)
    P = gpu_lib.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"], reltol=1e-12)
    assert P.structured
    h = P.forward(c["Ks"], c["dh"], c["Qs"])
    assert rel(h, ref["h"]) < HEAD_TOL
    dKs, ddh, dQs = P.adjoint(delta)
    assert rel(dKs, ref["dKs"]) < GRAD_TOL
    assert rel(ddh, ref["ddh"]) < GRAD_TOL
    assert rel(dQs, ref["dQs"]) < GRAD_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("mean", ["geometric", "harmonic"])
def test_logk_path_vs_oracle(gpu_lib, orc, precision, mean):
    c = steady_case(gpu_lib, (24, 20, 8), sigma=2.0, seed=4, ndir=1, mean=mean)
    kind = 0 if mean == "geometric" else 1
    rng = np.random.default_rng(3)
    obs = rng.choice(c["N"], 30, replace=False)
    P = gpu_lib.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"], reltol=1e-11, precision=precision)
    h, g = P.solve_grad_logk(c["logK"], c["dh"], c["Qs"], obs, mean=mean)
    O = orc.Problem(c["N"], c["nb"], c["aol"], c["dn"])
    Ks = orc.logk_to_faces(c["nb"], c["logK"], kind)
    h_or = O.steady(Ks, c["dh"], c["Qs"], reltol=1e-14)
    delta = np.zeros(c["N"])
    np.add.at(delta, obs, 2 * h_or[obs])
    dKs, _, _ = O.adjoint(c["dh"], delta, reltol=1e-14)
    g_or = orc.logk_to_faces_vjp(c["nb"], c["logK"], dKs, kind)
    assert rel(h, h_or) < HEAD_TOL
    assert rel(g, g_or) < GRAD_TOL


def test_logk_to_faces_and_vjp(gpu_lib, orc):
    c = steady_case(gpu_lib, (10, 9, 7), seed=12)
    P = gpu_lib.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"])
    rng = np.random.default_rng(2)
    dK = rng.standard_normal(len(c["nb"]))
    for kind, mean in ((0, "geometric"), (1, "harmonic")):
        K = P.logk_to_faces(c["logK"], mean)
        assert rel(K, orc.logk_to_faces(c["nb"], c["logK"], kind)) < 1e-14
        g = P.logk_to_faces_vjp(c["logK"], dK, mean)
        assert rel(g, orc.logk_to_faces_vjp(c["nb"], c["logK"], dK, kind)) < 1e-13


def test_forward_logk_matches_forward_ks(gpu_lib):
    c = steady_case(gpu_lib, (20, 18, 6), seed=21, ndir=3)
    P = gpu_lib.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"], reltol=1e-12)
    h1 = P.forward(c["Ks"], c["dh"], c["Qs"])
    h2 = P.forward_logk(c["logK"], c["dh"], c["Qs"])
    assert rel(h1, h2) < 1e-10
    delta = np.random.default_rng(0).standard_normal(c["N"])
    g2, ddh2, dQ2 = P.adjoint_logk(delta)
    P.forward(c["Ks"], c["dh"], c["Qs"])
    dK, ddh1, dQ1 = P.adjoint(delta)
    g1 = P.logk_to_faces_vjp(c["logK"], dK)
    assert rel(g1, g2) < 1e-9 and rel(ddh1, ddh2) < 1e-9 and rel(dQ1, dQ2) < 1e-9


def test_config1_parity(gpu_lib, orc):
    """100x100x10 over 50x50x5 m, layered Matern logK (ell 50 m, sigma 1, mean -9),
    Qs[0] = 1e-4, Dirichlet h = 0 at the last cell, reltol 1e-10."""
    pkg = gpu_lib
    c = steady_case(pkg, (100, 100, 10), mins=(0, 0, 0), maxs=(50, 50, 5), ell=50.0, sigma=1.0, seed=0, layered=True)
    P = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"])
    h = P.forward(c["Ks"], c["dh"], c["Qs"])
    ref = _oracle_steady(orc, c)
    assert rel(h, ref["h"]) < HEAD_TOL
    assert P.stats["iterations"] < 60


def test_config2_gradient_fd(gpu_lib, orc):
    """Forward + adjoint of J = sum h[obs]^2 over 100 seeded cells; gradient d/dlogK checked
    against the oracle and by central differences (step 1e-6) on 20 seeded cells."""
    pkg = gpu_lib
    c = steady_case(pkg, (100, 100, 10), mins=(0, 0, 0), maxs=(50, 50, 5), ell=50.0, sigma=1.0, seed=0, layered=True)
    rng = np.random.default_rng(2)
    obs = rng.choice(c["N"], 100, replace=False)
    P = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"], reltol=1e-12)
    h, g = P.solve_grad_logk(c["logK"], c["dh"], c["Qs"], obs)
    O = orc.Problem(c["N"], c["nb"], c["aol"], c["dn"])
    h_or = O.steady(orc.logk_to_faces(c["nb"], c["logK"]), c["dh"], c["Qs"], reltol=1e-14)
    delta = np.zeros(c["N"])
    delta[obs] = 2 * h_or[obs]
    dKs, _, _ = O.adjoint(c["dh"], delta, reltol=1e-14)
    g_or = orc.logk_to_faces_vjp(c["nb"], c["logK"], dKs)
    assert rel(h, h_or) < HEAD_TOL
    assert rel(g, g_or) < GRAD_TOL
    Q = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"], reltol=1e-13)

    def J(lk):
        hh = Q.forward_logk(lk, c["dh"], c["Qs"])
        return float(np.sum(hh[obs] ** 2))

    cells = rng.choice(c["N"], 20, replace=False)
    for i in cells:
        lp, lm = c["logK"].copy(), c["logK"].copy()
        lp[i] += 1e-6
        lm[i] -= 1e-6
        fd = (J(lp) - J(lm)) / 2e-6
        assert abs(fd - g[i]) <= 1e-4 * abs(fd) + 1e-6 * np.abs(g).max()


def test_mixed_precision_matches_fp64(gpu_lib, orc):
    c = steady_case(gpu_lib, (60, 50, 20), sigma=2.0, seed=8, ell=10.0)
    ref = _oracle_steady(orc, c)
    P = gpu_lib.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"], precision="mixed")
    h = P.forward(c["Ks"], c["dh"], c["Qs"])
    st = P.stats
    assert rel(h, ref["h"]) < HEAD_TOL
    assert st["outer"] >= 1 and st["relres"] <= 1e-9


def test_torch_device_buffers(gpu_lib, orc):
    import torch
    c = steady_case(gpu_lib, (16, 12, 8), seed=31, ndir=2)
    P = gpu_lib.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"], reltol=1e-12)
    dev = torch.device("cuda", 0)
    Ks = torch.tensor(c["Ks"], device=dev)
    h = P.forward(Ks, torch.tensor(c["dh"], device=dev), torch.tensor(c["Qs"], device=dev))
    assert isinstance(h, torch.Tensor) and h.is_cuda
    ref = _oracle_steady(orc, c)
    assert rel(h.cpu().numpy(), ref["h"]) < HEAD_TOL


def test_apply_operator_matches_oracle_matrix(gpu_lib, orc):
    c = steady_case(gpu_lib, (7, 6, 5), seed=2, ndir=3)
    P = gpu_lib.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"])
    P.forward(c["Ks"], c["dh"], c["Qs"])
    x = np.random.default_rng(0).standard_normal(c["N"])
    y = P.apply(x)
    O = orc.Problem(c["N"], c["nb"], c["aol"], c["dn"])
    A, b = O.assemble(c["Ks"], c["dh"], c["Qs"])
    isf = np.ones(c["N"], bool)
    isf[c["dn"]] = False
    # free rows: A_ff x_f plus the Dirichlet-face part folded into the diagonal; Dirichlet rows: identity
    assert rel(y[isf], A @ x[isf]) < 1e-13
    assert np.allclose(y[~isf], x[~isf])


def test_errors_are_reported(gpu_lib):
    pkg = gpu_lib
    c = steady_case(pkg, (5, 4, 3), seed=1)
    P = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"])
    with pytest.raises(pkg.DPFError) as e:
        P.adjoint(np.zeros(c["N"]))
    assert e.value.code == 7  # DPF_STATE: adjoint before forward
    with pytest.raises(pkg.DPFError) as e:
        pkg.GroundwaterProblem(c["nb"], c["aol"], [c["N"] + 5], N=c["N"])
    assert e.value.code == 1
    # no Dirichlet cell: the operator is singular and the coarsest factor reports it
    Q = pkg.GroundwaterProblem(c["nb"], c["aol"], [], N=c["N"])
    with pytest.raises(pkg.DPFError):
        Q.forward(c["Ks"], c["dh"], c["Qs"])
    # iteration cap: warns and returns the last iterate
    R = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"], maxiter=1, reltol=1e-15)
    with pytest.warns(RuntimeWarning):
        R.forward(c["Ks"], c["dh"], c["Qs"])


def test_nonfinite_input_reported(gpu_lib):
    pkg = gpu_lib
    c = steady_case(pkg, (6, 5, 4), seed=1)
    P = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"])
    Ks = c["Ks"].copy()
    Ks[3] = np.nan
    with pytest.raises(pkg.DPFError):
        P.forward(Ks, c["dh"], c["Qs"])
    # the handle stays usable
    h = P.forward(c["Ks"], c["dh"], c["Qs"])
    assert np.all(np.isfinite(h))
