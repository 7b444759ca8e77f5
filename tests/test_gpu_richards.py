"""The GPU Richards solver (Picard on the CG + AMG operator, adjoint fixed point) against the
oracle's Newton solve and rrule tangents (oracle/richards_oracle.py)."""
import numpy as np
import pytest

import richards_oracle as ro
from helpers import rel
from richards_cases import oracle_args, richards_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("ns,psi_top", [((8, 6, 4), -4.0), ((10, 9, 5), -1.5)])
def test_richards_vs_oracle(gpu_lib, precision, ns, psi_top):
    pkg = gpu_lib
    c = richards_case(pkg, ns=ns, psi_top=psi_top, seed=11)
    psi_or = ro.steady(c["psi0"], c["Ks"], c["nb"], c["aol"], c["dn"], c["dpsi"], c["z"], c["alphas"], c["Ns"],
                       c["Qs"], tol=1e-14)
    w = np.random.default_rng(5).standard_normal(c["N"])
    g_or = ro.pullback(psi_or, w, *oracle_args(c))
    psi, pb = pkg.rrule_richards_steadystate(c["psi0"], c["Ks"], c["nb"], c["aol"], c["dn"], c["dpsi"], c["coords"],
                                             c["alphas"], c["Ns"], c["Qs"], tol=1e-12, precision=precision,
                                             reltol=1e-12)
    assert rel(psi, psi_or) < 1e-9
    assert np.array_equal(psi[c["dn"]], c["dpsi"][c["dn"]])
    t = pb(w)
    assert t[0] is pkg.NoTangent and np.all(t[1] == 0)
    for got, want, name in ((t[2], g_or[0], "dKs"), (t[6], g_or[1], "ddirichletpsis"), (t[8], g_or[2], "dalphas"),
                            (t[9], g_or[3], "dNs"), (t[10], g_or[4], "dQs")):
        assert rel(got, want) < 1e-7, name
    st = pb.problem.richards_stats
    assert st["iterations"] > 1 and st["adjoint_iterations"] >= 1 and st["relres"] < 1e-12


def test_reference_example_setup(gpu_lib):
    """The reference example's configuration (examples/richards_steadystate_3d/inputdeck.jl: 30x30x3
    nodes over 50x50x1 m, alpha 0.375, N 1.25, Q = 1e-6 at the first cell, psi = 0 at the last) with
    a seeded lognormal K: GPU and oracle agree."""
    pkg = gpu_lib
    coords, nb, aol, _ = pkg.regulargrid3d((0.0, 0.0, 0.0), (50.0, 50.0, 1.0), (30, 30, 3))
    N = coords.shape[1]
    logK = -9.0 + np.random.default_rng(0).standard_normal(N)
    Ks = np.exp(0.5 * (logK[nb[:, 0]] + logK[nb[:, 1]]))
    Qs = np.zeros(N); Qs[0] = 1e-6
    dn = np.array([N - 1]); dpsi = np.zeros(N)
    alphas = np.full(len(nb), 0.375); Ns = np.full(len(nb), 1.25)
    psi = pkg.richards_steadystate(np.zeros(N), Ks, nb, aol, dn, dpsi, coords, alphas, Ns, Qs, tol=1e-12,
                                   reltol=1e-12)
    psi_or = ro.steady(np.zeros(N), Ks, nb, aol, dn, dpsi, coords[2], alphas, Ns, Qs, tol=1e-14)
    assert rel(psi, psi_or) < 1e-9


def test_structured_handle_is_refused(gpu_lib):
    pkg = gpu_lib
    c = richards_case(pkg, ns=(4, 4, 3))
    P = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"])
    assert P.structured
    with pytest.raises(pkg.DPFError) as e:
        P.richards_steady(c["psi0"], c["Ks"], c["dpsi"], c["z"], c["alphas"], c["Ns"], c["Qs"])
    assert e.value.code == pkg._lib.DPF_UNSUPPORTED


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_transient_richards_vs_oracle(gpu_lib, precision):
    from richards_cases import transient_case
    pkg = gpu_lib
    c = transient_case(pkg, ns=(8, 6, 4))
    st_or = ro.transient(c["psi0"], c["Ks"], c["nb"], c["aol"], c["dn"], c["dpsi"], c["z"], c["alphas"], c["Ns"],
                         c["Qs"], c["Ss"], c["vol"], c["dt"], c["nsteps"], tol=1e-14)
    g_or = ro.transient_pullback(st_or, c["obs"], c["w"], c["gT"], c["Ks"], c["nb"], c["aol"], c["dn"], c["z"],
                                 c["alphas"], c["Ns"], c["Qs"], c["Ss"], c["vol"], c["dt"])
    P = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"], volumes=c["vol"], general=True,
                               precision=precision, reltol=1e-12)
    psiT, st = P.richards_transient_forward(c["psi0"], c["Ks"], c["dpsi"], c["z"], c["alphas"], c["Ns"], c["Qs"],
                                            c["Ss"], c["dt"], c["nsteps"], tol=1e-12, return_states=True)
    assert rel(st, st_or) < 1e-9 and rel(psiT, st_or[-1]) < 1e-9
    g = P.richards_transient_adjoint(c["obs"], c["w"], c["gT"], tol=1e-11)
    for got, want, name in zip(g, g_or, ("dKs", "ddirichletpsis", "dalphas", "dNs", "dQs", "dpsi0")):
        assert rel(got, want) < 1e-7, name


def test_thiem_richards_matches_groundwater(gpu_lib):
    """The reference's Richards-against-groundwater check (test/thiem.jl:72-98) on the GPU: the
    saturated Richards solve and the groundwater solve of the Thiem setup agree to the solvers'
    tolerance (the reference asks 1e-4), and both give the Thiem drawdowns within 1e-1."""
    from test_oracle_richards import _thiem_setup
    pkg = gpu_lib
    t = _thiem_setup(pkg)
    h_gw = pkg.groundwater_steadystate(t["Ks"], t["nb"], t["aol"], t["dn"], t["dh"], t["Qs"], reltol=1e-12)
    psi = pkg.richards_steadystate(np.full(t["N"], t["steadyhead"]), t["Ks"], t["nb"], t["aol"], t["dn"], t["dh"],
                                   t["coords3"], t["alphas"], t["Ns"], t["Qs"], tol=1e-12, reltol=1e-12)
    dd_gw = t["steadyhead"] - h_gw[t["good"]]
    dd_r = t["steadyhead"] - psi[t["good"]]
    assert np.linalg.norm(dd_r - dd_gw) <= 1e-8 * np.linalg.norm(dd_gw)
    assert np.linalg.norm(t["thiem"] - dd_r) <= 1e-1 * max(np.linalg.norm(t["thiem"]), np.linalg.norm(dd_r))
