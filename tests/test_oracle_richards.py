"""The Richards oracle (a restatement of DPFEHM src/richards.jl) pinned by finite differences:
kr's derivatives, the Jacobian of the residual, the Newton solve and the rrule's tangents."""
import numpy as np
import pytest

import richards_oracle as ro
from richards_cases import oracle_args, richards_case


def test_kr_derivatives_match_finite_differences():
    rng = np.random.default_rng(1)
    psi = -rng.uniform(0.05, 3.0, 50)
    al = rng.uniform(0.2, 1.5, 50)
    n = rng.uniform(1.1, 2.5, 50)
    v, dp, da, dn = ro.kr(psi, al, n)
    h = 1e-6
    for d, args in ((dp, lambda e: (psi + e, al, n)), (da, lambda e: (psi, al + e, n)), (dn, lambda e: (psi, al, n + e))):
        fd = (ro.kr(*args(h))[0] - ro.kr(*args(-h))[0]) / (2 * h)
        assert np.allclose(d, fd, rtol=1e-6, atol=1e-10)
    # saturated: kr = 1, no derivatives
    v, dp, da, dn = ro.kr(np.array([0.0, 1.0]), 0.5, 1.5)
    assert np.all(v == 1) and np.all(dp == 0) and np.all(da == 0) and np.all(dn == 0)


def test_jacobian_matches_finite_differences(pkg):
    c = richards_case(pkg, ns=(5, 4, 3))
    psi = np.where(np.isin(np.arange(c["N"]), c["dn"]), c["dpsi"], -0.3 - 0.2 * np.random.default_rng(2).uniform(size=c["N"]))
    args = oracle_args(c)
    J = ro.jacobian(psi, *args).toarray()
    free = np.setdiff1d(np.arange(c["N"]), c["dn"])
    h = 1e-7
    for col, k in enumerate(free[:12]):
        e = np.zeros(c["N"]); e[k] = h
        fd = (ro.residual(psi + e, *args) - ro.residual(psi - e, *args)) / (2 * h)
        assert np.allclose(J[:, col], fd, rtol=1e-5, atol=1e-14 * np.abs(fd).max() + 1e-20)


def test_newton_solve_reaches_the_root(pkg):
    c = richards_case(pkg)
    psi = ro.steady(c["psi0"], c["Ks"], c["nb"], c["aol"], c["dn"], c["dpsi"], c["z"], c["alphas"], c["Ns"], c["Qs"])
    R = ro.residual(psi, *oracle_args(c))
    assert np.linalg.norm(R) <= 1e-12 * np.linalg.norm(c["Qs"])
    assert np.all(psi[c["dn"]] == c["dpsi"][c["dn"]])
    assert (psi < 0).sum() > c["N"] // 4          # the unsaturated regime is exercised


@pytest.mark.parametrize("which", ["Ks", "alphas", "Ns", "Qs", "dpsi"])
def test_pullback_matches_finite_differences(pkg, which):
    c = richards_case(pkg, ns=(5, 4, 4), seed=3)
    rng = np.random.default_rng(7)
    w = rng.standard_normal(c["N"])

    def J(cc):
        psi = ro.steady(cc["psi0"], cc["Ks"], cc["nb"], cc["aol"], cc["dn"], cc["dpsi"], cc["z"], cc["alphas"],
                        cc["Ns"], cc["Qs"], tol=1e-14)
        return float(w @ psi), psi

    _, psi = J(c)
    dK, ddp, dal, dN, dQ = ro.pullback(psi, w, *oracle_args(c))
    grad = {"Ks": dK, "alphas": dal, "Ns": dN, "Qs": dQ, "dpsi": ddp}[which]
    d = rng.standard_normal(len(c[which]))
    if which == "dpsi":
        d = np.where(np.isin(np.arange(c["N"]), c["dn"]), d, 0.0)
    scale = {"Ks": 1e-3 * c["Ks"], "alphas": 1e-4 * c["alphas"], "Ns": 1e-5, "Qs": 1e-9, "dpsi": 1e-5}[which]
    step = d * scale
    cp, cm = dict(c), dict(c)
    cp[which] = c[which] + step
    cm[which] = c[which] - step
    fd = (J(cp)[0] - J(cm)[0]) / 2
    assert fd == pytest.approx(float(grad @ step), rel=2e-4)


@pytest.mark.parametrize("which", ["Ks", "alphas", "Qs", "dpsi", "psi0"])
def test_transient_pullback_matches_finite_differences(pkg, which):
    from richards_cases import transient_case
    c = transient_case(pkg)

    def J(cc):
        st = ro.transient(cc["psi0"], cc["Ks"], cc["nb"], cc["aol"], cc["dn"], cc["dpsi"], cc["z"], cc["alphas"],
                          cc["Ns"], cc["Qs"], cc["Ss"], cc["vol"], cc["dt"], cc["nsteps"], tol=1e-14)
        j = sum(float(np.sum(c["w"] * s[c["obs"]] ** 2)) for s in st) + float(c["gT"] @ st[-1])
        return j, st

    _, st = J(c)
    g = ro.transient_pullback(st, c["obs"], c["w"], c["gT"], c["Ks"], c["nb"], c["aol"], c["dn"], c["z"], c["alphas"],
                              c["Ns"], c["Qs"], c["Ss"], c["vol"], c["dt"])
    grad = {"Ks": g[0], "dpsi": g[1], "alphas": g[2], "Qs": g[4], "psi0": g[5]}[which]
    rng = np.random.default_rng(9)
    d = rng.standard_normal(len(c[which]))
    isd = np.isin(np.arange(c["N"]), c["dn"])
    if which == "dpsi":
        d = np.where(isd, d, 0.0)
    if which == "psi0":
        d = np.where(isd, 0.0, d)
    scale = {"Ks": 1e-3 * c["Ks"], "alphas": 1e-4 * c["alphas"], "Qs": 1e-9, "dpsi": 1e-5, "psi0": 1e-5}[which]
    step = d * scale
    cp, cm = dict(c), dict(c)
    cp[which] = c[which] + step
    cm[which] = c[which] - step
    if which == "dpsi":   # the initial state carries the Dirichlet values too
        cp["psi0"] = np.where(isd, cp["dpsi"], c["psi0"])
        cm["psi0"] = np.where(isd, cm["dpsi"], c["psi0"])
    fd = (J(cp)[0] - J(cm)[0]) / 2
    assert fd == pytest.approx(float(grad @ step), rel=2e-4)


def _thiem_setup(pkg):
    """The reference's Thiem configuration (test/thiem.jl:27-47): a 101 x 101 grid, a sink at the
    centre, head 1000 m on the ring r >= 50 m (saturated everywhere, so kr = 1)."""
    steadyhead, sidelength, thickness, n = 1e3, 50.0, 10.0, 101
    coords, nb, aol, _ = pkg.regulargrid2d([-sidelength, -sidelength], [sidelength, sidelength], [n, n], thickness)
    N = coords.shape[1]
    k, Q = 1e-5, 1e-3
    Qs = np.zeros(N)
    Qs[n * ((n + 1) // 2 - 1) + (n + 1) // 2 - 1] = -Q
    r = np.sqrt(coords[0] ** 2 + coords[1] ** 2)
    dn = np.nonzero(r >= sidelength)[0]
    dh = np.zeros(N)
    dh[dn] = steadyhead
    coords3 = np.vstack([coords, np.zeros(N)])        # z = 0, as the reference's vcat(coords, zeros)
    good = np.nonzero((coords[1] == 0) & (coords[0] > 0.1))[0]
    thiem = Q * np.log(sidelength / coords[0, good]) / (2 * np.pi * thickness * k)
    return dict(N=N, nb=nb, aol=aol, Ks=np.full(len(nb), k), Qs=Qs, dn=dn, dh=dh, coords3=coords3, good=good,
                thiem=thiem, steadyhead=steadyhead, alphas=np.full(len(nb), 0.5), Ns=np.full(len(nb), 1.25))


def test_richards_thiem_matches_groundwater(orc, pkg):
    """The reference's Richards-against-groundwater check (test/thiem.jl:72-98): the saturated
    Richards solution on the Thiem setup gives the groundwater drawdowns (rtol 1e-4 there; the
    equations coincide when kr = 1, so here to the solvers' tolerance) and the Thiem drawdowns
    (rtol 1e-1)."""
    t = _thiem_setup(pkg)
    h_gw = orc.Problem(t["N"], t["nb"], t["aol"], t["dn"]).steady(t["Ks"], t["dh"], t["Qs"], reltol=1e-13)
    psi = ro.steady(np.full(t["N"], t["steadyhead"]), t["Ks"], t["nb"], t["aol"], t["dn"], t["dh"], t["coords3"][2],
                    t["alphas"], t["Ns"], t["Qs"], tol=1e-13)
    dd_gw = t["steadyhead"] - h_gw[t["good"]]
    dd_r = t["steadyhead"] - psi[t["good"]]
    assert np.linalg.norm(dd_r - dd_gw) <= 1e-8 * np.linalg.norm(dd_gw)
    assert np.linalg.norm(t["thiem"] - dd_r) <= 1e-1 * max(np.linalg.norm(t["thiem"]), np.linalg.norm(dd_r))
