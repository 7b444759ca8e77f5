"""The CPU oracle, pinned against the golden vectors and the reference's analytic checks (no GPU)."""
import os

import numpy as np
import pytest
import scipy.sparse.linalg as spl

from helpers import rel, steady_case

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return dict(np.load(os.path.join(GOLD, name)))


@pytest.mark.parametrize("name", ["steady_regular3d.npz", "steady_harmonic_multidir.npz", "steady_general_graph.npz"])
def test_oracle_matches_golden_steady(orc, name):
    g = _load(name)
    N = int(g["N"]) if "N" in g else int(np.prod(g["ns"]))
    P = orc.Problem(N, g["nb"], g["aol"], g["dn"])
    h = P.steady(g["Ks"], g["dh"], g["Qs"], reltol=1e-15)
    assert rel(h, g["h"]) < 1e-12
    assert np.array_equal(h[g["dn"]], g["dh"][g["dn"]])
    dKs, ddh, dQs = P.adjoint(g["dh"], g["delta"], reltol=1e-15)
    assert rel(dKs, g["dKs"]) < 1e-10
    assert rel(ddh, g["ddh"]) < 1e-10
    assert rel(dQs, g["dQs"]) < 1e-10


def test_oracle_matches_golden_twophase_pressure(orc):
    """The two-phase pressure system (transmissibility 2 aol K, src/twophase.jl:25) is the steady
    groundwater system with areas-over-lengths doubled; the oracle reproduces its golden case."""
    g = _load("twophase_pressure.npz")
    N = int(np.prod(g["ns"]))
    P = orc.Problem(N, g["nb"], 2.0 * g["aol"], g["dn"])
    h = P.steady(g["Ks"], g["dh"], g["Qs"], reltol=1e-15)
    assert rel(h, g["h"]) < 1e-12
    dKs, ddh, dQs = P.adjoint(g["dh"], g["delta"], reltol=1e-15)
    assert rel(dKs, g["dKs"]) < 1e-10
    assert rel(ddh, g["ddh"]) < 1e-10
    assert rel(dQs, g["dQs"]) < 1e-10


def test_oracle_matches_golden_transient(orc):
    g = _load("transient_regular3d.npz")
    N = int(np.prod(g["ns"]))
    P = orc.Problem(N, g["nb"], g["aol"], g["dn"])
    states = P.transient(g["Ks"], g["dh"], g["Qs"], g["Ss"], g["V"], float(g["dt"]), int(g["nsteps"]), g["h0"],
                         reltol=1e-15)
    assert rel(states, g["states"]) < 1e-11
    dKs, ddh, dQs, dh0 = P.transient_adjoint(g["dh"], g["obs"], reltol=1e-15)
    assert rel(dKs, g["dKs"]) < 1e-9
    assert rel(ddh, g["ddh"]) < 1e-9
    assert rel(dQs, g["dQs"]) < 1e-9
    assert rel(dh0, g["dh0"]) < 1e-9


def test_oracle_vs_direct_solver(orc, pkg):
    c = steady_case(pkg, (14, 11, 7), sigma=2.0, seed=3, ndir=4, nq=3)
    P = orc.Problem(c["N"], c["nb"], c["aol"], c["dn"])
    h = P.steady(c["Ks"], c["dh"], c["Qs"])
    A, b = P.assemble(c["Ks"], c["dh"], c["Qs"])
    x = spl.spsolve(A.tocsc(), b)
    isf = np.ones(c["N"], bool)
    isf[c["dn"]] = False
    assert rel(h[isf], x) < 1e-12
    assert P.last["levels"] >= 2


def test_oracle_adjoint_central_fd(orc, pkg):
    c = steady_case(pkg, (8, 7, 5), sigma=1.0, seed=5, ndir=3, nq=2)
    N = c["N"]
    P = orc.Problem(N, c["nb"], c["aol"], c["dn"])
    rng = np.random.default_rng(0)
    w = rng.standard_normal(N)
    h = P.steady(c["Ks"], c["dh"], c["Qs"])
    dKs, ddh, dQs = P.adjoint(c["dh"], w)

    def J(Ks=c["Ks"], dh=c["dh"], Qs=c["Qs"]):
        Q = orc.Problem(N, c["nb"], c["aol"], c["dn"])
        return w @ Q.steady(Ks, dh, Qs)

    for f in rng.choice(len(c["Ks"]), 5, replace=False):
        e = 1e-5 * c["Ks"][f]
        Kp, Km = c["Ks"].copy(), c["Ks"].copy()
        Kp[f] += e
        Km[f] -= e
        fd = (J(Ks=Kp) - J(Ks=Km)) / (2 * e)
        assert abs(fd - dKs[f]) <= 1e-5 * max(abs(fd), 1e-30) + 1e-9 * np.abs(dKs).max()
    k = c["dn"][0]
    dp, dm = c["dh"].copy(), c["dh"].copy()
    dp[k] += 1e-4
    dm[k] -= 1e-4
    fd = (J(dh=dp) - J(dh=dm)) / 2e-4
    assert abs(fd - ddh[k]) <= 1e-6 * abs(fd) + 1e-12
    i = int(np.nonzero(np.isin(np.arange(N), c["dn"], invert=True))[0][7])
    qp, qm = c["Qs"].copy(), c["Qs"].copy()
    qp[i] += 1e-7
    qm[i] -= 1e-7
    fd = (J(Qs=qp) - J(Qs=qm)) / 2e-7
    assert abs(fd - dQs[i]) <= 1e-6 * abs(fd)


@pytest.mark.parametrize("kind", [0, 1])
def test_oracle_logk_vjp_fd(orc, pkg, kind):
    c = steady_case(pkg, (5, 4, 3), seed=9)
    rng = np.random.default_rng(1)
    dK = rng.standard_normal(len(c["nb"]))
    g = orc.logk_to_faces_vjp(c["nb"], c["logK"], dK, kind)
    for i in [0, 7, 31, 59]:
        lp, lm = c["logK"].copy(), c["logK"].copy()
        lp[i] += 1e-6
        lm[i] -= 1e-6
        fd = dK @ (orc.logk_to_faces(c["nb"], lp, kind) - orc.logk_to_faces(c["nb"], lm, kind)) / 2e-6
        assert abs(fd - g[i]) <= 1e-7 * max(abs(fd), 1e-6 * np.abs(g).max())


def test_thiem_analytic(orc, pkg):
    """The reference's Thiem check (test/thiem.jl:27-67): drawdown around a well, rtol 1e-1."""
    steadyhead, sidelength, thickness = 1e3, 50.0, 10.0
    R = sidelength
    n = 101
    coords, nb, aol, vol = pkg.regulargrid2d([-sidelength, -sidelength], [sidelength, sidelength], [n, n], thickness)
    N = coords.shape[1]
    k = 1e-5
    Ks = np.full(len(nb), k)
    Q = 1e-3
    Qs = np.zeros(N)
    Qs[n * ((n + 1) // 2 - 1) + (n + 1) // 2 - 1] = -Q
    r = np.sqrt(coords[0] ** 2 + coords[1] ** 2)
    dn = np.nonzero(r >= R)[0]
    dh = np.zeros(N)
    dh[dn] = steadyhead
    P = orc.Problem(N, nb, aol, dn)
    h = P.steady(Ks, dh, Qs, reltol=1e-12)
    good = np.nonzero((coords[1] == 0) & (coords[0] > 0.1))[0]
    T = thickness * k
    thiem = Q * np.log(R / coords[0, good]) / (2 * np.pi * T)
    dd = -h[good] + steadyhead
    assert np.linalg.norm(thiem - dd) <= 1e-1 * max(np.linalg.norm(thiem), np.linalg.norm(dd))


def _theis_W(u):
    # polynomial / rational approximations of the well function (test/theis.jl:12-18)
    u = np.asarray(u, dtype=np.float64)
    small = -np.log(u) - 0.57721566 + 0.99999193 * u - 0.24991055 * u ** 2 + 0.05519968 * u ** 3 \
        - 0.00976004 * u ** 4 + 0.00107857 * u ** 5
    big = (u ** 2 + 2.334733 * u + 0.250621) / (u ** 2 + 3.330657 * u + 1.681534) * np.exp(-u) / u
    return np.where(u <= 1, small, big)


def test_theis_analytic(orc, pkg):
    """The reference's Theis check (test/theis.jl:36-102) with fixed-step backward Euler, atol 1e-1."""
    steadyhead, sidelength, thickness = 1e3, 50.0, 10.0
    n = 101
    coords, nb, aol, vol = pkg.regulargrid2d([-sidelength, -sidelength], [sidelength, sidelength], [n, n], thickness)
    N = coords.shape[1]
    k = 1e-5
    Ks = np.full(len(nb), k)
    T = thickness * k
    Q = 1e-3
    Ss = 0.1
    S = Ss * thickness
    Qs = np.zeros(N)
    Qs[n * ((n + 1) // 2 - 1) + (n + 1) // 2 - 1] = -Q
    dn = np.nonzero((np.abs(coords[0]) == sidelength) | (np.abs(coords[1]) == sidelength))[0]
    dh = np.zeros(N)
    dh[dn] = steadyhead
    P = orc.Problem(N, nb, aol, dn)
    tfinal = 60 * 60 * 24 * 1e1
    nsteps = 200
    h0 = np.full(P.nfree, steadyhead)
    states = P.transient(Ks, dh, Qs, np.full(N, Ss), vol, tfinal / nsteps, nsteps, h0, reltol=1e-12)
    isf, n2f, f2n = pkg.getfreenodes(N, dn)
    hT = pkg.addboundaryconditions(states[-1], dn, dh, isf, n2f)
    good = np.nonzero((coords[1] == 0) & (coords[0] > 0.1) & (coords[0] <= sidelength / 2))[0]
    rs = coords[0, good]
    theis = Q * _theis_W(rs ** 2 * S / (4 * T * tfinal)) / (4 * np.pi * T)
    dd = -hT[good] + steadyhead
    assert np.max(np.abs(theis - dd)) <= 1e-1


def test_oracle_transient_adjoint_fd(orc, pkg):
    c = steady_case(pkg, (6, 5, 4), seed=11, ndir=2, nq=2)
    N = c["N"]
    Ss = np.full(N, 1e-2)
    V = c["vol"]
    obs = np.array([3, 40, 77])

    def J(Ks):
        P = orc.Problem(N, c["nb"], c["aol"], c["dn"])
        st = P.transient(Ks, c["dh"], c["Qs"], Ss, V, 20.0, 5, np.zeros(P.nfree))
        isf, n2f, _ = pkg.getfreenodes(N, c["dn"])
        return sum((st[n][n2f[o]] ** 2) for n in range(5) for o in obs if isf[o])

    P = orc.Problem(N, c["nb"], c["aol"], c["dn"])
    P.transient(c["Ks"], c["dh"], c["Qs"], Ss, V, 20.0, 5, np.zeros(P.nfree))
    dKs, ddh, dQs, dh0 = P.transient_adjoint(c["dh"], obs)
    for f in [0, 13, 100]:
        e = 1e-5 * c["Ks"][f]
        Kp, Km = c["Ks"].copy(), c["Ks"].copy()
        Kp[f] += e
        Km[f] -= e
        fd = (J(Kp) - J(Km)) / (2 * e)
        assert abs(fd - dKs[f]) <= 1e-5 * abs(fd) + 1e-9 * np.abs(dKs).max()


def test_oracle_1m_accuracy_floor(orc, pkg):
    """At 1e-10 relative residual the oracle's 1M-cell-like solution is within 1e-9 of its 1e-14 solve
    (run at 100x100x25 to keep the CPU suite short)."""
    c = steady_case(pkg, (100, 100, 25), mins=(0, 0, 0), maxs=(50, 50, 10), ell=20.0, sigma=2.0, seed=1)
    orc.set_threads(os.cpu_count() or 1)
    try:
        P = orc.Problem(c["N"], c["nb"], c["aol"], c["dn"])
        h1 = P.steady(c["Ks"], c["dh"], c["Qs"], reltol=1e-10)
        h2 = P.steady(c["Ks"], c["dh"], c["Qs"], reltol=1e-14)
    finally:
        orc.set_threads(1)
    assert rel(h1, h2) < 1e-9


def test_philox_known_answers():
    """The sampler checker's Philox4x32-10 against the generator's published known-answer vectors."""
    import matern_oracle as mo
    kat = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
           ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
           ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
            (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, want in kat:
        got = mo.philox4x32_10(*ctr, *key)
        assert tuple(int(x) for x in got) == want


def test_matern_sampler_restatement_statistics():
    """The spectral-synthesis method (the GPU sampler's, restated in float64): mean, variance and
    the Matern (nu = 1) correlation at several lags, over an ensemble of seeds."""
    import matern_oracle as mo
    ell, sigma, mu, M = 4.0, 1.5, -9.0, 512
    lags = np.array([1.0, 2.0, 4.0, 8.0])
    vals, pairs = [], {lag: [] for lag in lags}
    for seed in range(40):
        w, phi = mo.modes(seed, ell, M)
        pts = np.array([[0.0, 0.0, 0.0]] + [[lag, 0.0, 0.0] for lag in lags])
        f = mu + sigma * np.sqrt(2.0 / M) * np.cos(pts @ w.T + phi).sum(axis=1)
        vals.append(f[0])
        for j, lag in enumerate(lags):
            pairs[lag].append((f[0] - mu) * (f[1 + j] - mu))
    vals = np.array(vals)
    assert abs(vals.mean() - mu) < 4 * sigma / np.sqrt(len(vals))
    # exact second moments of the method (expectation over modes): E[f^2] - mu^2 = sigma^2 and
    # E[(f(0)-mu)(f(r)-mu)] = sigma^2 E[cos(w . r)]; the characteristic function of the scale mixture
    # is the Matern correlation, checked here by the mode average over all seeds
    allw = np.concatenate([mo.modes(s, ell, M)[0] for s in range(40)])
    for lag in lags:
        emp = np.mean(np.cos(allw[:, 0] * lag))
        assert abs(emp - mo.matern_correlation(lag, ell)) < 0.02, lag
