"""Seeded Richards problems on small regular grids for the tests (unsaturated near a Dirichlet
top layer held at negative pressure head, a source and a sink, lognormal K, van Genuchten
parameters per face)."""
import numpy as np


def richards_case(pkg, ns=(8, 6, 4), seed=0, psi_top=-4.0, alpha=0.375, nvg=1.25, sigma=0.5):
    mins, maxs = (0.0, 0.0, 0.0), (7.0, 5.0, 3.0)
    coords, nb, aol, vol = pkg.regulargrid3d(mins, maxs, ns)
    N = coords.shape[1]
    rng = np.random.default_rng(seed)
    logK = -9.0 + sigma * rng.standard_normal(N)
    Ks = np.exp(0.5 * (logK[nb[:, 0]] + logK[nb[:, 1]]))
    z = coords[2]
    top = np.nonzero(np.isclose(z, maxs[2]))[0]
    dn = top.astype(np.int64)
    dpsi = np.zeros(N)
    dpsi[dn] = psi_top
    Qs = np.zeros(N)
    Qs[0] = 2e-5                      # a source in the bottom corner
    Qs[N // 2 - ns[2]] = -1e-5        # a sink
    F = len(nb)
    alphas = alpha * np.exp(0.1 * rng.standard_normal(F))
    Ns = nvg + 0.05 * rng.uniform(0, 1, F)
    psi0 = np.full(N, psi_top)
    return dict(coords=coords, nb=nb, aol=aol, N=N, F=F, Ks=Ks, dn=dn, dpsi=dpsi, z=z, Qs=Qs, alphas=alphas, Ns=Ns,
                psi0=psi0)


def oracle_args(c):
    return (c["Ks"], c["nb"], c["aol"], c["dn"], c["z"], c["alphas"], c["Ns"], c["Qs"])


def transient_case(pkg, ns=(5, 4, 4), seed=4):
    c = richards_case(pkg, ns=ns, seed=seed, psi_top=-1.0)
    mins, maxs = (0.0, 0.0, 0.0), (7.0, 5.0, 3.0)
    _, _, _, vol = pkg.regulargrid3d(mins, maxs, ns)
    c.update(vol=vol, Ss=np.full(c["N"], 0.2), dt=20000.0, nsteps=5,
             psi0=np.where(np.isin(np.arange(c["N"]), c["dn"]), c["dpsi"], -2.0))
    rng = np.random.default_rng(seed + 50)
    c["obs"] = rng.choice(np.setdiff1d(np.arange(c["N"]), c["dn"]), 6, replace=False)
    c["w"] = rng.uniform(0.5, 1.5, 6)
    c["gT"] = rng.standard_normal(c["N"]) * 0.1
    return c
