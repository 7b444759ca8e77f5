"""Shared problem builders for the tests (seeded synthetic inputs)."""
import numpy as np


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def steady_case(pkg, ns, mins=None, maxs=None, ell=None, sigma=1.0, seed=0, ndir=1, nq=1, layered=False,
                mean="geometric"):
    """A regulargrid3d problem with a seeded Matern logK, injection and Dirichlet cells."""
    mins = mins or (0.0, 0.0, 0.0)
    maxs = maxs or tuple(0.5 * (n - 1) for n in ns)
    ell = ell or 0.3 * max(maxs[0] - mins[0], maxs[1] - mins[1])
    coords, nb, aol, vol = pkg.regulargrid3d(mins, maxs, ns)
    N = coords.shape[1]
    if layered:
        logK = pkg.fields.layered_logk(ns, mins, maxs, ell, sigma, -9.0, seed)
    else:
        logK = pkg.fields.volume_logk(ns, mins, maxs, ell, sigma, -9.0, seed)
    rng = np.random.default_rng(seed + 1000)
    Qs = np.zeros(N)
    if nq == 1:
        Qs[0] = 1e-4
    else:
        Qs[rng.choice(N, nq, replace=False)] = rng.uniform(1e-5, 1e-3, nq)
    if ndir == 1:
        dn = np.array([N - 1], dtype=np.int64)
    else:
        dn = np.sort(rng.choice(N, ndir, replace=False)).astype(np.int64)
    dh = np.zeros(N)
    dh[dn] = rng.uniform(-1.0, 1.0, len(dn)) if ndir > 1 else 0.0
    if mean == "geometric":
        Ks = np.exp(0.5 * (logK[nb[:, 0]] + logK[nb[:, 1]]))
    else:
        Ks = 2.0 / (np.exp(-logK[nb[:, 0]]) + np.exp(-logK[nb[:, 1]]))
    return dict(coords=coords, nb=nb, aol=aol, vol=vol, N=N, logK=logK, Ks=Ks, Qs=Qs, dn=dn, dh=dh, ns=ns,
                mins=mins, maxs=maxs)
