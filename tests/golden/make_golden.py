"""Generate tests/golden/*.npz: small known-answer cases for the groundwater path.

The reference (DPFEHM.jl) holds no golden vectors and cannot run here (no
Julia), so these vectors come from an independent pure-Python restatement --
explicit loops over the face list exactly as written in src/groundwater.jl:1-21
(residual, and its derivatives with respect to h, Ks, dirichleths and Qs, as the
NonlinearEquations macro would form them), solved by scipy's direct sparse
solver, and the rrule formulas of src/groundwater.jl:93-107 applied literally
(-(gw_Ks' * lambda) etc.); likewise the two-phase pressure solve of
src/twophase.jl:22-82. The C oracle and the GPU library are both checked
against these files.

Run: python tests/golden/make_golden.py   (writes next to this script)
"""
import os

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl

HERE = os.path.dirname(os.path.abspath(__file__))


def getfreenodes(n, dn):
    isfree = np.ones(n, bool)
    isfree[list(dn)] = False
    n2f = -np.ones(n, np.int64)
    f2n = np.nonzero(isfree)[0]
    n2f[f2n] = np.arange(len(f2n))
    return isfree, n2f, f2n


def residual_terms(h, Ks, nb, aol, dn, dh, Qs, Ss, V):
    """Residual and Jacobians of src/groundwater.jl:4-20 by explicit loops (dense, small cases only)."""
    N = len(Qs)
    F = len(nb)
    isfree, n2f, f2n = getfreenodes(N, dn)
    m = len(f2n)
    R = np.zeros(m)
    Jh = np.zeros((m, m))
    JK = np.zeros((m, F))
    Jdh = np.zeros((m, N))
    JQ = np.zeros((m, N))
    for i in range(N):
        if isfree[i]:
            j = n2f[i]
            R[j] += -Qs[i] / (Ss[i] * V[i])
            JQ[j, i] += -1.0 / (Ss[i] * V[i])
    for f in range(F):
        a, b = nb[f]
        for n1, n2 in ((a, b), (b, a)):
            if not isfree[n1]:
                continue
            j1 = n2f[n1]
            s = 1.0 / (Ss[n1] * V[n1])
            if isfree[n2]:
                j2 = n2f[n2]
                R[j1] += Ks[f] * (h[j1] - h[j2]) * aol[f] * s
                Jh[j1, j1] += Ks[f] * aol[f] * s
                Jh[j1, j2] -= Ks[f] * aol[f] * s
                JK[j1, f] += (h[j1] - h[j2]) * aol[f] * s
            else:
                R[j1] += Ks[f] * (h[j1] - dh[n2]) * aol[f] * s
                Jh[j1, j1] += Ks[f] * aol[f] * s
                JK[j1, f] += (h[j1] - dh[n2]) * aol[f] * s
                Jdh[j1, n2] += -Ks[f] * aol[f] * s
    return R, Jh, JK, Jdh, JQ, isfree, n2f, f2n


def steady_and_rrule(Ks, nb, aol, dn, dh, Qs, delta):
    N = len(Qs)
    ones = np.ones(N)
    m = N - len(set(dn))
    R0, A, _, _, _, isfree, n2f, f2n = residual_terms(np.zeros(m), Ks, nb, aol, dn, dh, Qs, ones, ones)
    b = -R0
    hfree = spl.spsolve(sp.csc_matrix(A), b)
    h = np.where(isfree, hfree[np.maximum(n2f, 0)], dh)
    _, _, JK, Jdh, JQ, _, _, _ = residual_terms(hfree, Ks, nb, aol, dn, dh, Qs, ones, ones)
    lam = spl.spsolve(sp.csc_matrix(A.T), delta[isfree])
    dKs = -(JK.T @ lam)
    ddh = -(Jdh.T @ lam) + delta * (~isfree)
    dQs = -(JQ.T @ lam)
    return h, dKs, ddh, dQs


def pressure_and_rrule(Ks, nb, aol, dn, dh, Qs, delta):
    """Two-phase pressure solve and its rrule, src/twophase.jl:22-82 restated literally:
    residual -Q_i + sum over the faces of a free cell of (h_1 - h_2) * (tx K) with tx = 2 aol
    (the Dirichlet value for h_2 at Dirichlet neighbours), its Jacobians by explicit loops, a
    direct solve, and the pullback -(trans_Ks' lambda), -(trans_dirichleths' lambda) + delta at
    Dirichlet cells, -(trans_Qs' lambda)."""
    N, F = len(Qs), len(nb)
    isfree, n2f, f2n = getfreenodes(N, dn)
    m = len(f2n)
    tx = 2.0 * aol

    def terms(h):
        R = np.zeros(m); Jh = np.zeros((m, m)); JK = np.zeros((m, F)); Jdh = np.zeros((m, N)); JQ = np.zeros((m, N))
        for i in range(N):
            if isfree[i]:
                R[n2f[i]] += -Qs[i]
                JQ[n2f[i], i] += -1.0
        for f in range(F):
            a, b = nb[f]
            for n1, n2 in ((a, b), (b, a)):
                if not isfree[n1]:
                    continue
                j1 = n2f[n1]
                if isfree[n2]:
                    j2 = n2f[n2]
                    R[j1] += (h[j1] - h[j2]) * (tx[f] * Ks[f])
                    Jh[j1, j1] += tx[f] * Ks[f]
                    Jh[j1, j2] -= tx[f] * Ks[f]
                    JK[j1, f] += (h[j1] - h[j2]) * tx[f]
                else:
                    R[j1] += (h[j1] - dh[n2]) * (tx[f] * Ks[f])
                    Jh[j1, j1] += tx[f] * Ks[f]
                    JK[j1, f] += (h[j1] - dh[n2]) * tx[f]
                    Jdh[j1, n2] += -tx[f] * Ks[f]
        return R, Jh, JK, Jdh, JQ

    R0, A, _, _, _ = terms(np.zeros(m))
    hfree = spl.spsolve(sp.csc_matrix(A), -R0)
    h = np.where(isfree, hfree[np.maximum(n2f, 0)], dh)
    _, _, JK, Jdh, JQ = terms(hfree)
    lam = spl.spsolve(sp.csc_matrix(A.T), delta[isfree])
    return h, -(JK.T @ lam), -(Jdh.T @ lam) + delta * (~isfree), -(JQ.T @ lam)


def transient_and_adjoint(Ks, nb, aol, dn, dh, Qs, Ss, V, dt, nsteps, h0free, obs):
    """Fixed-step backward Euler of dh/dt = -R(h), J = sum_n sum_obs h^n[obs]^2, by dense linear algebra."""
    N = len(Qs)
    m = N - len(set(dn))
    R0, Jh, _, _, _, isfree, n2f, f2n = residual_terms(np.zeros(m), Ks, nb, aol, dn, dh, Qs, Ss, V)
    M = np.eye(m) + dt * Jh            # h^{n+1} + dt R(h^{n+1}) = h^n, R linear: R(h) = R0 + Jh h
    states = []
    h = h0free.copy()
    for _ in range(nsteps):
        h = np.linalg.solve(M, h - dt * R0)
        states.append(h.copy())
    # adjoint of G_n = M h^n - h^{n-1} + dt R0 = 0
    obs_free = [n2f[o] for o in obs if isfree[o]]
    dK = np.zeros(len(Ks))
    ddh = np.zeros(N)
    dQ = np.zeros(N)
    mu_next = np.zeros(m)
    for n in range(nsteps - 1, -1, -1):
        g = np.zeros(m)
        for j in obs_free:
            g[j] += 2.0 * states[n][j]
        mu = np.linalg.solve(M.T, g + mu_next)
        _, _, JK, Jdh, JQ, _, _, _ = residual_terms(states[n], Ks, nb, aol, dn, dh, Qs, Ss, V)
        dK -= dt * (JK.T @ mu)
        ddh -= dt * (Jdh.T @ mu)
        dQ -= dt * (JQ.T @ mu)
        mu_next = mu
    dh0 = mu_next.copy()
    return np.array(states), dK, ddh, dQ, dh0


def grid3d(ns, mins, maxs):
    n1, n2, n3 = ns
    xs = [np.linspace(mins[k], maxs[k], ns[k]) for k in range(3)]
    d = [x[1] - x[0] if len(x) > 1 else 1.0 for x in xs]
    nb, aol = [], []
    lin = lambda i1, i2, i3: i3 + n3 * i2 + n3 * n2 * i1
    for i1 in range(n1):
        for i2 in range(n2):
            for i3 in range(n3):
                if i1 < n1 - 1:
                    nb.append((lin(i1, i2, i3), lin(i1 + 1, i2, i3))); aol.append(d[1] * d[2] / d[0])
                if i2 < n2 - 1:
                    nb.append((lin(i1, i2, i3), lin(i1, i2 + 1, i3))); aol.append(d[0] * d[2] / d[1])
                if i3 < n3 - 1:
                    nb.append((lin(i1, i2, i3), lin(i1, i2, i3 + 1))); aol.append(d[0] * d[1] / d[2])
    return np.array(nb, np.int64), np.array(aol), d[0] * d[1] * d[2]


def main():
    rng = np.random.default_rng(20261203)
    # case A: 3-D regular grid, one Dirichlet cell, geometric face means
    ns = (6, 5, 4)
    nb, aol, vol = grid3d(ns, (0, 0, 0), (2.5, 2.0, 1.5))
    N = int(np.prod(ns))
    logK = -9.0 + rng.standard_normal(N)
    Ks = np.exp(0.5 * (logK[nb[:, 0]] + logK[nb[:, 1]]))
    Qs = np.zeros(N); Qs[0] = 1e-4
    dn = np.array([N - 1]); dh = np.zeros(N)
    delta = np.zeros(N); delta[[3, 17, 40]] = [1.0, -2.0, 0.5]
    h, dKs, ddh, dQs = steady_and_rrule(Ks, nb, aol, dn, dh, Qs, delta)
    np.savez(os.path.join(HERE, "steady_regular3d.npz"), ns=np.array(ns), nb=nb, aol=aol, logK=logK, Ks=Ks, Qs=Qs,
             dn=dn, dh=dh, delta=delta, h=h, dKs=dKs, ddh=ddh, dQs=dQs)
    # case B: 3-D regular grid, several Dirichlet cells with nonzero heads, several sources, harmonic means
    ns = (5, 4, 3)
    nb, aol, vol = grid3d(ns, (0, 0, 0), (4.0, 3.0, 1.0))
    N = int(np.prod(ns))
    logK = -8.0 + 1.5 * rng.standard_normal(N)
    Ks = 2.0 / (np.exp(-logK[nb[:, 0]]) + np.exp(-logK[nb[:, 1]]))
    Qs = np.zeros(N); Qs[[5, 22, 31]] = [2e-4, -1e-4, 5e-5]
    dn = np.array([0, 11, N - 1]); dh = np.zeros(N); dh[dn] = [1.5, -0.5, 2.0]
    delta = rng.standard_normal(N)
    h, dKs, ddh, dQs = steady_and_rrule(Ks, nb, aol, dn, dh, Qs, delta)
    np.savez(os.path.join(HERE, "steady_harmonic_multidir.npz"), ns=np.array(ns), nb=nb, aol=aol, logK=logK, Ks=Ks,
             Qs=Qs, dn=dn, dh=dh, delta=delta, h=h, dKs=dKs, ddh=ddh, dQs=dQs)
    # case C: general graph (grid with diagonal faces and one duplicated face)
    ns = (5, 5, 1)
    nb, aol, vol = grid3d(ns, (0, 0, 0), (4.0, 4.0, 1.0))
    extra = [(0, 6), (6, 12), (12, 18), (18, 24), (4, 8), (8, 12), (0, 6)]
    nb = np.concatenate([nb, np.array(extra, np.int64)])
    aol = np.concatenate([aol, np.full(len(extra), 0.35)])
    N = 25
    Ks = np.exp(-9.0 + 0.8 * rng.standard_normal(len(nb)))
    Qs = np.zeros(N); Qs[7] = 3e-4
    dn = np.array([20, 24]); dh = np.zeros(N); dh[dn] = [0.0, 1.0]
    delta = np.zeros(N); delta[[2, 13]] = [1.0, 1.0]
    h, dKs, ddh, dQs = steady_and_rrule(Ks, nb, aol, dn, dh, Qs, delta)
    np.savez(os.path.join(HERE, "steady_general_graph.npz"), nb=nb, aol=aol, Ks=Ks, Qs=Qs, dn=dn, dh=dh,
             delta=delta, h=h, dKs=dKs, ddh=ddh, dQs=dQs, N=np.array(N))
    # case D: transient backward Euler + adjoint on a small 3-D grid
    ns = (5, 4, 3)
    nb, aol, vol = grid3d(ns, (0, 0, 0), (2.0, 1.5, 1.0))
    N = int(np.prod(ns))
    logK = -7.0 + rng.standard_normal(N)
    Ks = np.exp(0.5 * (logK[nb[:, 0]] + logK[nb[:, 1]]))
    Qs = np.zeros(N); Qs[[2, 30]] = [1e-3, 5e-4]
    dn = np.array([N - 1, N - 2]); dh = np.zeros(N); dh[dn] = [0.0, 0.25]
    Ss = np.full(N, 1e-3)
    V = np.full(N, vol)
    dt, nsteps = 50.0, 6
    h0 = np.zeros(N - 2)
    obs = np.array([4, 17, 33])
    states, dK, ddh, dQ, dh0 = transient_and_adjoint(Ks, nb, aol, dn, dh, Qs, Ss, V, dt, nsteps, h0, obs)
    np.savez(os.path.join(HERE, "transient_regular3d.npz"), ns=np.array(ns), nb=nb, aol=aol, Ks=Ks, Qs=Qs, dn=dn,
             dh=dh, Ss=Ss, V=V, dt=np.array(dt), nsteps=np.array(nsteps), h0=h0, obs=obs, states=states, dKs=dK,
             ddh=ddh, dQs=dQ, dh0=dh0)
    # case E: two-phase pressure solve (transmissibility 2 aol K) and its rrule
    ns = (6, 4, 3)
    nb, aol, vol = grid3d(ns, (0, 0, 0), (3.0, 2.0, 1.0))
    N = int(np.prod(ns))
    Ks = np.exp(-8.0 + rng.standard_normal(len(nb)))
    Qs = np.zeros(N); Qs[[1, 40]] = [3e-4, -1e-4]
    dn = np.array([0, N - 1]); dh = np.zeros(N); dh[dn] = [2.0, -1.0]
    delta = rng.standard_normal(N)
    h, dKs, ddh, dQs = pressure_and_rrule(Ks, nb, aol, dn, dh, Qs, delta)
    np.savez(os.path.join(HERE, "twophase_pressure.npz"), ns=np.array(ns), nb=nb, aol=aol, Ks=Ks, Qs=Qs, dn=dn,
             dh=dh, delta=delta, h=h, dKs=dKs, ddh=ddh, dQs=dQs)


if __name__ == "__main__":
    main()
