"""CPU oracle for the steady Richards equation and its rrule (test infrastructure only).

A numpy/scipy restatement of DPFEHM's Richards path, used by the tests (and only there) to
check the GPU solver:
  * kr(psi, alpha, N): van Genuchten relative permeability, src/richards.jl:18-27;
  * hm(x, y) = 2 / (1/x + 1/y), src/richards.jl:50-52;
  * residuals at the free cells, steady (specificstorage = volumes = 1), src/richards.jl:98-118:
      R_j = Q_j + sum_{faces (j,k)} hm(kr_j, kr_k) K_f aol_f (psi_k + z_k - psi_j - z_j),
    psi_k = dirichletpsis[k] at a Dirichlet neighbour, one (alpha, N) per face;
  * richards_steadystate (src/richards.jl:148-167): the root of R, here by Newton's method with
    the exact sparse Jacobian and a direct solve (the reference uses NLsolve's trust region on
    the same Jacobian; the root is the same);
  * the rrule pullback (src/richards.jl:168-190): lambda = J^-T delta[free], dKs = -(dR/dKs)^T
    lambda, ddirichletpsis = -(dR/ddirichletpsis)^T lambda + delta at Dirichlet cells,
    dalphas, dNs, dQs likewise, zero for psi0.
The reference has no Richards tests or golden vectors, so this restatement is pinned by the
tests against central finite differences of its own solve ("parity unpinned" by reference
outputs).
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def kr(psi, alpha, N):
    """kr and its derivatives by psi, alpha and N (arrays broadcast); psi >= 0 gives 1."""
    psi = np.asarray(psi, float)
    alpha = np.broadcast_to(np.asarray(alpha, float), psi.shape)
    N = np.broadcast_to(np.asarray(N, float), psi.shape)
    neg = psi < 0
    v = np.ones_like(psi)
    dpsi = np.zeros_like(psi)
    dal = np.zeros_like(psi)
    dN = np.zeros_like(psi)
    if neg.any():
        p, a, n = psi[neg], alpha[neg], N[neg]
        m = (n - 1) / n
        u = np.abs(a * p)
        uN, uN1 = u ** n, u ** (n - 1)
        A = 1 + uN
        Am, Amh = A ** (-m), A ** (-m / 2)
        num = 1 - uN1 * Am
        v[neg] = num ** 2 * Amh
        uN2 = np.where(u > 0, uN1 / np.where(u > 0, u, 1), 0.0)
        dnum_du = -(n - 1) * uN2 * Am + m * n * uN1 * uN1 * Am / A
        dkr_du = 2 * num * dnum_du * Amh - 0.5 * m * num ** 2 * Amh / A * n * uN1
        dpsi[neg] = -a * dkr_du
        dal[neg] = np.abs(p) * dkr_du
        with np.errstate(divide="ignore", invalid="ignore"):
            lu = np.where(u > 0, np.log(np.where(u > 0, u, 1)), 0.0)
        lA = np.log(A)
        dm = 1 / n ** 2
        dA = uN * lu
        dAm = Am * (-dm * lA - m * dA / A)
        dnum = -(uN1 * lu * Am + uN1 * dAm)
        dAmh = Amh * (-0.5 * dm * lA - 0.5 * m * dA / A)
        dN[neg] = np.where(u > 0, 2 * num * dnum * Amh + num ** 2 * dAmh, 0.0)
    return v, dpsi, dal, dN


def _setup(N, neighbors, dirichletnodes):
    nb = np.asarray(neighbors, dtype=np.int64).reshape(-1, 2)
    isfree = np.ones(N, bool)
    isfree[np.asarray(dirichletnodes, dtype=np.int64)] = False
    free = np.nonzero(isfree)[0]
    fmap = -np.ones(N, np.int64)
    fmap[free] = np.arange(len(free))
    return nb, isfree, free, fmap


def _faces(psi, Ks, nb, aol, z, alphas, Ns):
    a, b = nb[:, 0], nb[:, 1]
    ka, dka, daa, dna = kr(psi[a], alphas, Ns)
    kb, dkb, dab, dnb = kr(psi[b], alphas, Ns)
    s = ka + kb
    H = 2 * ka * kb / s
    wa, wb = 2 * kb ** 2 / s ** 2, 2 * ka ** 2 / s ** 2
    D = psi[b] + z[b] - psi[a] - z[a]
    return dict(a=a, b=b, H=H, dHa=wa * dka, dHb=wb * dkb, dHal=wa * daa + wb * dab, dHN=wa * dna + wb * dnb, D=D,
                KA=np.asarray(Ks) * np.asarray(aol))


def residual(psi_full, Ks, neighbors, aol, dirichletnodes, z, alphas, Ns, Qs):
    """R at the free cells for a full-length psi (Dirichlet values in place)."""
    N = len(Qs)
    nb, isfree, free, fmap = _setup(N, neighbors, dirichletnodes)
    t = _faces(psi_full, Ks, nb, aol, z, alphas, Ns)
    flux = t["H"] * t["KA"] * t["D"]  # into a; -flux into b
    R = np.array(Qs, float).copy()
    np.add.at(R, t["a"], flux)
    np.add.at(R, t["b"], -flux)
    return R[free]


def jacobian(psi_full, Ks, neighbors, aol, dirichletnodes, z, alphas, Ns, Qs):
    """dR/dpsi at the free cells (sparse, free x free)."""
    N = len(Qs)
    nb, isfree, free, fmap = _setup(N, neighbors, dirichletnodes)
    t = _faces(psi_full, Ks, nb, aol, z, alphas, Ns)
    a, b, KA, H, D = t["a"], t["b"], t["KA"], t["H"], t["D"]
    dFa = KA * (t["dHa"] * D - H)   # d flux_into_a / d psi_a
    dFb = KA * (t["dHb"] * D + H)   # d flux_into_a / d psi_b
    rows, cols, vals = [], [], []
    # flux into a: rows a; flux into b is -flux_into_a: rows b
    for r_cell, sign in ((a, 1.0), (b, -1.0)):
        for c_cell, d in ((a, dFa), (b, dFb)):
            m = isfree[r_cell] & isfree[c_cell]
            rows.append(fmap[r_cell[m]])
            cols.append(fmap[c_cell[m]])
            vals.append(sign * d[m])
    n = len(free)
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def steady(psi0, Ks, neighbors, aol, dirichletnodes, dirichletpsis, z, alphas, Ns, Qs, tol=1e-13, maxiter=100):
    """Newton's method with the exact Jacobian and a backtracking line search; returns psi (N)."""
    N = len(Qs)
    nb, isfree, free, fmap = _setup(N, neighbors, dirichletnodes)
    psi = np.where(isfree, np.asarray(psi0, float), np.asarray(dirichletpsis, float))
    args = (Ks, neighbors, aol, dirichletnodes, z, alphas, Ns, Qs)
    R = residual(psi, *args)
    scale = max(np.linalg.norm(R), np.linalg.norm(np.asarray(Qs)[free]))
    for _ in range(maxiter):
        rn = np.linalg.norm(R)
        if rn <= tol * scale:
            break
        d = spla.spsolve(jacobian(psi, *args).tocsc(), -R)
        w = 1.0
        for _ in range(30):
            trial = psi.copy()
            trial[free] += w * d
            Rt = residual(trial, *args)
            if np.linalg.norm(Rt) < rn:
                break
            w *= 0.5
        psi, R = trial, Rt
    return psi


def r_transpose(psi, lfull, Ks, neighbors, aol, dirichletnodes, z, alphas, Ns, Qs):
    """(dR/dp)^T lambda at psi for lambda (N, zero at Dirichlet cells): the Ks, dirichletpsis,
    alphas, Ns and Qs parts (the dirichletpsis part only at Dirichlet cells)."""
    N = len(Qs)
    nb, isfree, free, fmap = _setup(N, neighbors, dirichletnodes)
    t = _faces(psi, Ks, nb, aol, z, alphas, Ns)
    a, b, D, H, KA = t["a"], t["b"], t["D"], t["H"], t["KA"]
    dl = lfull[a] - lfull[b]
    aolv = np.asarray(aol, float)
    gK = H * aolv * D * dl
    gal = KA * D * t["dHal"] * dl
    gN = KA * D * t["dHN"] * dl
    gQ = np.where(isfree, lfull, 0.0)
    gD = np.zeros(N)
    dFa = KA * (t["dHa"] * D - H)       # d flux_into_a / d psi_a
    dFb = KA * (t["dHb"] * D + H)       # d flux_into_a / d psi_b
    m = isfree[a] & ~isfree[b]          # k = b Dirichlet, j = a free: dR_a/dpsi_b = dFb
    np.add.at(gD, b[m], lfull[a[m]] * dFb[m])
    m = ~isfree[a] & isfree[b]          # k = a Dirichlet, j = b free: dR_b/dpsi_a = -dFa
    np.add.at(gD, a[m], -lfull[b[m]] * dFa[m])
    return gK, gD, gal, gN, gQ


def pullback(psi, delta, Ks, neighbors, aol, dirichletnodes, z, alphas, Ns, Qs):
    """The reference rrule's tangents at the solution psi (N): dKs, ddirichletpsis, dalphas, dNs, dQs."""
    N = len(Qs)
    nb, isfree, free, fmap = _setup(N, neighbors, dirichletnodes)
    args = (Ks, neighbors, aol, dirichletnodes, z, alphas, Ns, Qs)
    J = jacobian(psi, *args)
    lam = spla.spsolve(J.T.tocsc(), np.asarray(delta, float)[free])
    lfull = np.zeros(N)
    lfull[free] = lam
    gK, gD, gal, gN, gQ = r_transpose(psi, lfull, *args)
    ddp = np.where(isfree, 0.0, np.asarray(delta, float)) - gD
    return -gK, ddp, -gal, -gN, -gQ


def transient(psi0, Ks, neighbors, aol, dirichletnodes, dirichletpsis, z, alphas, Ns, Qs, Ss, vol, dt, nsteps,
              tol=1e-13, maxiter=100):
    """Fixed-step backward Euler of S V dpsi/dt = R(psi): each step the root of
    S V/dt (psi - psi_old) - R(psi) by Newton with the exact Jacobian; returns the states (nsteps, N)."""
    N = len(Qs)
    nb, isfree, free, fmap = _setup(N, neighbors, dirichletnodes)
    args = (Ks, neighbors, aol, dirichletnodes, z, alphas, Ns, Qs)
    shift = (np.asarray(Ss, float) * np.asarray(vol, float) / dt)[free]
    psi = np.where(isfree, np.asarray(psi0, float), np.asarray(dirichletpsis, float))
    out = []
    for _ in range(nsteps):
        old = psi.copy()

        def G(p):
            return shift * (p[free] - old[free]) - residual(p, *args)

        g = G(psi)
        scale = max(np.linalg.norm(g), np.linalg.norm(np.asarray(Qs)[free]))
        for _ in range(maxiter):
            gn = np.linalg.norm(g)
            if gn <= tol * scale:
                break
            Jg = sp.diags(shift) - jacobian(psi, *args)
            d = spla.spsolve(Jg.tocsc(), -g)
            w = 1.0
            for _ in range(30):
                trial = psi.copy()
                trial[free] += w * d
                gt = G(trial)
                if np.linalg.norm(gt) < gn:
                    break
                w *= 0.5
            psi, g = trial, gt
        out.append(psi.copy())
    return np.array(out)


def transient_pullback(states, obs, w, gT, Ks, neighbors, aol, dirichletnodes, z, alphas, Ns, Qs, Ss, vol, dt):
    """Discrete adjoint of `transient` for J = sum_n sum_k w_k psi^n[obs_k]^2 + gT . psi^nsteps:
    (dKs, ddirichletpsis, dalphas, dNs, dQs, dpsi0)."""
    N = len(Qs)
    nb, isfree, free, fmap = _setup(N, neighbors, dirichletnodes)
    args = (Ks, neighbors, aol, dirichletnodes, z, alphas, Ns, Qs)
    shift = np.asarray(Ss, float) * np.asarray(vol, float) / dt
    obs = np.asarray(obs, np.int64)
    w = np.ones(len(obs)) if w is None else np.asarray(w, float)
    nsteps = len(states)
    tot = None
    lam_next = np.zeros(N)
    for n in range(nsteps, 0, -1):
        psi = states[n - 1]
        seed = np.zeros(N)
        np.add.at(seed, obs, 2 * w * psi[obs])
        if n == nsteps and gT is not None:
            seed += np.asarray(gT, float)
        rhs = (seed + shift * lam_next)[free]
        Jg = sp.diags(shift[free]) - jacobian(psi, *args)
        lam = np.zeros(N)
        lam[free] = spla.spsolve(Jg.T.tocsc(), rhs)
        g = r_transpose(psi, lam, *args)
        g = (g[0], g[1] + np.where(isfree, 0.0, seed), g[2], g[3], g[4])
        tot = g if tot is None else tuple(x + y for x, y in zip(tot, g))
        lam_next = lam
    dpsi0 = np.where(isfree, shift * lam_next, 0.0)
    return tot + (dpsi0,)
