"""The CSR path for face lists that are not a regulargrid3d (unstructured meshes,
extra or duplicated faces) against the golden vectors and the oracle."""
import os

import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def random_mesh(n, seed, k=6):
    """A random 3-D point cloud joined to its k nearest neighbours (an unstructured mesh)."""
    rng = np.random.default_rng(seed)
    pts = rng.uniform(0, 10, (n, 3))
    d2 = ((pts[:, None, :] - pts[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d2, np.inf)
    nbr = np.argsort(d2, axis=1)[:, :k]
    pairs = {(min(i, j), max(i, j)) for i in range(n) for j in nbr[i]}
    nb = np.array(sorted(pairs), dtype=np.int64)
    lengths = np.sqrt(((pts[nb[:, 0]] - pts[nb[:, 1]]) ** 2).sum(1))
    areas = rng.uniform(0.5, 1.5, len(nb))
    return pts, nb, areas / lengths


def test_golden_general_graph(gpu_lib):
    pkg = gpu_lib
    g = dict(np.load(os.path.join(GOLD, "steady_general_graph.npz")))
    N = int(g["N"])
    h, back = pkg.rrule_groundwater_steadystate(g["Ks"], g["nb"], g["aol"], g["dn"], g["dh"], g["Qs"], reltol=1e-13)
    assert not back.problem.structured
    assert rel(h, g["h"]) < 1e-8
    _, dKs, _, _, _, ddh, dQs = back(g["delta"])
    assert rel(dKs, g["dKs"]) < 1e-6 and rel(ddh, g["ddh"]) < 1e-6 and rel(dQs, g["dQs"]) < 1e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n,ndir", [(400, 1), (3000, 5)])
def test_unstructured_vs_oracle(gpu_lib, orc, precision, n, ndir):
    pkg = gpu_lib
    pts, nb, aol = random_mesh(n, seed=n + ndir)
    rng = np.random.default_rng(3)
    logK = -9.0 + rng.standard_normal(n)
    Ks = np.exp(0.5 * (logK[nb[:, 0]] + logK[nb[:, 1]]))
    dn = rng.choice(n, ndir, replace=False)
    dh = np.zeros(n)
    dh[dn] = rng.uniform(0, 1, ndir)
    Qs = np.zeros(n)
    Qs[rng.choice(np.setdiff1d(np.arange(n), dn), 3, replace=False)] = [1e-4, 5e-5, -2e-5]
    delta = rng.standard_normal(n)
    P = pkg.GroundwaterProblem(nb, aol, dn, N=n, reltol=1e-12, precision=precision)
    assert not P.structured and P.levels >= 2
    h = P.forward(Ks, dh, Qs)
    dKs, ddh, dQs = P.adjoint(delta)
    O = orc.Problem(n, nb, aol, dn)
    h_or = O.steady(Ks, dh, Qs, reltol=1e-14)
    dKs_or, ddh_or, dQs_or = O.adjoint(dh, delta, reltol=1e-14)
    assert rel(h, h_or) < 1e-8
    assert rel(dKs, dKs_or) < 1e-6 and rel(ddh, ddh_or) < 1e-6 and rel(dQs, dQs_or) < 1e-6
    # logK path and face means through the same handle
    obs = rng.choice(n, 20, replace=False)
    h2, g2 = P.solve_grad_logk(logK, dh, Qs, obs)
    d2 = np.zeros(n)
    np.add.at(d2, obs, 2 * h_or[obs])
    dK2, _, _ = O.adjoint(dh, d2, reltol=1e-14)
    assert rel(h2, h_or) < 1e-8
    assert rel(g2, orc.logk_to_faces_vjp(nb, logK, dK2)) < 1e-6
    assert rel(P.logk_to_faces(logK, "harmonic"), orc.logk_to_faces(nb, logK, 1)) < 1e-14


def test_uge_mesh_roundtrip_solve(gpu_lib, orc, tmp_path):
    pkg = gpu_lib
    pts, nb, aol = random_mesh(600, seed=9)
    vols = np.full(600, 0.8)
    areas = aol * np.sqrt(((pts[nb[:, 0]] - pts[nb[:, 1]]) ** 2).sum(1))
    f = tmp_path / "mesh.uge"
    pkg.grid.write_uge(str(f), pts.T, vols, nb, areas)
    coords, volumes, nb2, areas2, lengths = pkg.load_uge(str(f))
    aol2 = areas2 / lengths
    n = coords.shape[1]
    Ks = np.full(len(nb2), 1e-5)
    Qs = np.zeros(n)
    Qs[10] = 1e-3
    dn = [0, 1]
    dh = np.zeros(n)
    dh[1] = 2.0
    h = pkg.groundwater_steadystate(Ks, nb2, aol2, dn, dh, Qs, reltol=1e-12)
    O = orc.Problem(n, nb2, aol2, dn)
    assert rel(h, O.steady(Ks, dh, Qs)) < 1e-8


def test_reordered_regular_grid_matches_structured(gpu_lib):
    pkg = gpu_lib
    coords, nb, aol, vol = pkg.regulargrid3d((0, 0, 0), (5, 4, 3), (11, 9, 7))
    N = coords.shape[1]
    rng = np.random.default_rng(1)
    logK = -9 + rng.standard_normal(N)
    Ks = np.exp(0.5 * (logK[nb[:, 0]] + logK[nb[:, 1]]))
    perm = rng.permutation(len(nb))
    Qs = np.zeros(N)
    Qs[5] = 1e-4
    dh = np.zeros(N)
    S = pkg.GroundwaterProblem(nb, aol, [N - 1], N=N, reltol=1e-12)
    G = pkg.GroundwaterProblem(nb[perm], aol[perm], [N - 1], N=N, reltol=1e-12)
    assert S.structured and not G.structured
    assert rel(G.forward(Ks[perm], dh, Qs), S.forward(Ks, dh, Qs)) < 1e-9


def test_general_transient_vs_oracle(gpu_lib, orc):
    pkg = gpu_lib
    pts, nb, aol = random_mesh(500, seed=21)
    n = 500
    rng = np.random.default_rng(5)
    Ks = np.exp(-8 + rng.standard_normal(len(nb)))
    dn = [3, 7]
    dh = np.zeros(n)
    Qs = np.zeros(n)
    Qs[100] = 1e-3
    Ss = np.full(n, 1e-3)
    vol = rng.uniform(0.5, 1.5, n)
    obs = [10, 50, 200]
    P = pkg.GroundwaterProblem(nb, aol, dn, N=n, volumes=vol, reltol=1e-12)
    hT, states = P.transient_forward(Ks, dh, Qs, Ss, 100.0, 6, np.zeros(n), return_states=True)
    dK, ddh, dQ, dh0 = P.transient_adjoint(obs)
    O = orc.Problem(n, nb, aol, dn)
    st = O.transient(Ks, dh, Qs, Ss, vol, 100.0, 6, np.zeros(O.nfree), reltol=1e-14)
    dK_or, ddh_or, dQ_or, dh0_or = O.transient_adjoint(dh, obs, reltol=1e-14)
    isf, _, _ = pkg.getfreenodes(n, dn)
    assert rel(states[:, isf], st) < 1e-8
    assert rel(dK, dK_or) < 1e-6 and rel(ddh, ddh_or) < 1e-6 and rel(dQ, dQ_or) < 1e-6
    assert rel(dh0[isf], dh0_or) < 1e-6


def _fracture_case(pkg, tmp_path):
    """A synthetic fracture network (1000 fractures with power-law sizes in a 100 m cube, about 64k
    cells, degrees up to 8) written as .uge and read back; one log-conductivity per fracture, h = 1
    on the cells within 5 m of x = 0 and h = 0 within 5 m of x = 100, two injection cells."""
    c, vol, nb, ar, ln, fr = pkg.grid.fracture_network(1000, 100.0, 1.0, 3)
    f = tmp_path / "dfn.uge"
    pkg.grid.write_uge(str(f), c, vol, nb, ar)
    coords, volumes, nb2, areas, lengths = pkg.load_uge(str(f))
    N = coords.shape[1]
    rng = np.random.default_rng(4)
    lk_frac = rng.normal(-9.0, 1.0, fr.max() + 1)
    logK = lk_frac[fr]
    Ks = np.exp(0.5 * (logK[nb2[:, 0]] + logK[nb2[:, 1]]))
    x = coords[0]
    dn = np.nonzero((x < 5.0) | (x > 95.0))[0]
    dh = np.zeros(N)
    dh[x < 5.0] = 1.0
    Qs = np.zeros(N)
    Qs[rng.choice(np.nonzero((x > 30) & (x < 70))[0], 2, replace=False)] = 1e-6
    return dict(N=N, nb=nb2, aol=areas / lengths, vol=volumes, dn=dn, dh=dh, Qs=Qs, Ks=Ks, logK=logK)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fracture_network_vs_oracle(gpu_lib, orc, tmp_path, precision):
    """Steady solve and rrule on the CSR path for a fracture-network mesh (irregular degrees, not a
    grid) read from a .uge file, against the oracle (heads 1e-8, tangents 1e-6)."""
    pkg = gpu_lib
    c = _fracture_case(pkg, tmp_path)
    P = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"], volumes=c["vol"], reltol=1e-12,
                               precision=precision)
    assert not P.structured
    h = P.forward(c["Ks"], c["dh"], c["Qs"])
    delta = np.random.default_rng(5).standard_normal(c["N"])
    dKs, ddh, dQs = P.adjoint(delta)
    O = orc.Problem(c["N"], c["nb"], c["aol"], c["dn"])
    h_or = O.steady(c["Ks"], c["dh"], c["Qs"], reltol=1e-14)
    dK_or, ddh_or, dQ_or = O.adjoint(c["dh"], delta, reltol=1e-14)
    assert rel(h, h_or) < 1e-8
    assert np.array_equal(h[c["dn"]], c["dh"][c["dn"]])
    assert rel(dKs, dK_or) < 1e-6 and rel(ddh, ddh_or) < 1e-6 and rel(dQs, dQ_or) < 1e-6


def test_general_path_profile_report(gpu_lib, tmp_path):
    """Per-kernel timing works on the CSR path too (the DF product, the updates and the V-cycle)."""
    pkg = gpu_lib
    c = _fracture_case(pkg, tmp_path)
    P = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"], reltol=1e-10, precision="mixed")
    P.profile(True)
    P.solve_grad_logk(c["logK"], c["dh"], c["Qs"], np.arange(0, c["N"], 997))
    rep = P.profile_report()
    P.profile(False)
    assert any(k.startswith("kg_df_spmv_pq<f32>/L0") for k in rep)
    assert any(k.startswith("kg_cheb_step<f32>/L1") for k in rep)
    assert all(v[0] > 0 and v[1] > 0 for v in rep.values())
