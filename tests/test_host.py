"""Host-side mirror of the reference's grid/bookkeeping functions (no GPU)."""
import numpy as np
import pytest


def test_grid2d_layout(pkg):
    # test/grid.jl:8-14: the 2-D grid goes over y first, then x
    ns, mins, maxs = [5, 10], [0, 0], [1, 1]
    coords, nb, aol, vol = pkg.regulargrid2d(mins, maxs, ns, 1.0)
    assert coords[1, 0] != coords[1, 1]
    assert coords[1, 0] == coords[1, ns[1]]
    assert coords[0, 0] != coords[0, ns[1]]
    assert np.all(coords[0, 0] == coords[0, : ns[1]])
    assert np.isclose(vol.sum(), np.prod(ns) * np.prod((np.array(maxs) - mins) / (np.array(ns) - 1)) * 1.0)
    assert len(nb) == 2 * 50 - 5 - 10


def test_grid3d_layout(pkg):
    # test/grid.jl:16-24: z first, then y, then x
    ns, mins, maxs = [5, 10, 20], [0, 0, 0], [1, 1, 1]
    coords, nb, aol, vol = pkg.regulargrid3d(mins, maxs, ns)
    assert coords[2, 0] != coords[2, 1]
    assert coords[2, 0] == coords[2, ns[2]]
    assert coords[1, 0] != coords[1, ns[2]]
    assert np.all(coords[1, 0] == coords[1, : ns[2]])
    assert coords[0, 0] != coords[0, ns[2] * ns[1]]
    assert np.all(coords[0, 0] == coords[0, : ns[1] * ns[2]])
    assert np.isclose(vol.sum(), np.prod(ns) * np.prod((np.array(maxs) - mins) / (np.array(ns) - 1)))
    F = 3 * 1000 - 50 - 100 - 200
    assert len(nb) == F == len(aol)


def test_grid3d_face_order_matches_loops(pkg):
    ns = (3, 4, 2)
    coords, nb, aol, vol = pkg.regulargrid3d((0, 0, 0), (2, 3, 1), ns)
    lin = lambda i1, i2, i3: i3 + ns[2] * i2 + ns[2] * ns[1] * i1
    exp = []
    for i1 in range(ns[0]):
        for i2 in range(ns[1]):
            for i3 in range(ns[2]):
                if i1 < ns[0] - 1:
                    exp.append((lin(i1, i2, i3), lin(i1 + 1, i2, i3)))
                if i2 < ns[1] - 1:
                    exp.append((lin(i1, i2, i3), lin(i1, i2 + 1, i3)))
                if i3 < ns[2] - 1:
                    exp.append((lin(i1, i2, i3), lin(i1, i2, i3 + 1)))
    assert np.array_equal(nb, np.array(exp))


def test_grid1d(pkg):
    coords, nb, aol, vol = pkg.regulargrid1d([0], [4], [5], 2.0, 3.0)
    assert len(nb) == 4 and len(aol) == 5 and np.allclose(aol, 6.0)


def test_getfreenodes_and_boundary(pkg):
    isf, n2f, f2n = pkg.getfreenodes(6, [1, 4])
    assert list(isf) == [True, False, True, True, False, True]
    assert list(n2f) == [0, -1, 1, 2, -1, 3]
    assert list(f2n) == [0, 2, 3, 5]
    h = pkg.addboundaryconditions(np.array([10.0, 20, 30, 40]), [1, 4], np.arange(6.0), isf, n2f)
    assert list(h) == [10, 1, 20, 30, 4, 40]


def test_uge_roundtrip(pkg, tmp_path):
    coords, nb, aol, vol = pkg.regulargrid3d((0, 0, 0), (2, 2, 1), (3, 3, 2))
    areas = np.arange(1, len(nb) + 1, dtype=float)
    f = tmp_path / "m.uge"
    pkg.grid.write_uge(str(f), coords, vol, nb, areas)
    c2, v2, nb2, a2, l2 = pkg.load_uge(str(f))
    assert np.allclose(c2, coords) and np.allclose(v2, vol) and np.array_equal(nb2, nb) and np.allclose(a2, areas)
    assert np.allclose(l2, np.sqrt(((coords[:, nb[:, 0]] - coords[:, nb[:, 1]]) ** 2).sum(0)))


def test_fracture_network_mesh(pkg, tmp_path):
    """The synthetic fracture network: seeded (same seed, same mesh), one connected component,
    irregular degrees (cells that several fractures cross have more than four neighbours), every
    face between two fractures' cells or two in-plane neighbours, and a .uge round trip that
    reproduces the areas over lengths the solver uses."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import connected_components
    c, vol, nb, ar, ln, fr = pkg.grid.fracture_network(1000, 100.0, 1.0, 3)
    c2, _, nb2, ar2, _, _ = pkg.grid.fracture_network(1000, 100.0, 1.0, 3)
    assert np.array_equal(nb, nb2) and np.array_equal(ar, ar2) and np.array_equal(c, c2)
    N = c.shape[1]
    assert N > 50000 and len(np.unique(fr)) > 100
    G = sp.coo_matrix((np.ones(len(nb)), (nb[:, 0], nb[:, 1])), shape=(N, N))
    assert connected_components(G, directed=False)[0] == 1
    deg = np.bincount(nb.ravel(), minlength=N)
    assert deg.min() >= 1 and deg.max() >= 7 and (deg > 4).sum() > 1000
    assert np.all(nb[:, 0] < nb[:, 1]) and len(np.unique(nb[:, 0] * N + nb[:, 1])) == len(nb)
    cross = fr[nb[:, 0]] != fr[nb[:, 1]]
    assert cross.any() and np.allclose(ln[~cross], 1.0) and np.all(ar / ln > 0)
    sub = np.nonzero((nb < 3000).all(axis=1))[0]  # a small piece for the file round trip
    keep = np.unique(nb[sub])
    f = tmp_path / "dfn.uge"
    pkg.grid.write_uge(str(f), c[:, :3000], vol[:3000], nb[sub], ar[sub])
    c3, v3, nb3, a3, l3 = pkg.load_uge(str(f))
    assert np.array_equal(nb3, nb[sub]) and np.allclose(a3 / l3, ar[sub] / ln[sub], rtol=1e-12)
    assert keep.size > 0


def test_matern_field_statistics(pkg):
    f = pkg.fields.matern_field((200, 200), (0.5, 0.5), 5.0, 2.0, -9.0, seed=3)
    assert f.shape == (200, 200)
    assert abs(f.mean() + 9.0) < 0.6
    assert 0.5 < f.std() < 3.0
    # neighbouring values are strongly correlated, far ones weakly
    a = f - f.mean()
    c1 = (a[:-1] * a[1:]).mean() / a.var()
    c50 = (a[:-50] * a[50:]).mean() / a.var()
    assert c1 > 0.9 and abs(c50) < c1
    g = pkg.fields.matern_field((200, 200), (0.5, 0.5), 5.0, 2.0, -9.0, seed=3)
    assert np.array_equal(f, g)


def test_layered_field(pkg):
    lk = pkg.fields.layered_logk((10, 8, 4), (0, 0, 0), (5, 4, 2), 3.0, 1.0, -9.0, 0)
    a = lk.reshape(10, 8, 4)
    assert np.all(a[:, :, 0:1] == a)


def test_options_reject_unknown(pkg):
    with pytest.raises(TypeError):
        pkg.default_options(bogus=1)
