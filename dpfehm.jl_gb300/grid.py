"""Mesh construction, mirroring DPFEHM's grid generators.

The index order and face enumeration are part of the drop-in contract: the GPU
library recognises a face list produced by ``regulargrid3d`` and switches to its
matrix-free 7-point path, so these functions reproduce the reference layout
exactly (cell index z fastest, then y, then x; faces emitted per cell in the
order +x, +y, +z when in range).

All indices returned here are 0-based; the reference is 1-based Julia.
"""
import numpy as np


def getpoints(lo, hi, n):
    """Node coordinates of one axis (src/grid.jl:27-29)."""
    return np.linspace(float(lo), float(hi), int(n))


def regulargrid1d(mins, maxs, ns, dy, dz):
    """src/grid.jl:79-96. Returns coords (1, n), neighbors (F, 2), areasoverlengths, volumes.

    The reference fills ``areasoverlengths`` with ``ns[1]`` entries although only
    ``ns[1]-1`` faces exist; the extra trailing entry is reproduced.
    """
    n = int(ns[0])
    xs = getpoints(mins[0], maxs[0], n)
    dx = xs[1] - xs[0]
    coords = xs[None, :].copy()
    nb = np.stack([np.arange(n - 1), np.arange(1, n)], axis=1).astype(np.int64)
    aol = np.full(n, dy * dz / dx)
    vol = np.full(n, dx * dy * dz)
    return coords, nb, aol, vol


def regulargrid2d(mins, maxs, ns, dz):
    """src/grid.jl:109-138: index i2 + ns[2]*(i1-1) (y fastest); faces +x then +y per cell."""
    n1, n2 = int(ns[0]), int(ns[1])
    xs = getpoints(mins[0], maxs[0], n1)
    ys = getpoints(mins[1], maxs[1], n2)
    dx = xs[1] - xs[0] if n1 > 1 else 1.0
    dy = ys[1] - ys[0] if n2 > 1 else 1.0
    i1, i2 = np.meshgrid(np.arange(n1), np.arange(n2), indexing="ij")
    lin = (i2 + n2 * i1).ravel()
    coords = np.empty((2, n1 * n2))
    coords[0, lin] = xs[i1.ravel()]
    coords[1, lin] = ys[i2.ravel()]
    # per-cell candidate faces in order (+x, +y); keep the in-range ones
    cand_b = np.stack([lin + n2, lin + 1], axis=1)
    valid = np.stack([i1.ravel() < n1 - 1, i2.ravel() < n2 - 1], axis=1)
    a = np.repeat(lin[:, None], 2, axis=1)[valid]
    b = cand_b[valid]
    aolc = np.broadcast_to(np.array([dy * dz / dx, dx * dz / dy]), valid.shape)[valid]
    nb = np.stack([a, b], axis=1).astype(np.int64)
    vol = np.full(n1 * n2, dx * dy * dz)
    return coords, nb, aolc.copy(), vol


def regulargrid3d(mins, maxs, ns):
    """src/grid.jl:150-188: index i3 + ns3*(i2-1) + ns3*ns2*(i1-1) (z fastest);
    faces per cell in the order +x, +y, +z when in range."""
    n1, n2, n3 = (int(v) for v in ns)
    xs = getpoints(mins[0], maxs[0], n1)
    ys = getpoints(mins[1], maxs[1], n2)
    zs = getpoints(mins[2], maxs[2], n3)
    # a single-node axis has no spacing in the reference (it indexes xs[2]); use 1
    dx, dy, dz = (v[1] - v[0] if len(v) > 1 else 1.0 for v in (xs, ys, zs))
    N = n1 * n2 * n3
    i1, i2, i3 = np.meshgrid(np.arange(n1), np.arange(n2), np.arange(n3), indexing="ij")
    i1 = i1.ravel(); i2 = i2.ravel(); i3 = i3.ravel()
    lin = i3 + n3 * i2 + n3 * n2 * i1  # equals arange(N) in this ordering
    coords = np.empty((3, N))
    coords[0, lin] = xs[i1]
    coords[1, lin] = ys[i2]
    coords[2, lin] = zs[i3]
    cand_b = np.stack([lin + n3 * n2, lin + n3, lin + 1], axis=1)
    valid = np.stack([i1 < n1 - 1, i2 < n2 - 1, i3 < n3 - 1], axis=1)
    a = np.repeat(lin[:, None], 3, axis=1)[valid]
    b = cand_b[valid]
    aolc = np.broadcast_to(np.array([dy * dz / dx, dx * dz / dy, dx * dy / dz]), valid.shape)[valid]
    nb = np.stack([a, b], axis=1).astype(np.int64)
    vol = np.full(N, dx * dy * dz)
    return coords, nb, aolc.copy(), vol


def load_uge(filename):
    """Read a PFLOTRAN explicit unstructured grid (.uge), src/grid.jl:38-65.

    Returns coords (3, N), volumes (N), neighbors (F, 2; 0-based), areas (F), lengths (F).
    File format: ``CELLS n`` then n lines ``id x y z volume``; ``CONNECTIONS m`` then m
    lines ``id1 id2 x y z area`` (ids 1-based in the file).
    """
    with open(filename) as fh:
        head = fh.readline().split()
        ncell = int(head[1])
        cells = np.loadtxt(fh, max_rows=ncell, ndmin=2) if ncell else np.zeros((0, 5))
        head = fh.readline().split()
        nconn = int(head[1])
        conns = np.loadtxt(fh, max_rows=nconn, ndmin=2) if nconn else np.zeros((0, 6))
    coords = np.ascontiguousarray(cells[:, 1:4].T)
    volumes = cells[:, 4].copy()
    nb = conns[:, 0:2].astype(np.int64) - 1
    areas = conns[:, 5].copy()
    lengths = np.sqrt(((coords[:, nb[:, 0]] - coords[:, nb[:, 1]]) ** 2).sum(axis=0))
    return coords, volumes, nb, areas, lengths


def write_uge(filename, coords, volumes, neighbors, areas):
    """Write a .uge file (the inverse of load_uge); neighbors are 0-based."""
    coords = np.asarray(coords)
    with open(filename, "w") as fh:
        fh.write(f"CELLS {coords.shape[1]}\n")
        for i in range(coords.shape[1]):
            fh.write("%d %.17g %.17g %.17g %.17g\n" % (i + 1, coords[0, i], coords[1, i], coords[2, i], volumes[i]))
        fh.write(f"CONNECTIONS {len(neighbors)}\n")
        for k, (a, b) in enumerate(neighbors):
            mid = 0.5 * (coords[:, a] + coords[:, b])
            fh.write("%d %d %.17g %.17g %.17g %.17g\n" % (a + 1, b + 1, mid[0], mid[1], mid[2], areas[k]))


def getfreenodes(n, dirichletnodes):
    """src/utilities.jl:10-24 (0-based): isfreenode, node->free index (-1 if Dirichlet), free->node."""
    isfree = np.ones(int(n), dtype=bool)
    isfree[np.asarray(dirichletnodes, dtype=np.int64)] = False
    node2free = np.full(int(n), -1, dtype=np.int64)
    free2node = np.nonzero(isfree)[0].astype(np.int64)
    node2free[free2node] = np.arange(free2node.size, dtype=np.int64)
    return isfree, node2free, free2node


def addboundaryconditions(hfree, dirichletnodes, dirichleths, isfreenode, nodei2freenodei):
    """src/utilities.jl:38-40."""
    h = np.array(dirichleths, dtype=np.float64, copy=True)
    h[isfreenode] = np.asarray(hfree)[nodei2freenodei[isfreenode]]
    return h


def fracture_network(nfrac, L, h, seed, smin=None, smax=None, alpha=2.6, aperture=1e-3):
    """A seeded synthetic discrete fracture network mesh, a stand-in for the dfnWorks meshes that
    DPFEHM reads with load_uge (examples/fracture_network_solver_scaling): square planar fractures
    with power-law side lengths (density s^-alpha on [smin, smax]), uniform centres in [0, L]^3 and
    uniformly random orientations, each meshed as a 2-D grid of cells of spacing h. Cells of one
    fracture are joined to their four in-plane neighbours (area h * aperture, length h); where two
    fractures cross, every cell of one that lies within h / 2 of the other's plane and inside it is
    joined to the nearest cell of the other (area h * aperture over the distance between the two
    centres, at least h / 2). Only the largest connected component is kept.

    Returns coords (3, N), volumes (N), neighbors (F, 2; 0-based), areas (F) and lengths (F) as
    load_uge does (areasoverlengths = areas / lengths), and the fracture of every cell (N). Degrees
    run from 2 at fracture corners to far above the in-plane four on cells that many fractures cross.
    """
    rng = np.random.default_rng(seed)
    smin = 4.0 * h if smin is None else smin
    smax = 0.5 * L if smax is None else smax
    a1 = 1.0 - alpha
    s = (smin ** a1 + rng.uniform(size=nfrac) * (smax ** a1 - smin ** a1)) ** (1.0 / a1)
    cen = rng.uniform(0.0, L, (nfrac, 3))
    nrm = rng.standard_normal((nfrac, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    ref = np.where(np.abs(nrm[:, :1]) < 0.9, np.array([[1.0, 0.0, 0.0]]), np.array([[0.0, 1.0, 0.0]]))
    u = np.cross(nrm, ref)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    v = np.cross(nrm, u)
    th = rng.uniform(0, 2 * np.pi, nfrac)[:, None]
    u, v = np.cos(th) * u + np.sin(th) * v, -np.sin(th) * u + np.cos(th) * v
    m = np.maximum(2, np.round(s / h).astype(np.int64))  # cells per side
    off = np.concatenate([[0], np.cumsum(m * m)])
    N0 = int(off[-1])
    frac = np.repeat(np.arange(nfrac), m * m)
    loc = np.arange(N0) - off[frac]
    ii, jj = loc // m[frac], loc % m[frac]
    half = 0.5 * m[frac]
    coords = (cen[frac] + ((ii + 0.5 - half) * h)[:, None] * u[frac] + ((jj + 0.5 - half) * h)[:, None] * v[frac])
    # in-plane neighbours
    ex, ey = np.nonzero(ii < m[frac] - 1)[0], np.nonzero(jj < m[frac] - 1)[0]
    a_list, b_list, kind = [ex, ey], [ex + m[frac[ex]], ey + 1], [np.zeros(len(ex), bool), np.zeros(len(ey), bool)]
    # crossings: candidate pairs whose bounding spheres overlap
    rad = 0.5 * np.sqrt(2.0) * m * h
    for A in range(nfrac):
        d = np.linalg.norm(cen - cen[A], axis=1)
        cand = np.nonzero((d < rad + rad[A]) & (np.arange(nfrac) != A))[0]
        if len(cand) == 0:
            continue
        cells = np.arange(off[A], off[A + 1])
        for B in cand:
            rel = coords[cells] - cen[B]
            dist = rel @ nrm[B]
            pu, pv = rel @ u[B], rel @ v[B]
            hb = 0.5 * m[B] * h
            near = (np.abs(dist) < 0.5 * h) & (np.abs(pu) < hb) & (np.abs(pv) < hb)
            if not near.any():
                continue
            ib = np.clip(np.floor(pu[near] / h + 0.5 * m[B]).astype(np.int64), 0, m[B] - 1)
            jb = np.clip(np.floor(pv[near] / h + 0.5 * m[B]).astype(np.int64), 0, m[B] - 1)
            a_list.append(cells[near])
            b_list.append(off[B] + ib * m[B] + jb)
            kind.append(np.ones(int(near.sum()), bool))
    a, b, cross = np.concatenate(a_list), np.concatenate(b_list), np.concatenate(kind)
    # one face per unordered pair
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    _, first = np.unique(lo * N0 + hi, return_index=True)
    lo, hi, cross = lo[first], hi[first], cross[first]
    # the largest connected component
    import scipy.sparse as sp
    from scipy.sparse.csgraph import connected_components
    G = sp.coo_matrix((np.ones(len(lo)), (lo, hi)), shape=(N0, N0))
    _, lab = connected_components(G, directed=False)
    keep = lab == np.argmax(np.bincount(lab))
    newid = np.full(N0, -1, np.int64)
    newid[keep] = np.arange(int(keep.sum()))
    ek = keep[lo] & keep[hi]
    nb = np.stack([newid[lo[ek]], newid[hi[ek]]], axis=1)
    coords = np.ascontiguousarray(coords[keep].T)
    lengths = np.sqrt(((coords[:, nb[:, 0]] - coords[:, nb[:, 1]]) ** 2).sum(axis=0))
    lengths = np.where(cross[ek], np.maximum(lengths, 1e-9 * h), h)
    # crossings: area over length = h aperture / max(length, h / 2)
    areas = np.where(cross[ek], h * aperture * lengths / np.maximum(lengths, 0.5 * h), h * aperture)
    volumes = np.full(coords.shape[1], h * h * aperture)
    return coords, volumes, nb, areas, lengths, frac[keep]
