"""The C-ABI library loads, exports every symbol declared in include/*.h, and its
host-only pieces work without a GPU (no compute calls here)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    for hdr in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(hdr).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(dpf_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def lib(pkg):
    import __graft_entry__ as g
    g._load_build_module().build()
    return pkg.load()


def test_header_declares_entry_points():
    names = _declared_symbols()
    for must in ["dpf_create", "dpf_steady_forward", "dpf_steady_adjoint", "dpf_logk_to_faces",
                 "dpf_transient_forward", "dpf_transient_adjoint", "dpf_batch_create", "dpf_destroy",
                 "dpf_last_error"]:
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in _declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header(pkg):
    from importlib import import_module
    _lib = import_module(pkg.__name__ + "._lib")
    assert set(_declared_symbols()) <= set(_lib.SIGNATURES)


def _c_options_fields():
    """(name, type) of struct dpf_options in include/dpfehm_gpu.h, in declaration order."""
    src = open(os.path.join(ROOT, "include", "dpfehm_gpu.h")).read()
    body = re.search(r"typedef struct dpf_options \{(.*?)\} dpf_options;", src, flags=re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    return [(m.group(2), m.group(1)) for m in re.finditer(r"\b(double|int)\s+([a-z0-9_]+)\s*;", body)]


def test_options_layout_matches_bindings(pkg):
    """The options struct is passed by pointer from Python (ctypes) and Julia (ccall with
    Ref{Options}): both mirrors must list the C fields in the same order with the same types,
    or every option after a mismatch would be read from the wrong bytes."""
    from importlib import import_module
    c_fields = _c_options_fields()
    assert len(c_fields) >= 20
    ct = {ctypes.c_double: "double", ctypes.c_int: "int"}
    _lib = import_module(pkg.__name__ + "._lib")
    py_fields = [(n, ct[t]) for n, t in _lib.Options._fields_]
    assert py_fields == c_fields
    jl = open(os.path.join(ROOT, "dpfehm.jl_gb300", "julia", "DPFEHMGPU.jl")).read()
    body = re.search(r"mutable struct Options\n(.*?)\nend", jl, flags=re.S).group(1)
    jt = {"Cdouble": "double", "Cint": "int"}
    jl_fields = [(m.group(1), jt[m.group(2)]) for m in re.finditer(r"^\s*([a-z0-9_]+)::(Cdouble|Cint)\s*$", body,
                                                                    flags=re.M)]
    assert jl_fields == c_fields
    # the Julia constructor call that default_options fills must pass one value per field
    ctor = re.search(r"o = Options\(([^)]*)\)", jl).group(1)
    assert len(ctor.split(",")) == len(c_fields)


def test_default_options(pkg, lib):
    o = pkg.default_options()
    assert o.reltol == 1e-10 and o.maxiter == 500 and o.precision == pkg.PREC_FP64
    assert o.cheb_degree == 0 and o.coarse_scale == 0.0 and o.max_coarse == 64 and o.blocks_per_sm == 16 and o.tail_cells == 4096 and o.plane == 1 and o.plane_cells == 1024
    assert o.plane_blocks_per_sm == 2 and o.df_plane_cells == 256 and o.df_plane_blocks_per_sm == 8
    assert o.tail_cluster == 1
    assert o.plane_levels == 0
    assert o.streams == 0
    assert o.fuse == -1
    assert o.solver == pkg.SOLVER_CG


@pytest.mark.parametrize("ns", [(4, 3, 2), (7, 1, 5), (1, 6, 3), (5, 4, 1), (9, 1, 1), (1, 1, 8), (3, 3, 3)])
def test_detect_regular3d(pkg, lib, ns):
    coords, nb, aol, vol = pkg.regulargrid3d((0, 0, 0), (1.5, 2.0, 3.0), [max(n, 1) for n in ns])
    N = coords.shape[1]
    a = np.ascontiguousarray(nb[:, 0])
    b = np.ascontiguousarray(nb[:, 1])
    dims = (ctypes.c_int * 3)()
    a3 = (ctypes.c_double * 3)()
    ok = lib.dpf_detect_regular3d(N, len(nb), a.ctypes.data, b.ctypes.data, aol.ctypes.data, dims, a3)
    assert ok == 1
    assert np.prod(list(dims)) == N
    # the detected grid regenerates the same face list (a unit axis may be reported in another slot)
    _, nb2, aol2, _ = pkg.regulargrid3d((0, 0, 0), (1, 1, 1), list(dims))
    assert np.array_equal(nb2, nb)
    d = np.array(list(dims))
    for k in range(3):
        if d[k] > 1:
            sel = (nb2[:, 1] - nb2[:, 0]) == int(np.prod(d[k + 1:]))
            assert np.allclose(aol[sel], a3[k])


def test_detect_rejects_general_graph(pkg, lib):
    coords, nb, aol, vol = pkg.regulargrid3d((0, 0, 0), (1, 1, 1), (4, 4, 4))
    nb2 = nb.copy()
    nb2[[3, 4]] = nb2[[4, 3]]  # reordered faces are no longer the regulargrid3d list
    a, b = np.ascontiguousarray(nb2[:, 0]), np.ascontiguousarray(nb2[:, 1])
    aol = np.ascontiguousarray(aol)
    assert lib.dpf_detect_regular3d(64, len(nb2), a.ctypes.data, b.ctypes.data, aol.ctypes.data, None, None) == 0
    aol2 = aol.copy()
    aol2[5] *= 1.01  # non-uniform areas over lengths
    a, b = np.ascontiguousarray(nb[:, 0]), np.ascontiguousarray(nb[:, 1])
    assert lib.dpf_detect_regular3d(64, len(nb), a.ctypes.data, b.ctypes.data, aol2.ctypes.data, None, None) == 0


def test_regulargrid2d_is_regular(pkg, lib):
    coords, nb, aol, vol = pkg.regulargrid2d((-1, -1), (1, 1), (6, 5), 3.0)
    a, b = np.ascontiguousarray(nb[:, 0]), np.ascontiguousarray(nb[:, 1])
    dims = (ctypes.c_int * 3)()
    a3 = (ctypes.c_double * 3)()
    assert lib.dpf_detect_regular3d(30, len(nb), a.ctypes.data, b.ctypes.data, np.ascontiguousarray(aol).ctypes.data,
                                    dims, a3) == 1
    assert tuple(dims) == (6, 5, 1)


def test_missing_library_fails_loudly(pkg, tmp_path):
    from importlib import import_module
    _lib = import_module(pkg.__name__ + "._lib")
    with pytest.raises(OSError):
        saved = _lib._lib
        _lib._lib = None
        try:
            _lib.load(str(tmp_path / "nope.so"))
        finally:
            _lib._lib = saved


def test_create_without_device_reports_no_device(pkg, lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(pkg.DPFError) as e:
        pkg.GroundwaterProblem.regular3d((0, 0, 0), (1, 1, 1), (3, 3, 3), [26])
    assert e.value.code == 6


def test_autotune_rejects_mismatched_lists(lib, pkg):
    """The per-problem lists are checked against the problem count on the host, before any
    device call: a single observation list for a batch of two is an error, not a list
    that silently goes to the first problem."""
    dims = [(4, 4, 4), (4, 4, 4)]
    N = 128
    z = np.zeros(N)
    with pytest.raises(ValueError):
        pkg.autotune_batch(dims, [(0, 0, 0)] * 2, [(3, 3, 3)] * 2, [[63], [63]], z, z, z, [np.array([1, 2])])
    with pytest.raises(ValueError):
        pkg.autotune_batch(dims, [(0, 0, 0)] * 2, [(3, 3, 3)] * 2, [[63]], z, z, z, [np.array([1]), np.array([2])])


def _bandwidth(perm, edges):
    """Half-bandwidth of the couplings `edges` (pairs of original rows) under the band order perm
    (perm[k] = original row of band row k)."""
    pos = np.empty(len(perm), dtype=np.int64)
    pos[perm] = np.arange(len(perm))
    return int(np.abs(pos[edges[:, 0]] - pos[edges[:, 1]]).max()) if len(edges) else 0


def _grid_edges(nx, ny, nz, off):
    """The 7-point couplings of an nx x ny x nz grid (cells z fastest) from cell offset off."""
    idx = off + np.arange(nx * ny * nz).reshape(nx, ny, nz)
    pairs = [np.stack([idx[1:].ravel(), idx[:-1].ravel()], 1), np.stack([idx[:, 1:].ravel(), idx[:, :-1].ravel()], 1),
             np.stack([idx[:, :, 1:].ravel(), idx[:, :, :-1].ravel()], 1)]
    return np.concatenate(pairs)


@pytest.mark.parametrize("grids", [[(20, 16, 1), (9, 9, 9), (30, 4, 6)], [(7, 1, 1)], [(1, 1, 1), (3, 50, 2)],
                                   [(200, 200, 25)]])
def test_band_order_grids(lib, grids):
    """The direct solver's band order for a batch of regular grids (host code, no device): a
    permutation of all cells, each grid's two shortest axes fastest, and the half-bandwidth it
    reports equal to the largest coupling distance, the largest product of a grid's two shorter
    extents."""
    dims = np.array(grids, dtype=np.int32).ravel()
    n = int(sum(a * b * c for a, b, c in grids))
    perm = np.empty(n, dtype=np.int64)
    w = ctypes.c_int64(-1)
    assert lib.dpf_debug_band_order_grids(len(grids), dims.ctypes.data, perm.ctypes.data, ctypes.byref(w)) == 0
    assert np.array_equal(np.sort(perm), np.arange(n))
    off, edges, expect = 0, [], 0
    for g in grids:
        edges.append(_grid_edges(*g, off))
        s = sorted(g)
        expect = max(expect, s[0] * s[1] if s[2] > 1 else 0)
        off += g[0] * g[1] * g[2]
    edges = np.concatenate(edges)
    assert w.value == _bandwidth(perm, edges) == expect
    assert lib.dpf_debug_band_order_grids(1, np.array([4, 0, 2], dtype=np.int32).ctypes.data, perm.ctypes.data,
                                          ctypes.byref(w)) == 1


def _csr(n, edges):
    a = np.concatenate([edges[:, 0], edges[:, 1]])
    b = np.concatenate([edges[:, 1], edges[:, 0]])
    order = np.lexsort((b, a))
    a, b = a[order], b[order]
    rp = np.zeros(n + 1, dtype=np.int32)
    np.add.at(rp, a + 1, 1)
    return np.cumsum(rp).astype(np.int32), b.astype(np.int32)


def test_band_order_graph_rcm(lib):
    """Reverse Cuthill-McKee on a shuffled 40 x 60 grid graph with a second component and isolated
    vertices (host code, no device): a permutation, the reported half-bandwidth equal to the
    largest coupling distance, and a band close to the grid's short side (the shuffled labels'
    band is thousands)."""
    rng = np.random.default_rng(3)
    g = _grid_edges(40, 60, 1, 0)
    tri = np.array([[0, 1], [1, 2], [2, 0]]) + 2400           # a second component
    n = 2400 + 3 + 5                                           # and five isolated vertices
    lab = rng.permutation(n)
    edges = lab[np.concatenate([g, tri])]
    rp, ci = _csr(n, edges)
    perm = np.empty(n, dtype=np.int64)
    w = ctypes.c_int64(-1)
    assert lib.dpf_debug_band_order_graph(n, rp.ctypes.data, ci.ctypes.data, perm.ctypes.data, ctypes.byref(w)) == 0
    assert np.array_equal(np.sort(perm), np.arange(n))
    assert w.value == _bandwidth(perm, edges)
    assert _bandwidth(np.arange(n), edges) > 1000
    assert 40 <= w.value <= 80
    bad = ci.copy()
    bad[0] = n
    assert lib.dpf_debug_band_order_graph(n, rp.ctypes.data, bad.ctypes.data, perm.ctypes.data, ctypes.byref(w)) == 1
