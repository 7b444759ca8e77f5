"""The double-float (hi + lo float pair) arithmetic of the mixed-precision CG product, emulated
in numpy float32 with the kernel's operation order (no GPU): on a smooth search direction near
a constant, the case that makes the operator nearly singular, the flux-form product keeps
about 48 bits, while the same product in plain FP32 loses almost everything."""
import numpy as np

F32, F64 = np.float32, np.float64


def _two_sum(a, b):
    s = (a + b).astype(F32)
    bb = (s - a).astype(F32)
    return s, ((a - (s - bb)) + (b - bb)).astype(F32)


def _quick(a, b):
    s = (a + b).astype(F32)
    return s, (b - (s - a)).astype(F32)


def df_add(a, b):
    s, e = _two_sum(a[0], b[0])
    return _quick(s, (e + (a[1] + b[1])).astype(F32))


def df_sub(a, b):
    return df_add(a, (-b[0], -b[1]))


def _fma(a, b, c):
    # a*b of two floats is exact in float64; one rounding to float32 as a fused multiply-add
    return (a.astype(F64) * b.astype(F64) + c.astype(F64)).astype(F32)


def df_mul(a, b):
    p = (a[0] * b[0]).astype(F32)
    e = _fma(a[0], b[0], -p)
    e = _fma(a[0], b[1], e)
    e = _fma(a[1], b[0], e)
    return _quick(p, e)


def _split(x):
    h = x.astype(F32)
    return h, (x - h.astype(F64)).astype(F32)


def _grid_operator(ns, seed):
    """Upper-face conductances (zero past the last cell of each axis) and the leak of one
    Dirichlet-adjacent cell, on an nx x ny x nz grid, z fastest."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = ns
    c = {}
    for ax, n_axis in (("z", 2), ("y", 1), ("x", 0)):
        v = np.exp(rng.normal(-9.0, 1.0, ns))
        idx = [slice(None)] * 3
        idx[n_axis] = -1
        v[tuple(idx)] = 0.0
        c[ax] = v.ravel()
    leak = np.zeros(nx * ny * nz)
    leak[-1] = 1e-4
    return c, leak


def _neighbours(ns):
    nx, ny, nz = ns
    i = np.arange(nx * ny * nz)
    iz, iy, ix = i % nz, (i // nz) % ny, i // (ny * nz)
    out = {}
    for ax, co, n, s in (("z", iz, nz, 1), ("y", iy, ny, nz), ("x", ix, nx, ny * nz)):
        out[ax] = (np.where(co + 1 < n, i + s, i), np.where(co > 0, i - s, i))
    return i, out


def test_double_float_flux_product_keeps_48_bits_on_a_smooth_direction():
    ns = (16, 12, 6)
    c, leak = _grid_operator(ns, 3)
    i, nbr = _neighbours(ns)
    N = len(i)
    p64 = 1.0 + 1e-9 * np.sin(np.linspace(0.0, 7.0, N)) + 1e-13 * np.random.default_rng(4).standard_normal(N)
    P = _split(p64)
    Pd = P[0].astype(F64) + P[1].astype(F64)           # the double-float value, exactly
    C = {k: _split(v) for k, v in c.items()}
    Cd = {k: v[0].astype(F64) + v[1].astype(F64) for k, v in C.items()}
    L = _split(leak)
    Ld = L[0].astype(F64) + L[1].astype(F64)
    # the exact product of the double-float operands
    ex = Ld.astype(np.longdouble) * Pd
    for ax, (up, dn) in nbr.items():
        ex += Cd[ax].astype(np.longdouble) * (Pd - Pd[up]) + Cd[ax][dn].astype(np.longdouble) * (Pd - Pd[dn])
    # the kernel's order: leak first, then each axis' upper and lower faces, each term renormalised
    pi = (P[0][i], P[1][i])
    acc = df_mul(L, pi)
    for ax, (up, dn) in nbr.items():
        acc = df_add(acc, df_mul(C[ax], df_sub(pi, (P[0][up], P[1][up]))))
        acc = df_add(acc, df_mul((C[ax][0][dn], C[ax][1][dn]), df_sub(pi, (P[0][dn], P[1][dn]))))
    got = acc[0].astype(F64) + acc[1].astype(F64)
    e = ex.astype(F64)
    # measured on the cells without a leak, where (A p)_i is all flux (the leak cell would dominate)
    m = leak == 0
    nrm = float(np.linalg.norm(e[m]))
    assert np.linalg.norm(got[m] - e[m]) <= 1e-12 * nrm           # emulated: 1.5e-15
    # plain FP32 on the same operands: the differences p_i - p_j vanish at 2^-24
    p32 = Pd.astype(F32)
    q32 = (leak.astype(F32) * p32).astype(F32)
    for ax, (up, dn) in nbr.items():
        c32 = c[ax].astype(F32)
        q32 = (q32 + c32 * (p32 - p32[up]) + c32[dn] * (p32 - p32[dn])).astype(F32)
    assert np.linalg.norm(q32[m].astype(F64) - e[m]) >= 0.5 * nrm     # emulated: 1.0
