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


def test_face_flux_is_antisymmetric_bit_for_bit():
    """The marching product computes each face flux c (p_i - p_j) once and hands its negation to
    the neighbour. That equals the neighbour's own term c (p_j - p_i) bit for bit (up to the sign
    of a zero) because the double-float difference and product are odd: round to nearest is
    symmetric and the two-sum error is exact."""
    rng = np.random.default_rng(11)
    n = 200000
    base = rng.normal(0.0, 1.0, n) * 10.0 ** rng.integers(-6, 3, n)
    a64 = base + rng.normal(0.0, 1.0, n) * 10.0 ** rng.integers(-16, 0, n) * np.abs(base)
    b64 = base.copy()
    a, b = _split(a64), _split(b64)
    c = _split(np.exp(rng.normal(-9.0, 2.0, n)))
    ab, ba = df_sub(a, b), df_sub(b, a)
    f_ab, f_ba = df_mul(c, ab), df_mul(c, ba)
    for k in range(2):
        assert np.array_equal(ab[k], -ba[k])
        assert np.array_equal(f_ab[k], -f_ba[k])


def split48_reference(v):
    """The bits of the library's split48 (integer-only 48-bit split), in numpy: v48 is v rounded to
    48 significant bits (half of the 5 dropped bits added, then dropped: to nearest, ties away from
    zero), hi its top 24 (exactly a float), lo = v48 - hi (exactly a float, a zero carrying v's
    sign); ok where v is zero or 2^-79 <= |v48| < 2^128."""
    v = np.asarray(v, dtype=F64)
    u0 = v.view(np.uint64)
    zero = (u0 << np.uint64(1)) == 0
    special = ((u0 >> np.uint64(52)) & np.uint64(0x7FF)) == np.uint64(0x7FF)
    u = np.where(zero, u0, (u0 + np.uint64(0x10)) & ~np.uint64(0x1F))
    e = ((u >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    ok = zero | (~special & (e != 0) & (e - 1023 >= -79) & (e - 1023 <= 127))
    v48 = np.where(ok, u.view(F64), 0.0)
    hi64 = np.where(ok, (u & ~np.uint64((1 << 29) - 1)).view(F64), 0.0)
    hi = hi64.astype(F32)
    lo = (v48 - hi64).astype(F32)
    lo = np.where(lo == 0, np.copysign(F32(0.0), v).astype(F32), lo)  # a zero lo carries v's sign
    return hi, lo, v48, ok


def test_split48_reference_is_exact():
    rng = np.random.default_rng(5)
    v = rng.normal(0.0, 1.0, 100000) * 10.0 ** rng.integers(-15, 20, 100000)
    hi, lo, v48, ok = split48_reference(v)
    assert ok.all()
    assert np.array_equal(hi.astype(F64) + lo.astype(F64), v48)     # exact in float64
    assert np.all(np.abs(v48 - v) <= np.abs(v) * 2.0 ** -48)          # rounded to nearest
    # nearly unbiased: only the ties (1 in 32) round away from zero, 1.1e-16 on average (truncation: 3.6e-15)
    assert abs(np.mean((v48 - v) / v)) < 2e-16
