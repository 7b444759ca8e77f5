"""The GPU Matern (nu = 1) field sampler (dpf_batch_sample_logk) against its float64 CPU restatement,
its reproducibility, and the fused draw-solve-differentiate loop.

Tolerances: a field is summed in FP32 on the GPU, so it agrees with the float64 restatement to
1e-4 absolute (sigma of order 1); reproducibility is bitwise.
"""
import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu


def _batch(pkg, grids, **kw):
    mins = [(0.5 * k, -1.0, 2.0) for k in range(len(grids))]
    maxs = [(m[0] + 0.5 * (g[0] - 1), m[1] + 0.5 * (g[1] - 1), m[2] + 0.5 * (g[2] - 1)) for m, g in zip(mins, grids)]
    dns = [[int(np.prod(g)) - 1] for g in grids]
    return pkg.GroundwaterBatch(grids, mins, maxs, dns, **kw), mins, maxs


def test_sampler_matches_restatement_and_repeats_bitwise(gpu_lib):
    import matern_oracle as mo
    pkg = gpu_lib
    grids = [(12, 10, 6), (20, 7, 9), (12, 10, 6)]
    B, mins, maxs = _batch(pkg, grids, precision="mixed")
    seeds = [11, 2 ** 40 + 7, 11]
    ell, sig, mu, M = [3.0, 5.0, 3.0], [1.5, 0.7, 1.5], [-9.0, -8.0, -9.0], 256
    f1 = B.sample_logk(seeds, ell, sig, mu, nmodes=M, out="host")
    f2 = B.sample_logk(seeds, ell, sig, mu, nmodes=M, out="cuda").cpu().numpy()
    assert np.array_equal(f1, f2)  # host and device outputs, two calls: bit for bit
    off = B.cell_offsets
    for p, g in enumerate(grids):
        ref = mo.field(g, mins[p], maxs[p], ell[p], sig[p], mu[p], seeds[p], M)
        assert np.max(np.abs(f1[off[p]:off[p + 1]] - ref)) < 1e-4, p
    # a field depends on its seed, grid and modes only, not on its place in the batch: the third
    # grid alone in a batch of its own gives the same values bit for bit
    C = pkg.GroundwaterBatch([grids[2]], [mins[2]], [maxs[2]], [[int(np.prod(grids[2])) - 1]], precision="mixed")
    f3 = C.sample_logk([seeds[2]], ell[2], sig[2], mu[2], nmodes=M, out="host")
    assert np.array_equal(f3, f1[off[2]:off[3]])
    # a new seed changes that problem's field only
    f4 = B.sample_logk([12, 2 ** 40 + 7, 11], ell, sig, mu, nmodes=M, out="host")
    assert not np.array_equal(f4[off[0]:off[1]], f1[off[0]:off[1]])
    assert np.array_equal(f4[off[1]:], f1[off[1]:])
    B.close()
    C.close()


def test_sampler_statistics_on_a_large_grid(gpu_lib):
    """One field over a domain much larger than the correlation length: mean, standard deviation
    and the correlation between cells ell apart, against the Matern (nu = 1) values."""
    import matern_oracle as mo
    pkg = gpu_lib
    grid, ell, sig, mu = (200, 200, 25), 2.0, 2.0, -9.0
    B = pkg.GroundwaterBatch([grid], [(0.0, 0.0, 0.0)], [(99.5, 99.5, 12.0)], [[0]], precision="mixed")
    f = B.sample_logk([5], ell, sig, mu, nmodes=1024, out="host").reshape(grid)
    assert abs(f.mean() - mu) < 0.2 and abs(f.std() - sig) < 0.2
    a = (f - f.mean()) / f.std()
    lag = 4  # cells of 0.5 m: 2 m = ell
    c_x = np.mean(a[:-lag] * a[lag:])
    assert abs(c_x - mo.matern_correlation(lag * 0.5, ell)) < 0.08
    B.close()


@pytest.mark.parametrize("streams", [1, 2])
def test_fused_sample_and_solve(gpu_lib, orc, streams):
    """Fields drawn into the handle and solved with logK = None give the same heads and gradients,
    bit for bit, as the same fields passed explicitly; the heads match the oracle. A NULL logK
    before any draw is refused."""
    pkg = gpu_lib
    grids = [(20, 16, 6), (14, 12, 5), (24, 10, 8)]
    B, mins, maxs = _batch(pkg, grids, precision="mixed", reltol=1e-11, streams=streams)
    N = B.N
    dh, Qs = np.zeros(N), np.zeros(N)
    Qs[B.cell_offsets[:-1]] = 1e-4
    obs = [np.arange(0, int(np.prod(g)), 37) for g in grids]
    with pytest.raises(pkg.DPFError) as e:
        B.solve_grad_logk(None, dh, Qs, obs)
    assert e.value.code == pkg._lib.DPF_STATE
    seeds, ell, sig, mu = [3, 4, 5], 4.0, 1.0, -9.0
    field = B.sample_logk(seeds, ell, sig, mu, nmodes=512, out="host")
    B.sample_logk(seeds, ell, sig, mu, nmodes=512)  # into the handle
    h1, g1 = B.solve_grad_logk(None, dh, Qs, obs)
    h2, g2 = B.solve_grad_logk(field, dh, Qs, obs)
    h1, g1 = h1.cpu().numpy(), g1.cpu().numpy()
    assert np.array_equal(h1, h2) and np.array_equal(g1, g2)
    # the explicit field was staged over the drawn ones: a NULL logK is refused again
    with pytest.raises(pkg.DPFError) as e:
        B.solve_grad_logk(None, dh, Qs, obs)
    assert e.value.code == pkg._lib.DPF_STATE
    for p, g in enumerate(grids):
        _, nb, aol, _ = pkg.regulargrid3d(mins[p], maxs[p], g)
        a, b = B.cell_offsets[p], B.cell_offsets[p + 1]
        O = orc.Problem(b - a, nb, aol, [b - a - 1])
        ho = O.steady(orc.logk_to_faces(nb, field[a:b]), dh[a:b], Qs[a:b], reltol=1e-14)
        assert rel(h1[a:b], ho) < 1e-8, p
    B.close()
