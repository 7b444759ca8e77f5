"""CPU restatement of the library's Matern (nu = 1) field sampler (dpf_sampler.cu), in float64 numpy.

TEST INFRASTRUCTURE ONLY: the checker of dpf_batch_sample_logk, imported by tests/ and never by the
shipped library. The reference samples its fields on the host with GaussianRandomFields.jl's
Karhunen-Loeve expansion (examples/gw_multigrid_inverse/inputdeck.jl:58-105, an external package
absent here); parity of the solves does not depend on the sampler, since the GPU and the solver
oracle consume the same saved field. This file restates the library's own method so that its GPU
output can be checked draw for draw:

  * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC 2011): ten rounds of two 32x32->64-bit
    multiplications by 0xD2511F53 and 0xCD9E8D57 with the key bumped by the Weyl constants
    0x9E3779B9 and 0xBB67AE85; pinned by the generator's published known-answer vectors
    (tests/test_oracle.py);
  * mode k of a problem: counters (k, 0, T, 0) and (k, 1, T, 0), T = 0x4d415445, key = the seed's low
    and high words; uniforms (x + 0.5) 2^-32; z ~ N(0, I_3) by Box-Muller; G = -log(u) ~ Gamma(1, 1);
    w = z / (ell sqrt(G)) (the Matern spectral density (2/ell^2 + |w|^2)^-(5/2) as a Gaussian scale
    mixture); phase phi = 2 pi u;
  * f(x) = mean + sigma sqrt(2 / M) sum_k cos(w_k . x + phi_k), cells at x0 + i dx.
"""
import numpy as np

M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
TAG = 0x4d415445
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10 over uint32-valued arrays; returns the four output words (uint64)."""
    c = [np.asarray(x, dtype=np.uint64) & _MASK for x in (c0, c1, c2, c3)]
    k0 = np.asarray(k0, dtype=np.uint64) & _MASK
    k1 = np.asarray(k1, dtype=np.uint64) & _MASK
    for _ in range(10):
        p0 = np.uint64(M0) * c[0]
        p1 = np.uint64(M1) * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & _MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & _MASK
        c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
        k0 = (k0 + np.uint64(W0)) & _MASK
        k1 = (k1 + np.uint64(W1)) & _MASK
    return c


def _u01(x):
    return (x.astype(np.float64) + 0.5) * 2.0 ** -32


def modes(seed, ell, M):
    """Frequencies (M, 3) and phases (M,) of one field."""
    k = np.arange(M, dtype=np.uint64)
    s = np.uint64(seed)
    k0, k1 = s & _MASK, s >> np.uint64(32)
    a = philox4x32_10(k, 0, TAG, 0, k0, k1)
    b = philox4x32_10(k, 1, TAG, 0, k0, k1)
    r1 = np.sqrt(-2.0 * np.log(_u01(a[0])))
    r2 = np.sqrt(-2.0 * np.log(_u01(a[2])))
    z = np.stack([r1 * np.cos(2 * np.pi * _u01(a[1])), r1 * np.sin(2 * np.pi * _u01(a[1])),
                  r2 * np.cos(2 * np.pi * _u01(a[3]))], axis=1)
    G = -np.log(_u01(b[0]))
    w = z / (ell * np.sqrt(G))[:, None]
    return w, 2 * np.pi * _u01(b[1])


def field(ns, mins, maxs, ell, sigma, mean, seed, M):
    """The field on regulargrid3d's cells (flat, z fastest), float64."""
    ns = [int(n) for n in ns]
    dx = [(maxs[d] - mins[d]) / (ns[d] - 1) if ns[d] > 1 else 1.0 for d in range(3)]
    w, phi = modes(seed, ell, M)
    ax = [mins[d] + dx[d] * np.arange(ns[d]) for d in range(3)]
    X, Y, Z = np.meshgrid(ax[0], ax[1], ax[2], indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    acc = np.zeros(len(pts))
    for j in range(0, M, 64):  # modest memory
        acc += np.cos(pts @ w[j:j + 64].T + phi[j:j + 64]).sum(axis=1)
    return mean + sigma * np.sqrt(2.0 / M) * acc


def matern_correlation(r, ell):
    """Matern (nu = 1) correlation (kappa r) K_1(kappa r), kappa = sqrt(2) / ell."""
    from scipy.special import kv
    x = np.sqrt(2.0) * np.asarray(r, dtype=np.float64) / ell
    with np.errstate(invalid="ignore"):
        c = x * kv(1, x)
    return np.where(x > 0, c, 1.0)
