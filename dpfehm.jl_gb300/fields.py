"""Seeded synthetic log-conductivity fields with Matern covariance.

The reference samples log-conductivity with GaussianRandomFields' Karhunen-Loeve
expansion (examples/gw_steadystate_3d/inputdeck.jl:30-36), a package absent here.
This module draws a stationary Gaussian field with Matern covariance
    C(r) = sigma^2 2^(1-nu)/Gamma(nu) (sqrt(2 nu) r / ell)^nu K_nu(sqrt(2 nu) r / ell)
by spectral (circulant-embedding style) synthesis on a padded periodic grid: white
noise is filtered by the square root of the Matern spectral density
    S(k) proportional to (2 nu / ell^2 + |k|^2)^-(nu + d/2)
normalised so each point has variance sigma^2. The GPU solve and the oracle both
consume the same saved field, so parity does not depend on this sampler.
"""
import numpy as np


def matern_field(ns, spacings, ell, sigma, mean, seed, nu=1.0):
    """Return an array of shape ``ns`` (node-centred axes with the given spacings)."""
    ns = tuple(int(n) for n in ns)
    d = len(ns)
    rng = np.random.default_rng(seed)
    pads = []
    for n, h in zip(ns, spacings):
        p = int(n + np.ceil(1.5 * ell / h))
        pads.append(p + (p % 2))
    freqs = np.meshgrid(*[np.fft.fftfreq(p, h) for p, h in zip(pads, spacings)], indexing="ij", sparse=True)
    k2 = sum((2.0 * np.pi * f) ** 2 for f in freqs)
    spec = (2.0 * nu / ell ** 2 + k2) ** (-(nu + d / 2.0))
    spec /= spec.mean()
    w = rng.standard_normal(pads)
    field = np.real(np.fft.ifftn(np.fft.fftn(w) * np.sqrt(spec)))
    sl = tuple(slice(0, n) for n in ns)
    return mean + sigma * np.ascontiguousarray(field[sl])


def _spacing(lo, hi, n):
    return (hi - lo) / (n - 1) if n > 1 and hi != lo else 1.0


def layered_logk(ns3, mins, maxs, ell, sigma, mean, seed):
    """2-D field in (x, y) copied to every z layer; returned flat in cell order (z fastest)."""
    n1, n2, n3 = ns3
    sp = [_spacing(mins[i], maxs[i], ns3[i]) for i in range(2)]
    f2 = matern_field((n1, n2), sp, ell, sigma, mean, seed)
    return np.repeat(f2[:, :, None], n3, axis=2).ravel()


def volume_logk(ns3, mins, maxs, ell, sigma, mean, seed):
    """Fully 3-D field; returned flat in cell order (z fastest)."""
    sp = [_spacing(mins[i], maxs[i], ns3[i]) for i in range(3)]
    return matern_field(ns3, sp, ell, sigma, mean, seed).ravel()


def volume_logk_torch(ns3, mins, maxs, ell, sigma, mean, seed, device="cuda"):
    """The spectral synthesis of matern_field (nu = 1) on a torch device (FFT by torch), for
    large batches of synthetic inputs; white noise from torch's generator, so the draws
    differ from the numpy sampler's for the same seed, and the periodic padding is capped
    at 2n per axis. Returns a flat float64 tensor (z fastest)."""
    import torch
    ns = tuple(int(n) for n in ns3)
    sp = [_spacing(mins[i], maxs[i], ns[i]) for i in range(3)]
    pads = []
    for n, h in zip(ns, sp):
        p = int(n + min(np.ceil(1.5 * ell / h), 2 * n))  # padding capped at 2n for long correlation lengths
        pads.append(p + (p % 2))
    f = [torch.fft.fftfreq(p, h, dtype=torch.float64, device=device) for p, h in zip(pads, sp)]
    k2 = ((2 * np.pi * f[0])[:, None, None] ** 2 + (2 * np.pi * f[1])[None, :, None] ** 2 +
          (2 * np.pi * f[2])[None, None, :] ** 2)
    spec = (2.0 / ell ** 2 + k2) ** (-(1.0 + 1.5))
    spec = spec / spec.mean()
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    w = torch.randn(pads, dtype=torch.float64, device=device, generator=g)
    field = torch.fft.ifftn(torch.fft.fftn(w) * torch.sqrt(spec)).real
    return (mean + sigma * field[: ns[0], : ns[1], : ns[2]]).contiguous().reshape(-1)
