"""Seeded Gaussian random fields by the FFT spectral (circulant-embedding) method.

Not in reference: the reference reads soil classes from files; the heterogeneous workloads need
continuous ln Ks / ln alpha fields.  A stationary field with exponential covariance
C(r) = exp(-sqrt((dx/lx)^2 + (dy/ly)^2 + (dz/lz)^2)) (lengths in cells) is drawn on the periodic
grid: the covariance evaluated at wrapped lags is diagonalised by the FFT, negative eigenvalues
are clipped to zero, and seeded white noise is coloured by the square-root spectrum.  The
realisation is then standardised to mean 0 and unit variance.
"""
from __future__ import annotations

import numpy as np


def _wrapped_lag(n: int) -> np.ndarray:
    k = np.arange(n, dtype=np.float64)
    return np.minimum(k, n - k)


def exponential_grf(shape, corr, seed: int) -> np.ndarray:
    """Standard-normal field of `shape` = (nz, ny, nx) with exponential covariance of
    correlation lengths `corr` = (lz, ly, lx) cells, seeded by `seed` (numpy PCG64)."""
    nz, ny, nx = shape
    lz, ly, lx = corr
    dz = _wrapped_lag(nz)[:, None, None] / lz
    dy = _wrapped_lag(ny)[None, :, None] / ly
    dx = _wrapped_lag(nx)[None, None, :] / lx
    cov = np.exp(-np.sqrt(dz * dz + dy * dy + dx * dx))
    lam = np.fft.rfftn(cov).real
    del cov
    np.maximum(lam, 0.0, out=lam)
    amp = np.sqrt(lam)
    del lam
    rng = np.random.Generator(np.random.PCG64(seed))
    noise = rng.standard_normal(shape)
    spec = np.fft.rfftn(noise)
    del noise
    spec *= amp
    field = np.fft.irfftn(spec, s=shape, axes=(0, 1, 2))
    field -= field.mean()
    field /= field.std()
    return np.ascontiguousarray(field)


def lnk_lnalpha_fields(shape, corr, seed_k: int, seed_a: int, ln_ks_mean: float, sigma_lnk: float,
                       ln_alpha_mean: float, sigma_lna: float, rho: float):
    """ln Ks = mean + sigma * xi_K;  ln alpha = mean + sigma_a (rho xi_K + sqrt(1-rho^2) xi')."""
    xk = exponential_grf(shape, corr, seed_k)
    xa = exponential_grf(shape, corr, seed_a)
    ln_ks = ln_ks_mean + sigma_lnk * xk
    ln_a = ln_alpha_mean + sigma_lna * (rho * xk + np.sqrt(1.0 - rho * rho) * xa)
    return ln_ks, ln_a
