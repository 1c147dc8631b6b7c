"""Seeded synthetic inputs of the benchmark workloads, in numpy alone.

This module imports nothing but numpy, so that a CPU-only caller (the CPU arm of the
benchmark, which runs Gridap's algorithm on the host) draws exactly the same coefficients
and sources as the device path without loading the CUDA library. `workloads.py` builds the
FE spaces around these arrays.

  - lognormal_inputs: kappa = exp(sigma g) per cell, g a unit-variance Gaussian random
    field of correlation length `corr_cells` (FFT filtering of white noise on the periodic
    cell grid, Gaussian covariance), sigma set so that max(kappa)/min(kappa) = contrast;
    f ~ N(0, 1) per node. Cells and nodes in Gridap's order (x fastest).
  - q2_jitter, elasticity_lame: node jitter of the Q2 workload and per-tet Lame
    coefficients of the elasticity workload.
  - sinsum_terms: the 2-D source f = sum_k a_k sin(pi m_k x) sin(pi n_k y), a_k ~ N(0, 1),
    m_k, n_k integers in 1..8.
"""
from __future__ import annotations

import numpy as np


def gaussian_random_field(shape, corr_cells: float, rng: np.random.Generator) -> np.ndarray:
    """Unit-variance stationary Gaussian field on a periodic cell grid with a Gaussian
    covariance of correlation length `corr_cells` cells (spectral filtering)."""
    white = rng.standard_normal(shape)
    k = [np.fft.fftfreq(n) * 2 * np.pi for n in shape]
    kk = np.zeros(shape)
    for d, kd in enumerate(k):
        sh = [1] * len(shape)
        sh[d] = shape[d]
        kk = kk + (kd.reshape(sh)) ** 2
    filt = np.exp(-0.25 * kk * corr_cells ** 2)
    g = np.real(np.fft.ifftn(np.fft.fftn(white) * filt))
    g -= g.mean()
    g /= g.std()
    return g


def lognormal_inputs(n: int = 128, seed: int = 5999, contrast: float = 1e4,
                     corr_cells: float = 8.0):
    """(kappa[n^3], f[(n+1)^3]) of the 3-D lognormal diffusion workload on n^3 cells."""
    rng = np.random.default_rng(seed)
    # cell grid in Gridap's cell order (x fastest): field indexed [k, j, i]
    g = gaussian_random_field((n, n, n), corr_cells, rng)
    sigma = np.log(contrast) / (g.max() - g.min())
    kappa = np.exp(sigma * (g - g.mean())).reshape(-1)
    f = rng.standard_normal((n + 1) ** 3)
    return kappa, f


def sinsum_terms(seed: int = 1) -> np.ndarray:
    """(8, 3) rows (a_k, m_k, n_k) of the 2-D sinusoid-sum source."""
    rng = np.random.default_rng(seed)
    return np.column_stack([rng.standard_normal(8), rng.integers(1, 9, 8),
                            rng.integers(1, 9, 8)]).astype(np.float64)


def q2_jitter(n: int = 64, seed: int = 2, amplitude: float = 0.2) -> np.ndarray:
    """Node displacements ((n+1)^3, 3) uniform in (-amplitude h, amplitude h)^3, h = 1/n, of
    the jittered Q2 workload; the model applies them to interior nodes only."""
    rng = np.random.default_rng(seed)
    return rng.uniform(-amplitude, amplitude, ((n + 1) ** 3, 3)) / n


def elasticity_lame(ncells: int, seed: int = 3) -> np.ndarray:
    """(ncells, 2) Lame coefficients (lambda, mu) = exp(N(0, 1)) normalised to mean 1."""
    rng = np.random.default_rng(seed)
    lame = np.exp(rng.standard_normal((ncells, 2)))
    lame /= lame.mean(axis=0)
    return lame


def lognormal_free_dofs(n: int) -> int:
    """Free dofs of the Q1 space on n^3 cells with Dirichlet data on the whole boundary."""
    return (n - 1) ** 3
