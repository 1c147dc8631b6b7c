"""Seeded synthetic problems with the shapes, sizes and value distributions of the
benchmark configurations (no dataset is involved; every input is generated here).

  - poisson_2d:      2-D Poisson on the unit square, 256 x 256 Q1 cells, quadrature degree
                     2, f = sum of 8 sinusoids with amplitudes ~ N(0,1) and integer
                     wavenumbers 1..8 (seed 1), homogeneous Dirichlet on "boundary".
  - lognormal_3d:    3-D diffusion on 128^3 Q1 cells, kappa = exp(sigma g) with g a
                     unit-variance Gaussian random field of correlation length 8h (FFT
                     filtering of white noise on the cell grid), sigma set so that
                     max(kappa)/min(kappa) = 1e4; f ~ N(0,1) per node; Dirichlet on
                     "boundary".
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .celldata import CellField, NodalField, SinSum
from .fespaces import FESpace, ReferenceFE, lagrangian
from .geometry import CartesianDiscreteModel, Measure, Triangulation
from .synthetic import (elasticity_lame, gaussian_random_field, lognormal_inputs,  # noqa: F401
                        q2_jitter, sinsum_terms)


@dataclass
class Workload:
    name: str
    model: CartesianDiscreteModel
    space: FESpace
    measure: Measure
    kappa: np.ndarray | None  # per cell
    source: object            # NodalField / SinSum / float
    rtol: float


def lognormal_3d(n: int = 128, seed: int = 5999, contrast: float = 1e4,
                 corr_cells: float = 8.0) -> Workload:
    model = CartesianDiscreteModel((0, 1, 0, 1, 0, 1), (n, n, n))
    V = FESpace(model, ReferenceFE(lagrangian, float, 1), dirichlet_tags="boundary")
    kappa, f = lognormal_inputs(n, seed, contrast, corr_cells)
    return Workload("lognormal_3d", model, V, Measure(Triangulation(model), 2), kappa,
                    NodalField(f), 1e-8)


def poisson_2d(n: int = 256, seed: int = 1) -> Workload:
    model = CartesianDiscreteModel((0, 1, 0, 1), (n, n))
    V = FESpace(model, ReferenceFE(lagrangian, float, 1), dirichlet_tags="boundary")
    terms = sinsum_terms(seed)
    return Workload("poisson_2d", model, V, Measure(Triangulation(model), 2), None,
                    SinSum(terms), 1e-10)


def coefficient(w: Workload):
    return None if w.kappa is None else CellField(w.kappa)


def batched_diffusion(nproblems: int = 256, seed: int = 7, nmin: int = 16, nmax: int = 64,
                      sigma: float = 1.5):
    """Independent diffusion problems on unit cubes: sizes n (n^3 cells) uniform in
    nmin..nmax, per-cell kappa = exp(sigma * N(0, 1)) in Gridap's cell order."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, nproblems)
    kappas = [np.exp(sigma * rng.standard_normal(int(n) ** 3)) for n in sizes]
    return [int(n) for n in sizes], kappas


def box_cell_dofs(n: int) -> np.ndarray:
    """Cell dof ids (cells x 8, int32, Gridap's 1-based free / negative Dirichlet convention) of
    the Q1 space on an (n, n, n) Cartesian box with dirichlet_tags="boundary": interior nodes
    are the free dofs in node order, boundary nodes the Dirichlet dofs in node order."""
    m = n + 1
    i, j, k = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
    i, j, k = (a.transpose(2, 1, 0).reshape(-1) for a in (i, j, k))  # node order: x fastest
    bnd = (i == 0) | (j == 0) | (k == 0) | (i == n) | (j == n) | (k == n)
    node_dof = np.empty(m ** 3, np.int64)
    node_dof[~bnd] = np.arange(1, (~bnd).sum() + 1)
    node_dof[bnd] = -np.arange(1, bnd.sum() + 1)
    c = np.arange(n)
    ci, cj, ck = np.meshgrid(c, c, c, indexing="ij")
    ci, cj, ck = (a.transpose(2, 1, 0).reshape(-1) for a in (ci, cj, ck))
    out = np.empty((n ** 3, 8), np.int32)
    for l in range(8):
        ii, jj, kk = ci + (l & 1), cj + ((l >> 1) & 1), ck + ((l >> 2) & 1)
        out[:, l] = node_dof[ii + m * (jj + m * kk)]
    return out


def elasticity_3d(n: int = 48, seed: int = 3):
    """Linear elasticity on simplexify(CartesianDiscreteModel((0,1)^3, (n,n,n))) with vector P2:
    per-cell Lamé coefficients exp(N(0,1)) normalised to mean 1 (independent draws for lambda
    and mu), body force (0, 0, -1), the x = 0 face clamped. Returns (model, V, measure,
    lame[ncells, 2], force)."""
    from .geometry import simplexify
    model = simplexify(CartesianDiscreteModel((0, 1, 0, 1, 0, 1), (n, n, n)))
    model.add_tag_from_vertex_filter("x0", lambda x: np.abs(x[:, 0]) < 1e-12)
    V = FESpace(model, ReferenceFE(lagrangian, 3, 2), dirichlet_tags="x0")
    lame = elasticity_lame(model.num_cells(), seed)
    return model, V, Measure(Triangulation(model), 4), lame, np.array([0.0, 0.0, -1.0])


def jittered_q2_3d(n: int = 64, seed: int = 2, amplitude: float = 0.2):
    """3-D Poisson on (0,1)^3 with n^3 hexahedra whose interior nodes are moved by a seeded
    uniform jitter in (-amplitude h, amplitude h)^3, Lagrangian Q2 with homogeneous Dirichlet
    data on the boundary, kappa = 1, f = 1, quadrature degree 4. Returns (model, V, measure)."""
    jit = q2_jitter(n, seed, amplitude)
    model = CartesianDiscreteModel((0, 1, 0, 1, 0, 1), (n, n, n), node_jitter=jit)
    V = FESpace(model, ReferenceFE(lagrangian, float, 2), dirichlet_tags="boundary")
    return model, V, Measure(Triangulation(model), 4)
