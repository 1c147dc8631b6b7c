"""Nonlinear FEOperators: residual and Jacobian re-assembly on the device, and Newton solves.

- residual!/jacobian! of quasilinear diffusion (p-Laplacian flux, polynomial α(u)) against
  the oracle's per-point restatement (pinned in the CPU suite by central differences of its
  own residual), Q1/Q2, 2-D/3-D, jittered cells, per-cell κ, point-wise f, Dirichlet data;
- the device Jacobian against central differences of the device residual;
- re-assembly into one Jacobian pattern is bit-identical across calls;
- Gridap's PLaplacianTests (test/GridapTests/PLaplacianTests.jl): p = 3, u = x + y imposed
  on the boundary, Newton from a random guess with the user Jacobian and with the law's exact
  derivative (Gridap's autodiff variant); Q2 here (Gridap uses Q3; u is linear, so both
  reproduce it), the solution equals u at every dof;
- a polynomial-coefficient problem -∇⋅((1+u²)∇u) = f with a non-symmetric Jacobian, solved
  by Newton with BiCGStab.
Tolerances: cell arrays are FP64 sums in another order than the oracle's: 1e-12 of the
largest entry.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _model(gg, part, jitter=0.0, seed=3):
    D = len(part)
    jit = None
    if jitter:
        nn = int(np.prod(np.array(part) + 1))
        jit = jitter * np.random.default_rng(seed).standard_normal((nn, D)) / max(part)
    return gg.CartesianDiscreteModel((0, 1) * D, part, node_jitter=jit)


def _operator(gg, m, order, law_kind, kappa=None, f=None, uD=None):
    tags = "tag_1" if m.dim == 2 else "tag_01"
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, order), dirichlet_tags=tags)
    U = gg.TrialFESpace(V, uD if uD is not None else 0.0)
    dO = gg.Measure(gg.Triangulation(m), 2 * order + 2)
    k = 1.0 if kappa is None else gg.CellField(kappa)
    if law_kind == "power":
        flux = gg.PowerLawFlux(3.0, 0.1)

        def res(u, v):
            t = k * gg.inner(gg.grad(v), flux(gg.grad(u)))
            return gg.integrate(t - f * v if f is not None else t, dO)

        def jac(u, du, v):
            return gg.integrate(k * gg.inner(gg.grad(v), flux.derivative(gg.grad(du),
                                                                         gg.grad(u))), dO)
        law, params = 1, (3.0, 0.1)
    else:
        alpha = gg.PolynomialCoefficient(1.0, 0.5, 1.0)

        def res(u, v):
            t = k * alpha(u) * gg.inner(gg.grad(v), gg.grad(u))
            return gg.integrate(t - f * v if f is not None else t, dO)

        def jac(u, du, v):
            return gg.integrate(k * alpha(u) * gg.inner(gg.grad(v), gg.grad(du))
                                + k * alpha.derivative(u) * du * gg.inner(gg.grad(v),
                                                                          gg.grad(u)), dO)
        law, params = 0, (1.0, 0.5, 1.0)
    return gg.FEOperator(res, jac, U, V), V, U, law, params, 2 * order + 2


@pytest.mark.parametrize("part,order,law_kind,jitter", [
    ((5, 4), 1, "power", 0.15), ((5, 4), 1, "poly", 0.15), ((3, 4), 2, "power", 0.15),
    ((3, 3), 2, "poly", 0.15), ((3, 3, 2), 1, "poly", 0.15), ((2, 2, 2), 2, "power", 0.15),
    # undistorted Q1 cells: the table-driven Cartesian kernel (symmetric and general)
    ((6, 5), 1, "power", 0.0), ((4, 3, 5), 1, "poly", 0.0), ((4, 3, 3), 1, "power", 0.0),
])
def test_residual_and_jacobian_match_oracle(gg, orc, part, order, law_kind, jitter):
    rng = np.random.default_rng(sum(part) + order)
    m = _model(gg, part, jitter=jitter)
    kappa = np.exp(0.3 * rng.standard_normal(m.num_cells()))
    f = lambda x: 1.0 + x[:, 0] * x[:, 1]  # noqa: E731
    uD = lambda x: 0.5 - x[:, 0]  # noqa: E731
    op, V, U, law, params, deg = _operator(gg, m, order, law_kind, kappa, f, uD)
    x = rng.standard_normal(V.num_free_dofs())
    b, A = op.residual_and_jacobian(x)
    mats, vecs = orc.quasilinear_cell_arrays(m.node_coords, m.cell_node_ids, V.cell_dof_ids,
                                             order, deg, x, U.dirichlet_values, law, params,
                                             kappa=kappa, f=f)
    bw = orc.assemble_vector(V.cell_dof_ids, vecs, V.num_free_dofs())
    assert np.abs(b - bw).max() <= RTOL * np.abs(bw).max()
    colptr, rowval, nzval = orc.assemble_csc(V.cell_dof_ids, V.cell_dof_ids, mats,
                                             V.num_free_dofs(), V.num_free_dofs())
    Aw = orc.to_scipy(colptr, rowval, nzval, V.num_free_dofs(), V.num_free_dofs()).toarray()
    Ad = A.to_scipy().toarray()
    assert np.abs(Ad - Aw).max() <= RTOL * np.abs(Aw).max()
    # the residual alone and the Jacobian alone give the same arrays
    assert np.array_equal(op.residual(x), b)
    A2 = op.jacobian(x)
    assert all(np.array_equal(s, t) for s, t in zip(A2.export_csr(0), A.export_csr(0)))


@pytest.mark.parametrize("law_kind,order", [("power", 1), ("poly", 2)])
def test_jacobian_is_the_derivative_of_the_device_residual(gg, law_kind, order):
    rng = np.random.default_rng(7)
    m = _model(gg, (4, 3, 3), jitter=0.1)
    op, V, _, _, _, _ = _operator(gg, m, order, law_kind, f=lambda x: x[:, 2])
    x = 0.5 * rng.standard_normal(V.num_free_dofs())
    d = rng.standard_normal(x.size)
    eps = 1e-6
    fd = (op.residual(x + eps * d) - op.residual(x - eps * d)) / (2 * eps)
    jd = op.jacobian(x).matvec(d)
    assert np.abs(fd - jd).max() <= 1e-7 * np.abs(jd).max()


def test_jacobian_reassembly_is_bit_identical(gg):
    rng = np.random.default_rng(9)
    m = _model(gg, (6, 5), jitter=0.1)
    op, V, _, _, _, _ = _operator(gg, m, 2, "poly", f=lambda x: x[:, 0])
    x1, x2 = rng.standard_normal((2, V.num_free_dofs()))
    A = op.jacobian(x1)
    ref = [a.copy() for a in A.export_csr(0)]
    op.jacobian_(A, x2)
    op.jacobian_(A, x1)
    assert all(np.array_equal(s, t) for s, t in zip(A.export_csr(0), ref))
    b = np.empty(V.num_free_dofs())
    op.residual_(b, x1)
    assert np.array_equal(b, op.residual(x1))


@pytest.mark.parametrize("autodiff", [False, True])
def test_plaplacian_newton_reproduces_linear_solution(gg, autodiff):
    """test/GridapTests/PLaplacianTests.jl: 4x4 box, p = 3, u = x + y on the boundary, f = 0,
    degree 2*order, Newton from a random initial guess."""
    m = gg.CartesianDiscreteModel((0, 1, 0, 1), (4, 4))
    order = 2
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, order), dirichlet_tags="boundary")
    u = lambda x: x[:, 0] + x[:, 1]  # noqa: E731
    U = gg.TrialFESpace(V, u)
    dO = gg.Measure(gg.Triangulation(m), 2 * order)
    flux = gg.PowerLawFlux(3.0)
    res = lambda u_, v: gg.integrate(gg.inner(gg.grad(v), flux(gg.grad(u_))), dO)  # noqa: E731

    def jac(u_, du, v):
        return gg.integrate(gg.inner(gg.grad(v), flux.derivative(gg.grad(du), gg.grad(u_))), dO)

    op = gg.FEOperator(res, U, V) if autodiff else gg.FEOperator(res, jac, U, V)
    nls = gg.NLSolver(show_trace=False, method="newton")
    x = np.random.default_rng(1).random(V.num_free_dofs())
    uh0 = gg.FEFunction(U, x)
    uh, _ = gg.solve_nonlinear_(uh0, gg.NonlinearFESolver(nls), op)
    fx, _, _, _ = V.dof_points()
    assert np.abs(uh.free_values - u(fx)).max() <= 1e-7
    assert 0 < nls.iterations < 30


def test_polynomial_coefficient_newton_with_bicgstab(gg):
    """-∇⋅((1+u²)∇u) = f with u = x + 2y (so f = -10u): u is in the Q1 space and every
    integral is exact at degree 4, so Newton (non-symmetric Jacobian, BiCGStab) reproduces u
    at the nodes; NewtonRaphsonSolver converges quadratically (a handful of steps)."""
    m = gg.CartesianDiscreteModel((0, 1, 0, 1), (8, 6))
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    u = lambda x: x[:, 0] + 2.0 * x[:, 1]  # noqa: E731
    U = gg.TrialFESpace(V, u)
    dO = gg.Measure(gg.Triangulation(m), 4)
    alpha = gg.PolynomialCoefficient(1.0, 0.0, 1.0)
    f = lambda x: -10.0 * u(x)  # noqa: E731
    res = lambda u_, v: gg.integrate(alpha(u_) * gg.inner(gg.grad(v), gg.grad(u_))  # noqa
                                     - f * v, dO)
    op = gg.FEOperator(res, U, V)
    nls = gg.NewtonRaphsonSolver(gg.BiCGStabSolver(rtol=1e-12), 1e-12, 20)
    uh = gg.solve(nls, op)
    assert np.abs(uh.nodal_values() - u(m.node_coords)).max() <= 1e-9
    assert nls.iterations <= 8
