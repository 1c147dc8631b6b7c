"""GPU parity of multi-field assembly (MultiFieldFESpace, consecutive and block styles)
against the oracle, through the C ABI.

The cases follow Gridap's own multi-field tests: the two- and three-field forms of
test/MultiFieldTests/BlockSparseMatrixAssemblersTests.jl (Q1 fields on a 5x5 grid, Dirichlet
data x1 + x2, monolithic against every block layout), the Taylor-Hood Stokes form of
test/GridapTests/StokesTaylorHoodTests.jl (vector Q2 velocity, Q1 pressure), and a coupled
manufactured solution that the FE space reproduces exactly.

Tolerances (written here, used below):
  - patterns: bit-exact (rowptr and column ids identical to the oracle's assembly);
  - matrix values: <= 1e-12 times the largest entry of their row (cell integrals computed
    in a different order than the oracle's dense contractions);
  - vectors: <= 1e-12 times max|b|;
  - block layouts against the monolithic assembly: bit-exact (same kernels, same order);
  - manufactured solution: nodal error <= 1e-8 (BiCGStab to rtol 1e-12).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _rowscaled(A, S):
    """max over rows of |A - S| / max|S row| for two scipy CSR matrices of one pattern."""
    err = 0.0
    for r in range(S.shape[0]):
        a, b = S.indptr[r], S.indptr[r + 1]
        if b > a:
            s = np.abs(S.data[a:b]).max()
            err = max(err, np.abs(A.data[a:b] - S.data[a:b]).max() / max(s, 1e-300))
    return err


def _check(A, b, S, bref):
    Ad = A.to_scipy() if hasattr(A, "to_scipy") else A
    Ad.sort_indices()
    assert np.array_equal(Ad.indptr, S.indptr) and np.array_equal(Ad.indices, S.indices)
    assert _rowscaled(Ad, S) <= TOL
    if b is not None:
        assert np.abs(b - bref).max() <= TOL * max(np.abs(bref).max(), 1e-300)


def _q1_setup(gg):
    model = gg.CartesianDiscreteModel((0.0, 1.0, 0.0, 1.0), (5, 5))
    V = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    U = gg.TrialFESpace(V, lambda x: x[:, 0] + x[:, 1])
    return model, V, U, gg.Measure(gg.Triangulation(model), 2)


def _forms(gg, n, dO):
    inner, grad, integrate = gg.inner, gg.grad, gg.integrate
    if n == 2:
        a = lambda x, y: integrate(  # noqa: E731
            inner(grad(x[0]), grad(y[0])) + x[1] * y[1] - x[0] * y[1], dO)
        l = lambda y: integrate(y[0] - y[1], dO)  # noqa: E731
        # oracle terms: (test field, test op, trial field, trial op, coef, cell coef, data)
        t = [(0, 1, 0, 1, 1.0, None, None), (1, 0, 1, 0, 1.0, None, None),
             (1, 0, 0, 0, -1.0, None, None), (0, 0, None, None, 1.0, None, None),
             (1, 0, None, None, -1.0, None, None)]
    else:
        a = lambda x, y: integrate(  # noqa: E731
            inner(grad(x[0]), grad(y[0])) + x[1] * y[1] - x[0] * y[1] - x[2] * y[1]
            - x[1] * y[2], dO)
        l = lambda y: integrate(y[0] - y[1] + 2.0 * y[2], dO)  # noqa: E731
        t = [(0, 1, 0, 1, 1.0, None, None), (1, 0, 1, 0, 1.0, None, None),
             (1, 0, 0, 0, -1.0, None, None), (1, 0, 2, 0, -1.0, None, None),
             (2, 0, 1, 0, -1.0, None, None), (0, 0, None, None, 1.0, None, None),
             (1, 0, None, None, -1.0, None, None), (2, 0, None, None, 2.0, None, None)]
    return a, l, t


def _oracle_q1(orc, model, V, U, n, terms):
    K, F = orc.multifield_cell_arrays(2, model.node_coords, model.cell_node_ids,
                                      [(1, 1)] * n, terms, 2)
    nf = V.num_free_dofs()
    ids = V.get_cell_dof_ids()
    cell_ids = [np.where(ids > 0, ids + i * nf, ids).astype(np.int32) for i in range(n)]
    return orc.multifield_assemble(cell_ids, [nf] * n, K, F,
                                   [U.get_dirichlet_dof_values()] * n)


@pytest.mark.parametrize("n", [2, 3])
def test_consecutive_assembly_matches_oracle(gg, orc, n):
    model, V, U, dO = _q1_setup(gg)
    a, l, terms = _forms(gg, n, dO)
    X = gg.MultiFieldFESpace([U] * n)
    Y = gg.MultiFieldFESpace([V] * n)
    assert X.num_free_dofs() == n * V.num_free_dofs() and gg.num_fields(X) == n
    op = gg.AffineFEOperator(a, l, X, Y)
    S, bref = _oracle_q1(orc, model, V, U, n, terms)
    _check(op.A, op.b, S, bref)
    # the untouched field pairs (e.g. test 1 / trial 2) add no entry
    Ad = op.A.to_scipy()
    nf = V.num_free_dofs()
    assert Ad[:nf, nf:2 * nf].nnz == 0


@pytest.mark.parametrize("n", [2, 3])
@pytest.mark.parametrize("trial_style,test_style", [("default", "default"),
                                                    ("split", "split"),
                                                    ("default", "split")])
def test_block_layouts_equal_the_monolithic_assembly(gg, n, trial_style, test_style):
    """BlockSparseMatrixAssemblersTests.jl: every block layout of trial and test spaces
    gives the monolithic matrix and vector, and the same products."""
    model, V, U, dO = _q1_setup(gg)
    a, l, _ = _forms(gg, n, dO)
    A, b = gg.assemble_matrix_and_vector(a, l, gg.MultiFieldFESpace([U] * n),
                                         gg.MultiFieldFESpace([V] * n))
    style = {"default": gg.BlockMultiFieldStyle(),
             "split": gg.BlockMultiFieldStyle(2, (1, n - 1))}
    Xb = gg.MultiFieldFESpace([U] * n, style=style[trial_style])
    Yb = gg.MultiFieldFESpace([V] * n, style=style[test_style])
    Ab, bb = gg.assemble_matrix_and_vector(a, l, Xb, Yb)
    M = A.to_scipy()
    Mb = Ab.to_scipy()
    M.sort_indices()
    Mb.sort_indices()
    assert np.array_equal(M.indptr, Mb.indptr) and np.array_equal(M.indices, Mb.indices)
    assert np.array_equal(M.data, Mb.data)
    assert np.array_equal(np.concatenate(bb), b)
    y = A.matvec(b)
    splits = np.cumsum(Ab.blocksizes(2))[:-1]
    yb = Ab.matvec(np.split(b, splits))
    assert np.allclose(np.concatenate(yb), y, rtol=1e-13, atol=1e-13)


def _stokes(gg, D, part):
    dom = (0.0, 2.0) * D
    model = gg.CartesianDiscreteModel(dom, part)
    if D == 2:
        u = lambda x: np.stack([x[:, 0] ** 2 + 2 * x[:, 1] ** 2, -x[:, 0] ** 2], axis=1)  # noqa
        f = lambda x: np.tile([-5.0, 5.0], (x.shape[0], 1))  # -lap u + grad p  # noqa: E731
        g = lambda x: 2 * x[:, 0]  # noqa: E731
    else:
        u = lambda x: np.stack([x[:, 1] ** 2, x[:, 2] ** 2 + x[:, 0], x[:, 0] * x[:, 1]], 1)  # noqa
        f = lambda x: np.tile([-1.0, 1.0, 3.0], (x.shape[0], 1))  # noqa: E731
        g = lambda x: 0.0 * x[:, 0]  # noqa: E731
    V = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, D, 2), dirichlet_tags="boundary")
    Q = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 1))
    U, P = gg.TrialFESpace(V, u), gg.TrialFESpace(Q)
    dO = gg.Measure(gg.Triangulation(model), 4)
    inner, grad, div, integrate = gg.inner, gg.grad, gg.div, gg.integrate
    a = lambda x, y: integrate(inner(grad(y[0]), grad(x[0])) - div(y[0]) * x[1]  # noqa: E731
                               + y[1] * div(x[0]), dO)
    l = lambda y: integrate(inner(y[0], f) + y[1] * g, dO)  # noqa: E731
    return model, V, Q, U, P, a, l, f, g


@pytest.mark.parametrize("D,part", [(2, (3, 3)), (2, (7, 5)), (3, (2, 3, 2))])
def test_stokes_taylor_hood_matches_oracle(gg, orc, D, part):
    """StokesTaylorHoodTests.jl's form a((u,p),(v,q)) = ∫ ∇v⊙∇u - (∇⋅v) p + q (∇⋅u) and
    l((v,q)) = ∫ v⋅f + q g with u = u_exact on the boundary (vector Q2 / Q1)."""
    model, V, Q, U, P, a, l, f, g = _stokes(gg, D, part)
    X, Y = gg.MultiFieldFESpace([U, P]), gg.MultiFieldFESpace([V, Q])
    op = gg.AffineFEOperator(a, l, X, Y)
    xq = orc.qpoints(D, model.cell_node_ids, model.node_coords, 4)
    pts = xq.reshape(-1, D)
    terms = [(0, 1, 0, 1, 1.0, None, None), (0, 2, 1, 0, -1.0, None, None),
             (1, 0, 0, 2, 1.0, None, None),
             (0, 0, None, None, 1.0, None, f(pts).reshape(xq.shape[0], xq.shape[1], D)),
             (1, 0, None, None, 1.0, None, g(pts).reshape(xq.shape[0], xq.shape[1], 1))]
    K, F = orc.multifield_cell_arrays(D, model.node_coords, model.cell_node_ids,
                                      [(2, D), (1, 1)], terms, 4)
    nu = V.num_free_dofs()
    ids_u = V.get_cell_dof_ids()
    ids_p = Q.get_cell_dof_ids()
    cell_ids = [ids_u, np.where(ids_p > 0, ids_p + nu, ids_p).astype(np.int32)]
    S, bref = orc.multifield_assemble(cell_ids, [nu, Q.num_free_dofs()], K, F,
                                      [U.get_dirichlet_dof_values(), None])
    _check(op.A, op.b, S, bref)
    # block layout: velocity / pressure blocks, the pressure-pressure block empty
    Xb = gg.MultiFieldFESpace([U, P], style=gg.BlockMultiFieldStyle())
    Yb = gg.MultiFieldFESpace([V, Q], style=gg.BlockMultiFieldStyle())
    Ab, bb = gg.assemble_matrix_and_vector(a, l, Xb, Yb)
    assert Ab[1, 1].nnz == 0 and Ab.shape == op.A.shape
    M = Ab.to_scipy()
    M.sort_indices()
    assert np.array_equal(M.indices, S.indices) and np.array_equal(M.indptr, S.indptr)
    assert np.array_equal(np.concatenate(bb), op.b)


def test_coupled_manufactured_solution_is_reproduced(gg):
    """a((u1,u2),(v1,v2)) = ∫ ∇v1⋅∇u1 + v2 u2 - v2 u1 with u1 = x² + xy + y² on the boundary
    and l = ∫ -4 v1: u1 solves -Δu1 = -4 and u2 is its projection, both exactly in Q2."""
    model = gg.CartesianDiscreteModel((0.0, 1.0, 0.0, 1.0), (6, 5))
    ex = lambda x: x[:, 0] ** 2 + x[:, 0] * x[:, 1] + x[:, 1] ** 2  # noqa: E731
    V1 = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 2), dirichlet_tags="boundary")
    V2 = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 2))
    X = gg.MultiFieldFESpace([gg.TrialFESpace(V1, ex), gg.TrialFESpace(V2)])
    Y = gg.MultiFieldFESpace([V1, V2])
    dO = gg.Measure(gg.Triangulation(model), 4)
    inner, grad, integrate = gg.inner, gg.grad, gg.integrate
    a = lambda x, y: integrate(inner(grad(y[0]), grad(x[0])) + y[1] * x[1]  # noqa: E731
                               - y[1] * x[0], dO)
    l = lambda y: integrate(-4.0 * y[0], dO)  # noqa: E731
    op = gg.AffineFEOperator(a, l, X, Y)
    xh = gg.solve(gg.BiCGStabSolver(rtol=1e-12), op)
    u1, u2 = xh
    assert xh.report.converged
    x1, _, _, _ = V1.dof_points()
    x2, _, _, _ = V2.dof_points()
    assert np.abs(np.asarray(u1.free_values) - ex(x1)).max() <= 1e-8
    assert np.abs(np.asarray(u2.free_values) - ex(x2)).max() <= 1e-8
