"""Conformance tests mirroring Gridap's own testers and driver tests for the drop-in path:

- `test_linear_solver` (Algebra/LinearSolvers.jl:138-161): solve(ls, A, b); symbolic_setup /
  numerical_setup / numerical_setup! / solve!(y, ns, b); solve!(y, ls, A, b); and the solve of
  an AffineOperator — for every solver the library provides;
- re-assembly into perturbed matrices and vectors reproduces the first assembly
  (test/FESpacesTests/AssemblersTests.jl:72-101; Gridap's bound 1e-14, here bit for bit);
- manufactured-solution exactness (test/GridapTests/PoissonTests.jl:87-120): a solution inside
  the FE space is reproduced to round-off (Q2 on a Cartesian box).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system(gg, part=(9, 8, 7), seed=40):
    rng = np.random.default_rng(seed)
    m = gg.CartesianDiscreteModel((0, 1) * 3, part)
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    dO = gg.Measure(gg.Triangulation(m), 2)
    kap = gg.CellField(np.exp(rng.standard_normal(m.num_cells())))
    a = lambda u, v: gg.integrate(kap * gg.inner(gg.grad(v), gg.grad(u)), dO)  # noqa: E731
    f = gg.NodalField(rng.standard_normal(m.num_nodes()))
    l = lambda v: gg.integrate(f * v, dO)  # noqa: E731
    return m, V, a, l


@pytest.mark.parametrize("kind", ["cg", "mixed", "ir", "fcg"])
def test_linear_solver_conformance(gg, kind):
    import scipy.sparse.linalg as sl
    _, V, a, l = _system(gg)
    A, b = gg.assemble_matrix_and_vector(a, l, V, V)
    x = sl.spsolve(A.to_scipy().tocsc(), b)
    rtol = 1e-10
    ls = {"cg": gg.CGSolver(rtol=rtol), "mixed": gg.MixedCGSolver(rtol=rtol),
          "ir": gg.IRCGSolver(rtol=rtol), "fcg": gg.FCGSolver(rtol=rtol)}[kind]
    close = lambda y: np.linalg.norm(y - x) <= 1e-7 * np.linalg.norm(x)  # noqa: E731
    y = gg.solve(ls, A, b)
    assert close(y)
    ss = gg.symbolic_setup(ls, A)
    ns = gg.numerical_setup(ss, A)
    gg.numerical_setup_(ns, A)
    y = np.zeros_like(b)
    gg.solve_(y, ns, b)
    assert close(y) and ns.report.converged
    y[:] = 0
    gg.solve_matrix_(y, ls, A, b)
    assert close(y)
    op = gg.AffineOperator(A, b)
    y = gg.solve(ls, op)
    assert close(y)
    assert np.linalg.norm(op.residual(y)) <= 1.01 * rtol * np.linalg.norm(b)


def test_reassembly_into_perturbed_matrix_and_vector(gg):
    rng = np.random.default_rng(41)
    _, V, a, l = _system(gg, seed=41)
    A1 = gg.assemble_matrix(a, V, V)
    b1 = gg.assemble_vector(l, V)
    A2, b2 = gg.assemble_matrix_and_vector(a, l, V, V)
    # perturb copies: random cell matrices into the same pattern, random vector entries
    assem = gg.SparseMatrixAssembler(V, V)
    ids = V.cell_dof_ids
    A12 = gg.symbolic_loop_matrix(assem, (None, ids, ids))
    gg.numeric_loop_matrix(A12, assem, (rng.standard_normal((ids.shape[0], 8, 8)), ids, ids))
    b12 = b1.copy()
    b12[0] = rng.random()
    A22 = gg.symbolic_loop_matrix(assem, (None, ids, ids))
    gg.numeric_loop_matrix(A22, assem, (rng.standard_normal((ids.shape[0], 8, 8)), ids, ids))
    b22 = b2.copy()
    b22[0] = rng.random()
    gg.assemble_matrix_(a, A12, V, V)
    gg.assemble_vector_(l, b12, V)
    gg.assemble_matrix_and_vector_(a, l, A22, b22, V, V)
    for X, Y in ((A12, A1), (A22, A2)):
        assert all(np.array_equal(s, t) for s, t in zip(X.export_csr(0), Y.export_csr(0)))
    assert np.array_equal(b12, b1) and np.array_equal(b22, b2)


def _q2_node_coords(D, part, V):
    """Physical coordinates of every free dof of a Q2 space on a Cartesian box, from the cell
    dof ids and Gridap's local node order (n-cube faces: vertices, edges, faces, interior;
    one node at each face centre)."""
    h = 1.0 / np.array(part)
    # local nodes in n-cube face order: the face's anchor and extrusion give the centre
    from oracle import oracle as orc
    exts, ancs = orc.ncube_faces(D)
    faces = list(zip(exts, ancs))
    ncell = int(np.prod(part))
    X = np.zeros((V.nfree, D))
    for c in range(ncell):
        idx = [(c // int(np.prod(part[:d]))) % part[d] for d in range(D)]
        for lf, (ext, anc) in enumerate(faces):
            centre = np.array([anc[d] + 0.5 * ext[d] for d in range(D)])
            dof = V.cell_dof_ids[c, lf]
            if dof > 0:
                X[dof - 1] = (np.array(idx) + centre) * h
    return X


def test_q2_manufactured_solution_is_exact(gg):
    """u = x(1-x) y(1-y) z(1-z) lies in Q2 and vanishes on the boundary; with f = -Δu
    integrated exactly (degree 4) the FE solution equals u at every node to round-off."""
    D, part = 3, (3, 4, 2)
    m = gg.CartesianDiscreteModel((0, 1) * D, part)
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 2), dirichlet_tags="boundary")
    dO = gg.Measure(gg.Triangulation(m), 4)

    def f(x):
        x, y, z = x[:, 0], x[:, 1], x[:, 2]
        q = lambda t: t * (1 - t)  # noqa: E731
        return 2 * (q(y) * q(z) + q(x) * q(z) + q(x) * q(y))

    op = gg.AffineFEOperator(lambda u, v: gg.integrate(gg.inner(gg.grad(v), gg.grad(u)), dO),
                             lambda v: gg.integrate(f * v, dO), V, V)
    uh = gg.solve(gg.LinearFESolver(gg.CGSolver(rtol=1e-13)), op)
    X = _q2_node_coords(D, part, V)
    u = np.prod(X * (1 - X), axis=1)
    assert np.abs(uh.free_values - u).max() <= 1e-10 * np.abs(u).max()


@pytest.mark.parametrize("kind", ["cg", "mixed", "fcg"])
def test_restart_from_saved_solution(gg, tmp_path, kind):
    """Checkpoint/restart: a solve stopped early is saved, reloaded and continued from that x
    (initial_guess); the continued solve meets the tolerance, needs fewer iterations than a
    cold start, and a converged guess returns at once."""
    _, V, a, l = _system(gg, seed=42)
    A, b = gg.assemble_matrix_and_vector(a, l, V, V)
    cls = {"cg": gg.CGSolver, "mixed": gg.MixedCGSolver, "fcg": gg.FCGSolver}[kind]
    cold = np.zeros_like(b)
    ns = gg.numerical_setup(gg.symbolic_setup(cls(rtol=1e-10), A), A)
    gg.solve_(cold, ns, b)
    cold_it = ns.report.iterations
    part = np.zeros_like(b)
    ns = gg.numerical_setup(gg.symbolic_setup(cls(rtol=1e-4), A), A)
    gg.solve_(part, ns, b)
    np.save(tmp_path / "x.npy", part)
    x = np.load(tmp_path / "x.npy")
    ns = gg.numerical_setup(gg.symbolic_setup(cls(rtol=1e-10, initial_guess=True), A), A)
    gg.solve_(x, ns, b)
    assert ns.report.converged and ns.report.relres <= 1e-10
    assert ns.report.iterations < cold_it
    r = b - A.to_scipy() @ x
    assert np.linalg.norm(r) <= 1.01e-10 * np.linalg.norm(b)
    ns = gg.numerical_setup(gg.symbolic_setup(cls(rtol=1e-6, initial_guess=True), A), A)
    y = x.copy()
    gg.solve_(y, ns, b)
    assert ns.report.converged and ns.report.iterations == 0 and np.array_equal(y, x)
