"""Boundary (Neumann) load terms ∫ g v dΓ on BoundaryTriangulations, against the oracle.

The oracle restates Gridap's facet enumeration and facet integration
(Geometry/BoundaryTriangulations.jl, Fields/FieldsInterfaces.jl:660-670) and is pinned by the
2x2 BoundaryTriangulation known-answer test; here the GPU facet vectors and their assembly
are compared with it for Q1 and Q2, 2-D and 3-D, constant and point-wise g, tag selections,
jittered cells and device vectors, and a Neumann problem is solved exactly (test/GridapTests/
PoissonTests.jl uses the same manufactured-solution check with a Neumann boundary).
Tolerance: the facet vectors are sums of a few FP64 products in another order than Gridap's,
so entries agree to 1e-13 relative to the vector's largest entry.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-13


def _space(gg, part, order, tags="boundary", jitter=0.0, seed=5):
    D = len(part)
    jit = None
    if jitter:
        nn = int(np.prod(np.array(part) + 1))
        jit = jitter * np.random.default_rng(seed).standard_normal((nn, D)) / max(part)
    m = gg.CartesianDiscreteModel((0, 1) * D, part, node_jitter=jit)
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, order), dirichlet_tags=tags)
    return m, V


def _oracle_b(orc, m, V, order, tags, degree, g, test_op=0):
    fc, fl = orc.boundary_facets(m.partition, tags)
    b, _ = orc.boundary_vector(m.partition, m.node_coords, m.cell_node_ids, V.cell_dof_ids,
                               order, fc, fl, degree, g, V.num_free_dofs(), test_op)
    return b


def _close(x, y):
    scale = max(np.abs(y).max(), 1e-300)
    assert np.abs(x - y).max() <= RTOL * scale, np.abs(x - y).max() / scale


G2 = lambda x: 1.0 + x[:, 0] ** 2 - 0.5 * x[:, 1]  # noqa: E731
G3 = lambda x: np.cos(x[:, 0]) + x[:, 1] * x[:, 2]  # noqa: E731


@pytest.mark.parametrize("part,order,btags,degree,g", [
    ((7, 5), 1, None, 2, 1.5),
    ((7, 5), 1, ["tag_6", "tag_8"], 3, G2),
    ((4, 6), 2, "tag_7", 4, G2),
    ((5, 4, 3), 1, None, 2, G3),
    ((5, 4, 3), 1, "tag_26", 2, -2.0),
    ((3, 4, 2), 2, ["tag_21", "tag_24"], 4, G3),
    ((3, 2, 3), 2, None, 5, 0.75),
])
def test_boundary_vector_matches_oracle(gg, orc, part, order, btags, degree, g):
    m, V = _space(gg, part, order, tags=["tag_1", "tag_2"] if len(part) == 2 else "tag_01")
    dG = gg.Measure(gg.BoundaryTriangulation(m, tags=btags), degree)
    b = gg.assemble_vector(lambda v: gg.integrate(g * v, dG), V)
    _close(b, _oracle_b(orc, m, V, order, btags, degree, g))


@pytest.mark.parametrize("order", [1, 2])
def test_boundary_plus_volume_and_jitter(gg, orc, order):
    """A volume source plus two boundary terms on a jittered model: the boundary part of the
    assembled vector equals the oracle's facet integrals (boundary facets are undistorted)."""
    m, V = _space(gg, (5, 4, 4), order, tags="tag_21", jitter=0.1)
    dO = gg.Measure(gg.Triangulation(m), 2 * order)
    G1 = gg.BoundaryTriangulation(m, tags="tag_26")
    G2_ = gg.BoundaryTriangulation(m, tags=["tag_22", "tag_23"])
    dG1, dG2 = gg.Measure(G1, 2 * order), gg.Measure(G2_, 2 * order)
    vol = gg.assemble_vector(lambda v: gg.integrate(3.0 * v, dO), V)
    b = gg.assemble_vector(lambda v: gg.integrate(3.0 * v, dO) + gg.integrate(G3 * v, dG1)
                           + gg.integrate(-1.0 * v, dG2), V)
    want = (_oracle_b(orc, m, V, order, "tag_26", 2 * order, G3)
            + _oracle_b(orc, m, V, order, ["tag_22", "tag_23"], 2 * order, -1.0))
    _close(b - vol, want)


def test_boundary_vector_on_device(gg, orc):
    torch = pytest.importorskip("torch")
    m, V = _space(gg, (6, 5, 4), 1, tags="tag_01")
    dG = gg.Measure(gg.BoundaryTriangulation(m), 2)
    l = lambda v: gg.integrate(G3 * v, dG)  # noqa: E731
    bh = gg.assemble_vector(l, V)
    bd = torch.full((V.num_free_dofs(),), 7.0, dtype=torch.float64, device="cuda")
    gg.assemble_vector_(l, bd, V)
    assert np.array_equal(bd.cpu().numpy(), bh)
    _close(bh, _oracle_b(orc, m, V, 1, None, 2, G3))
    assert np.abs(bh).max() > 0


def test_neumann_q2_manufactured_solution_is_exact(gg):
    """-Δu = f on (0,1)^3 with u = x(1-x) y(1-y) z(1-z) in Q2: u = 0 on every face but x = 1,
    where ∂u/∂n = -y(1-y) z(1-z) is imposed weakly. With exact quadrature the FE solution
    equals u at every node to round-off."""
    part = (3, 2, 4)
    m = gg.CartesianDiscreteModel((0, 1) * 3, part)
    diri = [f"tag_{i:02d}" for i in range(1, 26)]  # every entity but the x = 1 face
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 2), dirichlet_tags=diri)
    dO = gg.Measure(gg.Triangulation(m), 4)
    dG = gg.Measure(gg.BoundaryTriangulation(m, tags="tag_26"), 4)
    q = lambda t: t * (1 - t)  # noqa: E731

    def f(x):
        return 2 * (q(x[:, 1]) * q(x[:, 2]) + q(x[:, 0]) * q(x[:, 2]) + q(x[:, 0]) * q(x[:, 1]))

    def g(x):
        return -q(x[:, 1]) * q(x[:, 2])

    op = gg.AffineFEOperator(lambda u, v: gg.integrate(gg.inner(gg.grad(v), gg.grad(u)), dO),
                             lambda v: gg.integrate(f * v, dO) + gg.integrate(g * v, dG), V, V)
    uh = gg.solve(gg.LinearFESolver(gg.CGSolver(rtol=1e-13)), op)
    from test_gpu_conformance import _q2_node_coords
    X = _q2_node_coords(3, part, V)
    u = np.prod(q(X), axis=1)
    assert np.abs(uh.free_values - u).max() <= 1e-10 * np.abs(u).max()
    # the x = 1 face carries free dofs, so the Neumann data is what fixes them
    assert (X[:, 0] == 1.0).sum() > 0


def test_boundary_bad_facet_is_reported(gg):
    """An owner cell out of range is caught by the facet kernel's bounds check and comes back
    as an error status; the context stays usable."""
    import ctypes as C
    from importlib import import_module
    lib = gg._lib
    m, V = _space(gg, (4, 4), 1, tags="tag_1")
    A = import_module(gg.__name__ + ".assembly")
    dO = gg.Measure(gg.Triangulation(m), 2)
    prep = A.prepare_problem(V, V, dO, None, None)
    cells = np.array([0, 99], np.int32)
    lf = np.array([0, 1], np.int32)
    one = np.array([1.0])
    b = np.zeros(V.num_free_dofs())
    ctx = A.default_context()
    st = lib.load().gfe_assemble_boundary_vector(ctx.handle, C.byref(prep.p), 2, lib.ptr(cells),
                                                 lib.ptr(lf), 2, lib.GFE_BOP_VALUE,
                                                 lib.GFE_SRC_CONST,
                                                 lib.ptr(one), 1, lib.ptr(b))
    assert st == lib.GFE_ERR_INVALID_ARGUMENT
    G = gg.BoundaryTriangulation(m)
    b = gg.assemble_vector(lambda v: gg.integrate(1.0 * v, gg.Measure(G, 2)), V)
    # the next call succeeds; the free dofs carry the boundary's length 4 less the share of
    # the Dirichlet corner (0, 0): two half edges of size 1/4
    assert abs(b.sum() - (4.0 - 0.25)) < 1e-13


def _dense(A):
    return A.to_scipy().toarray()


@pytest.mark.parametrize("part,order,btags,coefs", [
    ((6, 5), 1, "tag_6", (40.0, -1.0, -1.0, 0.0)),
    ((4, 5), 2, ["tag_5", "tag_8"], (7.0, -1.0, -1.0, 0.5)),
    ((4, 3, 3), 1, None, (2.5, 0.0, 0.0, 0.0)),
    ((3, 3, 2), 2, "tag_24", (30.0, -1.0, -1.0, 0.0)),
])
def test_boundary_matrix_and_lift_match_oracle(gg, orc, part, order, btags, coefs):
    """Facet matrices (Nitsche, Robin, and an n⋅∇v n⋅∇u term) added into the volume matrix,
    their Dirichlet lift, and ∫ g (n⋅∇v) dΓ, against the oracle's facet integrals with
    gradients pushed forward through the owner cell."""
    D = len(part)
    m, V = _space(gg, part, order, tags=["tag_1", "tag_3"] if D == 2 else ["tag_01", "tag_22"])
    uD = (lambda x: 1.0 + x[:, 0] - 2.0 * x[:, 1]) if D == 2 else G3
    U = gg.TrialFESpace(V, uD)
    dO = gg.Measure(gg.Triangulation(m), 2 * order)
    G = gg.BoundaryTriangulation(m, tags=btags)
    dG = gg.Measure(G, 2 * order)
    n = gg.get_normal_vector(G)
    c0, c1, c2, c3 = coefs
    vol = lambda u, v: gg.integrate(gg.inner(gg.grad(v), gg.grad(u)), dO)  # noqa: E731

    def bnd(u, v):
        nu, nv = gg.inner(n, gg.grad(u)), gg.inner(n, gg.grad(v))
        return gg.integrate(c0 * v * u + c1 * v * nu + c2 * nv * u + c3 * nv * nu, dG)

    l0 = lambda v: gg.integrate(0.0 * v, dO)  # noqa: E731
    A0, b0 = gg.assemble_matrix_and_vector(vol, l0, U, V)
    A1, b1 = gg.assemble_matrix_and_vector(lambda u, v: vol(u, v) + bnd(u, v), l0, U, V)
    fc, fl = orc.boundary_facets(part, btags)
    K, lift = orc.boundary_matrix(m.node_coords, m.cell_node_ids, V.cell_dof_ids, order, fc, fl,
                                  2 * order, coefs, V.num_free_dofs(), U.dirichlet_values)
    dK = _dense(A1) - _dense(A0)
    assert np.abs(dK - K).max() <= RTOL * np.abs(K).max() * 10
    _close(b1 - b0, lift)
    # the n⋅∇v right-hand side
    g = G3 if D == 3 else G2
    bn = gg.assemble_vector(lambda v: gg.integrate(g * gg.inner(n, gg.grad(v)), dG), V)
    _close(bn, _oracle_b(orc, m, V, order, btags, 2 * order, g, 1))


@pytest.mark.parametrize("order,part", [(1, (6, 5, 4)), (2, (4, 3, 3)), (2, (5, 4))])
def test_dirichlet_lift_matches_oracle(gg, orc, order, part):
    """b of a(u,v), l(v) with TrialFESpace(V, u_D) minus b with u_D = 0 is the cell-wise lift
    -Σ_j K_ij u_D_j of the oracle's cell matrices."""
    D = len(part)
    m, V = _space(gg, part, order, tags="boundary", jitter=0.1 if order == 2 else 0.0)
    g = G3 if D == 3 else G2
    U = gg.TrialFESpace(V, g)
    dO = gg.Measure(gg.Triangulation(m), 2 * order)
    a = lambda u, v: gg.integrate(gg.inner(gg.grad(v), gg.grad(u)), dO)  # noqa: E731
    l = lambda v: gg.integrate(1.0 * v, dO)  # noqa: E731
    _, b0 = gg.assemble_matrix_and_vector(a, l, V, V)
    _, b1 = gg.assemble_matrix_and_vector(a, l, U, V)
    if order == 1:
        mats, _ = orc.q1_cell_arrays(D, m.cell_node_ids, m.node_coords, 2 * order,
                                     h=m.cell_sizes())
    else:
        mats, _ = orc.q2_cell_arrays(D, m.cell_node_ids, m.node_coords, 2 * order)
    want = orc.dirichlet_lift(V.cell_dof_ids, mats, U.dirichlet_values, V.num_free_dofs())
    _close(b1 - b0, want)
    assert np.abs(want).max() > 0


def test_poisson_nitsche_neumann_dirichlet_is_exact(gg):
    """Gridap's PoissonTests scalar case (test/GridapTests/PoissonTests.jl): Q2 on a 4x4 box,
    u = x² + y; Dirichlet data on tags 1, 2, 5, Neumann data n⋅∇u on tags 7, 8, Nitsche
    terms with γ = 10, h = 1/4 on tag 6, every measure of degree 2. u lies in the space and
    every integral is exact, so the solution equals u at every dof."""
    m = gg.CartesianDiscreteModel((0, 1, 0, 1), (4, 4))
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 2), dirichlet_tags=[1, 2, 5])
    u = lambda x: x[:, 0] ** 2 + x[:, 1]  # noqa: E731
    gradu = lambda x: np.stack([2 * x[:, 0], np.ones(x.shape[0])], axis=1)  # noqa: E731
    U = gg.TrialFESpace(V, u)
    dO = gg.Measure(gg.Triangulation(m), 2)
    Gn = gg.BoundaryTriangulation(m, tags=[7, 8])
    Gd = gg.BoundaryTriangulation(m, tags=6)
    dGn, dGd = gg.Measure(Gn, 2), gg.Measure(Gd, 2)
    nn, nd = gg.get_normal_vector(Gn), gg.get_normal_vector(Gd)
    gam, h = 10.0, 0.25

    def a(u_, v):
        return (gg.integrate(gg.inner(gg.grad(v), gg.grad(u_)), dO)
                + gg.integrate((gam / h) * v * u_ - v * gg.inner(nd, gg.grad(u_))
                               - gg.inner(nd, gg.grad(v)) * u_, dGd))

    def l(v):
        return (gg.integrate(-2.0 * v, dO) + gg.integrate(v * gg.inner(nn, gradu), dGn)
                + gg.integrate((gam / h) * v * u - gg.inner(nd, gg.grad(v)) * u, dGd))

    op = gg.AffineFEOperator(a, l, U, V)
    uh = gg.solve(gg.LinearFESolver(gg.CGSolver(rtol=1e-13)), op)
    fx, _, dx, _ = V.dof_points()
    assert np.abs(uh.free_values - u(fx)).max() <= 1e-10
    assert np.array_equal(uh.get_dirichlet_dof_values(), u(dx))
