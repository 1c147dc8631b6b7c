"""Free-dof reordering on the device (gfe_dof_permutation) against the oracle's literal
restatement of Gridap's compute_adjacency / RCM (George-Liu) / Sloan
(FESpaces/FESpaceReindexing.jl): integer results, compared exactly.

Cases: Q1 and Q2 in 2-D and 3-D with Dirichlet tags, vector P2 on a simplexified box, a graph
with several components, and Gridap's own check (test/FESpacesTests/FESpaceReindexingTests.jl:
counts preserved, RCM lowers the bandwidth of the assembled Laplacian). The reindexed
assembly is the permuted matrix P A Pᵀ entry for entry.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _space(gg, part, order, tags):
    m = gg.CartesianDiscreteModel((0, 1) * len(part), part)
    return m, gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, order), dirichlet_tags=tags)


@pytest.mark.parametrize("part,order,tags", [
    ((4, 4), 2, "boundary"), ((7, 5), 1, "tag_1"), ((6, 4, 3), 1, "boundary"),
    ((3, 3, 2), 2, ["tag_21", "tag_26"]), ((9, 2), 2, []),
])
@pytest.mark.parametrize("alg", ["rcm", "sloan"])
def test_permutation_matches_oracle(gg, orc, part, order, tags, alg):
    _, V = _space(gg, part, order, tags)
    ip = gg.compute_dof_permutation(V, alg)
    want = orc.dof_permutation(V.cell_dof_ids, V.num_free_dofs(), alg)
    assert np.array_equal(ip, want)


@pytest.mark.parametrize("alg", ["rcm", "sloan"])
def test_sloan_weights_and_p2_vector_space(gg, orc, alg):
    m = gg.simplexify(gg.CartesianDiscreteModel((0, 1, 0, 1, 0, 1), (3, 2, 2)))
    m.add_tag_from_vertex_filter("x0", lambda x: np.abs(x[:, 0]) < 1e-12)
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, 3, 2), dirichlet_tags="x0")
    kw = {"w1": 2, "w2": 1} if alg == "sloan" else {}
    ip = gg.compute_dof_permutation(V, alg, **kw)
    want = orc.dof_permutation(V.cell_dof_ids, V.num_free_dofs(), alg, **kw)
    assert np.array_equal(ip, want)


def test_disconnected_components(gg, orc):
    """Two meshes side by side in one dof table: components are numbered one after the other
    (seeded at the minimum-degree unnumbered dof) and RCM reverses the whole sequence."""
    _, V1 = _space(gg, (4, 3), 1, "tag_1")
    _, V2 = _space(gg, (3, 5), 2, [])
    n1 = V1.num_free_dofs()
    ids2 = V2.cell_dof_ids.copy()
    ids2[ids2 > 0] += n1
    # pad the Q1 cells to 9 dofs with inert ids (0 is neither free nor Dirichlet)
    ids1 = np.zeros((V1.cell_dof_ids.shape[0], 9), np.int32)
    ids1[:, :4] = V1.cell_dof_ids
    ids = np.ascontiguousarray(np.vstack([ids2, ids1]), np.int32)
    n = n1 + V2.num_free_dofs()
    ctx = gg.default_context()
    from gridap_gb300 import _lib
    for alg, code in (("rcm", _lib.GFE_REORDER_RCM), ("sloan", _lib.GFE_REORDER_SLOAN)):
        ip = np.empty(n, np.int64)
        _lib.check(_lib.load().gfe_dof_permutation(ctx.handle, ids.shape[0], 9, _lib.ptr(ids),
                                                   n, code, 1, 2, _lib.ptr(ip)))
        assert np.array_equal(ip, orc.dof_permutation(ids, n, alg))


def test_gridap_reindexing_check_and_permuted_assembly(gg):
    m, V = _space(gg, (4, 4), 2, "boundary")
    dO = gg.Measure(gg.Triangulation(m), 5)
    a = lambda u, v: gg.integrate(gg.inner(gg.grad(v), gg.grad(u)), dO)  # noqa: E731
    A = gg.assemble_matrix(a, V, V)
    for alg in ("rcm", "sloan", "coordinates"):
        W = gg.reindex_free_dof_ids(V, alg)
        assert W.num_free_dofs() == V.num_free_dofs()
        assert W.num_dirichlet_dofs() == V.num_dirichlet_dofs()
    W = gg.reindex_free_dof_ids(V, "rcm")
    Ar = gg.assemble_matrix(a, W, W)
    from gridap_gb300.reindexing import bandwidth
    assert bandwidth(Ar) < bandwidth(A)
    P = W.free_dof_permutation - 1
    D, Dr = A.to_scipy().toarray(), Ar.to_scipy().toarray()
    Dp = np.zeros_like(D)
    Dp[np.ix_(P, P)] = D
    assert np.abs(Dr - Dp).max() <= 1e-13 * np.abs(D).max()
