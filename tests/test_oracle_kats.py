"""The oracle against Gridap's own known-answer tests (tests/golden/gridap_kats.json, extracted
from Gridap's test files by tests/golden/extract_kats.py). These pin the CPU restatement
before it is trusted as the checker of the GPU library."""
import itertools

import numpy as np
import pytest


def test_quad_faces_match_gridap(orc, kats):
    ext, anc = orc.ncube_faces(2)
    dims = ext.sum(axis=1).tolist()
    assert dims == kats["quad_facedims"]["value"]
    # vertices of each edge: the face's anchor plus its extrusion span, vertex id 1 + x + 2y
    edges = []
    for e, a in zip(ext, anc):
        if e.sum() != 1:
            continue
        verts = []
        for t in (0, 1):
            p = a + t * e
            verts.append(1 + int(p[0]) + 2 * int(p[1]))
        edges.append(verts)
    assert edges == kats["quad_edge_vertices"]["value"]


def test_hex_faces_order():
    # 8 vertices, 12 edges (x-, y-, z-extruded), 6 faces (z-normal, y-normal, x-normal), 1 cell
    from oracle import oracle as orc
    ext, anc = orc.ncube_faces(3)
    assert ext.shape[0] == 27
    assert ext.sum(axis=1).tolist() == [0] * 8 + [1] * 12 + [2] * 6 + [3]
    faces = ext[20:26]
    assert faces.tolist() == [[1, 1, 0]] * 2 + [[1, 0, 1]] * 2 + [[0, 1, 1]] * 2
    assert anc[24].tolist() == [0, 0, 0] and anc[25].tolist() == [1, 0, 0]  # x=0 is tag 25


def test_gauss_legendre_matches_numpy(orc):
    for n in range(1, 12):
        x, w = orc.gauss_legendre01(n)
        xr, wr = np.polynomial.legendre.leggauss(n)
        assert np.allclose(x, (xr + 1) / 2, rtol=0, atol=2e-16 * 4)
        assert np.allclose(w, wr / 2, rtol=0, atol=4e-16 * 4)


@pytest.mark.parametrize("D", [2, 3])
def test_tensor_quadrature_exactness(orc, kats, D):
    k = kats["tensor_quadrature_exactness"]
    for degree in range(k["degrees"][0], k["degrees"][1] + 1):
        x, w = orc.tensor_quadrature(D, degree)
        assert abs(w.sum() - 1.0) < 1e-14
        errs, exact = [], []
        for expo in itertools.product(range(degree + 1), repeat=D):
            q = float(np.sum(w * np.prod(x ** np.array(expo), axis=1)))
            e = 1.0 / np.prod(np.array(expo) + 1.0)
            errs.append(abs(q - e))
            exact.append(abs(e))
        assert max(errs) / max(exact) < k["max_rel_err"]


def _clag(orc, kats, tags, ncomp, masks):
    k = kats["clagrangian_2x2"]
    coords, cells, ent = orc.cartesian_model(k["domain"], k["partition"])
    ntt = orc.node_tag_index(2, ent, tags) if tags else np.zeros(9, np.int8)
    return orc.clagrangian(ntt, cells, ncomp=ncomp, masks=masks)


def test_clagrangian_scalar(orc, kats):
    k = kats["clagrangian_2x2"]
    coords, cells, ent = orc.cartesian_model(k["domain"], k["partition"])
    node_dof, cell_dofs, nfree, ndiri = _clag(orc, kats, [], 1, None)
    assert np.array_equal(cell_dofs, cells)  # get_cell_dof_ids(V) == cell node ids
    assert nfree == 9 and ndiri == 0


def test_clagrangian_vector(orc, kats):
    k = kats["clagrangian_2x2"]
    node_dof, cell_dofs, nfree, ndiri = _clag(orc, kats, [], 2, None)
    assert cell_dofs.tolist() == k["vector_cell_dofs"]
    assert node_dof.tolist() == k["vector_node_and_comp_to_dof"]


def test_clagrangian_masked_scalar(orc, kats):
    k = kats["clagrangian_2x2"]
    masks = np.array(k["masks1"], np.uint8).reshape(-1, 1)
    node_dof, cell_dofs, nfree, ndiri = _clag(orc, kats, k["tags"], 1, masks)
    assert cell_dofs.tolist() == k["masked_cell_dofs"]
    assert node_dof[:, 0].tolist() == k["masked_node_and_comp_to_dof"]
    free_nodes = [i + 1 for i in range(9) if node_dof[i, 0] > 0]
    diri_nodes = [i + 1 for i in range(9) if node_dof[i, 0] < 0]
    assert free_nodes == k["masked_free_dof_to_node"]
    assert diri_nodes == k["masked_dirichlet_dof_to_node"]


def test_clagrangian_masked_vector(orc, kats):
    k = kats["clagrangian_2x2"]
    masks = np.array(k["masks2"], np.uint8)
    node_dof, cell_dofs, nfree, ndiri = _clag(orc, kats, k["tags"], 2, masks)
    assert cell_dofs.tolist() == k["masked_vector_cell_dofs"]
    assert node_dof.tolist() == k["masked_vector_node_and_comp_to_dof"]


def test_poisson_2x2_matrix_and_vector(orc, kats):
    k = kats["poisson_2x2_q1"]
    ref = orc.poisson_q1(k["domain"], k["partition"], k["dirichlet_tags"],
                         f_callable=lambda x: x[:, 1], degree=k["degree"])
    assert ref["nfree"] == 3
    A = orc.to_scipy(*ref["csc"], 3, 3).toarray()
    for i, j, v in k["mat_entries"]:
        assert abs(A[i - 1, j - 1] - v) <= 1e-13 * max(1.0, abs(v))
    assert np.allclose(ref["b"], k["vec"], rtol=1e-14, atol=1e-16)
    # the matrix Gridap prints is symmetric and its stored pattern is full 3x3 tridiagonal
    assert np.array_equal(A, A.T)


def test_oracle_csc_semantics(orc):
    """Pattern from InserterCSC equals the set of touched (row, col) pairs; values are the
    cell-order sums, checked against a dense accumulation."""
    rng = np.random.default_rng(0)
    ref = orc.poisson_q1((0, 1, 0, 1, 0, 1), (3, 4, 2), ("boundary",),
                         kappa=np.exp(rng.standard_normal(24)), fkind=orc.F_CONST,
                         fdata=np.array([1.0]))
    n = ref["nfree"]
    dense = np.zeros((n, n))
    touched = np.zeros((n, n), bool)
    for c, dofs in enumerate(ref["cell_dofs"]):
        for lj, j in enumerate(dofs):
            for li, i in enumerate(dofs):
                if i > 0 and j > 0:
                    dense[i - 1, j - 1] += ref["cellmats"][c, li, lj]
                    touched[i - 1, j - 1] = True
    A = orc.to_scipy(*ref["csc"], n, n)
    assert A.nnz == touched.sum()
    Ad = A.toarray()
    assert np.array_equal(Ad != 0, touched & (dense != 0))
    assert np.allclose(Ad, dense, rtol=1e-15, atol=1e-15)
    colptr, rowval, _ = ref["csc"]
    for j in range(n):  # sorted unique rows per column
        rows = rowval[colptr[j] - 1:colptr[j + 1] - 1]
        assert np.all(np.diff(rows) > 0)


def test_oracle_cg_matches_direct_solve(orc):
    import scipy.sparse.linalg as spla
    rng = np.random.default_rng(1)
    part = (8, 7, 6)
    nn = 9 * 8 * 7
    ref = orc.poisson_q1((0, 1, 0, 1, 0, 1), part, ("boundary",),
                         kappa=np.exp(rng.standard_normal(8 * 7 * 6)), fkind=orc.F_NODAL,
                         fdata=rng.standard_normal(nn))
    n = ref["nfree"]
    A = orc.to_scipy(*ref["csc"], n, n).tocsc()
    xd = spla.spsolve(A, ref["b"])
    for nt in (1, 2):
        x, it, rr = orc.pcg(*ref["csc"], ref["b"], 1e-12, nthreads=nt)
        assert rr <= 1e-12
        assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-9


def test_manufactured_nodal_solution(orc):
    """A discrete solution placed in the FE space is recovered exactly (to solver tolerance)."""
    rng = np.random.default_rng(2)
    ref = orc.poisson_q1((0, 2, 0, 1), (16, 9), ("boundary",), fkind=orc.F_NONE)
    n = ref["nfree"]
    u = rng.standard_normal(n)
    b = orc.csc_mul(*ref["csc"], u)
    x, it, rr = orc.pcg(*ref["csc"], b, 1e-13)
    assert np.linalg.norm(x - u) / np.linalg.norm(u) < 1e-10


def test_conforming_q2_matches_gridap_kat(orc, kats):
    k = kats["conforming_q2_3x3"]
    cd, nfree, ndiri = orc.conforming_q2(tuple(k["partition"]), k["dirichlet_tags"])
    assert cd.tolist() == k["cell_dofs"]
    assert (nfree, ndiri) == (k["nfree"], k["ndiri"])


def test_q2_shapes_partition_of_unity_and_nodality(orc):
    for D in (2, 3):
        # nodes at the face centres of the n-cube, in local order
        ext, anc = orc.ncube_faces(D)
        nodes = np.where(ext == 1, 0.5, anc.astype(float))
        phi, dphi = orc.q2_shapes(D, nodes)
        assert np.allclose(phi, np.eye(3 ** D), atol=1e-15)
        x, _ = orc.tensor_quadrature(D, 4)
        phi, dphi = orc.q2_shapes(D, x)
        assert np.allclose(phi.sum(axis=1), 1.0, atol=1e-14)
        assert np.allclose(dphi.sum(axis=1), 0.0, atol=1e-13)


# ---- simplexified boxes, P2 tets, Witherden-Vincent, elasticity ----------------------------
def test_extrusion_faces_restatement(orc, kats):
    quad = orc.extrusion_faces((1, 1))
    assert quad[1] == kats["quad_edge_vertices"]["value"]
    tet = orc.extrusion_faces((2, 2, 2))
    assert tet[1] == [[1, 2], [1, 3], [2, 3], [1, 4], [2, 4], [3, 4]]
    assert len(sum(tet, [])) == 15


def test_simplexify_matches_gridap_table(orc, kats):
    tv = orc.simplex_cells((1, 1, 1))
    assert tv.tolist() == kats["hex_simplexify"]["tets"]


def test_wv_tet_rule_matches_gridap_tables(orc, kats):
    x, w, res = orc.wv_tet_degree5()
    g = kats["wv_tet_degree4"]
    assert res < 1e-18
    assert np.abs(x - np.array(g["points"])).max() < 2e-16
    assert np.abs(w - np.array(g["weights"])).max() < 1e-17


def test_p2tet_nodal_basis(orc, kats):
    V = np.array(kats["tet_vertex_coordinates"]["value"], float)
    edges = orc.extrusion_faces((2, 2, 2))[1]
    nodes = np.vstack([V] + [(V[a - 1] + V[b - 1]) / 2 for a, b in edges])
    phi, dphi = orc.p2tet_shapes(nodes)
    assert np.abs(phi - np.eye(10)).max() < 1e-15
    # partition of unity and exact gradients of a quadratic
    x, w, _ = orc.wv_tet_degree5()
    phi, dphi = orc.p2tet_shapes(x)
    assert np.abs(phi.sum(1) - 1).max() < 1e-15
    f = lambda p: p[..., 0] ** 2 + 3 * p[..., 1] * p[..., 2] - p[..., 2]  # noqa: E731
    gx = np.stack([2 * x[:, 0], 3 * x[:, 2], 3 * x[:, 1] - 1], 1)
    assert np.abs(np.einsum("qn,n->q", phi, f(nodes)) - f(x)).max() < 1e-14
    assert np.abs(np.einsum("qnd,n->qd", dphi, f(nodes)) - gx).max() < 1e-13


def test_simplex_p2_numbering_counts(orc):
    for part in [(1, 1, 1), (2, 3, 2), (3, 3, 3)]:
        coords, _, _ = orc.cartesian_model((0, 1) * 3, part)
        vm = coords[:, 0] == 0.0
        cd, nf, nd = orc.simplex_p2_numbering(part, vm)
        nodes = np.prod([2 * n + 1 for n in part])
        assert nf + nd == 3 * nodes
        assert nd == 3 * (2 * part[1] + 1) * (2 * part[2] + 1)
        ids = cd.ravel()
        assert set(ids[ids > 0]) == set(range(1, nf + 1))
        assert set(-ids[ids < 0]) == set(range(1, nd + 1))
        # vertices are numbered before edges
        nv = int(np.prod([n + 1 for n in part]))
        vert = np.abs(cd[:, :4]).max()
        edge = np.abs(cd[:, 4:10][cd[:, 4:10] > 0]).min()
        assert vert <= 3 * nv and edge > 0


def test_elasticity_p2_invariants(orc):
    part = (2, 2, 2)
    rng = np.random.default_rng(0)
    lame = np.exp(rng.standard_normal((48, 2)))
    P = orc.elasticity_p2((0, 1) * 3, part, lame, clamp_x0=False)
    A = orc.to_scipy(*P["csc"], P["nfree"], P["nfree"])
    assert abs(A - A.T).max() <= 1e-15 * abs(A).max()
    cd = P["cell_dofs"]
    coords, _, _ = orc.cartesian_model((0, 1) * 3, part)
    # every dof's node position: vertices and edge midpoints
    tv = P["tet_vertices"]
    X = np.zeros((P["nfree"], 3))
    comp = np.zeros(P["nfree"], int)
    edges = orc.extrusion_faces((2, 2, 2))[1]
    for c in range(cd.shape[0]):
        xv = coords[tv[c] - 1]
        xn = np.vstack([xv] + [(xv[a - 1] + xv[b - 1]) / 2 for a, b in edges])
        for k in range(3):
            X[cd[c, k * 10:(k + 1) * 10] - 1] = xn
            comp[cd[c, k * 10:(k + 1) * 10] - 1] = k
    # rigid body modes are in the kernel
    for m in range(6):
        u = np.zeros(P["nfree"])
        if m < 3:
            u[comp == m] = 1.0
        else:
            a, b = [(1, 2), (2, 0), (0, 1)][m - 3]
            u[comp == a] = -X[comp == a, b]
            u[comp == b] = X[comp == b, a]
        assert np.abs(A @ u).max() < 1e-13 * abs(A).max()
    # energy of a linear field u = G x with constant lambda, mu
    P1 = orc.elasticity_p2((0, 1) * 3, part, np.tile([2.0, 0.5], 48), clamp_x0=False)
    A1 = orc.to_scipy(*P1["csc"], P1["nfree"], P1["nfree"])
    G = rng.standard_normal((3, 3))
    u = np.array([G[comp[i]] @ X[i] for i in range(P1["nfree"])])
    eps = 0.5 * (G + G.T)
    energy = 2.0 * np.trace(eps) ** 2 + 2 * 0.5 * np.sum(eps * eps)
    assert abs(u @ (A1 @ u) - energy) < 1e-12 * energy
    # body force: total load = int f over the box
    assert abs(P1["b"].reshape(-1)[comp == 2].sum() + 1.0) < 1e-14


def test_boundary_facets_2x2_kat(orc, kats):
    """Gridap's BoundaryTriangulation(model) on a 2x2 model of (0,4)^2: facet order, facet
    points in the owner cell and physical points at s = 0.25, 0.75
    (test/GeometryTests/BoundaryTriangulationsTests.jl)."""
    k = kats["boundary_facets_2x2"]
    part = tuple(k["partition"])
    cells, lfaces = orc.boundary_facets(part)
    coords, cell_nodes, _ = orc.cartesian_model(k["domain"], part)
    fverts = orc.extrusion_faces((1, 1))[1]
    refv = np.array([[(v >> d) & 1 for d in range(2)] for v in range(4)], np.float64)
    s = np.array(k["s"])[:, None]
    sphi, _ = orc.q1_shapes(1, s)
    assert len(cells) == len(k["cell_points"]) == 8
    for f in range(8):
        vs = [v - 1 for v in fverts[lfaces[f]]]
        np.testing.assert_allclose(sphi @ refv[vs], k["cell_points"][f], atol=0)
        X = coords[cell_nodes[cells[f], vs] - 1]
        np.testing.assert_allclose(sphi @ X, k["physical_points"][f], atol=1e-15)
    arrs = orc.facet_arrays(coords, cell_nodes, 1, cells, lfaces, 2)
    for f in range(8):
        np.testing.assert_allclose(arrs[f][4], k["normals"][f], atol=1e-15)


def test_facet_normal_derivatives(orc):
    """n⋅∇φ from the oracle's facet arrays equals the analytic outward derivative of the Q1
    and Q2 shape functions on an undistorted box (sum over the dofs of n⋅∇φ is 0, and for
    φ = 1 - x on the x = 0 facet, n⋅∇φ = +1/h)."""
    part, dom = (3, 2), (0, 3, 0, 1)
    coords, cell_nodes, _ = orc.cartesian_model(dom, part)
    cells, lfaces = orc.boundary_facets(part)
    for order in (1, 2):
        arrs = orc.facet_arrays(coords, cell_nodes, order, cells, lfaces, 4)
        for phi, dn, wm, xq, n in arrs:
            np.testing.assert_allclose(dn.sum(axis=1), 0.0, atol=1e-12)
            np.testing.assert_allclose(phi.sum(axis=1), 1.0, atol=1e-14)
    arrs = orc.facet_arrays(coords, cell_nodes, 1, cells, lfaces, 2)
    f = [i for i in range(len(cells)) if cells[i] == 0 and lfaces[i] == 2][0]  # x- of cell 0
    np.testing.assert_allclose(arrs[f][1][:, 0] + arrs[f][1][:, 2], 1.0, atol=1e-14)


def test_boundary_vector_measures(orc):
    """∫ 1 v dΓ summed over the dofs is the measure of Γ; the facet sizes of a jittered model
    are those of the box (its boundary nodes stay in place)."""
    for part, dom in (((3, 2), (0, 2, 0, 1)), ((2, 3, 2), (0, 1, 0, 2, 0, 3))):
        D = len(part)
        coords, cell_nodes, _ = orc.cartesian_model(dom, part)
        rng = np.random.default_rng(3)
        coords = orc.jitter_interior(part, coords, 0.05 * rng.standard_normal(coords.shape))
        ids = np.arange(cell_nodes.size, dtype=np.int32).reshape(cell_nodes.shape) + 1
        for tags, meas in ((None, None), ("tag_26" if D == 3 else "tag_8", None)):
            fc, fl = orc.boundary_facets(part, tags)
            b, _ = orc.boundary_vector(part, coords, cell_nodes, ids, 1, fc, fl, 2, 1.0,
                                       ids.size)
            L = [dom[2 * d + 1] - dom[2 * d] for d in range(D)]
            if tags is None:
                want = 2 * sum(np.prod([L[e] for e in range(D) if e != d]) for d in range(D))
            else:
                want = np.prod(L[1:])
            assert abs(b.sum() - want) <= 1e-13 * want


@pytest.mark.parametrize("law,params", [(0, (1.0, 0.5, 1.0)), (1, (3.0, 0.1)), (1, (4.0, 0.0))])
def test_quasilinear_jacobian_is_the_residual_derivative(orc, law, params):
    """The oracle's quasilinear Jacobian equals central differences of its residual (both on
    a jittered Q2 grid and a Q1 grid), so the law derivatives it restates are consistent."""
    rng = np.random.default_rng(11)
    for order, part in ((1, (3, 3)), (2, (2, 2))):
        coords, cells, _ = orc.cartesian_model((0, 1, 0, 1), part)
        coords = orc.jitter_interior(part, coords, 0.05 * rng.standard_normal(coords.shape))
        if order == 1:
            ids = np.arange(cells.size, dtype=np.int32).reshape(cells.shape) + 1
        else:
            ids, _, _ = orc.conforming_q2(part, [])
            ids = np.asarray(ids, np.int32)
        x = rng.random(int(ids.max()))
        f = lambda p: p[:, 0]  # noqa: E731
        M, _ = orc.quasilinear_cell_arrays(coords, cells, ids, order, 4, x, None, law, params,
                                           f=f)
        d = rng.standard_normal(x.size)
        eps = 1e-6
        _, vp = orc.quasilinear_cell_arrays(coords, cells, ids, order, 4, x + eps * d, None,
                                            law, params, f=f)
        _, vm = orc.quasilinear_cell_arrays(coords, cells, ids, order, 4, x - eps * d, None,
                                            law, params, f=f)
        jd = np.einsum("cij,cj->ci", M, d[ids - 1])
        assert np.abs((vp - vm) / (2 * eps) - jd).max() <= 1e-7 * np.abs(jd).max()


def test_reindexing_oracle_on_gridaps_case(orc):
    """test/FESpacesTests/FESpaceReindexingTests.jl: Q2 on a 4x4 box with Dirichlet
    boundary; every algorithm gives a permutation of the free dofs, RCM reduces the
    matrix bandwidth. A path graph is numbered end to end."""
    cd, nf, nd = orc.conforming_q2((4, 4), ["boundary"])

    def bw(c):
        m = 0
        for row in c:
            r = row[row > 0]
            if r.size:
                m = max(m, int(r.max() - r.min()))
        return m

    for alg in ("rcm", "sloan"):
        ip = orc.dof_permutation(cd, nf, alg)
        assert np.array_equal(np.sort(ip), np.arange(1, nf + 1))
    assert bw(orc.reindex_cell_dofs(cd, orc.dof_permutation(cd, nf, "rcm"))) < bw(cd)
    chain = np.array([[i + 1, i + 2] for i in range(5)], np.int32)
    for alg in ("rcm", "sloan"):
        ip = orc.dof_permutation(chain, 6, alg)
        assert list(ip) in ([6, 5, 4, 3, 2, 1], [1, 2, 3, 4, 5, 6])
    ptrs, data = orc.compute_adjacency(chain, 6)
    assert list(ptrs) == [1, 2, 4, 6, 8, 10, 11]
    assert list(data) == [2, 1, 3, 2, 4, 3, 5, 4, 6, 5]
