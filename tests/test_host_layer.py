"""CPU tests of the product's host layer: the C-ABI library loads and exports every symbol
include/gfe.h declares, and its host-side set-up (Cartesian model arrays, face labels, dof
numbering) equals the oracle's. No kernel is launched here (no GPU in this container)."""
import ctypes
import pathlib
import re

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def declared_symbols():
    src = (ROOT / "include" / "gfe.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(gfe_[a-z0-9_]+)\(", src, re.M)))


def test_library_exports_every_declared_symbol(gg):
    lib = gg._lib.load()
    names = declared_symbols()
    assert len(names) >= 19
    for n in names:
        assert hasattr(lib, n), n
    # the Python binding covers the whole header
    assert sorted(gg._lib.SIGNATURES) == names


def test_version_and_error_channel(gg):
    lib = gg._lib.load()
    assert b"sm_103a" in lib.gfe_version()
    # a host-only call with bad arguments returns a status and a message
    st = lib.gfe_cartesian_model(5, None, None, None, None, None)
    assert st == gg._lib.GFE_ERR_INVALID_ARGUMENT
    assert b"gfe_cartesian_model" in lib.gfe_last_error()


@pytest.mark.parametrize("part", [(2, 2), (5, 3), (3, 4, 2), (1, 1, 1)])
def test_cartesian_model_matches_oracle(gg, orc, part):
    D = len(part)
    dom = tuple(v for d in range(D) for v in (-0.5 + d, 1.25 + 2 * d))
    m = gg.CartesianDiscreteModel(dom, part)
    coords, cells, ent = orc.cartesian_model(dom, part)
    assert np.array_equal(m.cell_node_ids, cells)
    assert np.array_equal(m.labels.node_entity, ent)
    assert np.array_equal(m.node_coords, coords)


@pytest.mark.parametrize("tags", [["boundary"], [1, 2, 3, 4, 6, 5], ["tag_5", "tag_7"],
                                  ["interior"], []])
def test_clagrangian_scalar_matches_oracle(gg, orc, tags):
    part = (6, 5)
    m = gg.CartesianDiscreteModel((0, 1, 0, 1), part)
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags=tags)
    coords, cells, ent = orc.cartesian_model((0, 1, 0, 1), part)
    ntt = orc.node_tag_index(2, ent, tags) if tags else np.zeros(ent.shape[0], np.int8)
    node_dof, cell_dofs, nfree, ndiri = orc.clagrangian(ntt, cells)
    assert np.array_equal(V.cell_dof_ids, cell_dofs)
    assert (V.nfree, V.ndiri) == (nfree, ndiri)


def test_clagrangian_3d_boundary(gg, orc):
    part = (4, 3, 5)
    m = gg.CartesianDiscreteModel((0, 1, 0, 1, 0, 1), part)
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    assert V.nfree == 3 * 2 * 4
    coords, cells, ent = orc.cartesian_model((0, 1, 0, 1, 0, 1), part)
    ntt = orc.node_tag_index(3, ent, ["boundary"])
    _, cell_dofs, nfree, _ = orc.clagrangian(ntt, cells)
    assert np.array_equal(V.cell_dof_ids, cell_dofs)
    # tag_25 is the x=0 face of the box
    V25 = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="tag_25")
    x0 = np.isclose(m.node_coords[:, 0], 0) & ~np.isclose(m.node_coords[:, 1], 0) & \
        ~np.isclose(m.node_coords[:, 1], 1) & ~np.isclose(m.node_coords[:, 2], 0) & \
        ~np.isclose(m.node_coords[:, 2], 1)
    assert V25.ndiri == int(x0.sum())


def test_clagrangian_masked_vector_kat(gg, kats):
    k = kats["clagrangian_2x2"]
    m = gg.CartesianDiscreteModel(tuple(k["domain"]), tuple(k["partition"]))
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, 2, 1), dirichlet_tags=k["tags"],
                   dirichlet_masks=np.array(k["masks2"], np.uint8))
    assert V.cell_dof_ids.tolist() == k["masked_vector_cell_dofs"]
    assert V.node_comp_to_dof.tolist() == k["masked_vector_node_and_comp_to_dof"]
    V1 = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags=k["tags"],
                    dirichlet_masks=np.array(k["masks1"], np.uint8).reshape(-1, 1))
    assert V1.cell_dof_ids.tolist() == k["masked_cell_dofs"]


def test_weak_form_recognition(gg):
    m = gg.CartesianDiscreteModel((0, 1, 0, 1), (2, 2))
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    u, v = gg.get_trial_fe_basis(V), gg.get_fe_basis(V)
    from importlib import import_module
    cd = import_module("gridap_gb300.celldata")
    assert cd.classify_bilinear(gg.inner(gg.grad(v), gg.grad(u))) == ("diffusion", None)
    k = gg.CellField(np.ones(4))
    assert cd.classify_bilinear(k * gg.inner(gg.grad(v), gg.grad(u)))[1] is k
    assert cd.classify_bilinear(gg.inner(k * gg.grad(v), gg.grad(u)))[1] is k
    assert cd.classify_linear(3.0 * v) == ("source", 3.0)
    with pytest.raises(NotImplementedError):
        cd.classify_bilinear(gg.inner(gg.grad(v), gg.grad(v)))
    with pytest.raises(NotImplementedError):
        cd.classify_linear(gg.grad(v))


@pytest.mark.parametrize("part,tags", [((3, 3), ["tag_1", "tag_6"]), ((4, 5), ["boundary"]),
                                       ((3, 2, 4), ["boundary"]), ((2, 3, 2), ["tag_25", 7]),
                                       ((4, 4, 4), []), ((1, 2, 1), ["tag_21"])])
def test_conforming_q2_matches_oracle(gg, orc, part, tags):
    D = len(part)
    m = gg.CartesianDiscreteModel((0, 1) * D, part)
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 2), dirichlet_tags=tags)
    cd, nfree, ndiri = orc.conforming_q2(part, tags)
    assert np.array_equal(V.cell_dof_ids, cd)
    assert (V.nfree, V.ndiri) == (nfree, ndiri)


def test_conforming_q2_vector_components(gg, orc):
    """Vector Q2 (3 components) with a component mask: product vs oracle."""
    part = (2, 3, 2)
    masks = np.array([[1, 0, 1]], np.uint8)
    m = gg.CartesianDiscreteModel((0, 1) * 3, part)
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, 3, 2), dirichlet_tags=["tag_25"],
                   dirichlet_masks=masks)
    cd, nfree, ndiri = orc.conforming_q2(part, ["tag_25"], ncomp=3, masks=masks)
    assert np.array_equal(V.cell_dof_ids, cd)
    assert (V.nfree, V.ndiri) == (nfree, ndiri)


def test_box_cell_dofs_matches_fespace(gg):
    from gridap_gb300 import workloads
    for n in (2, 3, 5):
        m = gg.CartesianDiscreteModel((0, 1) * 3, (n, n, n))
        V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
        assert np.array_equal(workloads.box_cell_dofs(n), np.asarray(V.cell_dof_ids))


def test_batched_workload_sizes():
    import __graft_entry__ as ge
    ge.load_package()
    from gridap_gb300 import workloads
    sizes, kappas = workloads.batched_diffusion(256)
    assert len(sizes) == 256 and min(sizes) >= 16 and max(sizes) <= 64
    assert all(k.size == n ** 3 for n, k in zip(sizes, kappas))


@pytest.mark.parametrize("part,face", [((1, 1, 1), 0), ((2, 3, 2), 0), ((3, 2, 4), 1),
                                       ((4, 4, 4), None)])
def test_simplex_p2_numbering_matches_oracle(gg, orc, part, face):
    m = gg.simplexify(gg.CartesianDiscreteModel((0, 1) * 3, part))
    assert np.array_equal(m.cell_node_ids, orc.simplex_cells(part))
    coords, _, _ = orc.cartesian_model((0, 1) * 3, part)
    if face is None:
        vm = np.zeros(coords.shape[0], bool)
        tags = ()
    else:
        vm = np.abs(coords[:, face] - (0.0 if face == 0 else 1.0)) < 1e-12
        m.add_tag_from_vertex_filter("clamp", lambda x: np.abs(x[:, face] - (0.0 if face == 0
                                                                              else 1.0)) < 1e-12)
        tags = "clamp"
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, 3, 2), dirichlet_tags=tags)
    cd, nf, nd = orc.simplex_p2_numbering(part, vm)
    assert (V.nfree, V.ndiri) == (nf, nd)
    assert np.array_equal(V.cell_dof_ids, cd)
    # component mask: only z clamped
    if face is not None:
        V2 = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, 3, 2), dirichlet_tags=tags,
                        dirichlet_masks=[[0, 0, 1]])
        cd2, nf2, nd2 = orc.simplex_p2_numbering(part, vm, comp_mask=[0, 0, 1])
        assert np.array_equal(V2.cell_dof_ids, cd2) and (V2.nfree, V2.ndiri) == (nf2, nd2)


def test_elasticity_form_recognition(gg):
    from gridap_gb300.celldata import classify_bilinear, classify_linear
    u, v = gg.get_trial_fe_basis(None), gg.get_fe_basis(None)
    sigma = gg.isotropic_stress(2.0, 0.5)
    kind, lm = classify_bilinear(gg.inner(gg.ε(v), sigma(gg.ε(u))))
    assert kind == "elasticity" and lm == (2.0, 0.5)
    kind, f = classify_linear(gg.inner((0.0, 0.0, -1.0), v))
    assert kind == "body_force" and np.array_equal(f, [0, 0, -1])
    with pytest.raises(NotImplementedError):
        classify_bilinear(gg.inner(gg.ε(v), gg.ε(u)))


def test_boundary_facets_kat_and_order(gg, orc, kats):
    """The product's BoundaryTriangulation reproduces Gridap's 2x2 facet KAT and the oracle's
    facet order for tag selections in 2-D and 3-D."""
    k = kats["boundary_facets_2x2"]
    m = gg.CartesianDiscreteModel(k["domain"], k["partition"])
    G = gg.BoundaryTriangulation(m)
    ref, phys = G.facet_points(np.array(k["s"])[:, None])
    np.testing.assert_array_equal(ref, k["cell_points"])
    np.testing.assert_allclose(phys, k["physical_points"], atol=1e-15)
    np.testing.assert_array_equal(G.get_facet_normal() + 0.0, np.array(k["normals"])[:, 0] + 0.0)
    for part, tags in (((3, 2), None), ((3, 2), "tag_7"), ((4, 3), ["tag_5", 8]),
                       ((2, 3, 2), None), ((2, 3, 2), ["tag_21", "tag_24", "tag_26"]),
                       ((3, 1, 2), "boundary"), ((2, 2, 2), "interior")):
        m = gg.CartesianDiscreteModel((0, 1) * len(part), part)
        G = gg.BoundaryTriangulation(m, tags=tags)
        c, l = orc.boundary_facets(part, tags)
        assert np.array_equal(G.facet_cells, c) and np.array_equal(G.facet_lfaces, l)


def test_boundary_forms_and_facet_points(gg, orc):
    """Linear forms split into the volume source and the ∫ g v dΓ terms; the facet Gauss
    points handed to a callable g come in the oracle's order (facet by facet, first facet
    coordinate fastest), on a jittered model too."""
    from importlib import import_module
    A = import_module(gg.__name__ + ".assembly")
    part = (3, 2, 2)
    nn = int(np.prod(np.array(part) + 1))
    jit = 0.05 * np.random.default_rng(2).standard_normal((nn, 3))
    m = gg.CartesianDiscreteModel((0, 1, 0, 2, 0, 1), part, node_jitter=jit)
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="tag_01")
    dO = gg.Measure(gg.Triangulation(m), 2)
    G = gg.BoundaryTriangulation(m, tags=["tag_23", "tag_26"])
    dG = gg.Measure(G, 4)
    fo = A._forms(None, lambda v: gg.integrate(2.0 * v, dO) + gg.integrate(3.0 * v, dG), V, V)
    assert fo.source == 2.0 and fo.boundary == [(dG, [(0, 3.0, None)])]
    fo = A._forms(None, lambda v: gg.integrate(3.0 * v, dG), V, V)
    assert fo.source is None and len(fo.boundary) == 1
    # Nitsche terms: (γ/h) v u - v (n⋅∇u) - (n⋅∇v) u and (γ/h) v g - (n⋅∇v) g
    n = gg.get_normal_vector(G)
    g = lambda x: x[:, 0]  # noqa: E731
    fo = A._forms(lambda u, v: gg.integrate(gg.inner(gg.grad(v), gg.grad(u)), dO)
                  + gg.integrate(40.0 * v * u - v * gg.inner(n, gg.grad(u))
                                 - gg.inner(n, gg.grad(v)) * u, dG),
                  lambda v: gg.integrate(40.0 * v * g - gg.inner(n, gg.grad(v)) * g, dG), V, V)
    assert fo.boundary_mat == [(dG, (40.0, -1.0, -1.0, 0.0))]
    assert fo.boundary == [(dG, [(0, 40.0, g), (1, -1.0, g)])]
    with pytest.raises(NotImplementedError):  # a gradient term that is not along n
        A._forms(lambda u, v: gg.integrate(gg.inner(gg.grad(v), gg.grad(u)), dO)
                 + gg.integrate(gg.inner(gg.grad(v), gg.grad(u)), dG), None, V, V)
    g = lambda x: x[:, 0] + 10 * x[:, 1] + 100 * x[:, 2]  # noqa: E731
    xq = A._facet_qpoints(G, 4)
    assert xq.shape == (G.num_cells(), dG.num_points(), 3)
    _, gvals = orc.boundary_vector(part, m.node_coords, m.cell_node_ids, V.cell_dof_ids, 1,
                                   G.facet_cells, G.facet_lfaces, 4, g, V.num_free_dofs())
    np.testing.assert_allclose(g(xq.reshape(-1, 3)), gvals.reshape(-1), rtol=1e-14, atol=1e-14)


def test_quasilinear_forms_are_recognised(gg):
    """Residuals κ ∇v⋅flux(∇u) - f v and κ α(u) ∇v⋅∇u - f v are recognised, a matching
    Jacobian is accepted and one that drops a derivative term is refused."""
    from importlib import import_module
    cd = import_module(gg.__name__ + ".celldata")
    m = gg.CartesianDiscreteModel((0, 1, 0, 1), (3, 3))
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 2))
    u, v, du = cd._FEState(None), cd.get_fe_basis(V), cd.get_trial_fe_basis(V)
    k = gg.CellField(np.ones(9))
    f = lambda x: x[:, 0]  # noqa: E731
    flux, alpha = gg.PowerLawFlux(3.0, 0.1), gg.PolynomialCoefficient(1.0, 0.5, 1.0)
    F = cd.classify_residual(k * gg.inner(gg.grad(v), flux(gg.grad(u))) - f * v)
    assert F.law is flux and F.cells == [k] and F.source == (1.0, f)
    cd.check_jacobian(k * gg.inner(gg.grad(v), flux.derivative(gg.grad(du), gg.grad(u))), F)
    F = cd.classify_residual(2.0 * alpha(u) * gg.inner(gg.grad(v), gg.grad(u)))
    assert F.law is alpha and F.scale == 2.0 and F.source is None
    cd.check_jacobian(2.0 * alpha(u) * gg.inner(gg.grad(v), gg.grad(du))
                      + 2.0 * alpha.derivative(u) * du * gg.inner(gg.grad(v), gg.grad(u)), F)
    with pytest.raises(NotImplementedError):
        cd.check_jacobian(2.0 * alpha(u) * gg.inner(gg.grad(v), gg.grad(du)), F)
    with pytest.raises(NotImplementedError):
        cd.classify_residual(gg.inner(gg.grad(v), gg.grad(u)) * u)


def test_coordinate_reordering_matches_oracle(gg, orc):
    """reindex_free_dof_ids(V, "coordinates") sorts free dofs by their nodes' coordinates
    (lexicographic, stable), as the oracle's restatement of _coordinates_perm does."""
    for order, part in ((1, (4, 3)), (2, (3, 2, 2))):
        m = gg.CartesianDiscreteModel((0, 1) * len(part), part)
        V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, order), dirichlet_tags="tag_1"
                       if len(part) == 2 else "tag_01")
        ip = gg.compute_dof_permutation(V, "coordinates")
        fx, _, _, _ = V.dof_points()
        assert np.array_equal(ip, orc.dof_permutation(V.cell_dof_ids, V.num_free_dofs(),
                                                      "coordinates", coords=fx))
        W = gg.reindex_free_dof_ids(V, ip)
        assert W.num_free_dofs() == V.num_free_dofs()
        assert W.num_dirichlet_dofs() == V.num_dirichlet_dofs()
        fw, _, _, _ = W.dof_points()
        assert np.array_equal(fw[ip - 1], fx)


def test_block_field_offsets_kat(gg):
    """MultiFieldFESpacesTests.jl:121-145: field offsets and block sizes of permuted block
    layouts (there with Q1, Q2, Q3 fields; here Q1, Q2 and a vector Q1 field stand in)."""
    model = gg.CartesianDiscreteModel((0.0, 1.0, 0.0, 1.0), (2, 2))
    V1 = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 1))
    V2 = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 2))
    V3 = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, 2, 1))
    nd = [V.num_free_dofs() for V in (V1, V2, V3)]
    assert nd == [9, 25, 18]
    X1 = gg.MultiFieldFESpace([V1, V2, V3], style=gg.BlockMultiFieldStyle(2, (2, 1), (1, 2, 3)))
    X2 = gg.MultiFieldFESpace([V1, V2, V3], style=gg.BlockMultiFieldStyle(2, (2, 1), (3, 1, 2)))
    X3 = gg.MultiFieldFESpace([V1, V2, V3], style=gg.BlockMultiFieldStyle(2, (1, 2), (1, 3, 2)))
    assert gg.compute_field_offsets(X1) == (0, nd[0], 0)
    assert gg.compute_field_offsets(X2) == (nd[2], 0, 0)
    assert gg.compute_field_offsets(X3) == (0, nd[2], 0)
    assert X1.block_num_free_dofs() == [nd[0] + nd[1], nd[2]]
    assert X2.block_num_free_dofs() == [nd[2] + nd[0], nd[1]]
    assert X3.block_num_free_dofs() == [nd[0], nd[2] + nd[1]]
    # consecutive: offsets are the running sums; cell ids shift only the free dofs
    X = gg.MultiFieldFESpace([V1, V2, V3])
    assert gg.compute_field_offsets(X) == (0, nd[0], nd[0] + nd[1])
    ids = X.get_cell_dof_ids()
    assert ids.shape == (4, 4 + 9 + 8)
    assert np.array_equal(ids[:, :4], V1.get_cell_dof_ids())
    assert np.array_equal(ids[:, 4:13], V2.get_cell_dof_ids() + nd[0])
    x = np.arange(X.num_free_dofs(), dtype=float)
    assert np.array_equal(X.restrict_to_field(x, 2), x[nd[0] + nd[1]:])
    xb = X2.zero_free_values()
    assert [v.size for v in xb] == X2.block_num_free_dofs()


def test_multifield_forms_are_classified(gg):
    """Stokes' a((u,p),(v,q)) and l((v,q)) split into one term per operand pair."""
    import importlib
    cd = importlib.import_module(gg.__name__ + ".celldata")
    model = gg.CartesianDiscreteModel((0.0, 1.0, 0.0, 1.0), (2, 2))
    V = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, 2, 2), dirichlet_tags="boundary")
    Q = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 1))
    X = gg.MultiFieldFESpace([V, Q])
    (u, p), (v, q) = gg.get_trial_fe_basis(X), gg.get_fe_basis(X)
    kap = gg.CellField(np.ones(4))
    e = gg.inner(gg.grad(v), gg.grad(u)) - gg.div(v) * p + q * gg.div(u) + kap * (2.0 * q * p)
    terms = cd.classify_multifield(e, True)
    got = [(t.test_field, t.test_op, t.trial_field, t.trial_op, t.coef) for t in terms]
    assert got == [(0, cd.MOP_GRAD, 0, cd.MOP_GRAD, 1.0), (0, cd.MOP_DIV, 1, cd.MOP_VALUE, -1.0),
                   (1, cd.MOP_VALUE, 0, cd.MOP_DIV, 1.0), (1, cd.MOP_VALUE, 1, cd.MOP_VALUE, 2.0)]
    assert terms[3].cell_coef is not None
    f = lambda x: x  # noqa: E731
    lt = cd.classify_multifield(gg.inner(v, f) - 3.0 * q, False)
    assert [(t.test_field, t.test_op, t.trial_field, t.coef) for t in lt] == \
        [(0, cd.MOP_VALUE, None, 1.0), (1, cd.MOP_VALUE, None, -3.0)]
    assert lt[0].data is f and lt[1].data is None
    with pytest.raises(NotImplementedError):
        cd.classify_multifield(gg.inner(gg.grad(v), gg.grad(u)) * p, True)


def test_lagrangian_tables_reproduce_polynomials(gg):
    """Q1/Q2 shape tables in Gridap's node order interpolate their polynomials exactly."""
    import importlib
    mf = importlib.import_module(gg.__name__ + ".multifield")
    fs = importlib.import_module(gg.__name__ + ".fespaces")
    for D in (2, 3):
        qx, qw = mf.tensor_gauss(D, 4)
        assert abs(qw.sum() - 1.0) < 1e-14
        for order in (1, 2):
            phi, grads = mf.lagrangian_tables(D, order, qx)
            xn = fs.ncube_node_refs(D, order)
            c = np.arange(1, D + 1, dtype=float)
            if order == 1:
                p = lambda x: 1.0 + x @ c + np.prod(x[:, :2], axis=1)  # noqa: E731
            else:
                p = lambda x: 1.0 + x @ c + (x[:, 0] ** 2) * x[:, 1]  # noqa: E731
            assert np.abs(phi @ p(xn) - p(qx)).max() < 1e-13
            h = 1e-6
            for e in range(D):
                dx = np.zeros(D)
                dx[e] = h
                fd = (p(qx + dx) - p(qx - dx)) / (2 * h)
                assert np.abs(grads[:, :, e] @ p(xn) - fd).max() < 1e-8
