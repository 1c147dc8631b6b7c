"""GPU parity of vector P2 elasticity on simplexified Cartesian boxes (the configuration of
3-D linear elasticity with per-cell Lamé coefficients, body force (0, 0, -1) and the x = 0
face clamped).

Against the oracle (a literal restatement of Gridap's per-quadrature-point arithmetic and
InserterCSC assembly): the CSR pattern bit-exact, FP64 values within 1e-12 of each row's
largest entry, the load vector within 1e-12 of its largest entry. FP32 cell matrices
(scatter still FP64) within 1e-5 of the row maximum (FP32 keeps 24 bits; the tables and
Jacobians are formed in FP64 and rounded once, plus FP32 products).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_VAL = 1e-12


def _rowscaled_err(rp, nz, ref_nz):
    err = 0.0
    for r in range(rp.shape[0] - 1):
        a, b = rp[r], rp[r + 1]
        if b > a:
            s = np.abs(ref_nz[a:b]).max()
            err = max(err, np.abs(nz[a:b] - ref_nz[a:b]).max() / max(s, 1e-300))
    return err


def _space(gg, part):
    m = gg.simplexify(gg.CartesianDiscreteModel((0, 1) * 3, part))
    m.add_tag_from_vertex_filter("x0", lambda x: np.abs(x[:, 0]) < 1e-12)
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, 3, 2), dirichlet_tags="x0")
    return m, V


def _assemble(gg, V, m, lame, precision="fp64", geometry=None):
    import ctypes as C
    from gridap_gb300 import _lib
    dO = gg.Measure(gg.Triangulation(m), 4)
    lam, mu = gg.CellField(lame[:, 0]), gg.CellField(lame[:, 1])
    prep = gg.prepare_problem(V, V, dO, (lam, mu), np.array([0.0, 0.0, -1.0]),
                              precision=precision, geometry=geometry)
    assem = gg.SparseMatrixAssembler(V, V)
    A = gg.symbolic_loop_matrix(assem, (None, V.cell_dof_ids, V.cell_dof_ids))
    b = np.zeros(V.nfree)
    _lib.check(_lib.load().gfe_assemble_matrix_and_vector(
        assem.ctx.handle, C.byref(prep.p), A.handle, _lib.ptr(b)))
    return A, b


@pytest.mark.parametrize("part", [(2, 2, 2), (4, 3, 5)])
@pytest.mark.parametrize("geometry", [None, "nodal"])
def test_p2_elasticity_fp64_matches_oracle(gg, orc, part, geometry):
    rng = np.random.default_rng(80 + part[2])
    m, V = _space(gg, part)
    lame = np.exp(rng.standard_normal((m.num_cells(), 2)))
    ref = orc.elasticity_p2((0, 1) * 3, part, lame)
    assert V.nfree == ref["nfree"]
    A, b = _assemble(gg, V, m, lame, geometry=geometry)
    rp, cv, nz = A.export_csr(1)
    cp, rv, zv = ref["csc"]
    assert np.array_equal(rp, cp) and np.array_equal(cv, rv)  # symmetric: CSR == CSC
    assert _rowscaled_err(rp - 1, nz, zv) <= TOL_VAL
    assert np.abs(b - ref["b"]).max() <= TOL_VAL * np.abs(ref["b"]).max()


def test_p2_elasticity_fp32_cells_close(gg, orc):
    rng = np.random.default_rng(91)
    part = (3, 4, 3)
    m, V = _space(gg, part)
    lame = np.exp(rng.standard_normal((m.num_cells(), 2)))
    ref = orc.elasticity_p2((0, 1) * 3, part, lame)
    for geometry in (None, "nodal"):
        A, b = _assemble(gg, V, m, lame, precision="fp32", geometry=geometry)
        rp, cv, nz = A.export_csr(1)
        assert np.array_equal(cv, ref["csc"][1])
        assert _rowscaled_err(rp - 1, nz, ref["csc"][2]) <= 1e-5
        assert np.abs(b - ref["b"]).max() <= 1e-12 * np.abs(ref["b"]).max()


def test_p2_elasticity_affine_op_and_fcg_solve(gg, orc):
    """AffineFEOperator through the recognised weak form, then FCG (Jacobi) to 1e-8 against
    the oracle's own solve of its matrix."""
    rng = np.random.default_rng(92)
    part = (4, 4, 4)
    m, V = _space(gg, part)
    lame = np.exp(rng.standard_normal((m.num_cells(), 2)))
    dO = gg.Measure(gg.Triangulation(m), 4)
    sigma = gg.isotropic_stress(gg.CellField(lame[:, 0]), gg.CellField(lame[:, 1]))
    op = gg.AffineFEOperator(lambda u, v: gg.integrate(gg.inner(gg.ε(v), sigma(gg.ε(u))), dO),
                             lambda v: gg.integrate(gg.inner((0.0, 0.0, -1.0), v), dO), V, V)
    ref = orc.elasticity_p2((0, 1) * 3, part, lame)
    rp, cv, nz = op.A.export_csr(1)
    assert np.array_equal(cv, ref["csc"][1])
    assert _rowscaled_err(rp - 1, nz, ref["csc"][2]) <= TOL_VAL
    x = np.empty(V.nfree)
    ns = gg.numerical_setup(gg.symbolic_setup(gg.FCGSolver(rtol=1e-8), op.A), op.A)
    gg.solve_(x, ns, op.b)
    assert ns.report.converged and ns.report.relres <= 1e-8
    S = orc.to_scipy(*ref["csc"], V.nfree, V.nfree)
    r = ref["b"] - S @ x
    assert np.linalg.norm(r) / np.linalg.norm(ref["b"]) <= 1.01e-8
    import scipy.sparse.linalg as sl
    xs = sl.spsolve(S.tocsc(), ref["b"])
    assert np.linalg.norm(x - xs) <= 1e-5 * np.linalg.norm(xs)


def test_p2_elasticity_vector_only(gg, orc):
    rng = np.random.default_rng(93)
    part = (2, 3, 2)
    m, V = _space(gg, part)
    lame = np.exp(rng.standard_normal((m.num_cells(), 2)))
    ref = orc.elasticity_p2((0, 1) * 3, part, lame)
    dO = gg.Measure(gg.Triangulation(m), 4)
    b = gg.assemble_vector(lambda v: gg.integrate(gg.inner((0.0, 0.0, -1.0), v), dO), V)
    assert np.abs(b - ref["b"]).max() <= TOL_VAL * np.abs(ref["b"]).max()


def test_generic_numeric_loop_bit_exact_wide_cells(gg, orc):
    """Caller cell matrices with 30 dofs per cell (the warp-per-row gather) give exactly the
    oracle's InserterCSC sums: the same additions in the same cell order."""
    import scipy.sparse as sp
    rng = np.random.default_rng(94)
    part = (3, 3, 2)
    m, V = _space(gg, part)
    lame = np.exp(rng.standard_normal((m.num_cells(), 2)))
    ref = orc.elasticity_p2((0, 1) * 3, part, lame)
    cm = ref["cellmats"] * (1 + 1e-3 * rng.standard_normal(ref["cellmats"].shape))
    ids = ref["cell_dofs"]
    n = ref["nfree"]
    csc = orc.assemble_csc(ids, ids, cm, n, n)
    assem = gg.SparseMatrixAssembler(V, V)
    A = gg.symbolic_loop_matrix(assem, (None, ids, ids))
    gg.numeric_loop_matrix(A, assem, (cm, ids, ids))
    S = sp.csc_matrix((csc[2], csc[1] - 1, csc[0] - 1), shape=(n, n)).tocsr()
    S.sort_indices()
    rp, col, nz = A.export_csr(0)
    assert np.array_equal(rp, S.indptr) and np.array_equal(col, S.indices)
    assert np.array_equal(nz, S.data)


@pytest.mark.parametrize("part", [(6, 5, 4), (12, 12, 12)])
def test_p2_two_level_fcg(gg, orc, part):
    """Vector P2 elasticity on a simplexified box, flexible CG with the two-level
    preconditioner (Chebyshev-Jacobi on P2, the P1 elasticity matrix of the same tets solved
    approximately by Jacobi-PCG): the FP64 relative residual in the oracle's own system, in far
    fewer iterations than Jacobi-preconditioned FCG."""
    rng = np.random.default_rng(sum(part) + 11)
    m, V = _space(gg, part)
    lame = np.exp(rng.standard_normal((m.num_cells(), 2)))
    dO = gg.Measure(gg.Triangulation(m), 4)
    sigma = gg.isotropic_stress(gg.CellField(lame[:, 0]), gg.CellField(lame[:, 1]))
    op = gg.AffineFEOperator(lambda u, v: gg.integrate(gg.inner(gg.ε(v), sigma(gg.ε(u))), dO),
                             lambda v: gg.integrate(gg.inner((0.0, 0.0, -1.0), v), dO), V, V)
    reps = {}
    for name, solver in (("two_level", gg.FCGSolver(rtol=1e-8, pc="mg")),
                         ("jacobi", gg.FCGSolver(rtol=1e-8))):
        x = np.empty(V.nfree)
        ns = gg.numerical_setup(gg.symbolic_setup(solver, op.A), op.A)
        gg.solve_(x, ns, op.b)
        reps[name] = (x, ns.report)
    x, rep = reps["two_level"]
    assert rep.converged and rep.relres <= 1e-8
    assert rep.iterations < 0.25 * reps["jacobi"][1].iterations
    ref = orc.elasticity_p2((0, 1) * 3, part, lame)
    ro = ref["b"] - orc.csc_mul(*ref["csc"], x)
    assert np.linalg.norm(ro) <= 1.01e-8 * np.linalg.norm(ref["b"])


def _oracle_jittered(orc, part, lame, jit, f=(0.0, 0.0, -1.0)):
    """The oracle's elasticity_p2 on a simplexified box whose nodes are displaced by `jit`
    (the clamped face chosen on the undisplaced nodes, as the model's tag is)."""
    part = np.asarray(part, np.int64)
    coords, _, _ = orc.cartesian_model((0, 1) * 3, part)
    tv = orc.simplex_cells(part)
    vmask = np.abs(coords[:, 0]) < 1e-12
    cd, nfree, _ = orc.simplex_p2_numbering(part, vmask)
    x, w, _ = orc.wv_tet_degree5()
    xj = np.ascontiguousarray(coords + jit)
    nc = tv.shape[0]
    mats = np.empty((nc, 30, 30))
    vecs = np.empty((nc, 30))
    lm = np.ascontiguousarray(lame, np.float64).reshape(-1)
    fv = np.ascontiguousarray(f, np.float64)
    rc = orc.lib().orc_p2tet_cell_arrays_elasticity(nc, orc._p(tv), orc._p(xj), orc._p(lm), 14,
                                                    orc._p(x), orc._p(w), orc._p(fv),
                                                    orc._p(mats), orc._p(vecs))
    assert rc == 0
    mats = np.ascontiguousarray(np.transpose(mats, (0, 2, 1)))
    return dict(nfree=nfree, csc=orc.assemble_csc(cd, cd, mats, nfree, nfree),
                b=orc.assemble_vector(cd, vecs, nfree))


@pytest.mark.parametrize("part", [(3, 3, 2), (5, 4, 4)])
def test_p2_tensor_core_cells_jittered_match_oracle(gg, orc, part):
    """FP32 cell matrices of general affine tets from the tensor cores (tcgen05 kind::f16
    with split FP16 operands: about 22 significant bits) against the oracle's FP64 cell
    integrals on displaced nodes: within 1e-5 of each row's largest entry (the FP32 path's
    tolerance), the load vector (FP64) within 1e-12, the pattern bit-exact."""
    rng = np.random.default_rng(95 + part[0])
    m, V = _space(gg, part)
    h = 1.0 / np.asarray(part, np.float64)
    jit = rng.uniform(-0.1, 0.1, m.node_coords.shape) * h
    m.node_coords[:] += jit
    lame = np.exp(rng.standard_normal((m.num_cells(), 2)))
    ref = _oracle_jittered(orc, part, lame, jit)
    assert V.nfree == ref["nfree"]
    A, b = _assemble(gg, V, m, lame, precision="fp32", geometry="nodal")
    rp, cv, nz = A.export_csr(1)
    cp, rv, zv = ref["csc"]
    assert np.array_equal(rp, cp) and np.array_equal(cv, rv)
    assert _rowscaled_err(rp - 1, nz, zv) <= 1e-5
    assert np.abs(b - ref["b"]).max() <= 1e-12 * np.abs(ref["b"]).max()
    # and the FP64 path on the same displaced nodes
    A64, b64 = _assemble(gg, V, m, lame, precision="fp64", geometry="nodal")
    _, _, nz64 = A64.export_csr(1)
    assert _rowscaled_err(rp - 1, nz64, zv) <= TOL_VAL
