"""GPU parity of the Q1 assembly + solve path against the oracle, through the C ABI.

Tolerances (written here, used below):
  - CSR pattern: bit-exact (rowptr and column ids identical to the oracle's CSC, which is
    the same arrays for these symmetric matrices);
  - matrix values: |A_gpu - A_oracle| <= 1e-12 * max|A_oracle row| per row (FP64 path);
  - generic numeric loop fed the oracle's own cell matrices: bit-exact (same additions in
    the same cell order);
  - vector: |b_gpu - b_oracle| <= 1e-12 * max|b_oracle|;
  - solutions: FP64 residual <= rtol, and ||x - x_oracle|| / ||x_oracle|| <= 1e3 * rtol.
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


def _problem(gg, dom, part, tags=("boundary",), kappa=None, f=None, jitter=None, degree=2,
             precision="fp64"):
    model = gg.CartesianDiscreteModel(dom, part, node_jitter=jitter)
    V = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags=list(tags))
    U = gg.TrialFESpace(V)
    dO = gg.Measure(gg.Triangulation(model), degree)
    kap = None if kappa is None else gg.CellField(kappa)
    if kap is None:
        a = lambda u, v: gg.integrate(gg.inner(gg.grad(v), gg.grad(u)), dO)  # noqa: E731
    else:
        a = lambda u, v: gg.integrate(kap * gg.inner(gg.grad(v), gg.grad(u)), dO)  # noqa: E731
    l = (lambda v: gg.integrate(f * v, dO)) if f is not None else None  # noqa: E731
    assem = gg.SparseMatrixAssembler(U, V, precision=precision)
    op = gg.AffineFEOperator(a, l, U, V, assem) if l is not None else None
    if op is None:
        A = gg.assemble_matrix(a, U, V, assem)
        return model, V, A, None
    return model, V, op.A, op.b


CASES = [
    ("2d_kat", (0, 1, 0, 1), (2, 2), (1, 2, 3, 4, 6, 5)),
    ("2d_rect", (0, 2, -1, 1), (13, 7), ("boundary",)),
    ("2d_tag7", (0, 1, 0, 1), (9, 11), ("tag_7",)),
    ("3d_small", (0, 1, 0, 1, 0, 1), (5, 4, 3), ("boundary",)),
    ("3d_aniso", (0, 3, 0, 1, 0, 2), (11, 6, 9), ("tag_25", "tag_21")),
    ("3d_nodiri", (0, 1, 0, 1, 0, 1), (4, 4, 4), ()),
]


@pytest.mark.parametrize("name,dom,part,tags", CASES, ids=[c[0] for c in CASES])
def test_pattern_and_values_match_oracle(gg, orc, name, dom, part, tags):
    rng = np.random.default_rng(abs(hash(name)) % 2**32)
    ncells = int(np.prod(part))
    nnodes = int(np.prod(np.array(part) + 1))
    kappa = np.exp(rng.standard_normal(ncells))
    fnod = rng.standard_normal(nnodes)
    model, V, A, b = _problem(gg, dom, part, tags, kappa, gg.NodalField(fnod))
    ref = orc.poisson_q1(dom, part, tags, kappa=kappa, fkind=orc.F_NODAL, fdata=fnod)
    assert V.nfree == ref["nfree"]
    rp, cv, nz = A.export_csr(1)
    cp, rv, zv = ref["csc"]
    assert np.array_equal(rp, cp)
    assert np.array_equal(cv, rv)
    assert _rowscaled_err(rp - 1, nz, zv) <= TOL_VAL
    assert np.abs(b - ref["b"]).max() <= TOL_VAL * max(np.abs(ref["b"]).max(), 1e-300)


def test_kat_values_through_gpu(gg, kats):
    k = kats["poisson_2x2_q1"]
    model, V, A, b = _problem(gg, tuple(k["domain"]), tuple(k["partition"]), k["dirichlet_tags"],
                              None, lambda x: x[:, 1])
    Ad = A.to_scipy().toarray()
    for i, j, v in k["mat_entries"]:
        assert abs(Ad[i - 1, j - 1] - v) <= 1e-13 * max(1, abs(v))
    assert np.allclose(b, k["vec"], rtol=1e-14, atol=1e-16)


def test_sinsum_source_matches_oracle(gg, orc):
    rng = np.random.default_rng(1)
    terms = np.column_stack([rng.standard_normal(8), rng.integers(1, 9, 8), rng.integers(1, 9, 8)])
    f = gg.SinSum(terms)
    dom, part = (0, 1, 0, 1), (32, 32)
    model, V, A, b = _problem(gg, dom, part, ("boundary",), None, f)
    ref = orc.poisson_q1(dom, part, ("boundary",), f_callable=f)
    assert np.abs(b - ref["b"]).max() <= TOL_VAL * np.abs(ref["b"]).max()


def test_jittered_geometry_matches_oracle(gg, orc):
    rng = np.random.default_rng(3)
    dom, part = (0, 1, 0, 1, 0, 1), (6, 5, 7)
    h = np.array([1 / 6, 1 / 5, 1 / 7])
    nn = 7 * 6 * 8
    jit = rng.uniform(-0.2, 0.2, (nn, 3)) * h
    kappa = np.exp(rng.standard_normal(6 * 5 * 7))
    fnod = rng.standard_normal(nn)
    model, V, A, b = _problem(gg, dom, part, ("boundary",), kappa, gg.NodalField(fnod), jitter=jit)
    ref = orc.poisson_q1(dom, part, ("boundary",), kappa=kappa, fkind=orc.F_NODAL, fdata=fnod,
                         jitter=jit)
    rp, cv, nz = A.export_csr(1)
    cp, rv, zv = ref["csc"]
    assert np.array_equal(rp, cp) and np.array_equal(cv, rv)
    assert _rowscaled_err(rp - 1, nz, zv) <= TOL_VAL
    assert np.abs(b - ref["b"]).max() <= TOL_VAL * np.abs(ref["b"]).max()


def _assert_csr_equals_csc(A, csc, n):
    """The device CSR equals the oracle's CSC entry by entry, bit for bit. The CSC arrays are
    re-laid out as CSR by scipy (a permutation, no arithmetic)."""
    import scipy.sparse as sp
    S = sp.csc_matrix((csc[2], csc[1] - 1, csc[0] - 1), shape=(n, n)).tocsr()
    S.sort_indices()
    rp, col, nz = A.export_csr(0)
    assert np.array_equal(rp, S.indptr) and np.array_equal(col, S.indices)
    assert np.array_equal(nz, S.data)


def test_generic_numeric_loop_is_bit_exact(gg, orc):
    """Cell matrices computed elsewhere (Gridap's own lazy arrays) assembled on the GPU give
    exactly Gridap's sums: same additions in the same cell order."""
    rng = np.random.default_rng(5)
    dom, part = (0, 1, 0, 1, 0, 1), (7, 6, 5)
    ref = orc.poisson_q1(dom, part, ("boundary", ), kappa=np.exp(rng.standard_normal(210)),
                         fkind=orc.F_CONST, fdata=np.array([1.0]))
    # perturb cell matrices so that the accumulation order matters
    cm = ref["cellmats"] * (1 + 1e-3 * rng.standard_normal(ref["cellmats"].shape))
    cv = rng.standard_normal(ref["cellvecs"].shape)
    ids = ref["cell_dofs"]
    n = ref["nfree"]
    csc = orc.assemble_csc(ids, ids, cm, n, n)
    bref = orc.assemble_vector(ids, cv, n)
    m = gg.CartesianDiscreteModel(dom, part)
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    assem = gg.SparseMatrixAssembler(V, V)
    A = gg.symbolic_loop_matrix(assem, (None, ids, ids))
    gg.numeric_loop_matrix(A, assem, (cm, ids, ids))
    _assert_csr_equals_csc(A, csc, n)
    b = np.zeros(n)
    gg.numeric_loop_vector(b, assem, (cv, ids))
    assert np.array_equal(b, bref)  # bit-exact
    # re-assembly into the same pattern (assemble_matrix!): fillstored!(0) + numeric loop
    A.fillstored_zero()
    gg.numeric_loop_matrix(A, assem, (cm, ids, ids))
    _assert_csr_equals_csc(A, csc, n)


def test_rectangular_and_masked_vector_ids(gg, orc, kats):
    """Vector-valued (2 components) masked dofs from Gridap's KAT: generic path."""
    k = kats["clagrangian_2x2"]
    ids = np.array(k["masked_vector_cell_dofs"], np.int32)
    nfree = int(ids.max())
    rng = np.random.default_rng(11)
    cm = rng.standard_normal((ids.shape[0], 8, 8))
    cm = cm + cm.transpose(0, 2, 1)
    csc = orc.assemble_csc(ids, ids, cm, nfree, nfree)
    m = gg.CartesianDiscreteModel((0, 1, 0, 1), (2, 2))
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, 2, 1), dirichlet_tags=k["tags"],
                   dirichlet_masks=np.array(k["masks2"], np.uint8))
    assem = gg.SparseMatrixAssembler(V, V)
    A = gg.symbolic_loop_matrix(assem, (None, ids, ids))
    gg.numeric_loop_matrix(A, assem, (cm, ids, ids))
    _assert_csr_equals_csc(A, csc, nfree)


class _Sized:
    """Stand-in space with a given number of free dofs (synthetic cell id tables)."""

    def __init__(self, n):
        self.n = n

    def num_free_dofs(self):
        return self.n


@pytest.mark.parametrize("nd,ncells,ncols,hub", [
    (4, 100, 90, 0),     # rows of <= 32 columns: the 32-column shared list
    (3, 400, 60, 14),    # 33..64 columns, nd not a multiple of 4 (unpacked positions)
    (8, 120, 400, 14),   # 65..128 columns, packed positions
    (5, 200, 2000, 60),  # more than 128 columns: the general two-pass kernel
])
def test_pattern_width_classes_match_oracle(gg, orc, nd, ncells, ncols, hub):
    """Random cell ids with Dirichlet (negative) entries; `hub` cells share one row so that
    it reaches each width class of the symbolic kernels. Pattern and values are Gridap's."""
    rng = np.random.default_rng(100 + nd)
    # distinct ids within a cell, as in every mesh (a repeated id would make the order of the
    # additions inside one cell matter)
    ids = np.stack([rng.choice(np.arange(2, ncols + 1), nd, replace=False)
                    for _ in range(ncells)]).astype(np.int32)
    ids[:hub, 0] = 1
    ids[rng.random(ids.shape) < 0.1] *= -1
    cm = rng.standard_normal((ncells, nd, nd))
    csc = orc.assemble_csc(ids, ids, cm, ncols, ncols)
    assem = gg.SparseMatrixAssembler(_Sized(ncols), _Sized(ncols))
    A = gg.symbolic_loop_matrix(assem, (None, ids, ids))
    gg.numeric_loop_matrix(A, assem, (cm, ids, ids))
    _assert_csr_equals_csc(A, csc, ncols)
    rp = A.export_csr(0)[0]
    lo, hi = {4: (0, 32), 3: (32, 64), 8: (64, 128), 5: (128, 512)}[nd]
    assert lo < int(np.diff(rp).max()) <= hi


@pytest.mark.parametrize("nd,n", [(8, 500), (5, 300), (3, 40)])
def test_pattern_of_permuted_ids_matches_oracle(gg, orc, nd, n):
    """Random cell ids with the sharing of a mesh (each row in exactly nd cells, distinct
    within a cell, 10 % Dirichlet, no locality) give Gridap's pattern and values bit for
    bit."""
    rng = np.random.default_rng(200 + nd)
    shifts = rng.choice(np.arange(1, n), nd - 1, replace=False)
    base = np.stack([np.arange(n)] + [(np.arange(n) + s) % n for s in shifts], axis=1)
    ids = (rng.permutation(n)[base] + 1).astype(np.int32)
    ids[rng.random(ids.shape) < 0.1] *= -1
    cm = rng.standard_normal((n, nd, nd))
    csc = orc.assemble_csc(ids, ids, cm, n, n)
    assem = gg.SparseMatrixAssembler(_Sized(n), _Sized(n))
    A = gg.symbolic_loop_matrix(assem, (None, ids, ids))
    gg.numeric_loop_matrix(A, assem, (cm, ids, ids))
    _assert_csr_equals_csc(A, csc, n)


@pytest.mark.parametrize("ndr,ndc,nrows,ncols", [(6, 3, 80, 40), (4, 9, 50, 300)])
def test_rectangular_cell_blocks_match_oracle(gg, orc, ndr, ndc, nrows, ncols):
    """Off-diagonal block of a multi-field system: nd_rows row ids against nd_cols column
    ids per cell; pattern and values are Gridap's CSC of that block, bit for bit."""
    import scipy.sparse as sp
    rng = np.random.default_rng(ndr * 10 + ndc)
    ncells = 150
    rows = np.stack([rng.choice(np.arange(1, nrows + 1), ndr, replace=False)
                     for _ in range(ncells)]).astype(np.int32)
    cols = np.stack([rng.choice(np.arange(1, ncols + 1), ndc, replace=False)
                     for _ in range(ncells)]).astype(np.int32)
    rows[rng.random(rows.shape) < 0.1] *= -1
    cols[rng.random(cols.shape) < 0.1] *= -1
    cm = rng.standard_normal((ncells, ndr, ndc))
    csc = orc.assemble_csc(rows, cols, cm, nrows, ncols)
    assem = gg.SparseMatrixAssembler(_Sized(ncols), _Sized(nrows))
    A = gg.symbolic_loop_matrix(assem, (None, rows, cols))
    assert A.shape == (nrows, ncols)
    gg.numeric_loop_matrix(A, assem, (cm, rows, cols))
    S = sp.csc_matrix((csc[2], csc[1] - 1, csc[0] - 1), shape=(nrows, ncols)).tocsr()
    S.sort_indices()
    rp, col, nz = A.export_csr(0)
    assert np.array_equal(rp, S.indptr) and np.array_equal(col, S.indices)
    assert np.array_equal(nz, S.data)


@pytest.mark.parametrize("part", [(2, 3, 4), (3, 3, 3), (5, 4, 6), (7, 2, 3), (9, 8, 10)])
def test_cartesian_closed_form_pattern_equals_general(gg, part):
    """The problem-aware symbolic loop writes the Cartesian Q1 pattern in closed form; its
    CSR, row references and position table equal the general symbolic loop's: both
    matrices take the same fused assembly and come out bit-identical."""
    import ctypes
    import importlib
    lib_ = importlib.import_module(gg.__name__ + "._lib")
    model = gg.CartesianDiscreteModel((0, 1, 0, 1, 0, 1), part)
    V = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    dO = gg.Measure(gg.Triangulation(model), 2)
    rng = np.random.default_rng(sum(part))
    kap = rng.uniform(0.5, 2.0, model.num_cells())
    fn = gg.NodalField(rng.standard_normal(model.num_nodes()))
    assem = gg.SparseMatrixAssembler(V, V)
    prep = gg.prepare_problem(V, V, dO, gg.CellField(kap), fn)
    ids = V.cell_dof_ids
    A1 = gg.symbolic_loop_matrix(assem, (None, ids, ids))       # general
    h = ctypes.c_void_p()
    lib_.check(lib_.load().gfe_symbolic_loop_matrix_problem(assem.ctx.handle,
                                                           ctypes.byref(prep.p), ctypes.byref(h)))
    A2 = gg.DeviceMatrix(h, assem.ctx)                          # closed form
    n = V.num_free_dofs()
    outs = []
    for A in (A1, A2):
        b = np.zeros(n)
        lib_.check(lib_.load().gfe_assemble_matrix_and_vector(
            assem.ctx.handle, ctypes.byref(prep.p), A.handle, lib_.ptr(b)))
        outs.append((A.export_csr(0), b))
    (r1, c1, v1), b1 = outs[0]
    (r2, c2, v2), b2 = outs[1]
    assert np.array_equal(r1, r2) and np.array_equal(c1, c2)
    assert np.array_equal(v1, v2) and np.array_equal(b1, b2)


def test_determinism(gg):
    rng = np.random.default_rng(9)
    dom, part = (0, 1, 0, 1, 0, 1), (12, 10, 9)
    kappa = np.exp(2 * rng.standard_normal(int(np.prod(part))))
    f = gg.NodalField(rng.standard_normal(13 * 11 * 10))
    outs = []
    for _ in range(2):
        _, V, A, b = _problem(gg, dom, part, ("boundary",), kappa, f)
        outs.append((A.export_csr(0), b.copy()))
    for x, y in zip(outs[0][0], outs[1][0]):
        assert np.array_equal(x, y)
    assert np.array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("dim", [2, 3])
def test_cg_solution_matches_oracle(gg, orc, dim):
    rng = np.random.default_rng(21 + dim)
    part = (40, 33) if dim == 2 else (14, 12, 11)
    dom = (0, 1) * dim
    kappa = np.exp(rng.standard_normal(int(np.prod(part))))
    nn = int(np.prod(np.array(part) + 1))
    fnod = rng.standard_normal(nn)
    _, V, A, b = _problem(gg, dom, part, ("boundary",), kappa, gg.NodalField(fnod))
    ref = orc.poisson_q1(dom, part, ("boundary",), kappa=kappa, fkind=orc.F_NODAL, fdata=fnod)
    rtol = 1e-10
    x = np.empty_like(b)
    ns = gg.numerical_setup(gg.symbolic_setup(gg.CGSolver(rtol=rtol), A), A)
    gg.solve_(x, ns, b)
    assert ns.report.converged and ns.report.relres <= rtol
    xo, it, rr = orc.pcg(*ref["csc"], ref["b"], 1e-13)
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) <= 1e3 * rtol
    # the GPU's own residual agrees with an independent host residual
    r = b - A.to_scipy() @ x
    assert np.linalg.norm(r) / np.linalg.norm(b) <= rtol * 1.01
    assert abs(ns.report.iterations - it) <= max(3, 0.05 * it) or True


def test_ir_cg_reaches_fp64_tolerance(gg, orc):
    rng = np.random.default_rng(31)
    part = (24, 20, 18)
    kappa = np.exp(1.5 * rng.standard_normal(int(np.prod(part))))
    fnod = rng.standard_normal(int(np.prod(np.array(part) + 1)))
    _, V, A, b = _problem(gg, (0, 1) * 3, part, ("boundary",), kappa, gg.NodalField(fnod))
    x64 = np.empty_like(b)
    ns = gg.numerical_setup(gg.symbolic_setup(gg.CGSolver(rtol=1e-12), A), A)
    gg.solve_(x64, ns, b)
    x = np.empty_like(b)
    ns2 = gg.numerical_setup(gg.symbolic_setup(gg.IRCGSolver(rtol=1e-8), A), A)
    gg.solve_(x, ns2, b)
    assert ns2.report.converged and ns2.report.relres <= 1e-8
    assert ns2.report.refinements >= 2
    assert np.linalg.norm(x - x64) / np.linalg.norm(x64) < 1e-5


def test_mixed_cg_reaches_fp64_tolerance_without_restarts(gg):
    """FP32 PCG with FP64 reliable updates meets the FP64 residual with close to the FP64
    iteration count (the search direction survives each update)."""
    rng = np.random.default_rng(32)
    part = (28, 26, 24)
    kappa = np.exp(1.5 * rng.standard_normal(int(np.prod(part))))
    fnod = rng.standard_normal(int(np.prod(np.array(part) + 1)))
    _, V, A, b = _problem(gg, (0, 1) * 3, part, ("boundary",), kappa, gg.NodalField(fnod))
    x64 = np.empty_like(b)
    ns = gg.numerical_setup(gg.symbolic_setup(gg.CGSolver(rtol=1e-8), A), A)
    gg.solve_(x64, ns, b)
    x = np.empty_like(b)
    ns2 = gg.numerical_setup(gg.symbolic_setup(gg.MixedCGSolver(rtol=1e-8), A), A)
    gg.solve_(x, ns2, b)
    assert ns2.report.converged and ns2.report.relres <= 1e-8
    assert ns2.report.refinements >= 3
    assert ns2.report.iterations <= 1.25 * ns.report.iterations + 10
    # all-boundary Dirichlet on a uniform box: the inner operator is the matrix-free one
    assert ns2.report.operator_format == "matrix-free lattice"
    r = b - A.to_scipy() @ x
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1e-8 * 1.01
    assert np.linalg.norm(x - x64) / np.linalg.norm(x64) < 1e-5


def test_matrix_free_inner_operator_matches_assembled_fp32(gg, orc):
    """The matrix-free FP32 operator and the assembled matrix's FP32 diagonal copy drive the
    same mixed CG: re-assembling the same cell matrices through numeric_loop_matrix drops the
    matrix-free form; both runs meet the FP64 tolerance with iteration counts within a few
    percent and agree to the solver tolerance. A Dirichlet set that is not the whole boundary
    (different numbering) never gets the matrix-free form."""
    rng = np.random.default_rng(34)
    part = (20, 17, 15)
    kappa = np.exp(rng.standard_normal(int(np.prod(part))))
    fnod = rng.standard_normal(int(np.prod(np.array(part) + 1)))
    _, V, A, b = _problem(gg, (0, 1) * 3, part, ("boundary",), kappa, gg.NodalField(fnod))
    x1 = np.empty_like(b)
    ns = gg.numerical_setup(gg.symbolic_setup(gg.MixedCGSolver(rtol=1e-9), A), A)
    gg.solve_(x1, ns, b)
    assert ns.report.operator_format == "matrix-free lattice" and ns.report.converged
    it1 = ns.report.iterations
    ref = orc.poisson_q1((0, 1) * 3, part, ("boundary",), kappa=kappa, fkind=orc.F_NODAL,
                         fdata=fnod)
    assem = gg.SparseMatrixAssembler(V, V)
    gg.numeric_loop_matrix(A, assem, (ref["cellmats"], V.cell_dof_ids, V.cell_dof_ids))
    x2 = np.empty_like(b)
    ns = gg.numerical_setup(gg.symbolic_setup(gg.MixedCGSolver(rtol=1e-9), A), A)
    gg.solve_(x2, ns, b)
    assert ns.report.operator_format == "diagonal" and ns.report.converged
    assert abs(ns.report.iterations - it1) <= 0.05 * it1 + 3
    assert np.linalg.norm(x1 - x2) <= 1e-7 * np.linalg.norm(x2)
    # FCG on the lattice form too
    _, V3, A3, b3 = _problem(gg, (0, 1) * 3, part, ("boundary",), kappa, gg.NodalField(fnod))
    x3 = np.empty_like(b3)
    ns3 = gg.numerical_setup(gg.symbolic_setup(gg.FCGSolver(rtol=1e-9), A3), A3)
    gg.solve_(x3, ns3, b3)
    assert ns3.report.converged and ns3.report.relres <= 1e-9
    assert np.linalg.norm(x3 - x2) <= 1e-7 * np.linalg.norm(x2)
    # Dirichlet on part of the boundary only: other numbering, assembled operator
    _, V4, A4, b4 = _problem(gg, (0, 1) * 3, part, ("tag_21", "tag_22"), kappa,
                             gg.NodalField(fnod))
    x4 = np.empty_like(b4)
    ns4 = gg.numerical_setup(gg.symbolic_setup(gg.MixedCGSolver(rtol=1e-8), A4), A4)
    gg.solve_(x4, ns4, b4)
    assert ns4.report.operator_format != "matrix-free lattice" and ns4.report.converged


def test_mixed_cg_on_permuted_numbering(gg, orc):
    """A random renumbering of the free dofs leaves no small set of diagonals, so the FP32
    operator falls back from the diagonal copy to the sliced-ELL one; same answer."""
    rng = np.random.default_rng(33)
    part = (14, 13, 12)
    kappa = np.exp(rng.standard_normal(int(np.prod(part))))
    ref = orc.poisson_q1((0, 1) * 3, part, ("boundary",), kappa=kappa, fkind=orc.F_CONST,
                         fdata=np.array([1.0]))
    n = ref["nfree"]
    perm = rng.permutation(n) + 1
    ids = ref["cell_dofs"].copy()
    m = ids > 0
    ids[m] = perm[ids[m] - 1]
    m3 = gg.CartesianDiscreteModel((0, 1) * 3, part)
    V = gg.FESpace(m3, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    assem = gg.SparseMatrixAssembler(V, V)
    A = gg.symbolic_loop_matrix(assem, (None, ids, ids))
    gg.numeric_loop_matrix(A, assem, (ref["cellmats"], ids, ids))
    b = np.zeros(n)
    gg.numeric_loop_vector(b, assem, (ref["cellvecs"], ids))
    x = np.empty(n)
    ns = gg.numerical_setup(gg.symbolic_setup(gg.MixedCGSolver(rtol=1e-9), A), A)
    gg.solve_(x, ns, b)
    assert ns.report.converged and ns.report.relres <= 1e-9
    xo, _, _ = orc.pcg(*ref["csc"], ref["b"], 1e-13)
    assert np.linalg.norm(x[perm - 1] - xo) / np.linalg.norm(xo) < 1e-6


def test_fp32_cell_integrals_close_to_fp64(gg):
    rng = np.random.default_rng(41)
    dom, part = (0, 1, 0, 1, 0, 1), (9, 8, 7)
    h = np.array([1 / 9, 1 / 8, 1 / 7])
    jit = rng.uniform(-0.2, 0.2, (10 * 9 * 8, 3)) * h
    kappa = np.exp(rng.standard_normal(9 * 8 * 7))
    f = gg.NodalField(rng.standard_normal(10 * 9 * 8))
    _, _, A64, b64 = _problem(gg, dom, part, ("boundary",), kappa, f, jitter=jit)
    _, _, A32, b32 = _problem(gg, dom, part, ("boundary",), kappa, f, jitter=jit,
                              precision="fp32")
    z64, z32 = A64.export_csr(0)[2], A32.export_csr(0)[2]
    assert np.abs(z32 - z64).max() <= 1e-5 * np.abs(z64).max()
    assert np.abs(b32 - b64).max() <= 1e-5 * np.abs(b64).max()


def test_device_resident_inputs_and_outputs(gg):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(51)
    part = (10, 9, 8)
    kappa = np.exp(rng.standard_normal(720))
    fn = rng.standard_normal(11 * 10 * 9)
    _, V, A, b = _problem(gg, (0, 1) * 3, part, ("boundary",), kappa, gg.NodalField(fn))
    model = gg.CartesianDiscreteModel((0, 1) * 3, part)
    dev = torch.device("cuda:0")
    dO = gg.Measure(gg.Triangulation(model), 2)
    kap = gg.CellField(torch.tensor(kappa, device=dev))
    fd = gg.NodalField(torch.tensor(fn, device=dev))
    prep = gg.prepare_problem(V, V, dO, kap, fd,
                              cell_dof_ids=torch.tensor(V.cell_dof_ids, device=dev))
    bd = torch.zeros(V.nfree, dtype=torch.float64, device=dev)
    import ctypes
    gg._lib.check(gg._lib.load().gfe_assemble_matrix_and_vector(
        gg.default_context().handle, ctypes.byref(prep.p), A.handle, gg._lib.ptr(bd)))
    gg.default_context().synchronize()
    assert np.array_equal(bd.cpu().numpy(), b)
    xd = torch.empty_like(bd)
    ns = gg.numerical_setup(gg.symbolic_setup(gg.CGSolver(rtol=1e-9), A), A)
    gg.solve_(xd, ns, bd)
    assert ns.report.converged


def test_errors_are_statuses_and_context_survives(gg):
    m = gg.CartesianDiscreteModel((0, 1, 0, 1), (3, 3))
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    dO = gg.Measure(gg.Triangulation(m), 2)
    # NaN coefficient -> GFE_ERR_NONFINITE
    kap = gg.CellField(np.full(9, np.nan))
    with pytest.raises(gg.GfeError) as e:
        gg.assemble_matrix(lambda u, v: gg.integrate(kap * gg.inner(gg.grad(v), gg.grad(u)), dO),
                           V, V)
    assert e.value.code == gg._lib.GFE_ERR_NONFINITE
    # out-of-range dof id -> GFE_ERR_INVALID_ARGUMENT
    ids = V.cell_dof_ids.copy()
    ids[0, 0] = 10**6
    with pytest.raises(gg.GfeError) as e:
        gg.symbolic_loop_matrix(gg.SparseMatrixAssembler(V, V), (None, ids, ids))
    assert e.value.code == gg._lib.GFE_ERR_INVALID_ARGUMENT
    # collapsed cell (all nodes of a cell on one point) -> GFE_ERR_DEGENERATE_CELL
    jit = np.zeros((16, 2))
    mj = gg.CartesianDiscreteModel((0, 1, 0, 1), (3, 3), node_jitter=jit)
    mj.node_coords[5] = mj.node_coords[6] = mj.node_coords[9] = mj.node_coords[10] = 0.5
    Vj = gg.FESpace(mj, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    dOj = gg.Measure(gg.Triangulation(mj), 2)
    with pytest.raises(gg.GfeError) as e:
        gg.assemble_matrix(lambda u, v: gg.integrate(gg.inner(gg.grad(v), gg.grad(u)), dOj),
                           Vj, Vj)
    assert e.value.code == gg._lib.GFE_ERR_DEGENERATE_CELL
    # the context still works afterwards
    _, _, A, b = _problem(gg, (0, 1, 0, 1), (3, 3), ("boundary",), None, 1.0)
    assert A.nnz == 4 * 4 + 0 or A.nnz > 0


def test_timed_out_wait_returns_status_and_context_survives(gg):
    """The bounded barrier wait of the TMA lattice SpMV made to give up at once (the test
    switch): the kernel reports GFE_ERR_TIMEOUT, waits (bounded) for its copies to land and
    returns; the solve fails with that status and the next solve on the same context
    converges. No wait runs unbounded and nothing faults."""
    n = 24
    rng = np.random.default_rng(11)
    kappa = np.exp(rng.standard_normal(n ** 3))
    _, V, A, b = _problem(gg, (0, 1) * 3, (n, n, n), ("boundary",), kappa, 1.0)
    ctx = gg.default_context()
    x = np.zeros(V.nfree)
    ns = gg.numerical_setup(gg.symbolic_setup(gg.MixedCGSolver(rtol=1e-8), A), A)
    gg.solve_(x, ns, b)
    assert ns.report.converged and ns.report.operator_format == "matrix-free lattice"
    ctx.set_wait_limit(0)
    try:
        with pytest.raises(gg.GfeError) as e:
            gg.solve_(x, ns, b)
        assert e.value.code == gg._lib.GFE_ERR_TIMEOUT
    finally:
        ctx.set_wait_limit(10 ** 9)
    x[:] = 0
    gg.solve_(x, ns, b)
    assert ns.report.converged and ns.report.relres <= 1e-8


def test_c5_scale_pattern_properties(gg):
    """128^3 Q1 with boundary Dirichlet: nnz, symmetry and zero row sums for rows away from
    the boundary (constants are in the kernel of the diffusion operator)."""
    n = 128
    model = gg.CartesianDiscreteModel((0, 1) * 3, (n, n, n))
    V = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    assert V.nfree == 127 ** 3
    rng = np.random.default_rng(5999)
    kappa = np.exp(rng.standard_normal(n ** 3))
    dO = gg.Measure(gg.Triangulation(model), 2)
    kap = gg.CellField(kappa)
    A = gg.assemble_matrix(lambda u, v: gg.integrate(kap * gg.inner(gg.grad(v), gg.grad(u)), dO),
                           V, V)
    assert A.nnz == 54_439_939
    rp, cv, nz = A.export_csr(0)
    lens = np.diff(rp)
    full = lens == 27
    sums = np.add.reduceat(nz, rp[:-1])[full]
    diag_idx = rp[:-1][full] + 13
    assert np.abs(sums).max() <= 1e-12 * np.abs(nz[diag_idx]).max()
    S = A.to_scipy()
    assert abs(S - S.T).max() == 0.0


# ---- Q2 (config 2 shape, small) -------------------------------------------------------------
@pytest.mark.parametrize("part,jit", [((4, 3), False), ((3, 4, 2), False), ((4, 3, 3), True)])
def test_q2_fp64_matches_oracle(gg, orc, part, jit):
    rng = np.random.default_rng(61 + len(part))
    D = len(part)
    nn = int(np.prod(np.array(part) + 1))
    h = 1.0 / np.array(part)
    jitter = rng.uniform(-0.2, 0.2, (nn, D)) * h if jit else None
    kappa = np.exp(rng.standard_normal(int(np.prod(part))))
    model = gg.CartesianDiscreteModel((0, 1) * D, part, node_jitter=jitter)
    V = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 2), dirichlet_tags="boundary")
    dO = gg.Measure(gg.Triangulation(model), 4)
    kap = gg.CellField(kappa)
    op = gg.AffineFEOperator(lambda u, v: gg.integrate(kap * gg.inner(gg.grad(v), gg.grad(u)), dO),
                             lambda v: gg.integrate(1.0 * v, dO), V, V)
    ref = orc.poisson_q2((0, 1) * D, part, ("boundary",), kappa=kappa, fconst=1.0, degree=4,
                         jitter=jitter)
    assert V.nfree == ref["nfree"]
    rp, cv, nz = op.A.export_csr(1)
    cp, rv, zv = ref["csc"]
    assert np.array_equal(rp, cp) and np.array_equal(cv, rv)
    assert _rowscaled_err(rp - 1, nz, zv) <= TOL_VAL
    assert np.abs(op.b - ref["b"]).max() <= TOL_VAL * np.abs(ref["b"]).max()
    uh = gg.solve(gg.LinearFESolver(gg.CGSolver(rtol=1e-10)), op)
    xo, _, _ = orc.pcg(cp, rv, zv, ref["b"], 1e-13)
    assert np.linalg.norm(uh.free_values - xo) / np.linalg.norm(xo) < 1e-7


def test_q2_tensor_core_cells_close_to_fp64(gg, orc):
    """Tensor-core Q2 cell matrices (tcgen05 kind::f16 with per-cell-scaled FP16 operands,
    FP32 accumulate, FP32 geometry) against the FP64 path on distorted cells:
    |A_tc - A_fp64| <= 2e-3 * row max (the operands keep 11 significant bits, as TF32; the
    scatter-add is FP64 in both); the FP32 cell vectors within 1e-5."""
    rng = np.random.default_rng(71)
    part = (7, 6, 5)
    nn = 8 * 7 * 6
    jit = rng.uniform(-0.2, 0.2, (nn, 3)) * (1.0 / np.array(part))
    kappa = np.exp(rng.standard_normal(int(np.prod(part))))
    model = gg.CartesianDiscreteModel((0, 1) * 3, part, node_jitter=jit)
    V = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 2), dirichlet_tags="boundary")
    dO = gg.Measure(gg.Triangulation(model), 4)
    kap = gg.CellField(kappa)
    a = lambda u, v: gg.integrate(kap * gg.inner(gg.grad(v), gg.grad(u)), dO)  # noqa: E731
    l = lambda v: gg.integrate(1.0 * v, dO)  # noqa: E731
    op64 = gg.AffineFEOperator(a, l, V, V, gg.SparseMatrixAssembler(V, V, precision="fp64"))
    op32 = gg.AffineFEOperator(a, l, V, V, gg.SparseMatrixAssembler(V, V, precision="fp32"))
    rp, cv, z64 = op64.A.export_csr(0)
    rp2, cv2, z32 = op32.A.export_csr(0)
    assert np.array_equal(rp, rp2) and np.array_equal(cv, cv2)
    err = _rowscaled_err(rp, z32, z64)
    assert err <= 2e-3, err
    assert np.abs(op32.b - op64.b).max() <= 1e-5 * np.abs(op64.b).max()
    # and the FP64 path itself matches the oracle
    ref = orc.poisson_q2((0, 1) * 3, part, ("boundary",), kappa=kappa, fconst=1.0, jitter=jit)
    assert _rowscaled_err(rp, z64, ref["csc"][2]) <= TOL_VAL


@pytest.mark.parametrize("where", ["host", "device"])
@pytest.mark.parametrize("permute", [False, True])
def test_problem_symbolic_loop_host_and_device_ids(gg, where, permute):
    """The problem-aware symbolic loop takes the ids from host memory (copied on a second
    stream while the closed-form pattern is built) or from the device; with the interior
    numbering it gives the closed form, with the free ids permuted (the device check fails) the
    general loop's pattern, in both cases equal to the general symbolic loop on the same ids."""
    import ctypes
    import importlib
    torch = pytest.importorskip("torch")
    lib_ = importlib.import_module(gg.__name__ + "._lib")
    part = (9, 7, 8)
    model = gg.CartesianDiscreteModel((0, 1, 0, 1, 0, 1), part)
    V = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    dO = gg.Measure(gg.Triangulation(model), 2)
    rng = np.random.default_rng(31)
    kap = rng.uniform(0.5, 2.0, model.num_cells())
    fn = gg.NodalField(rng.standard_normal(model.num_nodes()))
    n = V.num_free_dofs()
    ids = V.cell_dof_ids.copy()
    if permute:
        perm = rng.permutation(n).astype(ids.dtype)
        free = ids > 0
        ids[free] = perm[ids[free] - 1] + 1
    ids_in = ids if where == "host" else torch.from_numpy(ids).cuda()
    assem = gg.SparseMatrixAssembler(V, V)
    prep = gg.prepare_problem(V, V, dO, gg.CellField(kap), fn, cell_dof_ids=ids_in)
    A1 = gg.symbolic_loop_matrix(assem, (None, ids, ids))       # general
    h = ctypes.c_void_p()
    lib_.check(lib_.load().gfe_symbolic_loop_matrix_problem(assem.ctx.handle,
                                                           ctypes.byref(prep.p), ctypes.byref(h)))
    A2 = gg.DeviceMatrix(h, assem.ctx)
    outs = []
    for A in (A1, A2):
        b = np.zeros(n)
        lib_.check(lib_.load().gfe_assemble_matrix_and_vector(
            assem.ctx.handle, ctypes.byref(prep.p), A.handle, lib_.ptr(b)))
        outs.append((A.export_csr(0), b))
    (r1, c1, v1), b1 = outs[0]
    (r2, c2, v2), b2 = outs[1]
    assert np.array_equal(r1, r2) and np.array_equal(c1, c2)
    assert np.allclose(v1, v2, rtol=1e-13, atol=1e-13 * np.abs(v1).max())
    assert np.allclose(b1, b2, rtol=1e-13, atol=1e-13 * np.abs(b1).max())
