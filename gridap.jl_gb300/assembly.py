"""Assemblers and affine FE operators over libgfe, mirroring Gridap's
SparseMatrixAssembler / assemble_* / AffineFEOperator API (FESpaces/SparseMatrixAssemblers.jl,
FESpaces/Assemblers.jl, FESpaces/AffineFEOperators.jl).

Gridap's `!`-suffixed functions appear here without the `!` (Python names cannot carry it):
`symbolic_loop_matrix`, `numeric_loop_matrix`, `numeric_loop_vector`, `assemble_matrix_`.
Matrices stay on the GPU inside a `DeviceMatrix`; vectors are numpy arrays (host) or torch
CUDA tensors (device), whichever the caller passes.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _lib
from .celldata import (CellField, NodalField, SinSum, classify_bilinear,
                       classify_boundary_bilinear, classify_boundary_linear, classify_linear)
from .fespaces import FESpace, TrialFESpace, _space
from .geometry import BoundaryTriangulation, Measure, SimplexDiscreteModel, Triangulation

_CTX = {}


class Context:
    """One GPU, one CUDA stream (gfe_ctx)."""

    def __init__(self, device: int = 0):
        lib = _lib.load()
        h = C.c_void_p()
        _lib.check(lib.gfe_ctx_create(device, C.byref(h)))
        self.handle = h
        self.device = device
        self._children = weakref.WeakSet()

    def _own(self, obj) -> None:
        """Registers an object holding a handle of this context (matrix, batch, learned
        preconditioner); close() releases it before the context itself."""
        self._children.add(obj)

    def close(self) -> None:
        for obj in list(self._children):
            obj._release()
        if self.handle:
            h, self.handle = self.handle, None
            _lib.load().gfe_ctx_destroy(h)

    def stream(self) -> int:
        s = C.c_void_p()
        _lib.check(_lib.load().gfe_ctx_stream(self.handle, C.byref(s)))
        return s.value or 0

    def synchronize(self) -> None:
        _lib.check(_lib.load().gfe_ctx_synchronize(self.handle))

    def kernel_launches(self) -> int:
        n = C.c_int64()
        _lib.check(_lib.load().gfe_ctx_kernel_launches(self.handle, C.byref(n)))
        return n.value

    def set_timing(self, enable: bool) -> None:
        _lib.check(_lib.load().gfe_ctx_set_timing(self.handle, int(enable)))

    def set_wait_limit(self, first_wait_ns: int) -> None:
        """Limit of the first bounded barrier wait in the lattice SpMV (0: give up at once, a
        switch for tests of the timeout path; default 1 s)."""
        _lib.check(_lib.load().gfe_ctx_set_wait_limit(self.handle, int(first_wait_ns)))

    def kernel_time(self, kind: int) -> tuple[float, int]:
        """(total milliseconds, launches) of a kernel class since timing was enabled."""
        ms, n = C.c_double(), C.c_int64()
        _lib.check(_lib.load().gfe_ctx_kernel_time(self.handle, kind, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def default_context(device: int = 0) -> Context:
    if device not in _CTX:
        _CTX[device] = Context(device)
    return _CTX[device]


class DeviceMatrix:
    """A sparse matrix resident on the GPU (gfe_matrix): CSR with sorted unique columns."""

    def __init__(self, handle, ctx: Context):
        self.handle = handle
        self.ctx = ctx
        ctx._own(self)
        r, c, z = C.c_int64(), C.c_int64(), C.c_int64()
        _lib.check(_lib.load().gfe_matrix_info(handle, C.byref(r), C.byref(c), C.byref(z)))
        self.shape = (r.value, c.value)
        self.nnz = z.value

    def export_csr(self, index_base: int = 0):
        """(rowptr, colval, nzval) as int64/int64/float64 host arrays."""
        rp = np.empty(self.shape[0] + 1, dtype=np.int64)
        cv = np.empty(self.nnz, dtype=np.int64)
        nz = np.empty(self.nnz, dtype=np.float64)
        _lib.check(_lib.load().gfe_matrix_export_csr(self.handle, index_base, _lib.ptr(rp),
                                                     _lib.ptr(cv), _lib.ptr(nz)))
        return rp, cv, nz

    def to_scipy(self):
        import scipy.sparse as sp
        rp, cv, nz = self.export_csr(0)
        return sp.csr_matrix((nz, cv, rp), shape=self.shape)

    def matvec(self, x, y=None):
        if y is None:
            y = np.empty(self.shape[0]) if isinstance(x, np.ndarray) else x.new_empty(self.shape[0])
        _lib.check(_lib.load().gfe_matrix_mul(self.ctx.handle, self.handle, _lib.ptr(x),
                                              _lib.ptr(y)))
        return y

    def fillstored_zero(self):
        _lib.check(_lib.load().gfe_matrix_fillstored_zero(self.handle))

    def _release(self):
        # a context already closed (garbage cycles finalise in any order) took the matrix's
        # device memory with it: only the handle is dropped then
        h, self.handle = self.handle, None
        if h and self.ctx.handle:
            _lib.load().gfe_matrix_destroy(h)

    def __del__(self):
        try:
            self._release()
        except Exception:
            pass


class SparseMatrixAssembler:
    """SparseMatrixAssembler(U, V): assembles into device CSR matrices and dense vectors.
    `precision` selects the arithmetic of fused cell integrals ("fp64" or "fp32"); the
    scatter-add always accumulates in FP64."""

    def __init__(self, trial, test, precision: str = "fp64", ctx: Context | None = None):
        self.trial = _space(trial)
        self.test = _space(test)
        if precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        self.precision = precision
        self.ctx = ctx or default_context()

    def get_rows(self):
        return self.test.num_free_dofs()

    def get_cols(self):
        return self.trial.num_free_dofs()


# ---- protocol-level entry points (FESpaces/SparseMatrixAssemblers.jl:174-316) ------------
def symbolic_loop_matrix(assem: SparseMatrixAssembler, matdata) -> DeviceMatrix:
    """Pattern of assembling matdata = (cellmats, cell_rows, cell_cols) (cellmats unused).
    cell_rows and cell_cols may have different widths (a rectangular block)."""
    _, rows, cols = matdata
    rows = _as_ids(rows)
    cols = _as_ids(cols)
    if rows.shape[0] != cols.shape[0]:
        raise ValueError("cell_rows and cell_cols cover different numbers of cells")
    h = C.c_void_p()
    lib = _lib.load()
    if rows.shape[1] == cols.shape[1]:
        _lib.check(lib.gfe_symbolic_loop_matrix(
            assem.ctx.handle, rows.shape[0], rows.shape[1], _lib.ptr(rows), _lib.ptr(cols),
            assem.get_rows(), assem.get_cols(), C.byref(h)))
    else:
        _lib.check(lib.gfe_symbolic_loop_matrix_rect(
            assem.ctx.handle, rows.shape[0], rows.shape[1], cols.shape[1], _lib.ptr(rows),
            _lib.ptr(cols), assem.get_rows(), assem.get_cols(), C.byref(h)))
    return DeviceMatrix(h, assem.ctx)


def symbolic_loop_problem(assem: SparseMatrixAssembler, prep) -> DeviceMatrix:
    """The pattern of a prepared problem's cell ids, built with the model in hand
    (gfe_symbolic_loop_matrix_problem: closed form for the interior numbering of Cartesian
    Q1 grids, the general symbolic loop otherwise)."""
    h = C.c_void_p()
    _lib.check(_lib.load().gfe_symbolic_loop_matrix_problem(assem.ctx.handle, C.byref(prep.p),
                                                            C.byref(h)))
    return DeviceMatrix(h, assem.ctx)


def numeric_loop_matrix(A: DeviceMatrix, assem: SparseMatrixAssembler, matdata) -> DeviceMatrix:
    """Adds cell matrices (ncells, nd, nd) [row, col] into A in cell order."""
    cellmats = matdata[0]
    cm = _cellmats_colmajor(cellmats)
    _lib.check(_lib.load().gfe_numeric_loop_matrix(assem.ctx.handle, A.handle, _lib.ptr(cm)))
    return A


def numeric_loop_vector(b, assem: SparseMatrixAssembler, vecdata):
    cellvecs, rows = vecdata
    rows = _as_ids(rows)
    cv = np.ascontiguousarray(cellvecs, dtype=np.float64) if isinstance(cellvecs, np.ndarray) \
        else cellvecs.contiguous()
    _lib.check(_lib.load().gfe_numeric_loop_vector(
        assem.ctx.handle, rows.shape[0], rows.shape[1], _lib.ptr(rows), _lib.ptr(cv),
        b.shape[0], _lib.ptr(b)))
    return b


def _as_ids(a):
    if isinstance(a, np.ndarray):
        return np.ascontiguousarray(a, dtype=np.int32)
    return a.contiguous()


def _cellmats_colmajor(cellmats):
    """Gridap cell matrices are column-major nd x nd; numpy (ncells, nd, nd)[c, i, j] is
    transposed into that layout."""
    if isinstance(cellmats, np.ndarray):
        return np.ascontiguousarray(np.transpose(cellmats, (0, 2, 1)), dtype=np.float64)
    return cellmats.transpose(1, 2).contiguous()


# ---- weak-form driven assembly ------------------------------------------------------------
class _Prepared:
    """A gfe_problem plus the arrays it points to (kept alive for the call)."""

    def __init__(self):
        self.keep = []
        self.p = _lib.Problem()


def _coef_to_problem(prep: _Prepared, coef, ncells):
    p = prep.p
    if coef is None:
        p.coef_kind = _lib.GFE_COEF_ONE
    elif isinstance(coef, (int, float)):
        arr = np.array([float(coef)])
        prep.keep.append(arr)
        p.coef_kind, p.coef = _lib.GFE_COEF_CONST, _lib.ptr(arr)
    elif isinstance(coef, CellField):
        v = coef.values
        if isinstance(v, np.ndarray):
            v = np.ascontiguousarray(v, dtype=np.float64)
        if v.shape[0] != ncells:
            raise ValueError("per-cell coefficient has the wrong length")
        prep.keep.append(v)
        p.coef_kind, p.coef = _lib.GFE_COEF_CELL, _lib.ptr(v)
    else:
        raise NotImplementedError(f"coefficient of type {type(coef)}")


def _qpoints(model, measure: Measure) -> np.ndarray:
    """Physical quadrature points of every cell (host glue for Python-callable sources)."""
    D = model.dim
    n = measure.degree // 2 + 1
    x1, w1 = np.polynomial.legendre.leggauss(n)
    x1 = (x1 + 1) / 2
    k = np.arange(n ** D)
    xi = np.stack([x1[(k // n ** d) % n] for d in range(D)], axis=1)  # first coord fastest
    nv = 2 ** D
    phi = np.ones((xi.shape[0], nv))
    for a in range(nv):
        for d in range(D):
            phi[:, a] *= xi[:, d] if (a >> d) & 1 else 1 - xi[:, d]
    X = model.node_coords[model.cell_node_ids - 1]  # (ncells, nv, D)
    return np.einsum("qa,cad->cqd", phi, X)


def _source_to_problem(prep: _Prepared, f, model, measure):
    p = prep.p
    if f is None:
        p.source_kind = _lib.GFE_SRC_NONE
    elif isinstance(f, (int, float)):
        arr = np.array([float(f)])
        prep.keep.append(arr)
        p.source_kind, p.source, p.source_len = _lib.GFE_SRC_CONST, _lib.ptr(arr), 1
    elif isinstance(f, NodalField):
        v = f.values
        if isinstance(v, np.ndarray):
            v = np.ascontiguousarray(v, dtype=np.float64)
        prep.keep.append(v)
        p.source_kind, p.source, p.source_len = _lib.GFE_SRC_NODAL, _lib.ptr(v), v.shape[0]
    elif isinstance(f, SinSum) and model.cartesian:
        arr = np.concatenate([[f.terms.shape[0]], f.terms.reshape(-1)]).astype(np.float64)
        prep.keep.append(arr)
        p.source_kind, p.source, p.source_len = _lib.GFE_SRC_SINSUM, _lib.ptr(arr), arr.size
    elif callable(f):
        xq = _qpoints(model, measure)
        vals = np.ascontiguousarray(
            np.asarray(f(xq.reshape(-1, model.dim)), dtype=np.float64).reshape(-1))
        prep.keep.append(vals)
        p.source_kind, p.source, p.source_len = _lib.GFE_SRC_QPOINT, _lib.ptr(vals), vals.size
    else:
        raise NotImplementedError(f"source of type {type(f)}")


def _lame_to_problem(prep: _Prepared, lame, ncells):
    """(λ, μ), each a number or a per-cell CellField -> interleaved (λ, μ) array."""
    p = prep.p
    if lame is None:
        p.coef_kind = _lib.GFE_COEF_ONE
        return
    lam, mu = lame
    if all(isinstance(c, (int, float)) for c in (lam, mu)):
        arr = np.array([float(lam), float(mu)])
        p.coef_kind = _lib.GFE_COEF_CONST
    else:
        cols = []
        for c in (lam, mu):
            vals = c.values if isinstance(c, CellField) else c
            if isinstance(vals, (int, float)):
                vals = np.full(ncells, float(vals))
            vals = np.asarray(vals.cpu() if hasattr(vals, "cpu") else vals, np.float64)
            if vals.shape != (ncells,):
                raise ValueError("per-cell Lamé coefficient has the wrong length")
            cols.append(vals)
        arr = np.ascontiguousarray(np.stack(cols, axis=1).reshape(-1))
        p.coef_kind = _lib.GFE_COEF_CELL
    prep.keep.append(arr)
    p.coef = _lib.ptr(arr)


def _prepare_elasticity(V, measure, lame, force, precision, cell_dof_ids, geometry):
    model = V.model
    prep = _Prepared()
    p = prep.p
    p.dim, p.ncomp, p.degree = 3, V.reffe.ncomp, measure.degree
    p.reffe = _lib.GFE_REFFE_P2_TET
    p.ncells = model.num_cells()
    p.nd = V.ndofs_per_cell()
    ids = V.cell_dof_ids if cell_dof_ids is None else cell_dof_ids
    prep.keep.append(ids)
    p.cell_dof_ids = _lib.ptr(ids)
    p.nfree = V.num_free_dofs()
    for d in range(3):
        p.partition[d] = model.partition[d]
        p.domain[2 * d] = model.domain[2 * d]
        p.domain[2 * d + 1] = model.domain[2 * d + 1]
    p.nnodes = model.num_nodes()
    prep.keep += [model.node_coords, model.cell_node_ids]
    p.node_coords = _lib.ptr(model.node_coords)
    p.cell_node_ids = _lib.ptr(model.cell_node_ids)
    p.geometry = _lib.GFE_GEOM_NODAL if geometry == "nodal" else _lib.GFE_GEOM_CARTESIAN
    p.form = _lib.GFE_FORM_ELASTICITY
    _lame_to_problem(prep, lame, p.ncells)
    if force is None:
        p.source_kind = _lib.GFE_SRC_NONE
    else:
        fv = np.ascontiguousarray(force, np.float64).reshape(3)
        prep.keep.append(fv)
        p.source_kind, p.source, p.source_len = _lib.GFE_SRC_CONST, _lib.ptr(fv), 3
    p.precision = _lib.GFE_PREC_FP32 if precision == "fp32" else _lib.GFE_PREC_FP64
    return prep


def prepare_problem(U, V, measure: Measure, coef=None, source=None, precision="fp64",
                    cell_dof_ids=None, geometry=None) -> _Prepared:
    """The gfe_problem for ∫ coef ∇v⋅∇u dΩ and ∫ source v dΩ on V (U == V for square); on a
    simplexified model, for ∫ ε(v) ⊙ σ(ε(u)) dΩ with coef = (λ, μ) and ∫ f⋅v dΩ with
    source = f. geometry="nodal" forces the general (node-coordinate) element path."""
    uD = U.dirichlet_values if isinstance(U, TrialFESpace) else None
    V = _space(V)
    model = V.model
    if isinstance(model, SimplexDiscreteModel):
        prep = _prepare_elasticity(V, measure, coef, source, precision, cell_dof_ids, geometry)
        _dirichlet_to_problem(prep, uD)
        return prep
    prep = _Prepared()
    p = prep.p
    D = model.dim
    q2 = V.reffe.order == 2
    p.dim, p.ncomp, p.degree = D, V.reffe.ncomp, measure.degree
    p.reffe = _lib.GFE_REFFE_Q2 if q2 else _lib.GFE_REFFE_Q1
    p.ncells = model.num_cells()
    p.nd = V.ndofs_per_cell()
    ids = V.cell_dof_ids if cell_dof_ids is None else cell_dof_ids
    prep.keep.append(ids)
    p.cell_dof_ids = _lib.ptr(ids)
    p.nfree = V.num_free_dofs()
    for d in range(D):
        p.partition[d] = model.partition[d]
        p.domain[2 * d] = model.domain[2 * d]
        p.domain[2 * d + 1] = model.domain[2 * d + 1]
    p.nnodes = model.num_nodes()
    if model.cartesian and not q2:
        p.geometry = _lib.GFE_GEOM_CARTESIAN
    else:
        p.geometry = _lib.GFE_GEOM_NODAL
        prep.keep.append(model.node_coords)
        p.node_coords = _lib.ptr(model.node_coords)
        prep.keep.append(model.cell_node_ids)
        p.cell_node_ids = _lib.ptr(model.cell_node_ids)
    p.form = _lib.GFE_FORM_DIFFUSION
    _coef_to_problem(prep, coef, p.ncells)
    _source_to_problem(prep, source, model, measure)
    p.precision = _lib.GFE_PREC_FP32 if precision == "fp32" else _lib.GFE_PREC_FP64
    _dirichlet_to_problem(prep, uD)
    return prep


def _dirichlet_to_problem(prep: _Prepared, uD) -> None:
    if uD is None:
        return
    uD = np.ascontiguousarray(uD, np.float64)
    prep.keep.append(uD)
    prep.p.dirichlet_values, prep.p.ndirichlet = _lib.ptr(uD), uD.size


class _Forms:
    """User forms evaluated into the volume measure, coefficient and source, plus the
    boundary terms: bilinear [(measure, (c0, c1, c2, c3))] and linear
    [(measure, [(test_op, scale, data)])] on BoundaryTriangulation measures."""

    def __init__(self, meas, coef, source, boundary, boundary_mat):
        self.meas, self.coef, self.source = meas, coef, source
        self.boundary, self.boundary_mat = boundary, boundary_mat

    def __iter__(self):
        return iter((self.meas, self.coef, self.source))


def _forms(a, l, U, V) -> _Forms:
    """Evaluates user forms a(u,v), l(v): one volume term in each, and any number of terms on
    BoundaryTriangulation measures (Neumann, Nitsche and Robin terms)."""
    from .celldata import get_fe_basis, get_trial_fe_basis
    u, v = get_trial_fe_basis(U), get_fe_basis(V)
    coef = source = None
    meas = None
    boundary, boundary_mat = [], []
    if a is not None:
        dc = a(u, v)
        vol = [(e, m) for e, m in dc.terms if not m.on_boundary]
        boundary_mat = [(m, classify_boundary_bilinear(e)) for e, m in dc.terms if m.on_boundary]
        if len(vol) != 1:
            raise NotImplementedError("one bilinear term over the cells is provided")
        expr, meas = vol[0]
        _, coef = classify_bilinear(expr)
    if l is not None:
        dc = l(v)
        vol = [(e, m) for e, m in dc.terms if not m.on_boundary]
        boundary = [(m, classify_boundary_linear(e)) for e, m in dc.terms if m.on_boundary]
        if len(vol) > 1:
            raise NotImplementedError("one linear term over the cells is provided")
        if vol:
            expr, m2 = vol[0]
            if meas is not None and m2.degree != meas.degree:
                raise NotImplementedError("bilinear and linear forms on different measures")
            meas = m2
            _, source = classify_linear(expr)
    if meas is None:
        # boundary terms only: the volume pass assembles no source
        meas = Measure(Triangulation(_space(V).model), 2)
    return _Forms(meas, coef, source, boundary, boundary_mat)


def _facet_qpoints(trian: BoundaryTriangulation, degree: int) -> np.ndarray:
    """Physical Gauss points of every facet (tensor Gauss-Legendre of `degree`, first facet
    coordinate fastest): host glue for Python-callable boundary data."""
    D = trian.model.dim
    n = degree // 2 + 1
    x1, _ = np.polynomial.legendre.leggauss(n)
    x1 = (x1 + 1) / 2
    k = np.arange(n ** (D - 1))
    s = np.stack([x1[(k // n ** d) % n] for d in range(D - 1)], axis=1)
    return trian.facet_points(s)[1]


def _facet_data(trian: BoundaryTriangulation, degree: int, terms):
    """Sum of scale * data over terms at every facet Gauss point: (kind, values)."""
    if all(d is None for _, _, d in terms):
        return _lib.GFE_SRC_CONST, np.array([sum(c for _, c, _ in terms)])
    xq = _facet_qpoints(trian, degree)
    nf, nq, D = xq.shape
    x = xq.reshape(-1, D)
    tot = np.zeros(nf * nq)
    for _, c, d in terms:
        if d is None:
            tot += c
        elif isinstance(d, tuple):  # n . G(x)
            G = np.asarray(d[1](x), np.float64)
            if G.shape != (x.shape[0], D):
                G = np.array([np.asarray(d[1](xi), np.float64) for xi in x])
            n = np.repeat(trian.get_facet_normal(), nq, axis=0)
            tot += c * np.einsum("pd,pd->p", n, G)
        else:
            g = np.asarray(d(x), np.float64)
            if g.shape != (x.shape[0],):
                g = np.array([float(d(xi)) for xi in x])
            tot += c * g
    return _lib.GFE_SRC_QPOINT, np.ascontiguousarray(tot)


def _assemble_boundary(ctx, prep: _Prepared, forms: _Forms, A, b) -> None:
    """A += the facet matrices of the bilinear boundary terms (with their Dirichlet lift into
    b) and b += the linear boundary terms: gfe_assemble_boundary_matrix / _vector."""
    if not forms.boundary and not forms.boundary_mat:
        return
    p = prep.p
    if p.reffe not in (_lib.GFE_REFFE_Q1, _lib.GFE_REFFE_Q2) or p.ncomp != 1:
        raise NotImplementedError("boundary terms are provided for scalar Q1/Q2 spaces")
    L = _lib.load()
    if A is not None:
        for meas, coefs in forms.boundary_mat:
            G = meas.trian
            cf = np.array(coefs, np.float64)
            _lib.check(L.gfe_assemble_boundary_matrix(
                ctx.handle, C.byref(p), A.handle, _lib.ptr(b) if b is not None else None,
                G.num_cells(), _lib.ptr(G.facet_cells), _lib.ptr(G.facet_lfaces), meas.degree,
                _lib.ptr(cf)))
    if b is None:
        return
    for meas, terms in forms.boundary:
        G = meas.trian
        for op in (_lib.GFE_BOP_VALUE, _lib.GFE_BOP_NORMAL_GRAD):
            sel = [t for t in terms if t[0] == op]
            if not sel:
                continue
            kind, vals = _facet_data(G, meas.degree, sel)
            _lib.check(L.gfe_assemble_boundary_vector(
                ctx.handle, C.byref(p), G.num_cells(), _lib.ptr(G.facet_cells),
                _lib.ptr(G.facet_lfaces), meas.degree, op, kind, _lib.ptr(vals), vals.size,
                _lib.ptr(b)))


def assemble_matrix_and_vector(a, l, U, V, assem: SparseMatrixAssembler | None = None,
                               b_out=None):
    """(A, b) for the weak forms a(u,v), l(v) (FESpaces/Assemblers.jl:372-400)."""
    from .multifield import MultiFieldFESpace
    if isinstance(U, MultiFieldFESpace) or isinstance(V, MultiFieldFESpace):
        from . import multifield
        return multifield.assemble_matrix_and_vector(a, l, U, V, assem)
    assem = assem or SparseMatrixAssembler(U, V)
    forms = _forms(a, l, U, V)
    meas, coef, source = forms
    Vs = _space(V)
    prep = prepare_problem(U, V, meas, coef, source if l is not None else None, assem.precision)
    prep.model = Vs.model
    A = None
    if a is not None:
        A = symbolic_loop_problem(assem, prep)
    b = None
    if l is not None:
        b = np.zeros(Vs.num_free_dofs()) if b_out is None else b_out
    _lib.check(_lib.load().gfe_assemble_matrix_and_vector(
        assem.ctx.handle, C.byref(prep.p), A.handle if A is not None else None,
        _lib.ptr(b) if b is not None else None))
    _assemble_boundary(assem.ctx, prep, forms, A, b)
    return A, b


def assemble_matrix_and_vector_(a, l, A: DeviceMatrix, b, U, V,
                                assem: SparseMatrixAssembler | None = None):
    """assemble_matrix_and_vector!(a, l, A, b, U, V): re-assembles into A's existing pattern
    (fillstored!(A, 0) then the numeric loop, FESpaces/SparseMatrixAssemblers.jl:60-68) and
    overwrites b."""
    assem = assem or SparseMatrixAssembler(U, V)
    forms = _forms(a, l, U, V)
    meas, coef, source = forms
    prep = prepare_problem(U, V, meas, coef, source if l is not None else None, assem.precision)
    prep.model = _space(V).model
    if A is not None:
        A.fillstored_zero()
    if b is not None:
        b[...] = 0
    ctx = A.ctx if A is not None else assem.ctx
    _lib.check(_lib.load().gfe_assemble_matrix_and_vector(
        ctx.handle, C.byref(prep.p),
        A.handle if A is not None else None, _lib.ptr(b) if b is not None else None))
    _assemble_boundary(ctx, prep, forms, A, b)
    return A, b


def assemble_matrix_(a, A: DeviceMatrix, U, V, assem: SparseMatrixAssembler | None = None):
    """assemble_matrix!(a, A, U, V)."""
    return assemble_matrix_and_vector_(a, None, A, None, U, V, assem)[0]


def assemble_vector_(l, b, V, assem: SparseMatrixAssembler | None = None):
    """assemble_vector!(l, b, V)."""
    return assemble_matrix_and_vector_(None, l, None, b, V, V, assem)[1]


def assemble_matrix(a, U, V, assem: SparseMatrixAssembler | None = None) -> DeviceMatrix:
    return assemble_matrix_and_vector(a, None, U, V, assem)[0]


def assemble_vector(l, V, assem: SparseMatrixAssembler | None = None):
    return assemble_matrix_and_vector(None, l, V, V, assem)[1]


class AffineFEOperator:
    """AffineFEOperator(a, l, U, V[, assem]): the assembled system A x = b
    (FESpaces/AffineFEOperators.jl:23-54)."""

    def __init__(self, a, l, U, V, assem: SparseMatrixAssembler | None = None):
        self.trial = U
        self.test = V
        self.assem = assem or SparseMatrixAssembler(U, V)
        self.A, self.b = assemble_matrix_and_vector(a, l, U, V, self.assem)

    def get_matrix(self) -> DeviceMatrix:
        return self.A

    def get_vector(self):
        return self.b

    def get_trial(self):
        return self.trial

    def get_test(self):
        return self.test
