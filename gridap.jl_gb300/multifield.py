"""Multi-field FE spaces and their assembly, mirroring Gridap's MultiField module.

`MultiFieldFESpace([U, P])` couples single-field Lagrangian spaces on one model. With
`ConsecutiveMultiFieldStyle()` (the default) the free dofs of the fields are concatenated and
a weak form assembles into one matrix; with `BlockMultiFieldStyle(NB, SB, P)` the fields are
grouped into NB blocks (SB fields each, in the order of the permutation P) and the assembly
returns an NB x NB grid of matrices, as `BlockSparseMatrixAssembler` does
(MultiField/MultiFieldFESpaces.jl:1-110, MultiField/BlockSparseMatrixAssemblers.jl:1-140).

The cell integrals and their assembly run on the device (gfe_multifield_assemble): per cell
the geometry and the physical gradients of every field at the quadrature points, then the
cell matrices and vectors of a block, then the row-gather numeric loops of the single-field
path. Here on the host: the numbering, the reference tables, and Python-callable data
evaluated at the quadrature points.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .celldata import classify_multifield
from .fespaces import FEFunction, TrialFESpace, _space, ncube_node_refs


class ConsecutiveMultiFieldStyle:
    """Free dofs of field i follow those of fields 1..i-1 (MultiFieldFESpaces.jl:6-11)."""


class BlockMultiFieldStyle:
    """BlockMultiFieldStyle(NB, SB, P): NB blocks of SB[k] fields each, taken in the order of
    the 1-based permutation P (MultiFieldFESpaces.jl:13-57). BlockMultiFieldStyle() makes
    one block per field."""

    def __init__(self, NB: int = 0, SB=None, P=None):
        self.NB = int(NB)
        self.SB = None if SB is None else tuple(int(s) for s in SB)
        self.P = None if P is None else tuple(int(p) for p in P)

    def resolved(self, nfields: int) -> "BlockMultiFieldStyle":
        if self.NB == 0:
            return BlockMultiFieldStyle(nfields, (1,) * nfields, tuple(range(1, nfields + 1)))
        SB = self.SB if self.SB is not None else (1,) * self.NB
        P = self.P if self.P is not None else tuple(range(1, sum(SB) + 1))
        if len(SB) != self.NB or sum(SB) != len(P) or sorted(P) != list(range(1, nfields + 1)):
            raise ValueError("BlockMultiFieldStyle: SB must have NB entries summing to the "
                             "number of fields, and P must be a permutation of the fields")
        return BlockMultiFieldStyle(self.NB, SB, P)


def get_block_ranges(NB: int, SB, P):
    """Field indices (0-based) of every block, in the order of P (MultiFieldFESpaces.jl:62-67)."""
    ptr = np.concatenate([[0], np.cumsum(SB)])
    return [[P[k] - 1 for k in range(ptr[i], ptr[i + 1])] for i in range(NB)]


class MultiFieldFESpace:
    """MultiFieldFESpace(spaces; style): single-field spaces (FESpace or TrialFESpace) of one
    model (MultiFieldFESpaces.jl:99-150)."""

    def __init__(self, spaces, style=None):
        self.spaces = list(spaces)
        if not self.spaces:
            raise ValueError("MultiFieldFESpace needs at least one field")
        models = {id(_space(S).model) for S in self.spaces}
        if len(models) != 1:
            raise NotImplementedError("the fields of a MultiFieldFESpace share one model")
        style = style or ConsecutiveMultiFieldStyle()
        if isinstance(style, BlockMultiFieldStyle):
            style = style.resolved(len(self.spaces))
        self.style = style

    # collection protocol (Base.iterate / getindex / length)
    def __iter__(self):
        return iter(self.spaces)

    def __getitem__(self, i):
        return self.spaces[i]

    def __len__(self):
        return len(self.spaces)

    def num_fields(self) -> int:
        return len(self.spaces)

    @property
    def model(self):
        return _space(self.spaces[0]).model

    def is_block(self) -> bool:
        return isinstance(self.style, BlockMultiFieldStyle)

    def block_ranges(self):
        """Fields of every assembly block (one block holding every field when consecutive)."""
        if self.is_block():
            s = self.style
            return get_block_ranges(s.NB, s.SB, s.P)
        return [list(range(len(self.spaces)))]

    def num_free_dofs(self) -> int:
        return sum(_space(S).num_free_dofs() for S in self.spaces)

    def block_num_free_dofs(self):
        return [sum(_space(self.spaces[f]).num_free_dofs() for f in r)
                for r in self.block_ranges()]

    def compute_field_offsets(self):
        """Offset of every field's free dofs inside its block (the whole vector when
        consecutive): MultiFieldFESpaces.jl:335-364."""
        off = [0] * len(self.spaces)
        for r in self.block_ranges():
            acc = 0
            for f in r:
                off[f] = acc
                acc += _space(self.spaces[f]).num_free_dofs()
        return tuple(off)

    def field_cell_dof_ids(self, f: int) -> np.ndarray:
        """Cell dof ids of field f with its offset added to the free (positive) ids, Dirichlet
        ids unchanged (_sum_if_first_positive, MultiFieldFESpaces.jl:460-488)."""
        ids = _space(self.spaces[f]).get_cell_dof_ids()
        o = self.compute_field_offsets()[f]
        return np.where(ids > 0, ids + o, ids).astype(np.int32)

    def get_cell_dof_ids(self) -> np.ndarray:
        """The fields' cell ids side by side (one row per cell)."""
        return np.ascontiguousarray(
            np.concatenate([self.field_cell_dof_ids(f) for f in range(len(self.spaces))],
                           axis=1))

    def zero_free_values(self):
        if self.is_block():
            return [np.zeros(n) for n in self.block_num_free_dofs()]
        return np.zeros(self.num_free_dofs())

    def _block_of(self, f: int) -> int:
        for k, r in enumerate(self.block_ranges()):
            if f in r:
                return k
        raise IndexError(f)

    def restrict_to_field(self, free_values, f: int):
        """The free values of field f (MultiFieldFESpaces.jl:289-330): a view."""
        o = self.compute_field_offsets()[f]
        n = _space(self.spaces[f]).num_free_dofs()
        if self.is_block() and isinstance(free_values, (list, tuple)):
            return free_values[self._block_of(f)][o:o + n]
        if self.is_block():  # a flat vector laid out block after block
            starts = np.concatenate([[0], np.cumsum(self.block_num_free_dofs())])
            o += int(starts[self._block_of(f)])
        return free_values[o:o + n]


def compute_field_offsets(X: MultiFieldFESpace):
    return X.compute_field_offsets()


def num_fields(X) -> int:
    return X.num_fields() if isinstance(X, MultiFieldFESpace) else 1


class MultiFieldFEFunction:
    """FEFunction(X, free_values) on a MultiFieldFESpace: one FEFunction per field, unpacked
    as `uh, ph = xh` (MultiField/MultiFieldFEFunctions.jl)."""

    def __init__(self, X: MultiFieldFESpace, free_values):
        self.space = X
        self.free_values = free_values
        self.fields = [FEFunction(U, X.restrict_to_field(free_values, i))
                       for i, U in enumerate(X.spaces)]

    def __iter__(self):
        return iter(self.fields)

    def __getitem__(self, i):
        return self.fields[i]

    def get_free_dof_values(self):
        return self.free_values


# ---- reference tables ------------------------------------------------------------------------
def tensor_gauss(D: int, degree: int):
    """Tensor Gauss-Legendre rule on [0,1]^D with degree//2+1 points per direction, the first
    coordinate fastest (Quadrature(QUAD/HEX, degree))."""
    n = degree // 2 + 1
    x1, w1 = np.polynomial.legendre.leggauss(n)
    x1, w1 = (x1 + 1) / 2, w1 / 2
    k = np.arange(n ** D)
    i = np.stack([(k // n ** d) % n for d in range(D)], axis=1)
    return np.ascontiguousarray(x1[i]), np.ascontiguousarray(np.prod(w1[i], axis=1))


def lagrangian_tables(D: int, order: int, qx: np.ndarray):
    """Values (nq, nn) and reference gradients (nq, nn, D) of the Lagrangian Q_order shape
    functions at the points qx, nodes in Gridap's order (ncube_node_refs): tensor products of
    the 1-D Lagrange polynomials on the equispaced nodes of [0, 1]."""
    z = np.linspace(0.0, 1.0, order + 1)
    idx = np.rint(ncube_node_refs(D, order) * order).astype(int)  # (nn, D)
    L = np.empty((order + 1,) + qx.shape)
    dL = np.empty_like(L)
    for j in range(order + 1):
        others = [m for m in range(order + 1) if m != j]
        den = np.prod([z[j] - z[m] for m in others])
        L[j] = np.prod([qx - z[m] for m in others], axis=0) / den
        dL[j] = sum(np.prod([qx - z[m] for m in others if m != k] or [np.ones_like(qx)],
                            axis=0) for k in others) / den
    dims = np.arange(D)
    vals = L[idx[:, None, :], np.arange(qx.shape[0])[None, :, None], dims]  # (nn, nq, D)
    ders = dL[idx[:, None, :], np.arange(qx.shape[0])[None, :, None], dims]
    phi = np.prod(vals, axis=2).T
    grads = np.empty((qx.shape[0], idx.shape[0], D))
    for e in range(D):
        fac = vals.copy()
        fac[:, :, e] = ders[:, :, e]
        grads[:, :, e] = np.prod(fac, axis=2).T
    return np.ascontiguousarray(phi), np.ascontiguousarray(grads)


def _eval_points(f, x: np.ndarray) -> np.ndarray:
    """f at the points x (N, D) as an (N, k) array: f a constant (number or sequence) or a
    callable vectorised over rows or of one point."""
    if not callable(f):
        v = np.asarray(f, np.float64).reshape(-1)
        return np.ascontiguousarray(np.broadcast_to(v, (x.shape[0], v.size)))
    try:
        v = np.asarray(f(x), np.float64)
        if v.ndim == 0 or v.shape[0] != x.shape[0]:
            raise ValueError
    except (TypeError, IndexError, ValueError):
        v = np.array([np.asarray(f(xi), np.float64) for xi in x])
    return np.ascontiguousarray(v.reshape(x.shape[0], -1))


# ---- assembly -------------------------------------------------------------------------------
class BlockDeviceMatrix:
    """An NB_rows x NB_cols grid of device matrices (the BlockArray of sparse matrices that
    BlockSparseMatrixAssembler builds)."""

    def __init__(self, blocks, row_sizes, col_sizes):
        self.blocks = blocks
        self.row_sizes, self.col_sizes = list(row_sizes), list(col_sizes)
        self.shape = (sum(self.row_sizes), sum(self.col_sizes))

    def __getitem__(self, ij):
        i, j = ij
        return self.blocks[i][j]

    def blocksizes(self, dim: int):
        return list(self.row_sizes if dim == 1 else self.col_sizes)

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.bmat([[B.to_scipy() for B in row] for row in self.blocks], format="csr")

    def matvec(self, x):
        """y = A x for a list of block vectors (numpy)."""
        ys = [np.zeros(n) for n in self.row_sizes]
        for i, row in enumerate(self.blocks):
            for j, B in enumerate(row):
                if B.nnz:
                    ys[i] += B.matvec(np.ascontiguousarray(x[j], np.float64))
        return ys


class _MfContext:
    """gfe_mf_problem of one quadrature degree: tables, geometry and terms (the arrays are
    kept alive with the structure)."""

    def __init__(self, X, Y, degree, terms):
        model = X.model
        D = model.dim
        self.keep = []
        qx, qw = tensor_gauss(D, degree)
        phi1, g1 = lagrangian_tables(D, 1, qx)
        self.nq = qx.shape[0]
        self.fields = (_lib.MfField * X.num_fields())()
        for f, S in enumerate(X.spaces):
            Vf, Wf = _space(S), _space(Y.spaces[f])
            if Vf.reffe.order != Wf.reffe.order or Vf.reffe.ncomp != Wf.reffe.ncomp:
                raise NotImplementedError("test and trial spaces of a field use one reffe")
            if Vf.reffe.ncomp not in (1, D):
                raise NotImplementedError("fields are scalar or have dim components")
            phi, gr = lagrangian_tables(D, Vf.reffe.order, qx)
            self.keep += [phi, gr]
            self.fields[f].ncomp, self.fields[f].nnodes = Vf.reffe.ncomp, phi.shape[1]
            self.fields[f].shapes, self.fields[f].grads = _lib.ptr(phi), _lib.ptr(gr)
        coords = np.ascontiguousarray(model.node_coords, np.float64)
        cells = np.ascontiguousarray(model.cell_node_ids, np.int32)
        self.keep += [coords, cells, qw, g1]
        xq = None
        self.terms = (_lib.MfTerm * max(len(terms), 1))()
        for k, t in enumerate(terms):
            T = self.terms[k]
            T.test_field, T.test_op = t.test_field, t.test_op
            T.trial_field = -1 if t.trial_field is None else t.trial_field
            T.trial_op = 0 if t.trial_op is None else t.trial_op
            T.coef = t.coef
            if t.cell_coef is not None:
                self.keep.append(t.cell_coef)
                T.cell_coef = _lib.ptr(t.cell_coef)
            if t.data is not None:
                if xq is None:
                    X0 = coords[cells - 1].transpose(0, 2, 1)  # (ncells, D, 2^D)
                    xq = np.ascontiguousarray((X0 @ phi1.T).transpose(0, 2, 1)).reshape(-1, D)
                vals = _eval_points(t.data, xq)
                self.keep.append(vals)
                T.qdata, T.qdata_ncomp = _lib.ptr(vals), vals.shape[1]
        p = self.p = _lib.MfProblem()
        p.dim, p.ncells, p.nnodes = D, model.num_cells(), model.num_nodes()
        p.node_coords, p.cell_node_ids = _lib.ptr(coords), _lib.ptr(cells)
        p.nq, p.qweights, p.geo_grads = self.nq, _lib.ptr(qw), _lib.ptr(g1)
        p.nfields, p.fields = X.num_fields(), C.cast(self.fields, C.c_void_p)
        p.nterms, p.terms = len(terms), C.cast(self.terms, C.c_void_p)


def _forms(a, l, X, Y):
    """(bilinear terms, degree) and [(linear terms, degree)] of user forms a(x, y), l(y) on
    a multi-field space."""
    from .celldata import get_fe_basis, get_trial_fe_basis
    xs, ys = get_trial_fe_basis(X), get_fe_basis(Y)
    bil, deg = [], None
    if a is not None:
        for expr, m in a(xs, ys).terms:
            if m.on_boundary:
                raise NotImplementedError("multi-field boundary terms are not provided")
            if deg is not None and m.degree != deg:
                raise NotImplementedError("the bilinear form integrates with one measure")
            deg = m.degree
            bil += classify_multifield(expr, True)
    lin = {}
    if l is not None:
        for expr, m in l(ys).terms:
            if m.on_boundary:
                raise NotImplementedError("multi-field boundary terms are not provided")
            lin.setdefault(m.degree, []).extend(classify_multifield(expr, False))
    return bil, deg, lin


def _dirichlet(X: MultiFieldFESpace, fields):
    """Column ids of `fields` with field f's Dirichlet ids shifted past those of the fields
    before it, and the matching concatenated Dirichlet values (None when all vanish)."""
    ids, vals, shift = [], [], 0
    any_nonzero = False
    for f in fields:
        U = X.spaces[f]
        cid = X.field_cell_dof_ids(f)
        ids.append(np.where(cid < 0, cid - shift, cid))
        nd = _space(U).num_dirichlet_dofs()
        v = U.get_dirichlet_dof_values() if isinstance(U, TrialFESpace) else np.zeros(nd)
        any_nonzero = any_nonzero or bool(np.any(v))
        vals.append(np.asarray(v, np.float64))
        shift += nd
    uD = np.ascontiguousarray(np.concatenate(vals)) if any_nonzero else None
    return np.ascontiguousarray(np.concatenate(ids, axis=1).astype(np.int32)), uD


def _coupling_mask(X, Y, rfields, cfields, terms):
    """local_mask[li + lj*ndr]: 1 where the (row field, column field) pair of a local entry
    has a bilinear term."""
    pairs = {(t.test_field, t.trial_field) for t in terms}
    rsz = [_space(Y.spaces[f]).ndofs_per_cell() for f in rfields]
    csz = [_space(X.spaces[f]).ndofs_per_cell() for f in cfields]
    rown = np.repeat(rfields, rsz)
    coln = np.repeat(cfields, csz)
    M = np.array([[(r, c) in pairs for c in coln] for r in rown], np.uint8)
    return np.ascontiguousarray(M.T), M.all()  # column-major bytes


def _assemble_block(ctx, X, Y, rfields, cfields, mfc, terms, want_A, b, nrows, ncols):
    """One call of gfe_multifield_assemble: the block (rfields x cfields) into a new matrix
    (want_A) and/or b."""
    L = _lib.load()
    row_ids = np.ascontiguousarray(
        np.concatenate([Y.field_cell_dof_ids(f) for f in rfields], axis=1).astype(np.int32))
    col_ids, uD = _dirichlet(X, cfields)
    A = None
    if want_A:
        from .assembly import DeviceMatrix
        mask, full = _coupling_mask(X, Y, rfields, cfields, terms)
        h = C.c_void_p()
        nc = row_ids.shape[0]
        if full and row_ids.shape[1] == col_ids.shape[1]:
            _lib.check(L.gfe_symbolic_loop_matrix(ctx.handle, nc, row_ids.shape[1],
                                                  _lib.ptr(row_ids), _lib.ptr(col_ids), nrows,
                                                  ncols, C.byref(h)))
        else:
            _lib.check(L.gfe_symbolic_loop_matrix_masked(
                ctx.handle, nc, row_ids.shape[1], col_ids.shape[1], _lib.ptr(row_ids),
                _lib.ptr(col_ids), _lib.ptr(mask), nrows, ncols, C.byref(h)))
        A = DeviceMatrix(h, ctx)
    rf = np.array(rfields, np.int32)
    cf = np.array(cfields, np.int32)
    _lib.check(L.gfe_multifield_assemble(
        ctx.handle, C.byref(mfc.p), rf.size, _lib.ptr(rf), cf.size, _lib.ptr(cf),
        _lib.ptr(row_ids), _lib.ptr(col_ids), _lib.ptr(uD), 0 if uD is None else uD.size,
        A.handle if A is not None else None, nrows, _lib.ptr(b)))
    return A


def assemble_matrix_and_vector(a, l, X, Y, assem=None):
    """(A, b) of the multi-field forms a(x, y), l(y): one DeviceMatrix and vector with the
    consecutive style, a BlockDeviceMatrix and a list of block vectors with the block style
    (FESpaces/Assemblers.jl:372-400 through MultiField/BlockSparseMatrixAssemblers.jl:
    236-255). b carries the Dirichlet lift -a(u_D, y) of the trial spaces' data."""
    from .assembly import default_context
    ctx = assem.ctx if assem is not None else default_context()
    if not isinstance(X, MultiFieldFESpace) or not isinstance(Y, MultiFieldFESpace) \
            or X.num_fields() != Y.num_fields():
        raise ValueError("trial and test spaces are MultiFieldFESpaces with the same fields")
    if X.is_block() != Y.is_block():
        raise ValueError("trial and test spaces use the same multi-field style")
    bil, deg, lin = _forms(a, l, X, Y)
    rblocks, cblocks = Y.block_ranges(), X.block_ranges()
    rsz, csz = Y.block_num_free_dofs(), X.block_num_free_dofs()
    allf = list(range(X.num_fields()))
    bs = [np.zeros(n) for n in rsz] if l is not None else None
    A = None
    if a is not None:
        fused = bs is not None and not X.is_block() and (deg in lin or not lin)
        terms = bil + (lin.get(deg, []) if fused else [])
        mfc = _MfContext(X, Y, deg, terms)
        A = [[_assemble_block(ctx, X, Y, rf, cf, mfc, terms, True,
                              bs[0] if fused else None, nr, nc)
              for cf, nc in zip(cblocks, csz)] for rf, nr in zip(rblocks, rsz)]
        if fused:
            lin = {k: v for k, v in lin.items() if k != deg}
        elif bs is not None:
            # the lift with the bilinear form's quadrature, linear terms of that degree too
            terms = bil + lin.pop(deg, [])
            mfc = _MfContext(X, Y, deg, terms)
            for I, rf in enumerate(rblocks):
                _assemble_block(ctx, X, Y, rf, allf, mfc, terms, False, bs[I], rsz[I],
                                X.num_free_dofs())
    for d, terms in (lin or {}).items():
        mfc = _MfContext(X, Y, d, terms)
        for I, rf in enumerate(rblocks):
            _assemble_block(ctx, X, Y, rf, rf, mfc, terms, False, bs[I], rsz[I], rsz[I])
    if X.is_block():
        Am = BlockDeviceMatrix(A, rsz, csz) if A is not None else None
        return Am, bs
    return (A[0][0] if A is not None else None), (bs[0] if bs is not None else None)


def assemble_matrix(a, X, Y, assem=None):
    return assemble_matrix_and_vector(a, None, X, Y, assem)[0]


def assemble_vector(l, Y, assem=None):
    return assemble_matrix_and_vector(None, l, Y, Y, assem)[1]
