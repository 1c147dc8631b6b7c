"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the oracle (libgfe_oracle.so), the CPU
restatement of Gridap.jl v0.20.8's assembly and solve path (gfe_oracle.c).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline / reference legs use it, as
the checker or the timed CPU baseline. The product (gridap.jl_gb300/) never imports it.
"""
from __future__ import annotations

import ctypes as C
import math
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libgfe_oracle.so"

F_NONE, F_CONST, F_NODAL, F_QPOINT = 0, 1, 2, 3
GEOM_CARTESIAN, GEOM_NODAL = 0, 1

_lib = None


def build() -> pathlib.Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


class _CSC(C.Structure):
    _fields_ = [("nrows", C.c_int64), ("ncols", C.c_int64), ("nnz", C.c_int64),
                ("colptr", C.POINTER(C.c_int64)), ("rowval", C.POINTER(C.c_int64)),
                ("nzval", C.POINTER(C.c_double))]


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        P = C.c_void_p
        L.orc_ncube_faces.argtypes = [C.c_int, P, P]
        L.orc_cartesian_coords.argtypes = [C.c_int, P, P, P]
        L.orc_cartesian_cell_nodes.argtypes = [C.c_int, P, P]
        L.orc_cartesian_node_entity.argtypes = [C.c_int, P, P]
        L.orc_node_tag_index.argtypes = [C.c_int64, P, C.c_int, P, P, P]
        L.orc_jitter_interior.argtypes = [C.c_int, P, P, P]
        L.orc_clagrangian_numbering.argtypes = [C.c_int64, P, C.c_int, P, C.c_int64, C.c_int, P,
                                                P, P, P, P, P]
        L.orc_conforming_q2.argtypes = [C.c_int, P, C.c_int, P, P, P, P, P]
        L.orc_q2_shapes.argtypes = [C.c_int, C.c_int, P, P, P]
        L.orc_q2_cell_arrays_diffusion.argtypes = [C.c_int, C.c_int64, P, P, P, C.c_int, P, P,
                                                   C.c_int, P, P, P]
        L.orc_gauss_legendre01.argtypes = [C.c_int, P, P]
        L.orc_tensor_quadrature.argtypes = [C.c_int, C.c_int, P, P]
        L.orc_q1_shapes.argtypes = [C.c_int, C.c_int, P, P, P]
        L.orc_q1_cell_qpoints.argtypes = [C.c_int, C.c_int64, P, P, C.c_int, P, P]
        L.orc_q1_cell_arrays_diffusion.argtypes = [C.c_int, C.c_int64, P, P, C.c_int, P, P,
                                                   C.c_int, P, P, C.c_int, P, P, P]
        L.orc_assemble_matrix_csc.argtypes = [C.c_int64, C.c_int, P, P, P, C.c_int64, C.c_int64,
                                              C.POINTER(_CSC)]
        L.orc_assemble_matrix_csc_rect.argtypes = [C.c_int64, C.c_int, C.c_int, P, P, P,
                                                   C.c_int64, C.c_int64, C.POINTER(_CSC)]
        L.orc_csc_free.argtypes = [C.POINTER(_CSC)]
        L.orc_assemble_vector.argtypes = [C.c_int64, C.c_int, P, P, P]
        L.orc_pcg.argtypes = [C.POINTER(_CSC), P, P, C.c_double, C.c_int, C.c_int, C.c_int, P]
        L.orc_csc_mul.argtypes = [C.POINTER(_CSC), P, P]
        L.orc_simplex_cells.argtypes = [P, P]
        L.orc_simplex_p2_numbering.argtypes = [P, C.c_int, P, P, P, P, P]
        L.orc_p2tet_shapes.argtypes = [C.c_int, P, P, P]
        L.orc_wv_tet_degree5.argtypes = [P, P]
        L.orc_wv_tet_degree5.restype = C.c_double
        L.orc_p2tet_cell_arrays_elasticity.argtypes = [C.c_int64, P, P, P, C.c_int, P, P, P,
                                                       P, P]
        L.orc_compute_adjacency.argtypes = [C.c_int64, C.c_int, P, C.c_int64,
                                            C.POINTER(C.POINTER(C.c_int64)),
                                            C.POINTER(C.POINTER(C.c_int32))]
        L.orc_free.argtypes = [P]
        L.orc_set_cell_threads.argtypes = [C.c_int]
        L.orc_color_cells.argtypes = [C.c_int64, C.c_int, P, C.c_int64, P]
        L.orc_assemble_csc_colored.argtypes = [C.c_int64, C.c_int, P, P, P, C.c_int64, C.c_int,
                                               P, P, C.c_int, C.POINTER(_CSC), P]
        L.orc_rcm_perm.argtypes = [C.c_int64, P, P, P]
        L.orc_sloan_perm.argtypes = [C.c_int64, P, P, C.c_int64, C.c_int64, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data if a is not None else None


# ---- geometry ----------------------------------------------------------------------------
def ncube_faces(D):
    ext = np.zeros((27, D), np.int32)
    anc = np.zeros((27, D), np.int32)
    n = lib().orc_ncube_faces(D, _p(ext), _p(anc))
    return ext[:n], anc[:n]


def cartesian_model(domain, partition):
    D = len(partition)
    part = np.asarray(partition, np.int64)
    dom = np.asarray(domain, np.float64)
    nn = int(np.prod(part + 1))
    nc = int(np.prod(part))
    coords = np.empty((nn, D))
    cells = np.empty((nc, 2 ** D), np.int32)
    ent = np.empty(nn, np.int32)
    L = lib()
    L.orc_cartesian_coords(D, _p(part), _p(dom), _p(coords))
    L.orc_cartesian_cell_nodes(D, _p(part), _p(cells))
    L.orc_cartesian_node_entity(D, _p(part), _p(ent))
    return coords, cells, ent


def jitter_interior(partition, coords, jitter):
    D = len(partition)
    part = np.asarray(partition, np.int64)
    out = np.ascontiguousarray(coords.copy())
    lib().orc_jitter_interior(D, _p(part), _p(np.ascontiguousarray(jitter, np.float64)), _p(out))
    return out


def cartesian_tags(D):
    """Gridap's Cartesian tags: tag_<i> per boundary entity, 'interior', 'boundary'."""
    interior = 3 ** D
    width = math.ceil(math.log10(interior))
    names, ents = [], []
    for i in range(1, interior):
        names.append(f"tag_{str(i).zfill(width)}")
        ents.append([i])
    names += ["interior", "boundary"]
    ents += [[interior], list(range(1, interior))]
    return names, ents


def node_tag_index(D, node_entity, tags):
    names, ents = cartesian_tags(D)
    sel = []
    for t in tags:
        sel.append(ents[t - 1] if isinstance(t, (int, np.integer)) else ents[names.index(t)])
    ptrs = np.zeros(len(sel) + 1, np.int32)
    for i, e in enumerate(sel):
        ptrs[i + 1] = ptrs[i] + len(e)
    flat = np.asarray([x for e in sel for x in e] or [0], np.int32)
    out = np.zeros(node_entity.shape[0], np.int8)
    lib().orc_node_tag_index(node_entity.shape[0], _p(np.ascontiguousarray(node_entity)),
                             len(sel), _p(ptrs), _p(flat), _p(out))
    return out


# ---- dofs -------------------------------------------------------------------------------
def clagrangian(node_to_tag, cell_nodes, ncomp=1, masks=None, lmap=None):
    nn = node_to_tag.shape[0]
    nc, nv = cell_nodes.shape
    ntags = max(int(node_to_tag.max(initial=0)), 1)
    if masks is None:
        masks = np.ones((ntags, ncomp), np.uint8)
    masks = np.ascontiguousarray(masks, np.uint8)
    if lmap is None:
        lmap = np.array([[c * nv + a + 1 for c in range(ncomp)] for a in range(nv)], np.int32)
    node_dof = np.empty((nn, ncomp), np.int32)
    cell_dofs = np.empty((nc, nv * ncomp), np.int32)
    nf = np.zeros(1, np.int32)
    ndr = np.zeros(1, np.int32)
    lib().orc_clagrangian_numbering(nn, _p(node_to_tag), ncomp, _p(masks), nc, nv,
                                    _p(np.ascontiguousarray(cell_nodes)), _p(lmap), _p(node_dof),
                                    _p(cell_dofs), _p(nf), _p(ndr))
    return node_dof, cell_dofs, int(nf[0]), int(ndr[0])


def conforming_q2(partition, tags, ncomp=1, masks=None):
    """Q2 conforming numbering: (cell_dofs, nfree, ndiri)."""
    D = len(partition)
    names, ents = cartesian_tags(D)
    ent_to_tag = np.zeros(3 ** D, np.int8)
    for e in range(1, 3 ** D + 1):
        for k, t in enumerate(tags):
            te = ents[t - 1] if isinstance(t, (int, np.integer)) else ents[names.index(t)]
            if e in te:
                ent_to_tag[e - 1] = k + 1
                break
    ntags = max(len(tags), 1)
    if masks is None:
        masks = np.ones((ntags, ncomp), np.uint8)
    masks = np.ascontiguousarray(masks, np.uint8)
    part = np.asarray(partition, np.int64)
    nc = int(np.prod(part))
    cd = np.empty((nc, 3 ** D * ncomp), np.int32)
    nf = np.zeros(1, np.int32)
    nd = np.zeros(1, np.int32)
    lib().orc_conforming_q2(D, _p(part), ncomp, _p(ent_to_tag), _p(masks), _p(cd), _p(nf),
                            _p(nd))
    return cd, int(nf[0]), int(nd[0])


def q2_shapes(D, pts):
    pts = np.ascontiguousarray(pts, np.float64)
    nn = 3 ** D
    phi = np.empty((pts.shape[0], nn))
    dphi = np.empty((pts.shape[0], nn, D))
    lib().orc_q2_shapes(D, pts.shape[0], _p(pts), _p(phi), _p(dphi))
    return phi, dphi


def q2_cell_arrays(D, cell_vertices, coords, degree, kappa=None, fkind=F_NONE, fdata=None):
    qx, qw = tensor_quadrature(D, degree)
    nc = cell_vertices.shape[0]
    nn = 3 ** D
    mats = np.zeros((nc, nn, nn))
    vecs = np.zeros((nc, nn))
    kap = None if kappa is None else np.ascontiguousarray(kappa, np.float64)
    fd = None if fdata is None else np.ascontiguousarray(fdata, np.float64)
    st = lib().orc_q2_cell_arrays_diffusion(
        D, nc, _p(np.ascontiguousarray(cell_vertices)), _p(np.ascontiguousarray(coords)),
        _p(kap), qx.shape[0], _p(qx), _p(qw), fkind, _p(fd), _p(mats), _p(vecs))
    if st != 0:
        raise RuntimeError("oracle: degenerate cell")
    return np.ascontiguousarray(np.transpose(mats, (0, 2, 1))), vecs


def poisson_q2(domain, partition, dirichlet_tags=("boundary",), kappa=None, fconst=None,
               degree=4, jitter=None):
    """Gridap's Q2 problem: numbering, cell arrays, CSC matrix and vector."""
    D = len(partition)
    coords, cells, ent = cartesian_model(domain, partition)
    if jitter is not None:
        coords = jitter_interior(partition, coords, jitter)
    cd, nfree, ndiri = conforming_q2(partition, list(dirichlet_tags))
    fk = F_NONE if fconst is None else F_CONST
    fd = None if fconst is None else np.array([float(fconst)])
    mats, vecs = q2_cell_arrays(D, cells, coords, degree, kappa, fk, fd)
    out = dict(coords=coords, cells=cells, cell_dofs=cd, nfree=nfree, ndiri=ndiri,
               cellmats=mats, cellvecs=vecs)
    out["csc"] = assemble_csc(cd, cd, mats, nfree, nfree)
    out["b"] = assemble_vector(cd, vecs, nfree)
    return out


# ---- quadrature / shapes -------------------------------------------------------------------
def gauss_legendre01(n):
    x = np.empty(n)
    w = np.empty(n)
    lib().orc_gauss_legendre01(n, _p(x), _p(w))
    return x, w


def tensor_quadrature(D, degree):
    n = (degree // 2 + 1) ** D
    x = np.empty((n, D))
    w = np.empty(n)
    lib().orc_tensor_quadrature(D, degree, _p(x), _p(w))
    return x, w


def q1_shapes(D, pts):
    pts = np.ascontiguousarray(pts, np.float64)
    nv = 2 ** D
    phi = np.empty((pts.shape[0], nv))
    dphi = np.empty((pts.shape[0], nv, D))
    lib().orc_q1_shapes(D, pts.shape[0], _p(pts), _p(phi), _p(dphi))
    return phi, dphi


# ---- cell arrays ---------------------------------------------------------------------------
def qpoints(D, cell_nodes, coords, degree):
    qx, _ = tensor_quadrature(D, degree)
    nc = cell_nodes.shape[0]
    xq = np.empty((nc, qx.shape[0], D))
    lib().orc_q1_cell_qpoints(D, nc, _p(np.ascontiguousarray(cell_nodes)),
                              _p(np.ascontiguousarray(coords)), qx.shape[0], _p(qx), _p(xq))
    return xq


def q1_cell_arrays(D, cell_nodes, coords, degree, geom=GEOM_CARTESIAN, h=None, kappa=None,
                   fkind=F_NONE, fdata=None, want_mat=True, want_vec=True):
    """Cell matrices (ncells, nd, nd)[c, i, j] and vectors (ncells, nd)."""
    qx, qw = tensor_quadrature(D, degree)
    nc, nv = cell_nodes.shape
    mats = np.zeros((nc, nv, nv)) if want_mat else None  # filled col-major per cell
    vecs = np.zeros((nc, nv)) if want_vec else None
    hh = np.asarray(h if h is not None else [1.0] * D, np.float64)
    kap = None if kappa is None else np.ascontiguousarray(kappa, np.float64)
    fd = None if fdata is None else np.ascontiguousarray(fdata, np.float64)
    st = lib().orc_q1_cell_arrays_diffusion(
        D, nc, _p(np.ascontiguousarray(cell_nodes)), _p(np.ascontiguousarray(coords)), geom,
        _p(hh), _p(kap), qx.shape[0], _p(qx), _p(qw), fkind, _p(fd), _p(mats), _p(vecs))
    if st != 0:
        raise RuntimeError("oracle: degenerate cell")
    if mats is not None:
        mats = np.ascontiguousarray(np.transpose(mats, (0, 2, 1)))  # col-major -> [c, i, j]
    return mats, vecs


# ---- assembly ------------------------------------------------------------------------------
def assemble_csc(cell_rows, cell_cols, cellmats, nrows, ncols):
    """Gridap's SparseMatrixCSC{Float64,Int}: returns (colptr, rowval, nzval), 1-based.
    cellmats[c, i, j] pairs cell_rows[c, i] with cell_cols[c, j]; the two id tables may have
    different widths (a rectangular block)."""
    cell_rows = np.ascontiguousarray(cell_rows, np.int32)
    cell_cols = np.ascontiguousarray(cell_cols, np.int32)
    nc, ndr = cell_rows.shape
    ndc = cell_cols.shape[1]
    cm = None
    if cellmats is not None:
        cm = np.ascontiguousarray(np.transpose(cellmats, (0, 2, 1)), np.float64)  # col-major
    out = _CSC()
    st = lib().orc_assemble_matrix_csc_rect(nc, ndr, ndc, _p(cell_rows), _p(cell_cols), _p(cm),
                                            nrows, ncols, C.byref(out))
    if st != 0:
        raise MemoryError("oracle assembly failed")
    nnz = out.nnz
    colptr = np.ctypeslib.as_array(out.colptr, (ncols + 1,)).copy()
    rowval = np.ctypeslib.as_array(out.rowval, (max(nnz, 1),))[:nnz].copy()
    nzval = np.ctypeslib.as_array(out.nzval, (max(nnz, 1),))[:nnz].copy()
    lib().orc_csc_free(C.byref(out))
    return colptr, rowval, nzval


def set_cell_threads(n):
    """Threads of the oracle's per-cell loops (1 = serial, the default). The cell arrays are
    the same for every thread count."""
    lib().orc_set_cell_threads(int(n))


class cell_threads:
    """`with cell_threads(n):` runs the per-cell loops on n threads, then restores 1."""

    def __init__(self, n):
        self.n = n

    def __enter__(self):
        set_cell_threads(self.n)

    def __exit__(self, *a):
        set_cell_threads(1)


def color_cells(cell_dofs, nfree):
    """Greedy first-fit colours of the cells (cells of one colour share no free dof)."""
    cd = np.ascontiguousarray(cell_dofs, np.int32)
    col = np.empty(cd.shape[0], np.int32)
    k = lib().orc_color_cells(cd.shape[0], cd.shape[1], _p(cd), nfree, _p(col))
    if k < 0:
        raise RuntimeError("oracle: more than 64 colours")
    return col, k


def assemble_colored(cell_dofs, cellmats, cellvecs, n, nthreads, colors=None):
    """Colour-parallel InserterCSC assembly of a square system on `nthreads` threads:
    (colptr, rowval, nzval) 1-based and b. Same pattern as assemble_csc; values are the same
    sums in colour-then-cell order."""
    cd = np.ascontiguousarray(cell_dofs, np.int32)
    col, k = colors if colors is not None else color_cells(cd, n)
    order = np.argsort(col, kind="stable").astype(np.int64)
    cptr = np.zeros(k + 1, np.int64)
    cptr[1:] = np.cumsum(np.bincount(col, minlength=k))
    cm = np.ascontiguousarray(np.transpose(cellmats, (0, 2, 1)), np.float64)  # col-major
    cv = None if cellvecs is None else np.ascontiguousarray(cellvecs, np.float64)
    b = np.zeros(n) if cv is not None else None
    out = _CSC()
    st = lib().orc_assemble_csc_colored(cd.shape[0], cd.shape[1], _p(cd), _p(cm), _p(cv), n, k,
                                        _p(cptr), _p(order), nthreads, C.byref(out), _p(b))
    if st != 0:
        raise MemoryError("oracle colour-parallel assembly failed")
    nnz = out.nnz
    colptr = np.ctypeslib.as_array(out.colptr, (n + 1,)).copy()
    rowval = np.ctypeslib.as_array(out.rowval, (max(nnz, 1),))[:nnz].copy()
    nzval = np.ctypeslib.as_array(out.nzval, (max(nnz, 1),))[:nnz].copy()
    lib().orc_csc_free(C.byref(out))
    return (colptr, rowval, nzval), b


def to_scipy(colptr, rowval, nzval, nrows, ncols):
    import scipy.sparse as sp
    return sp.csc_matrix((nzval, rowval - 1, colptr - 1), shape=(nrows, ncols))


def assemble_vector(cell_rows, cellvecs, nrows):
    b = np.zeros(nrows)
    cell_rows = np.ascontiguousarray(cell_rows, np.int32)
    lib().orc_assemble_vector(cell_rows.shape[0], cell_rows.shape[1], _p(cell_rows),
                              _p(np.ascontiguousarray(cellvecs, np.float64)), _p(b))
    return b


def _csc_struct(colptr, rowval, nzval, n):
    s = _CSC()
    s.nrows = n
    s.ncols = n
    s.nnz = nzval.shape[0]
    s.colptr = colptr.ctypes.data_as(C.POINTER(C.c_int64))
    s.rowval = rowval.ctypes.data_as(C.POINTER(C.c_int64))
    s.nzval = nzval.ctypes.data_as(C.POINTER(C.c_double))
    return s


def pcg(colptr, rowval, nzval, b, rtol, maxit=100000, precond=1, nthreads=1):
    n = b.shape[0]
    s = _csc_struct(colptr, rowval, nzval, n)
    x = np.zeros(n)
    rr = np.zeros(1)
    it = lib().orc_pcg(C.byref(s), _p(np.ascontiguousarray(b)), _p(x), rtol, maxit, precond,
                       nthreads, _p(rr))
    return x, it, float(rr[0])


def csc_mul(colptr, rowval, nzval, x):
    n = colptr.shape[0] - 1
    s = _csc_struct(colptr, rowval, nzval, n)
    y = np.zeros(n)
    lib().orc_csc_mul(C.byref(s), _p(np.ascontiguousarray(x)), _p(y))
    return y


# ---- a whole Gridap-style problem ----------------------------------------------------------
def poisson_q1(domain, partition, dirichlet_tags=("boundary",), kappa=None, fkind=F_NONE,
               fdata=None, f_callable=None, degree=2, jitter=None, assemble=True):
    """Everything Gridap computes for  a = ∫ κ ∇v⋅∇u dΩ,  l = ∫ f v dΩ  on a Q1 space:
    returns a dict with model arrays, dofs, cell arrays, the CSC matrix (1-based) and b."""
    D = len(partition)
    coords, cells, ent = cartesian_model(domain, partition)
    geom = GEOM_CARTESIAN
    if jitter is not None:
        coords = jitter_interior(partition, coords, jitter)
        geom = GEOM_NODAL
    h = [(domain[2 * d + 1] - domain[2 * d]) / partition[d] for d in range(D)]
    ntt = node_tag_index(D, ent, list(dirichlet_tags))
    node_dof, cell_dofs, nfree, ndiri = clagrangian(ntt, cells)
    if f_callable is not None:
        xq = qpoints(D, cells, coords, degree)
        fkind = F_QPOINT
        fdata = np.asarray(f_callable(xq.reshape(-1, D)), np.float64).reshape(-1)
    mats, vecs = q1_cell_arrays(D, cells, coords, degree, geom, h, kappa, fkind, fdata)
    out = dict(coords=coords, cells=cells, node_entity=ent, node_to_tag=ntt, node_dof=node_dof,
               cell_dofs=cell_dofs, nfree=nfree, ndiri=ndiri, cellmats=mats, cellvecs=vecs)
    if assemble:
        out["csc"] = assemble_csc(cell_dofs, cell_dofs, mats, nfree, nfree)
        out["b"] = assemble_vector(cell_dofs, vecs, nfree)
    return out


# ---- simplexified boxes, P2 tets, elasticity ------------------------------------------------
def simplex_cells(partition):
    part = np.ascontiguousarray(partition, np.int64)
    tv = np.empty((int(np.prod(part)) * 6, 4), np.int32)
    lib().orc_simplex_cells(_p(part), _p(tv))
    return tv


def simplex_p2_numbering(partition, vertex_mask, ncomp=3, comp_mask=None):
    part = np.ascontiguousarray(partition, np.int64)
    vm = np.ascontiguousarray(vertex_mask, np.uint8)
    cm = np.ascontiguousarray(np.ones(ncomp) if comp_mask is None else comp_mask, np.uint8)
    cd = np.empty((int(np.prod(part)) * 6, 10 * ncomp), np.int32)
    nf = np.zeros(1, np.int32)
    nd = np.zeros(1, np.int32)
    lib().orc_simplex_p2_numbering(_p(part), ncomp, _p(vm), _p(cm), _p(cd), _p(nf), _p(nd))
    return cd, int(nf[0]), int(nd[0])


def p2tet_shapes(pts):
    pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
    phi = np.empty((pts.shape[0], 10))
    dphi = np.empty((pts.shape[0], 10, 3))
    lib().orc_p2tet_shapes(pts.shape[0], _p(pts), _p(phi), _p(dphi))
    return phi, dphi


def wv_tet_degree5():
    x = np.empty((14, 3))
    w = np.empty(14)
    res = lib().orc_wv_tet_degree5(_p(x), _p(w))
    return x, w, res


def elasticity_p2(domain, partition, lame, f=(0.0, 0.0, -1.0), clamp_x0=True, assemble=True):
    """Everything Gridap computes for a(u,v) = int eps(v) : (lambda tr eps(u) I + 2 mu eps(u)),
    l(v) = int f . v on vector P2 over simplexify(CartesianDiscreteModel(domain, partition))
    with the x = x0 face clamped (all components)."""
    part = np.asarray(partition, np.int64)
    coords, _, _ = cartesian_model(domain, partition)
    tv = simplex_cells(part)
    vmask = (np.abs(coords[:, 0] - domain[0]) < 1e-12) if clamp_x0 else np.zeros(len(coords), bool)
    cd, nfree, ndiri = simplex_p2_numbering(part, vmask)
    x, w, _ = wv_tet_degree5()
    lame = np.ascontiguousarray(lame, np.float64).reshape(-1)
    fv = np.ascontiguousarray(f, np.float64)
    nc = tv.shape[0]
    mats = np.empty((nc, 30, 30))  # filled col-major per cell
    vecs = np.empty((nc, 30))
    rc = lib().orc_p2tet_cell_arrays_elasticity(nc, _p(tv), _p(np.ascontiguousarray(coords)),
                                                _p(lame), 14, _p(x), _p(w), _p(fv), _p(mats),
                                                _p(vecs))
    if rc != 0:
        raise RuntimeError("degenerate tet")
    mats = np.ascontiguousarray(np.transpose(mats, (0, 2, 1)))  # col-major -> [c, i, j]
    out = dict(coords=coords, tet_vertices=tv, cell_dofs=cd, nfree=nfree, ndiri=ndiri,
               cellmats=mats, cellvecs=vecs, qx=x, qw=w)
    if assemble:
        out["csc"] = assemble_csc(cd, cd, mats, nfree, nfree)
        out["b"] = assemble_vector(cd, vecs, nfree)
    return out


def extrusion_faces(extrusion):
    """Faces of an extrusion polytope as 1-based vertex lists per dimension, by the
    generation and ordering rules of ReferenceFEs/ExtrusionPolytopes.jl:460-531
    (_polytopenfaces / _nfaceboundary!; HEX_AXIS = 1, TET_AXIS = 2)."""
    D = len(extrusion)

    def boundary(anchor, ext, extend, isanchor, lst):
        lst.append((anchor, ext))
        newext = extend
        for i in range(D):
            curex = newext[i]
            if curex > 0:
                newext = tuple(0 if j == i else newext[j] for j in range(D))
                edim = tuple(1 if j == i else 0 for j in range(D))
                tetp = tuple(anchor[j] if j >= i else 0 for j in range(D))
                if curex == 1:
                    boundary(tuple(a + e for a, e in zip(anchor, edim)), ext, newext, False, lst)
                elif isanchor:
                    boundary(tuple(a + e for a, e in zip(tetp, edim)), ext, newext, False, lst)
                boundary(anchor, tuple(x + e * curex for x, e in zip(ext, edim)), newext, False,
                         lst)
        return lst

    def nfaces(anchor, ext):
        lst = boundary(anchor, (0,) * D, ext, True, [])
        for i in range(D):
            lst.sort(key=lambda f: f[0][i])  # stable sorts, as Julia's sort!
        for i in range(D):
            lst.sort(key=lambda f: f[1][i])
        lst.sort(key=lambda f: sum(1 for x in f[1] if x))
        return lst

    dim = lambda f: sum(1 for x in f[1] if x)  # noqa: E731
    allf = nfaces((0,) * D, tuple(extrusion))
    ids = {f: k + 1 for k, f in enumerate(allf)}
    out = []
    for d in range(D + 1):
        out.append([[ids[s] for s in nfaces(f[0], f[1]) if dim(s) == 0]
                    for f in allf if dim(f) == d])
    return out


# ---- boundary (Neumann) terms --------------------------------------------------------------
def boundary_facets(partition, tags=None):
    """(owner cell, local facet) of the boundary facets of a Cartesian model selected by
    `tags` (None: every boundary facet), in Gridap's BoundaryTriangulation order.

    Facet ids come from the first-touch numbering of the grid topology: cells in order, the
    local faces of each cell in n-cube order, a new id for every face not met before
    (Geometry/GridTopologies.jl:1184-1240); a boundary facet has one cell around, so its id
    order is the (cell, local facet) order. BoundaryTriangulation keeps findall(mask), i.e.
    ascending ids (Geometry/BoundaryTriangulations.jl:174-203). The entity of a boundary
    facet is its local facet's position in the n-cube face list
    (Geometry/CartesianDiscreteModels.jl:215-240), and a tag selects the facets whose entity it
    lists. Normal axis and side are read off the n-cube faces: the axis the face does not
    extend along, and the anchor's coordinate on it."""
    D = len(partition)
    ext, anc = ncube_faces(D)
    fids = [k for k in range(ext.shape[0]) if int(ext[k].sum()) == D - 1]
    names, ents = cartesian_tags(D)
    if tags is None:
        sel = set(ents[names.index("boundary")])
    else:
        sel = set()
        for t in ([tags] if isinstance(tags, (str, int)) else tags):
            sel |= set(ents[t - 1] if isinstance(t, int) else ents[names.index(t)])
    axes = [(int(np.nonzero(ext[k] == 0)[0][0]), int(anc[k][np.nonzero(ext[k] == 0)[0][0]]))
            for k in fids]
    cells, lfaces = [], []
    nc = int(np.prod(partition))
    stride = [int(np.prod(partition[:d])) for d in range(D)]
    for c in range(nc):
        idx = [(c // stride[d]) % partition[d] for d in range(D)]
        for lf, k in enumerate(fids):
            ax, side = axes[lf]
            if idx[ax] == (0 if side == 0 else partition[ax] - 1) and (k + 1) in sel:
                cells.append(c)
                lfaces.append(lf)
    return np.array(cells, np.int32), np.array(lfaces, np.int32)


def facet_arrays(coords, cell_nodes, order, facet_cells, facet_lfaces, degree):
    """Per facet, at the Gauss points of the facet polytope (Quadrature(QUAD/SEGMENT,
    degree)): the owner cell's shape values phi (nq, nn), their outward normal derivatives
    dn (nq, nn), the integration factors w_q |J_q| (nq), the physical points (nq, D) and
    the unit normals (nq, D).

    The facet points are mapped into the owner cell through the facet's vertex list (the
    n-cube face-to-vertex table; the reference face map interpolates those vertices'
    reference coordinates). |J| = sqrt(det(JᵀJ)) with J the facet map's Jacobian from the
    facet's physical vertices. Gradients are pushed forward with the owner cell's Q1 map
    (∇φ = J_c⁻ᵀ ∇_ξ φ) and the normal is the unit vector orthogonal to the facet's tangents,
    pointing away from the cell's centre (get_facet_normal)."""
    D = coords.shape[1]
    fverts = extrusion_faces((1,) * D)[D - 1]
    refv = np.array([[(v >> d) & 1 for d in range(D)] for v in range(2 ** D)], np.float64)
    sx, sw = tensor_quadrature(D - 1, degree)
    sphi, sdphi = q1_shapes(D - 1, sx)
    out = []
    for f in range(facet_cells.shape[0]):
        c, lf = int(facet_cells[f]), int(facet_lfaces[f])
        vs = [v - 1 for v in fverts[lf]]
        cellpts = sphi @ refv[vs]
        Xc = coords[cell_nodes[c] - 1]  # owner cell vertices
        X = Xc[vs]
        xq = sphi @ X
        if order == 1:
            phi, dphi = q1_shapes(D, cellpts)
        else:
            phi, dphi = q2_shapes(D, cellpts)
        _, gdphi = q1_shapes(D, cellpts)  # geometry map
        centre = Xc.mean(axis=0)
        dn = np.zeros_like(phi)
        wm = np.zeros(sw.shape[0])
        nrm = np.zeros((sw.shape[0], D))
        for q in range(sw.shape[0]):
            T = sdphi[q].T @ X  # (D-1, D) tangents
            wm[q] = sw[q] * math.sqrt(np.linalg.det(T @ T.T))
            if D == 2:
                n = np.array([T[0, 1], -T[0, 0]])
            else:
                n = np.cross(T[0], T[1])
            n /= np.linalg.norm(n)
            if np.dot(n, xq[q] - centre) < 0:
                n = -n
            nrm[q] = n
            Jc = gdphi[q].T @ Xc  # (D, D): Jc[k, l] = d x_l / d xi_k
            grad = np.linalg.solve(Jc, dphi[q].T)  # (D, nn) physical gradients
            dn[q] = n @ grad
        out.append((phi, dn, wm, xq, nrm))
    return out


def boundary_vector(partition, coords, cell_nodes, cell_dofs, order, facet_cells,
                    facet_lfaces, degree, g, nfree, test_op=0):
    """Gridap's assemble_vector of ∫ g v dΓ (test_op 0) or ∫ g (n⋅∇v) dΓ (test_op 1) on a
    BoundaryTriangulation: the facet vector r_i = Σ_q g_q op(φ_i)(q) w_q |J_q| in the order of
    Fields/FieldsInterfaces.jl:660-670, added with the owner cell's dof ids in facet order
    (FESpaces/SparseMatrixAssemblers.jl:287-316). g: a number or a callable on physical
    points (npoints, D); returns (b, g values at the points, facet by facet)."""
    arrs = facet_arrays(coords, cell_nodes, order, facet_cells, facet_lfaces, degree)
    nf = facet_cells.shape[0]
    vecs = np.zeros((nf, cell_dofs.shape[1]))
    nq = arrs[0][2].shape[0] if nf else 0
    gvals = np.zeros((nf, nq))
    for f, (phi, dn, wm, xq, _) in enumerate(arrs):
        op = phi if test_op == 0 else dn
        gq = (np.full(nq, float(g)) if not callable(g)
              else np.asarray(g(xq), np.float64).reshape(-1))
        gvals[f] = gq
        for q in range(nq):
            for i in range(op.shape[1]):
                vecs[f, i] += gq[q] * op[q, i] * wm[q]
    b = assemble_vector(cell_dofs[facet_cells], vecs, nfree)
    return b, gvals


def boundary_matrix(coords, cell_nodes, cell_dofs, order, facet_cells, facet_lfaces, degree,
                    coefs, nfree, uD=None):
    """Dense sum of the facet matrices of ∫ c0 v u + c1 v (n⋅∇u) + c2 (n⋅∇v) u
    + c3 (n⋅∇v)(n⋅∇u) dΓ over the free rows and columns, and the Dirichlet lift
    -Σ_j M_ij u_D_j of the Dirichlet columns (AttachDirichletMap, CellData/AttachDirichlet.jl)."""
    arrs = facet_arrays(coords, cell_nodes, order, facet_cells, facet_lfaces, degree)
    K = np.zeros((nfree, nfree))
    lift = np.zeros(nfree)
    c0, c1, c2, c3 = coefs
    for f, (phi, dn, wm, _, _) in enumerate(arrs):
        M = np.zeros((phi.shape[1], phi.shape[1]))
        for q in range(wm.shape[0]):
            M += (c0 * np.outer(phi[q], phi[q]) + c1 * np.outer(phi[q], dn[q])
                  + c2 * np.outer(dn[q], phi[q]) + c3 * np.outer(dn[q], dn[q])) * wm[q]
        ids = cell_dofs[facet_cells[f]]
        for i, r in enumerate(ids):
            if r <= 0:
                continue
            for j, s in enumerate(ids):
                if s > 0:
                    K[r - 1, s - 1] += M[i, j]
                elif uD is not None:
                    lift[r - 1] -= M[i, j] * uD[-s - 1]
    return K, lift


def dirichlet_lift(cell_dofs, cellmats, uD, nfree):
    """-Σ_j K_ij u_D_j over every cell's Dirichlet columns, added by row (the vector part of
    AttachDirichletMap, CellData/AttachDirichlet.jl:59-110). cellmats[c][i][j]: i test row."""
    b = np.zeros(nfree)
    for c in range(cell_dofs.shape[0]):
        ids = cell_dofs[c]
        neg = ids < 0
        if not neg.any():
            continue
        lv = -(cellmats[c][:, neg] @ uD[-ids[neg] - 1])
        for i, r in enumerate(ids):
            if r > 0:
                b[r - 1] += lv[i]
    return b


# ---- quasilinear diffusion (nonlinear FEOperator) --------------------------------------------
LAW_POLY, LAW_POWER = 0, 1


def quasilinear_cell_arrays(coords, cell_nodes, cell_dofs, order, degree, state, uD, law,
                            params, kappa=None, f=None):
    """Cell residuals and Jacobians of  r(u; v) = ∫ κ α(u, ∇u) ∇u⋅∇v - f v  at the FE function
    u (free values `state`, Dirichlet values `uD`), by Gridap's per-point evaluation of
    res(uh, v) and jac(uh, du, v) (CellData/CellQuadratures.jl:138-170): geometry from the cell's
    Q1 map, ∇φ = J⁻ᵀ ∇ξφ, u_q = Σ u_i φ_i, ∇u_q = Σ u_i ∇φ_i, then
      r_i  += κ α ∇u⋅∇φ_i dV - f φ_i dV,
      J_ij += κ (α ∇φ_j⋅∇φ_i + α_u φ_j ∇u⋅∇φ_i + γ (∇u⋅∇φ_j)(∇u⋅∇φ_i)) dV
    with the laws POLY α = c0 + c1 u + c2 u² (α_u = c1 + 2 c2 u, γ = 0) and POWER
    α = (e + |∇u|²)^((p-2)/2), γ = (p-2)(e + |∇u|²)^((p-4)/2) (params p, e): the derivative of
    the p-Laplacian flux (test/GridapTests/PLaplacianTests.jl dflux). f: a number or a
    callable of the points. Returns (mats [c, i, j] (i test), vecs)."""
    D = coords.shape[1]
    qx, qw = tensor_quadrature(D, degree)
    phi1, dphi1 = q1_shapes(D, qx)
    phi, dref = (phi1, dphi1) if order == 1 else q2_shapes(D, qx)
    nc, nn = cell_dofs.shape
    mats = np.zeros((nc, nn, nn))
    vecs = np.zeros((nc, nn))
    for c in range(nc):
        X = coords[cell_nodes[c] - 1]
        ids = cell_dofs[c]
        uc = np.array([state[i - 1] if i > 0 else (uD[-i - 1] if uD is not None else 0.0)
                       for i in ids])
        kap = 1.0 if kappa is None else (float(kappa) if np.ndim(kappa) == 0 else kappa[c])
        for q in range(qw.shape[0]):
            Jt = dphi1[q].T @ X
            dV = qw[q] * abs(np.linalg.det(Jt))
            g = np.linalg.solve(Jt, dref[q].T).T  # (nn, D)
            u = phi[q] @ uc
            gu = g.T @ uc
            n2 = gu @ gu
            if law == LAW_POLY:
                c0, c1, c2 = params[:3]
                al, be, ga = c0 + c1 * u + c2 * u * u, c1 + 2 * c2 * u, 0.0
            else:
                p, e = params[:2]
                al, be, ga = (e + n2) ** ((p - 2) / 2), 0.0, (p - 2) * (e + n2) ** ((p - 4) / 2)
            xq = phi1[q] @ X
            fq = 0.0 if f is None else (float(f(xq[None, :])[0]) if callable(f) else float(f))
            a = g @ gu
            vecs[c] += kap * al * a * dV - fq * phi[q] * dV
            mats[c] += kap * (al * (g @ g.T) + be * np.outer(a, phi[q])
                              + ga * np.outer(a, a)) * dV
    return mats, vecs


# ---- free-dof reordering ---------------------------------------------------------------------
def compute_adjacency(cell_dofs, nfree):
    """Gridap's compute_adjacency: (ptrs (nfree+1), data), 1-based like its Table."""
    cd = np.ascontiguousarray(cell_dofs, np.int32)
    pp = C.POINTER(C.c_int64)()
    dp = C.POINTER(C.c_int32)()
    L = lib()
    if L.orc_compute_adjacency(C.c_int64(cd.shape[0]), cd.shape[1], _p(cd), C.c_int64(nfree),
                               C.byref(pp), C.byref(dp)) != 0:
        raise MemoryError("oracle adjacency")
    ptrs = np.ctypeslib.as_array(pp, (nfree + 1,)).copy()
    nnz = int(ptrs[-1] - 1)
    data = np.ctypeslib.as_array(dp, (max(nnz, 1),))[:nnz].copy()
    L.orc_free(C.cast(pp, C.c_void_p))
    L.orc_free(C.cast(dp, C.c_void_p))
    return ptrs, data


def dof_permutation(cell_dofs, nfree, algorithm="rcm", w1=1, w2=2, coords=None):
    """compute_dof_permutation (FESpaceReindexing.jl:264-300): iperm[old-1] = new (1-based).
    'coordinates' sorts the free dofs' points lexicographically (stable sortperm by Tuple)."""
    if algorithm == "coordinates":
        X = np.asarray(coords, np.float64)
        order = np.lexsort(tuple(X[:, d] for d in range(X.shape[1] - 1, -1, -1)))
        iperm = np.empty(nfree, np.int64)
        iperm[order] = np.arange(1, nfree + 1)
        return iperm
    ptrs, data = compute_adjacency(cell_dofs, nfree)
    iperm = np.empty(nfree, np.int64)
    L = lib()
    if algorithm == "rcm":
        st = L.orc_rcm_perm(C.c_int64(nfree), _p(ptrs), _p(data), _p(iperm))
    elif algorithm == "sloan":
        st = L.orc_sloan_perm(C.c_int64(nfree), _p(ptrs), _p(data), C.c_int64(w1),
                              C.c_int64(w2), _p(iperm))
    else:
        raise ValueError(algorithm)
    if st != 0:
        raise MemoryError("oracle permutation")
    return iperm


def reindex_cell_dofs(cell_dofs, iperm):
    """PosNegReindex of free ids (Dirichlet ids unchanged)."""
    cd = np.asarray(cell_dofs)
    out = cd.copy()
    m = cd > 0
    out[m] = iperm[cd[m] - 1]
    return out.astype(np.int32)


# ---- multi-field cell arrays (MultiFieldFESpace, Stokes-like forms) ------------------------
MOP_VALUE, MOP_GRAD, MOP_DIV = 0, 1, 2


def _mf_operand(op, ncomp, phi, P, D):
    """Dense operand of every local basis function at every point: phi (nq, nn) values and
    P (nc, nq, nn, D) physical gradients -> (nc, nq, nd) + shape, with nd = ncomp * nn and
    local dof l = comp * nn + node (component-major, as Gridap's vector Lagrangian reffes).
    value: phi (scalar) or e_c phi; grad: grad phi or e_c (x) grad phi (row c of the D x D
    gradient, Fields/DiffOperators.jl); div = tr(grad) (DiffOperators.jl:7)."""
    nc, nq, nn, _ = P.shape
    if ncomp == 1:
        if op == MOP_VALUE:
            return np.broadcast_to(phi[None], (nc, nq, nn))
        if op == MOP_GRAD:
            return P
        raise ValueError("div of a scalar field")
    nd = ncomp * nn
    if op == MOP_VALUE:
        out = np.zeros((nc, nq, nd, D))
        for c in range(D):
            out[:, :, c * nn:(c + 1) * nn, c] = phi[None]
        return out
    if op == MOP_GRAD:
        out = np.zeros((nc, nq, nd, D, D))
        for c in range(D):
            out[:, :, c * nn:(c + 1) * nn, c, :] = P
        return out
    out = np.zeros((nc, nq, nd))
    for c in range(D):
        out[:, :, c * nn:(c + 1) * nn] = P[..., c]
    return out


def multifield_cell_arrays(D, coords, cell_nodes, fields, terms, degree):
    """Cell matrices per field pair and cell vectors per field of a multi-field form, by
    Gridap's per-point evaluation (CellData/CellQuadratures.jl:138-170: sum over the
    tensor Gauss points of integrand(x_q) w_q |det J_q|, J from the cell's Q1 map,
    grad = J^-T grad_xi) of each product term (MultiField/MultiFieldCellFields.jl: one block
    per (test field, trial field)), the operands contracted fully (inner / ⊙,
    TensorValues/Operations.jl).
    fields: [(order, ncomp)]; terms: [(test_field, test_op, trial_field or None, trial_op,
    coef, cell_coef or None, qdata or None (ncells, nq, k))]. Returns (K, F): K[(i, j)] of
    shape (ncells, nd_i, nd_j) [c, row, col] and F[i] (ncells, nd_i)."""
    qx, qw = tensor_quadrature(D, degree)
    phi1, g1 = q1_shapes(D, qx)
    X = coords[cell_nodes - 1]                             # (nc, 2^D, D)
    J = np.einsum("cad,qae->cqde", X, g1)                  # dx_d / dxi_e
    det = np.linalg.det(J)
    if np.any(det <= 0):
        raise RuntimeError("oracle: degenerate cell")
    JinvT = np.linalg.inv(J).transpose(0, 1, 3, 2)
    dV = det * qw[None, :]                                 # (nc, nq)
    tabs = []
    for order, ncomp in fields:
        phi, dphi = (q1_shapes(D, qx) if order == 1 else q2_shapes(D, qx))
        P = np.einsum("cqde,qne->cqnd", JinvT, dphi)
        tabs.append((phi, P, ncomp))
    nc = cell_nodes.shape[0]
    K, F = {}, {}
    for tf, top, uf, uop, coef, cell_coef, qdata in terms:
        phi_t, P_t, nc_t = tabs[tf]
        Tt = _mf_operand(top, nc_t, phi_t, P_t, D)
        w = dV * coef * (1.0 if cell_coef is None else np.asarray(cell_coef)[:, None])
        nq, nd = Tt.shape[1], Tt.shape[2]
        Ts = Tt.reshape(nc, nq, nd, -1)  # trailing operand dims flattened: the contraction
        if uf is None:
            f = (np.ones((nc, nq, 1)) if qdata is None
                 else np.asarray(qdata).reshape(nc, nq, -1))
            if f.shape[2] != Ts.shape[3]:
                raise ValueError("data of another shape than the test operand")
            val = np.einsum("cq,cqls,cqs->cl", w, Ts, f)
            F[tf] = F.get(tf, 0.0) + val
            continue
        phi_u, P_u, nc_u = tabs[uf]
        Tu = _mf_operand(uop, nc_u, phi_u, P_u, D)
        if Tt.shape[3:] != Tu.shape[3:]:
            raise ValueError("operands of different shapes")
        Us = Tu.reshape(nc, nq, Tu.shape[2], -1)
        val = np.einsum("cq,cqis,cqjs->cij", w, Ts, Us)
        K[(tf, uf)] = K.get((tf, uf), 0.0) + val
    return K, F


def multifield_assemble(cell_ids, nfree_fields, K, F, uD_fields, rows_of=None):
    """Gridap's monolithic assembly of a consecutive multi-field system: cell ids per field
    (free ids already offset, Dirichlet ids field-local), K/F from multifield_cell_arrays,
    Dirichlet values per field. The matrix is the sum of the per-block assemblies (each
    (row, col) entry belongs to one field pair, whose contributions arrive in cell order);
    the vector is sum over cells of F_c - K_c u_D,c (AttachDirichletMap,
    CellData/AttachDirichlet.jl:59-110). Returns (scipy CSR of the matrix, b)."""
    import scipy.sparse as sp
    n = sum(nfree_fields)
    nf = len(cell_ids)
    # the blocks' entries are disjoint: their triplets side by side (a sparse sum would drop
    # the structural zeros, e.g. the cross-component entries of a vector field's block)
    rr, cc, vv = [], [], []
    for (i, j), Kij in K.items():
        cp, rv, nz = assemble_csc(cell_ids[i], cell_ids[j], Kij, n, n)
        rr.append(rv - 1)
        cc.append(np.repeat(np.arange(n), np.diff(cp)))
        vv.append(nz)
    A = sp.coo_matrix((np.concatenate(vv), (np.concatenate(rr), np.concatenate(cc))),
                      shape=(n, n)).tocsr()
    nc = cell_ids[0].shape[0]
    rows = np.concatenate(cell_ids, axis=1)
    vec = np.zeros((nc, rows.shape[1]))
    starts = np.concatenate([[0], np.cumsum([c.shape[1] for c in cell_ids])])
    for i in range(nf):
        if i in F:
            vec[:, starts[i]:starts[i + 1]] += F[i]
    for i in range(nf):
        lift = np.zeros((nc, cell_ids[i].shape[1]))
        for j in range(nf):
            if (i, j) not in K or uD_fields[j] is None:
                continue
            ids = cell_ids[j]
            u = np.where(ids < 0, np.asarray(uD_fields[j])[np.maximum(-ids, 1) - 1], 0.0)
            lift += np.einsum("cij,cj->ci", K[(i, j)], u)
        vec[:, starts[i]:starts[i + 1]] -= lift
    b = assemble_vector(rows, vec, n)
    A.sort_indices()
    return A, b
