"""FE spaces: reference FEs, dof numbering and FE functions, mirroring Gridap's
`FESpace(model, ReferenceFE(lagrangian, T, order); dirichlet_tags)` for the Lagrangian
spaces the device kernels integrate.

Q1 spaces on linear grids use the CLagrangian numbering (FESpaces/CLagrangianFESpaces.jl:
155-380): free dofs are the untagged (or unmasked) nodes in node order, Dirichlet dofs get
-1, -2, ... in node order, vector fields are node-major with interleaved components.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .geometry import CartesianDiscreteModel, SimplexDiscreteModel

lagrangian = "lagrangian"


class ReferenceFE:
    """ReferenceFE(lagrangian, T, order); T is float (scalar) or an int number of components."""

    def __init__(self, kind: str, T=float, order: int = 1):
        if kind != lagrangian:
            raise NotImplementedError(f"reference FE {kind!r}")
        self.kind = kind
        self.ncomp = 1 if T in (float, np.float64) else int(T)
        self.order = int(order)


class FESpace:
    def __init__(self, model: CartesianDiscreteModel, reffe: ReferenceFE, dirichlet_tags=(),
                 dirichlet_masks=None):
        if reffe.order not in (1, 2):
            raise NotImplementedError("Lagrangian spaces of order 1 and 2 are provided")
        lib = _lib.load()
        self.model = model
        self.reffe = reffe
        if isinstance(dirichlet_tags, (str, int)):
            dirichlet_tags = [dirichlet_tags]
        self.dirichlet_tags = list(dirichlet_tags)
        nc = reffe.ncomp
        if isinstance(model, SimplexDiscreteModel):
            self._simplex_p2(lib, dirichlet_masks)
            return
        if reffe.order == 2:
            self._conforming(lib, dirichlet_masks)
            return
        node_to_tag = model.get_face_labeling().get_face_tag_index(self.dirichlet_tags, 0)
        ntags = max(len(self.dirichlet_tags), 1)
        if dirichlet_masks is None:
            masks = np.ones((ntags, nc), dtype=np.uint8)
        else:
            masks = np.asarray(dirichlet_masks, dtype=np.uint8).reshape(len(self.dirichlet_tags), nc)
        nv = 2 ** model.dim
        # local dof of (local node, comp): component-major inside the cell
        lmap = np.array([[c * nv + a + 1 for c in range(nc)] for a in range(nv)], dtype=np.int32)
        self.node_comp_to_dof = np.empty((model.num_nodes(), nc), dtype=np.int32)
        self.cell_dof_ids = np.empty((model.num_cells(), nv * nc), dtype=np.int32)
        nfree = np.zeros(1, dtype=np.int32)
        ndiri = np.zeros(1, dtype=np.int32)
        _lib.check(lib.gfe_clagrangian_dofs(
            model.num_nodes(), _lib.ptr(node_to_tag), nc, _lib.ptr(np.ascontiguousarray(masks)),
            model.num_cells(), nv, _lib.ptr(model.cell_node_ids), _lib.ptr(lmap),
            _lib.ptr(self.node_comp_to_dof), _lib.ptr(self.cell_dof_ids), _lib.ptr(nfree),
            _lib.ptr(ndiri)))
        self.nfree = int(nfree[0])
        self.ndiri = int(ndiri[0])

    def _conforming(self, lib, dirichlet_masks):
        """Q2 numbering (ConformingFESpaces.jl:367-636) through gfe_cartesian_conforming_dofs."""
        model, nc = self.model, self.reffe.ncomp
        labels = model.get_face_labeling()
        D = model.dim
        ntags = max(len(self.dirichlet_tags), 1)
        ent_to_tag = np.zeros(3 ** D, dtype=np.int8)
        for e in range(1, 3 ** D + 1):
            for k, t in enumerate(self.dirichlet_tags):
                if e in labels.tag_entities[labels._tag_index(t)]:
                    ent_to_tag[e - 1] = k + 1
                    break
        if dirichlet_masks is None:
            masks = np.ones((ntags, nc), dtype=np.uint8)
        else:
            masks = np.asarray(dirichlet_masks, dtype=np.uint8).reshape(len(self.dirichlet_tags), nc)
        part = np.asarray(model.partition, dtype=np.int64)
        self.cell_dof_ids = np.empty((model.num_cells(), 3 ** D * nc), dtype=np.int32)
        nfree = np.zeros(1, dtype=np.int32)
        ndiri = np.zeros(1, dtype=np.int32)
        _lib.check(lib.gfe_cartesian_conforming_dofs(
            D, 2, _lib.ptr(part), nc, _lib.ptr(ent_to_tag), _lib.ptr(np.ascontiguousarray(masks)),
            _lib.ptr(self.cell_dof_ids), _lib.ptr(nfree), _lib.ptr(ndiri)))
        self.nfree = int(nfree[0])
        self.ndiri = int(ndiri[0])
        self.node_comp_to_dof = None

    def _simplex_p2(self, lib, dirichlet_masks):
        """P2 on a simplexified box (ConformingFESpaces.jl:367-636) via gfe_simplex_p2_dofs.
        dirichlet_tags name vertex-filter tags of the model; with several tags they must share
        one component mask."""
        model, nc = self.model, self.reffe.ncomp
        if self.reffe.order != 2:
            raise NotImplementedError("simplexified models carry P2 spaces")
        vmask = np.zeros(model.num_nodes(), dtype=np.uint8)
        for t in self.dirichlet_tags:
            if t not in model.vertex_tags:
                raise ValueError(f"unknown tag {t!r} (add it with add_tag_from_vertex_filter)")
            vmask |= model.vertex_tags[t].astype(np.uint8)
        if dirichlet_masks is None:
            cmask = np.ones(nc, dtype=np.uint8)
        else:
            m = np.asarray(dirichlet_masks, dtype=np.uint8).reshape(-1, nc)
            if (m != m[0]).any():
                raise NotImplementedError("one component mask for all Dirichlet tags")
            cmask = np.ascontiguousarray(m[0])
        part = np.asarray(model.partition, dtype=np.int64)
        self.cell_dof_ids = np.empty((model.num_cells(), 10 * nc), dtype=np.int32)
        nfree = np.zeros(1, dtype=np.int32)
        ndiri = np.zeros(1, dtype=np.int32)
        _lib.check(lib.gfe_simplex_p2_dofs(_lib.ptr(part), nc, _lib.ptr(vmask), _lib.ptr(cmask),
                                           _lib.ptr(self.cell_dof_ids), _lib.ptr(nfree),
                                           _lib.ptr(ndiri)))
        self.nfree = int(nfree[0])
        self.ndiri = int(ndiri[0])
        self.node_comp_to_dof = None

    def num_free_dofs(self) -> int:
        return self.nfree

    def dof_points(self):
        """Physical node of every dof and its component: (free_x, free_comp, diri_x, diri_comp),
        the node positions mapped through each cell's geometry (the Q1 map of a hexahedron, the
        affine map of a tet), as Lagrangian dof values are point evaluations there."""
        model, nc = self.model, self.reffe.ncomp
        D = model.dim
        X = model.node_coords[model.cell_node_ids - 1]  # (ncells, nverts, D)
        if isinstance(model, SimplexDiscreteModel):
            lam = np.zeros((10, 4))
            lam[np.arange(4), np.arange(4)] = 1.0
            for k, (i, j) in enumerate(((0, 1), (0, 2), (1, 2), (0, 3), (1, 3), (2, 3))):
                lam[4 + k, [i, j]] = 0.5
            P = np.einsum("na,cad->cnd", lam, X)
        else:
            ref = ncube_node_refs(D, self.reffe.order)
            nv = 2 ** D
            phi = np.ones((ref.shape[0], nv))
            for a in range(nv):
                for d in range(D):
                    phi[:, a] *= ref[:, d] if (a >> d) & 1 else 1 - ref[:, d]
            P = np.einsum("na,cad->cnd", phi, X)
        nn = P.shape[1]
        ids = self.cell_dof_ids
        comp = np.broadcast_to(np.arange(ids.shape[1]) // nn, ids.shape)
        node = np.arange(ids.shape[1]) % nn
        pts = P[:, node, :]  # (ncells, nd, D)
        fx, fc = np.zeros((self.nfree, D)), np.zeros(self.nfree, np.int32)
        dx, dc = np.zeros((self.ndiri, D)), np.zeros(self.ndiri, np.int32)
        f = ids > 0
        fx[ids[f] - 1], fc[ids[f] - 1] = pts[f], comp[f]
        d = ids < 0
        dx[-ids[d] - 1], dc[-ids[d] - 1] = pts[d], comp[d]
        return fx, fc, dx, dc

    def num_dirichlet_dofs(self) -> int:
        return self.ndiri

    def get_cell_dof_ids(self) -> np.ndarray:
        return self.cell_dof_ids

    def ndofs_per_cell(self) -> int:
        return self.cell_dof_ids.shape[1]


def ncube_node_refs(D: int, order: int) -> np.ndarray:
    """Reference coordinates of the Lagrangian nodes of the D-cube: order 1, the vertices
    (coordinate bit d of vertex a is (a >> d) & 1); order 2, one node at the centre of every
    n-cube face in Gridap's face order (ReferenceFEs/ExtrusionPolytopes.jl:460-531): faces
    by dimension, within one dimension by extrusion pattern with the first axis as the most
    significant bit, descending, then by anchor over the fixed axes, the first fastest."""
    if order == 1:
        return np.array([[(a >> d) & 1 for d in range(D)] for a in range(2 ** D)], np.float64)
    out = []
    for k in range(D + 1):
        exts = [e for e in range(2 ** D) if bin(e).count("1") == k]
        # e encodes the extrusion with axis 0 as the most significant bit
        for e in sorted(exts, reverse=True):
            span = [(e >> (D - 1 - d)) & 1 for d in range(D)]
            fixed = [d for d in range(D) if not span[d]]
            for a in range(2 ** len(fixed)):
                x = [0.5 if span[d] else 0.0 for d in range(D)]
                for i, d in enumerate(fixed):
                    x[d] = float((a >> i) & 1)
                out.append(x)
    return np.array(out, np.float64)


def _eval_data(u_D, x: np.ndarray, comp: np.ndarray) -> np.ndarray:
    """u_D at the points x (n, D), component comp of each: u_D is a number, a sequence with
    one constant per component, or a callable of the points (vectorised over rows, or of one
    point) returning one value (scalar field) or one value per component."""
    if callable(u_D):
        try:
            vals = np.asarray(u_D(x), np.float64)
            if vals.ndim == 0 or vals.shape[0] != x.shape[0]:
                raise ValueError
        except (TypeError, IndexError, ValueError):
            vals = np.array([np.asarray(u_D(xi), np.float64) for xi in x])
        if vals.ndim == 1:
            return vals
        return vals[np.arange(x.shape[0]), comp]
    vals = np.asarray(u_D, np.float64)
    if vals.ndim == 0:
        return np.full(x.shape[0], float(vals))
    return vals[comp]


class TrialFESpace:
    """TrialFESpace(V, u_D): V with Dirichlet values u_D (a number, a per-component
    sequence, or a callable of x) interpolated at the Dirichlet dofs' nodes
    (FESpaces/TrialFESpaces.jl, interpolate_dirichlet). The assembly of a(u,v), l(v) then
    lifts them into the right-hand side (b -= A_free,D u_D cell by cell)."""

    def __init__(self, V: FESpace, u_D=0.0):
        self.space = V
        self.u_D = u_D
        homogeneous = not callable(u_D) and not np.any(np.asarray(u_D, np.float64))
        self.dirichlet_values = None
        if not homogeneous and V.num_dirichlet_dofs() > 0:
            _, _, dx, dc = V.dof_points()
            self.dirichlet_values = np.ascontiguousarray(_eval_data(u_D, dx, dc))

    def __getattr__(self, k):
        return getattr(self.space, k)

    def get_dirichlet_dof_values(self) -> np.ndarray:
        if self.dirichlet_values is None:
            return np.zeros(self.space.num_dirichlet_dofs())
        return self.dirichlet_values


def _space(S):
    return S.space if isinstance(S, TrialFESpace) else S


class FEFunction:
    """FEFunction(U, free_values): free values plus the trial space's Dirichlet values
    (zero for a test space or homogeneous data)."""

    def __init__(self, U, free_values):
        self.space = _space(U)
        self.free_values = free_values
        self.dirichlet_values = (U.get_dirichlet_dof_values() if isinstance(U, TrialFESpace)
                                 else np.zeros(self.space.num_dirichlet_dofs()))

    def get_free_dof_values(self):
        return self.free_values

    def get_dirichlet_dof_values(self) -> np.ndarray:
        return self.dirichlet_values

    def dof_values(self, ids) -> np.ndarray:
        """Values of the dofs with Gridap ids (positive free, negative Dirichlet)."""
        fv = np.asarray(self.free_values.cpu() if hasattr(self.free_values, "cpu")
                        else self.free_values)
        ids = np.asarray(ids)
        return np.where(ids > 0, fv[np.maximum(ids, 1) - 1],
                        self.dirichlet_values[np.maximum(-ids, 1) - 1]
                        if self.dirichlet_values.size else 0.0)

    def nodal_values(self) -> np.ndarray:
        """Values at every mesh node (scalar Q1 spaces)."""
        return self.dof_values(self.space.node_comp_to_dof[:, 0])


def get_cell_dof_ids(V):
    return _space(V).get_cell_dof_ids()


def num_free_dofs(V) -> int:
    return _space(V).num_free_dofs()
