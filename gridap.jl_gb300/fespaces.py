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

    def num_dirichlet_dofs(self) -> int:
        return self.ndiri

    def get_cell_dof_ids(self) -> np.ndarray:
        return self.cell_dof_ids

    def ndofs_per_cell(self) -> int:
        return self.cell_dof_ids.shape[1]


class TrialFESpace:
    """TrialFESpace(V) with homogeneous Dirichlet values (u_D = 0)."""

    def __init__(self, V: FESpace, u_D=0.0):
        if u_D != 0.0:
            raise NotImplementedError("only homogeneous Dirichlet data is provided")
        self.space = V

    def __getattr__(self, k):
        return getattr(self.space, k)


def _space(S):
    return S.space if isinstance(S, TrialFESpace) else S


class FEFunction:
    """FEFunction(U, free_values): free values plus zero Dirichlet values."""

    def __init__(self, U, free_values):
        self.space = _space(U)
        self.free_values = free_values

    def get_free_dof_values(self):
        return self.free_values

    def nodal_values(self) -> np.ndarray:
        """Values at every mesh node (scalar spaces), Dirichlet nodes at 0."""
        fv = np.asarray(self.free_values.cpu() if hasattr(self.free_values, "cpu")
                        else self.free_values)
        d = self.space.node_comp_to_dof[:, 0]
        out = np.zeros(d.shape[0])
        m = d > 0
        out[m] = fv[d[m] - 1]
        return out


def get_cell_dof_ids(V):
    return _space(V).get_cell_dof_ids()


def num_free_dofs(V) -> int:
    return _space(V).num_free_dofs()
