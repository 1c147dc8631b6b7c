"""Discrete models, face labels, triangulations and measures (the host-side set-up that
fixes node and cell numbering), mirroring Gridap's Geometry / CellData constructors.

Cartesian models follow Geometry/CartesianGrids.jl:108-171 and
Geometry/CartesianDiscreteModels.jl:133-189; the arrays are produced by libgfe
(`gfe_cartesian_model`).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib


class FaceLabeling:
    """Vertex labels of a Cartesian model: the box entity (n-cube face id) of every node and
    the tags Gridap defines on top of them: "tag_<id>" for each boundary entity (zero padded
    to the width of the interior id), "interior", and "boundary" (all boundary entities).
    Integer tags are 1-based positions in that tag list, as in Gridap."""

    def __init__(self, dim: int, node_entity: np.ndarray):
        self.dim = dim
        self.node_entity = node_entity
        nfaces = 3 ** dim
        interior = nfaces
        width = math.ceil(math.log10(interior))
        self.tag_names: list[str] = []
        self.tag_entities: list[list[int]] = []
        for i in range(1, interior):
            self.tag_names.append(f"tag_{str(i).zfill(width)}")
            self.tag_entities.append([i])
        self.tag_names.append("interior")
        self.tag_entities.append([interior])
        self.tag_names.append("boundary")
        self.tag_entities.append(list(range(1, interior)))

    def _tag_index(self, tag) -> int:
        if isinstance(tag, (int, np.integer)):
            if not 1 <= tag <= len(self.tag_names):
                raise ValueError(f"unknown tag {tag}")
            return int(tag) - 1
        if tag in self.tag_names:
            return self.tag_names.index(tag)
        raise ValueError(f"unknown tag {tag!r}")

    def get_face_tag_index(self, tags, d: int = 0) -> np.ndarray:
        """FaceLabelings.jl:411-427 for vertices: the 1-based position in `tags` of the first
        tag containing each node's entity, 0 if none."""
        if d != 0:
            raise NotImplementedError("only vertex labels are provided")
        if isinstance(tags, (str, int, np.integer)):
            tags = [tags]
        out = np.zeros(self.node_entity.shape[0], dtype=np.int8)
        unset = np.ones_like(out, dtype=bool)
        for k, t in enumerate(tags):
            ents = self.tag_entities[self._tag_index(t)]
            hit = unset & np.isin(self.node_entity, ents)
            out[hit] = k + 1
            unset &= ~hit
        return out


class CartesianDiscreteModel:
    """CartesianDiscreteModel(domain, partition). `node_jitter` (nnodes x D) displaces the
    nodes that are not on the domain boundary, which turns the model into one with general
    (distorted) cells: Jacobians are then computed from node coordinates per quadrature point."""

    def __init__(self, domain, partition, node_jitter: np.ndarray | None = None):
        lib = _lib.load()
        self.partition = tuple(int(n) for n in partition)
        self.dim = D = len(self.partition)
        if len(domain) != 2 * D:
            raise ValueError("domain must have 2*D entries")
        self.domain = tuple(float(x) for x in domain)
        part = np.asarray(self.partition, dtype=np.int64)
        dom = np.asarray(self.domain, dtype=np.float64)
        nn = int(np.prod(part + 1))
        nc = int(np.prod(part))
        coords = np.empty((nn, D), dtype=np.float64)
        cells = np.empty((nc, 2 ** D), dtype=np.int32)
        ent = np.empty(nn, dtype=np.int32)
        _lib.check(lib.gfe_cartesian_model(D, _lib.ptr(part), _lib.ptr(dom), _lib.ptr(coords),
                                           _lib.ptr(cells), _lib.ptr(ent)))
        self.node_coords = coords
        self.cell_node_ids = cells
        self.labels = FaceLabeling(D, ent)
        self.cartesian = node_jitter is None
        if node_jitter is not None:
            jit = np.asarray(node_jitter, dtype=np.float64).reshape(nn, D)
            interior = self.labels.node_entity == 3 ** D
            self.node_coords = coords + np.where(interior[:, None], jit, 0.0)

    def num_cells(self) -> int:
        return self.cell_node_ids.shape[0]

    def num_nodes(self) -> int:
        return self.node_coords.shape[0]

    def get_node_coordinates(self) -> np.ndarray:
        return self.node_coords

    def get_cell_node_ids(self) -> np.ndarray:
        return self.cell_node_ids

    def get_face_labeling(self) -> FaceLabeling:
        return self.labels

    def cell_sizes(self) -> tuple[float, ...]:
        return tuple((self.domain[2 * d + 1] - self.domain[2 * d]) / self.partition[d]
                     for d in range(self.dim))


class SimplexDiscreteModel:
    """simplexify(CartesianDiscreteModel(domain, partition)) in 3-D: every hexahedron c is
    split into the 6 tets of the oriented 3-cube simplexification, tet 6c+t
    (Geometry/Grids.jl:487-558, Geometry/UnstructuredDiscreteModels.jl:85-200). The vertices
    (and their coordinates) are the Cartesian model's nodes. Dirichlet regions are tags made
    with `add_tag_from_vertex_filter` (face_labeling_from_vertex_filter: a vertex, edge, face
    or tet carries the tag when all its vertices pass the filter)."""

    def __init__(self, cart: CartesianDiscreteModel):
        if cart.dim != 3 or not cart.cartesian:
            raise NotImplementedError("simplexify is provided for 3-D Cartesian models")
        self.cart = cart
        self.dim = 3
        self.partition = cart.partition
        self.domain = cart.domain
        self.node_coords = cart.node_coords
        self.cartesian = True
        part = np.asarray(self.partition, dtype=np.int64)
        self.cell_node_ids = np.empty((int(np.prod(part)) * 6, 4), dtype=np.int32)
        _lib.check(_lib.load().gfe_simplex_model(_lib.ptr(part), _lib.ptr(self.cell_node_ids)))
        self.vertex_tags: dict[str, np.ndarray] = {}

    def add_tag_from_vertex_filter(self, name: str, filt):
        """filt(coords[nverts, 3]) -> bool mask, or a per-vertex callable."""
        x = self.node_coords
        try:
            m = np.asarray(filt(x), dtype=bool)
            if m.shape != (x.shape[0],):
                raise ValueError
        except (ValueError, TypeError, IndexError):
            m = np.array([bool(filt(xi)) for xi in x])
        self.vertex_tags[name] = m
        return self

    def num_cells(self) -> int:
        return self.cell_node_ids.shape[0]

    def num_nodes(self) -> int:
        return self.node_coords.shape[0]

    def get_node_coordinates(self) -> np.ndarray:
        return self.node_coords

    def get_cell_node_ids(self) -> np.ndarray:
        return self.cell_node_ids


def simplexify(model: CartesianDiscreteModel) -> SimplexDiscreteModel:
    return SimplexDiscreteModel(model)


class Triangulation:
    def __init__(self, model: CartesianDiscreteModel):
        self.model = model

    def num_cells(self) -> int:
        return self.model.num_cells()


def facet_axis(D: int, lf: int) -> tuple[int, int]:
    """Normal axis and side (0 lower, 1 upper) of local facet lf of the D-cube in Gridap's
    face order: the facets come by normal axis from the last to the first, lower side first
    (3-D: z-, z+, y-, y+, x-, x+; 2-D: y-, y+, x-, x+)."""
    return D - 1 - lf // 2, lf & 1


class BoundaryTriangulation:
    """BoundaryTriangulation(model; tags) (Geometry/BoundaryTriangulations.jl:174-208): the
    boundary facets of a Cartesian model whose entity one of `tags` lists (None: all boundary
    facets), in ascending facet id. Facet ids are numbered first-touch over the cells
    (Geometry/GridTopologies.jl:1184-1240), so a boundary facet, which has one cell, comes in
    (owner cell, local facet) order; its entity is the local facet's position in the n-cube
    face list (Geometry/CartesianDiscreteModels.jl:215-240).

    facet_cells: owner cell of each facet (0-based); facet_lfaces: its local facet (0-based)."""

    def __init__(self, model: CartesianDiscreteModel, tags=None):
        if isinstance(model, SimplexDiscreteModel):
            raise NotImplementedError("boundary terms are provided on hexahedral Cartesian models")
        self.model = model
        D = model.dim
        part = np.asarray(model.partition, np.int64)
        nc = int(np.prod(part))
        c = np.arange(nc, dtype=np.int64)
        stride = np.concatenate([[1], np.cumprod(part)[:-1]])
        idx = (c[:, None] // stride[None, :]) % part[None, :]
        offset = 4 if D == 2 else 20  # faces of lower dimension in the n-cube face list
        labels = model.get_face_labeling()
        if tags is None:
            sel = set(labels.tag_entities[labels._tag_index("boundary")])
        else:
            sel = set()
            for t in ([tags] if isinstance(tags, (str, int, np.integer)) else tags):
                sel |= set(labels.tag_entities[labels._tag_index(t)])
        mask = np.zeros((nc, 2 * D), dtype=bool)
        for lf in range(2 * D):
            ax, side = facet_axis(D, lf)
            if offset + lf + 1 in sel:
                mask[:, lf] = idx[:, ax] == (0 if side == 0 else part[ax] - 1)
        cells, lfaces = np.nonzero(mask)  # row-major: (cell, local facet) order
        self.facet_cells = np.ascontiguousarray(cells, dtype=np.int32)
        self.facet_lfaces = np.ascontiguousarray(lfaces, dtype=np.int32)

    def num_cells(self) -> int:
        return int(self.facet_cells.shape[0])

    def facet_points(self, s: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """Facet points s (npoints x D-1, facet reference coordinates) in every facet's owner
        cell: reference-cell coordinates (nfacets x npoints x D; the facet's spanned axes in
        increasing order carry s, the normal axis is fixed at the facet's side) and physical
        coordinates through the owner cell's Q1 map (glue.tface_to_mface_map and
        get_cell_map of Geometry/BoundaryTriangulations.jl)."""
        model = self.model
        D = model.dim
        s = np.asarray(s, np.float64).reshape(-1, D - 1)
        nv = 2 ** D
        ref = np.empty((self.num_cells(), s.shape[0], D))
        phys = np.empty_like(ref)
        X = model.node_coords[model.cell_node_ids[self.facet_cells] - 1]  # (nf, nv, D)
        for lf in range(2 * D):
            ax, side = facet_axis(D, lf)
            xi = np.empty((s.shape[0], D))
            xi[:, ax] = side
            xi[:, [d for d in range(D) if d != ax]] = s
            phi = np.ones((xi.shape[0], nv))
            for a in range(nv):
                for d in range(D):
                    phi[:, a] *= xi[:, d] if (a >> d) & 1 else 1 - xi[:, d]
            sel = self.facet_lfaces == lf
            ref[sel] = xi
            phys[sel] = np.einsum("qa,fad->fqd", phi, X[sel])
        return ref, phys

    def get_facet_normal(self) -> np.ndarray:
        """Outward unit normal of every facet (nfacets x D); the box's facets are flat."""
        D = self.model.dim
        n = np.zeros((self.num_cells(), D))
        for lf in range(2 * D):
            ax, side = facet_axis(D, lf)
            n[self.facet_lfaces == lf, ax] = 1.0 if side else -1.0
        return n

    get_normal_vector = get_facet_normal


Boundary = BoundaryTriangulation


class Measure:
    """Measure(trian, degree): tensor-product Gauss-Legendre of the given degree
    (ReferenceFEs/Quadratures.jl:157-182), on the cells of a Triangulation or on the facets of
    a BoundaryTriangulation."""

    def __init__(self, trian, degree: int):
        self.trian = trian
        self.degree = int(degree)

    @property
    def on_boundary(self) -> bool:
        return isinstance(self.trian, BoundaryTriangulation)

    def num_points(self) -> int:
        if self.on_boundary:
            return (self.degree // 2 + 1) ** (self.trian.model.dim - 1)
        if isinstance(self.trian.model, SimplexDiscreteModel):
            if self.degree not in (4, 5):
                raise NotImplementedError("tet quadrature of degree 4 or 5 is provided")
            return 14  # Witherden-Vincent degree 4/5 (ReferenceFEs/WitherdenVincentQuadratures.jl)
        return (self.degree // 2 + 1) ** self.trian.model.dim
