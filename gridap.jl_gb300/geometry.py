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


class Measure:
    """Measure(trian, degree): tensor-product Gauss-Legendre of the given degree
    (ReferenceFEs/Quadratures.jl:157-182)."""

    def __init__(self, trian: Triangulation, degree: int):
        self.trian = trian
        self.degree = int(degree)

    def num_points(self) -> int:
        if isinstance(self.trian.model, SimplexDiscreteModel):
            if self.degree not in (4, 5):
                raise NotImplementedError("tet quadrature of degree 4 or 5 is provided")
            return 14  # Witherden-Vincent degree 4/5 (ReferenceFEs/WitherdenVincentQuadratures.jl)
        return (self.degree // 2 + 1) ** self.trian.model.dim
