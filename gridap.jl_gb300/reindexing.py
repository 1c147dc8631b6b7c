"""Free-dof reordering: compute_dof_permutation / reindex_free_dof_ids
(FESpaces/FESpaceReindexing.jl:264-343).

  - "rcm":         Reverse Cuthill-McKee with George-Liu pseudo-peripheral nodes; every
                   breadth-first search runs on the device (gfe_dof_permutation);
  - "sloan":       Sloan's wavefront ordering (w1, w2 as Gridap's), device searches plus the
                   heap-driven numbering on the host;
  - "coordinates": free dofs sorted by their nodes' coordinates, lexicographically (x, y, z),
                   or by a key function `by` of each point.

Permutations follow Gridap's convention iperm[old-1] = new (1-based). The reindexed space has
the same Dirichlet ids; its cell dof ids carry the new free ids, so a matrix assembled on it
is P A Pᵀ of the original.
"""
from __future__ import annotations

import copy

import numpy as np

from . import _lib
from .fespaces import FESpace, _space


def compute_dof_permutation(space, algorithm: str = "rcm", by=None, w1: int = 1, w2: int = 2,
                            ctx=None) -> np.ndarray:
    V = _space(space)
    n = V.num_free_dofs()
    if algorithm == "coordinates":
        X, _, _, _ = V.dof_points()
        if by is None:
            order = np.lexsort(tuple(X[:, d] for d in range(X.shape[1] - 1, -1, -1)))
        else:
            keys = [by(x) for x in X]
            order = np.array(sorted(range(n), key=lambda i: keys[i]), dtype=np.int64)
        iperm = np.empty(n, np.int64)
        iperm[order] = np.arange(1, n + 1)
        return iperm
    alg = {"rcm": _lib.GFE_REORDER_RCM, "sloan": _lib.GFE_REORDER_SLOAN}.get(algorithm)
    if alg is None:
        raise ValueError(f"Unknown algorithm {algorithm!r}. Supported: rcm, sloan, coordinates")
    if ctx is None:
        from .assembly import default_context
        ctx = default_context()
    ids = np.ascontiguousarray(V.cell_dof_ids, np.int32)
    iperm = np.empty(n, np.int64)
    _lib.check(_lib.load().gfe_dof_permutation(ctx.handle, ids.shape[0], ids.shape[1],
                                               _lib.ptr(ids), n, alg, int(w1), int(w2),
                                               _lib.ptr(iperm)))
    return iperm


def reindex_free_dof_ids(space, perm="rcm", **kwargs) -> FESpace:
    """A copy of the space whose free dof k is numbered perm[k-1] (perm: an algorithm name or
    a permutation iperm with iperm[old-1] = new)."""
    V = _space(space)
    iperm = (compute_dof_permutation(V, perm, **kwargs) if isinstance(perm, str)
             else np.asarray(perm, np.int64))
    n = V.num_free_dofs()
    if iperm.shape != (n,) or not np.array_equal(np.sort(iperm), np.arange(1, n + 1)):
        raise ValueError("not a permutation of the free dofs")
    W = copy.copy(V)
    ids = V.cell_dof_ids
    new = ids.copy()
    m = ids > 0
    new[m] = iperm[ids[m] - 1].astype(np.int32)
    W.cell_dof_ids = np.ascontiguousarray(new, np.int32)
    if getattr(V, "node_comp_to_dof", None) is not None:
        nc = V.node_comp_to_dof.copy()
        m = nc > 0
        nc[m] = iperm[nc[m] - 1].astype(nc.dtype)
        W.node_comp_to_dof = nc
    W.free_dof_permutation = iperm
    return W


def bandwidth(A) -> int:
    """max |i - j| over the stored entries of a DeviceMatrix (CSR export)."""
    rowptr, colval, _ = A.export_csr(0)
    rows = np.repeat(np.arange(len(rowptr) - 1), np.diff(rowptr))
    return int(np.abs(rows - colval).max()) if colval.size else 0
