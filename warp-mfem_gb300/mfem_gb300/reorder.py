"""Vertex reordering for the persistent PCG.

The fast PCG forms keep, per CTA, the contiguous range of rows its columns
reach (its "window") in shared memory; that range is narrow when the vertex
order is banded.  Meshes from generators or files are often not: reverse
Cuthill-McKee on the vertex adjacency graph restores a narrow band.  The
solver works on any order (it falls back to gathering from L2), so this is an
optional preprocessing step of the model.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
from scipy.sparse.csgraph import reverse_cuthill_mckee


def vertex_adjacency(tet_indices: np.ndarray, n: int) -> sp.csr_matrix:
    tets = np.asarray(tet_indices, dtype=np.int64)
    rows = np.repeat(tets, 4, axis=1).ravel()
    cols = np.tile(tets, (1, 4)).ravel()
    A = sp.coo_matrix((np.ones(rows.shape[0], dtype=np.int8), (rows, cols)), shape=(n, n)).tocsr()
    A.sum_duplicates()
    return A


def bandwidth(tet_indices: np.ndarray) -> int:
    """Largest |i - j| over the vertex pairs that share a tet."""
    tets = np.asarray(tet_indices, dtype=np.int64)
    if tets.size == 0:
        return 0
    return int((tets.max(axis=1) - tets.min(axis=1)).max())


def rcm_order(tet_indices: np.ndarray, n: int) -> np.ndarray:
    """Permutation `order` (new vertex i is old vertex order[i]) from reverse
    Cuthill-McKee on the vertex adjacency graph."""
    return np.asarray(reverse_cuthill_mckee(vertex_adjacency(tet_indices, n), symmetric_mode=True), dtype=np.int64)


def permute_vertices(order: np.ndarray, tet_indices: np.ndarray, *vertex_arrays):
    """Applies a vertex permutation: returns the renumbered tets followed by
    each vertex array reordered (rows taken in `order`)."""
    order = np.asarray(order, dtype=np.int64)
    inverse = np.empty_like(order)
    inverse[order] = np.arange(order.shape[0])
    new_tets = inverse[np.asarray(tet_indices, dtype=np.int64)].astype(np.int32)
    return (new_tets,) + tuple(np.asarray(a)[order] for a in vertex_arrays)
