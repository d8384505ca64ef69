"""Card-mesh edge topology.

``build_edges_from_triangles`` returns the unique undirected edges of a triangle mesh and,
per edge, up to two adjacent triangles (-1 where there is none), like the reference's
``build_edges_from_triangles`` (``pystrns2cards/__init__.py:19-40``,
``src/mesh_utils.cpp:52-95``).  The reference emits edges in ``std::unordered_map``
iteration order, which is implementation-defined; here the order is fixed: edges sorted by
(min vertex, max vertex), each stored as (min, max), and the adjacent triangles are the
first two triangles (in triangle order) that contain the edge, as the reference's
``push_back`` order gives for each edge.
"""
from __future__ import annotations

from typing import Tuple

import numpy as np


def build_edges_from_triangles(tri: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    if not isinstance(tri, np.ndarray):
        raise TypeError("Input must be a NumPy ndarray.")
    if tri.dtype != np.int32:
        raise TypeError("Triangle indices must be int32.")
    if tri.ndim != 2 or tri.shape[1] != 3:
        raise ValueError("Input triangle array must have shape (T, 3).")
    T = tri.shape[0]
    if T == 0:
        return np.zeros((0, 2), np.int32), np.zeros((0, 2), np.int32)
    t64 = tri.astype(np.int64)
    a = np.stack([t64[:, 0], t64[:, 1], t64[:, 2]], 1).reshape(-1)
    b = np.stack([t64[:, 1], t64[:, 2], t64[:, 0]], 1).reshape(-1)
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    owner = np.repeat(np.arange(T, dtype=np.int64), 3)
    order = np.lexsort((owner, hi, lo))
    lo, hi, owner = lo[order], hi[order], owner[order]
    first = np.ones(lo.shape[0], dtype=bool)
    first[1:] = (lo[1:] != lo[:-1]) | (hi[1:] != hi[:-1])
    starts = np.nonzero(first)[0]
    edges = np.stack([lo[starts], hi[starts]], 1).astype(np.int32)
    e2t = np.full((starts.shape[0], 2), -1, dtype=np.int32)
    e2t[:, 0] = owner[starts]
    nxt = starts + 1
    has2 = nxt < lo.shape[0]
    has2[has2] = ~first[nxt[has2]]
    e2t[has2, 1] = owner[nxt[has2]]
    return edges, e2t
