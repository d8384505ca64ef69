"""Card-mesh edge topology.

``build_edges_from_triangles`` returns the unique undirected edges of a triangle mesh and,
per edge, up to two adjacent triangles (-1 where there is none), like the reference's
``build_edges_from_triangles`` (``pystrns2cards/__init__.py:19-40``,
``src/mesh_utils.cpp:52-95``), computed by libs2c's host C++ builder.  The reference emits
edges in ``std::unordered_map`` iteration order, which is implementation-defined; here the
order is fixed: edges sorted by (min vertex, max vertex), each stored as (min, max), and
the adjacent triangles are the first two triangles (in triangle order) that contain the
edge, as the reference's ``push_back`` order gives for each edge.
"""
from __future__ import annotations

from typing import Tuple

import numpy as np

from . import _core


def build_edges_from_triangles(tri: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    if not isinstance(tri, np.ndarray):
        raise TypeError("Input must be a NumPy ndarray.")
    if tri.dtype != np.int32:
        raise TypeError("Triangle indices must be int32.")
    if tri.ndim != 2 or tri.shape[1] != 3:
        raise ValueError("Input triangle array must have shape (T, 3).")
    return _core.build_edges_from_triangles(np.ascontiguousarray(tri))
