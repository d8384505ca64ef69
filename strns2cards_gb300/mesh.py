"""Card-mesh edge topology.

``build_edges_from_triangles`` returns the unique undirected edges of a triangle mesh and,
per edge, up to two adjacent triangles (-1 where there is none), like the reference's
``build_edges_from_triangles`` (``pystrns2cards/__init__.py:19-40``,
``src/mesh_utils.cpp:52-95``), computed by libs2c's host C++ builder.  The reference emits
edges in ``std::unordered_map`` iteration order, which is implementation-defined; here the
order is fixed: edges sorted by (min vertex, max vertex), each stored as (min, max), and
the adjacent triangles are the first two triangles (in triangle order) that contain the
edge, as the reference's ``push_back`` order gives for each edge.

Given a CUDA tensor the edges are built on the device (same edges, same order, same
adjacency) and come back as CUDA tensors; ``build_edges_from_triangles_device`` does the
same without any host synchronisation, for a serving loop that rebuilds card topology.
"""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np
import torch

from . import _core


def build_edges_from_triangles_device(tri: torch.Tensor, num_verts: int):
    """(edges (3T, 2), edge2tri (3T, 2), counts int64 (2,) = [num_edges, num_bad]) on the
    device, the first num_edges rows holding the edges; no host synchronisation.
    ``num_bad`` counts half-edges with a vertex outside [0, num_verts) (left out)."""
    return _core.build_edges_device(tri.to(torch.int32).contiguous(), num_verts)


def build_edges_from_triangles(tri, num_verts: Optional[int] = None):
    if isinstance(tri, torch.Tensor) and tri.is_cuda:
        if tri.dtype != torch.int32:
            raise TypeError("Triangle indices must be int32.")
        if tri.ndim != 2 or tri.shape[1] != 3:
            raise ValueError("Input triangle array must have shape (T, 3).")
        t = tri.contiguous()
        if num_verts is None:
            num_verts = int(t.max()) + 1 if t.numel() else 0
            if t.numel() and int(t.min()) < 0:
                raise ValueError("Triangle indices must be non-negative.")
        edges, e2t, counts = _core.build_edges_device(t, num_verts)
        E, bad = (int(x) for x in counts.tolist())
        if bad:
            raise ValueError(f"{bad} half-edges reference vertices outside [0, {num_verts}).")
        return edges[:E], e2t[:E]
    if not isinstance(tri, np.ndarray):
        raise TypeError("Input must be a NumPy ndarray.")
    if tri.dtype != np.int32:
        raise TypeError("Triangle indices must be int32.")
    if tri.ndim != 2 or tri.shape[1] != 3:
        raise ValueError("Input triangle array must have shape (T, 3).")
    return _core.build_edges_from_triangles(np.ascontiguousarray(tri))
