"""DDA line rasterisation ops (the reference's ``pystrns2cards/dda.py``).

``dda_compute_fragments`` keeps the reference's signature, checks and outputs
(``dda.py:5-76``); its fragments come out in primitive order (the order of an in-order
compaction), where the reference's order depends on block scheduling.
``dda_cluster_bitset`` is the fused hot path: strand segments straight to the per-pixel
cluster bitset, bit-identical to ``cluster_mask_from_fragments(dda_compute_fragments(...))``.
"""
from __future__ import annotations

from typing import Optional, Tuple

import torch

from . import _core


def dda_compute_fragments(
    resolution: Tuple[int, int],
    pos: torch.Tensor,
    edges: torch.Tensor,
    edge_ids: Optional[torch.Tensor] = None,
) -> Tuple[torch.Tensor, torch.Tensor]:
    """Rasterise line segments into fragments.

    Returns ``frag_pix`` (N, 3) int32 = (view, row, col) and ``frag_attrs`` (N, 4) float32 =
    (axis, t1, z_ndc, edge_id + 1), as ``dda.py:5-76``.
    """
    H, W = resolution
    if not pos.is_cuda or not edges.is_cuda:
        raise ValueError("Input tensors must be on CUDA.")
    if pos.dtype != torch.float32 or edges.dtype != torch.int32:
        raise ValueError("`pos` must be float32 and `edges` must be int32.")
    if pos.ndim != 3 or pos.shape[2] != 4:
        raise ValueError("`pos` must have shape (B, V, 4).")
    if edges.ndim != 2 or edges.shape[1] != 2:
        raise ValueError("`edges` must have shape (E, 2).")
    if not pos.is_contiguous() or not edges.is_contiguous():
        raise ValueError("Input tensors must be contiguous.")
    B, V, _ = pos.shape
    E = edges.shape[0]
    dev = pos.device
    if edge_ids is None:
        edge_ids = torch.arange(B * E, dtype=torch.int32, device=dev)
    elif not edge_ids.is_cuda or edge_ids.dtype != torch.int32 or edge_ids.ndim != 1:
        raise ValueError("`edge_ids` must be a 1D int32 CUDA tensor.")
    edge_ids = edge_ids.contiguous()
    P = edge_ids.shape[0]
    prefix = torch.empty((P,), dtype=torch.int32, device=dev)
    slopes = torch.empty((P, 2), dtype=torch.float32, device=dev)
    spans = torch.empty((P, 4), dtype=torch.float32, device=dev)
    F = _core.dda_compute_span(edge_ids, H, W, pos, edges, prefix, slopes, spans)
    # the reference writes every DDA step (-1 where rejected) and compacts the list
    # (dda.py:50-76); here the accepted steps are counted and written straight into a list of
    # their own: the same fragments in the same order
    return _core.dda_compact_fragments(prefix, edge_ids, slopes, spans, H, W, pos, edges, F)


class DDAInterpolateAttributes(torch.autograd.Function):
    """``dda.py:79-120``: image = (1 - t1) a[v0] + t1 a[v1] per pixel of a line raster."""

    @staticmethod
    def forward(ctx, rast: torch.Tensor, attr: torch.Tensor, edges: torch.Tensor) -> torch.Tensor:
        if not rast.is_cuda or not attr.is_cuda or not edges.is_cuda:
            raise ValueError("All input tensors must be CUDA tensors.")
        if rast.dtype != torch.float32 or attr.dtype != torch.float32:
            raise ValueError("`rast` and `attr` must be float32.")
        if edges.dtype != torch.int32:
            raise ValueError("`edges` must be int32.")
        if rast.ndim != 4 or rast.shape[-1] != 4:
            raise ValueError("`rast` must have shape (B, H, W, 4).")
        if attr.ndim != 2:
            raise ValueError("`attr` must have shape (V, C).")
        if edges.ndim != 2 or edges.shape[1] != 2:
            raise ValueError("`edges` must have shape (E, 2).")
        B, H, W, _ = rast.shape
        V, C = attr.shape
        image = torch.zeros((B, H, W, C), dtype=torch.float32, device=rast.device)
        _core.dda_interpolate_attributes(rast.contiguous(), attr.contiguous(), edges.contiguous(), image)
        ctx.save_for_backward(rast, attr, edges)
        return image

    @staticmethod
    def backward(ctx, d_image: torch.Tensor):
        rast, attr, edges = ctx.saved_tensors
        d_attr = torch.zeros_like(attr)
        _core.backward_dda_interpolate_attributes(rast.contiguous(), d_image.contiguous(), edges.contiguous(), d_attr)
        return None, d_attr, None


def dda_interpolate_attributes(rast: torch.Tensor, attr: torch.Tensor, edges: torch.Tensor) -> torch.Tensor:
    """Differentiable interpolation of per-vertex attributes along rasterised lines (``dda.py:123-136``)."""
    return DDAInterpolateAttributes.apply(rast, attr, edges)


def dda_cluster_bitset(
    resolution: Tuple[int, int],
    pos: torch.Tensor,
    edges: torch.Tensor,
    edge2cluster: torch.Tensor,
    cluster_count: int,
    edge_ids: Optional[torch.Tensor] = None,
    out: Optional[torch.Tensor] = None,
    workspace: Optional[torch.Tensor] = None,
) -> torch.Tensor:
    """Per-pixel cluster bitset (B, H, W, ceil(K/32)) int32 of line segments, fused.

    Same bits as ``cluster_mask_from_fragments(resolution, *dda_compute_fragments(...),
    edge2cluster, cluster_count)`` (the target bitset of ``3_fitting.py:254-261``), except
    that B is ``pos.shape[0]`` rather than inferred from the last view that has fragments.
    No fragment list is built and the call does not synchronise with the host.
    """
    H, W = resolution
    if not (pos.is_cuda and edges.is_cuda and edge2cluster.is_cuda):
        raise ValueError("Input tensors must be on CUDA.")
    if pos.dtype != torch.float32 or edges.dtype != torch.int32 or edge2cluster.dtype != torch.int32:
        raise ValueError("`pos` must be float32, `edges` and `edge2cluster` int32.")
    if pos.ndim != 3 or pos.shape[2] != 4:
        raise ValueError("`pos` must have shape (B, V, 4).")
    if edges.ndim != 2 or edges.shape[1] != 2:
        raise ValueError("`edges` must have shape (E, 2).")
    if edge2cluster.ndim != 1 or edge2cluster.shape[0] != edges.shape[0]:
        raise ValueError("`edge2cluster` must have shape (E,).")
    if cluster_count <= 0:
        raise ValueError("`cluster_count` must be positive.")
    B = pos.shape[0]
    S = (int(cluster_count) + 31) // 32
    if out is None:
        out = torch.empty((B, H, W, S), dtype=torch.int32, device=pos.device)
    elif tuple(out.shape) != (B, H, W, S) or out.dtype != torch.int32 or not out.is_contiguous():
        raise ValueError(f"`out` must be a contiguous int32 tensor of shape {(B, H, W, S)}.")
    return _core.dda_cluster_bitset(pos.contiguous(), edges.contiguous(), edge2cluster.contiguous(), out,
                                    None if edge_ids is None else edge_ids.contiguous(), workspace)


def dda_cluster_bitset_workspace_bytes(num_prims: int, B: int, H: int, W: int, cluster_count: int) -> int:
    from . import _lib
    return int(_lib.lib().s2c_dda_cluster_bitset_workspace_size(num_prims, B, H, W, (cluster_count + 31) // 32))
