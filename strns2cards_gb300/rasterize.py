"""Triangle rasterisation and fragment -> bitset ops (the reference's ``pystrns2cards/rasterize.py``)."""
from __future__ import annotations

from typing import Optional, Tuple

import torch

from . import _core


def cluster_mask_from_fragments(
    resolution: Tuple[int, int],
    frag_pix: torch.Tensor,
    frag_attrs: torch.Tensor,
    tri2cluster: torch.Tensor,
    cluster_count: Optional[int] = None,
) -> torch.Tensor:
    """Per-pixel OR of ``1 << cluster`` over fragments (``rasterize.py:170-214``).

    As in the reference, B is one more than the largest view index among the fragments
    and the cluster count defaults to ``tri2cluster.max() + 1`` (both read on the host).
    """
    H, W = resolution
    if frag_pix.dtype != torch.int32 or frag_pix.ndim != 2 or frag_pix.shape[1] != 3:
        raise ValueError("frag_pix must be a (N, 3) int32 tensor.")
    if frag_attrs.dtype != torch.float32 or frag_attrs.ndim != 2 or frag_attrs.shape[1] != 4:
        raise ValueError("frag_attrs must be a (N, 4) float32 tensor.")
    if tri2cluster.dtype != torch.int32 or tri2cluster.ndim != 1:
        raise ValueError("tri2cluster must be a (T,) int32 tensor.")
    if not (frag_pix.is_cuda and frag_attrs.is_cuda and tri2cluster.is_cuda):
        raise ValueError("All input tensors must be CUDA tensors.")
    B = int(frag_pix[:, 0].max().item()) + 1
    K = cluster_count if cluster_count is not None else int(tri2cluster.max().item()) + 1
    S = (K + 31) // 32
    bitset = torch.zeros((B, H, W, S), dtype=torch.int32, device=frag_pix.device)
    _core.cluster_mask_from_fragments(frag_pix.contiguous(), frag_attrs.contiguous(), tri2cluster.contiguous(), bitset)
    return bitset
