"""Bitset reductions (the reference's ``pystrns2cards/bitset_utils.py``)."""
from __future__ import annotations

import torch

from . import _core


def accumulate_bitset_rgb(bitset: torch.Tensor, cluster_rgb: torch.Tensor) -> torch.Tensor:
    """Sum of the cluster colours of the set bits per pixel, (B, H, W, 3) (``bitset_utils.py:6-32``)."""
    if not bitset.is_cuda or not cluster_rgb.is_cuda:
        raise ValueError("All inputs must be on CUDA")
    if bitset.dtype != torch.int32:
        raise TypeError("bitset must be int32")
    if cluster_rgb.dtype != torch.float32:
        raise TypeError("cluster_rgb must be float32")
    if cluster_rgb.shape[1] != 3:
        raise ValueError("cluster_rgb must have shape (num_clusters, 3)")
    B, H, W, _ = bitset.shape
    out = torch.zeros((B, H, W, 3), dtype=torch.float32, device=bitset.device)
    _core.accumulate_bitset_rgb(bitset.contiguous(), cluster_rgb.contiguous(), out)
    return out


def popcount_bitset(bitset: torch.Tensor) -> torch.Tensor:
    """Number of set bits per pixel as float32 (B, H, W) (``bitset_utils.py:35-55``)."""
    if not bitset.is_cuda:
        raise ValueError("bitset must be on CUDA")
    if bitset.dtype != torch.int32:
        raise TypeError("bitset must be int32")
    B, H, W, _ = bitset.shape
    out = torch.zeros((B, H, W), dtype=torch.float32, device=bitset.device)
    _core.popcount_bitset(bitset.contiguous(), out)
    return out


def xor_error(bitset: torch.Tensor, target_bitset: torch.Tensor) -> torch.Tensor:
    """Number of mismatching (pixel, cluster) bits as a float32 scalar: the
    ``count_xor_error`` loss of ``antialias.py:124-126`` in one pass."""
    return _core.xor_popcount(bitset.contiguous(), target_bitset.contiguous()).to(torch.float32)[0]


def cluster_iou(bitset: torch.Tensor, target_bitset: torch.Tensor, cluster_count: int):
    """Per-cluster (per-card) bitset IoU: |pred_k & target_k| / |pred_k | target_k| over
    pixels, with the integer intersection and union counts (NaN where the union is 0)."""
    inter, uni = _core.cluster_iou_counts(bitset.contiguous(), target_bitset.contiguous(), int(cluster_count))
    iou = inter.to(torch.float64) / uni.to(torch.float64)
    return iou, inter, uni
