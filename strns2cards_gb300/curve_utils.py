"""Strand curve operators with the reference's ``pystrns2cards.curve_utils`` signatures
(``curve_utils.py:167-240``): ``compute_arclength``, ``smooth_strands``, ``skinning``.

``smooth_strands`` and ``skinning`` run as one launch each: the kernel computes the
arclength of the strands it stages instead of reading a separately computed tensor.
"""
from __future__ import annotations

import torch

from . import _core


def compute_arclength(strands: torch.Tensor) -> torch.Tensor:
    """Cumulative arclength (N, V) of strands (N, V, 3), 0 at the root
    (``curve_utils.py:167-180``)."""
    if not strands.is_cuda:
        raise ValueError("compute_arclength: Input tensor must be on CUDA.")
    if strands.ndim != 3 or strands.shape[-1] != 3:
        raise ValueError("compute_arclength: Input tensor must have shape (N, V, 3).")
    s = strands.contiguous()
    out = torch.empty(s.shape[:2], dtype=torch.float32, device=s.device)
    _core.compute_arclength(s, out)
    return out


def smooth_strands(strands: torch.Tensor, beta: float) -> torch.Tensor:
    """Gaussian smoothing in arclength with a 3-beta cutoff (``curve_utils.py:182-206``)."""
    if not strands.is_cuda:
        raise ValueError("smooth_strands: Input tensor must be on CUDA.")
    if strands.ndim != 3 or strands.shape[-1] != 3:
        raise ValueError("smooth_strands: Input tensor must have shape (N, V, 3).")
    s = strands.contiguous()
    out = torch.empty_like(s)
    _core.smooth_strands(s, None, out, beta)
    return out


def skinning(strands: torch.Tensor, handle_strands: torch.Tensor, canonical_handles: torch.Tensor,
             R: torch.Tensor, beta: float) -> torch.Tensor:
    """Arclength-weighted rigid skinning of strands to per-point handle frames
    (``curve_utils.py:209-240``)."""
    if not (strands.is_cuda and handle_strands.is_cuda and canonical_handles.is_cuda and R.is_cuda):
        raise ValueError("skinning: All input tensors must be on CUDA.")
    N, V, _ = strands.shape
    if handle_strands.shape != (N, V, 3) or canonical_handles.shape != (N, V, 3) or R.shape != (N, V, 3, 3):
        raise ValueError("skinning: Input tensor shapes do not match the expected dimensions.")
    s = strands.contiguous()
    out = torch.empty_like(s)
    _core.skinning(s, None, handle_strands.contiguous(), canonical_handles.contiguous(), R.contiguous(), out, beta)
    return out
