"""Triangle rasterisation and fragment -> bitset ops (the reference's ``pystrns2cards/rasterize.py``)."""
from __future__ import annotations

from typing import Optional, Tuple

import torch

from . import _core, _lib


def compute_fragments(
    resolution: Tuple[int, int],
    pos: torch.Tensor,
    tri: torch.Tensor,
) -> Tuple[torch.Tensor, torch.Tensor]:
    """Triangle fragments (``rasterize.py:6-53``): ``frag_pix`` (N, 3) int32 = (view, row, col),
    ``frag_attrs`` (N, 4) float32 = (b0, b1, z, triangle_id + 1), in (view, triangle,
    row-major pixel) order."""
    H, W = resolution
    if not pos.is_cuda or not tri.is_cuda:
        raise ValueError("Input tensors must be on CUDA.")
    if pos.dtype != torch.float32 or tri.dtype != torch.int32:
        raise ValueError("`pos` must be float32 and `tri` must be int32.")
    if pos.ndim != 3 or pos.shape[2] != 4:
        raise ValueError("`pos` must have shape (B, V, 4).")
    if tri.ndim != 2 or tri.shape[1] != 3:
        raise ValueError("`tri` must have shape (T, 3).")
    if not pos.is_contiguous() or not tri.is_contiguous():
        raise ValueError("Input tensors must be contiguous.")
    B = pos.shape[0]
    T = tri.shape[0]
    dev = pos.device
    rects = torch.empty((B * T, 4), dtype=torch.int32, device=dev)
    prefix = torch.empty((B * T,), dtype=torch.int32, device=dev)
    F = _core.compute_triangle_rects(H, W, pos, tri, rects, prefix)
    # the reference lists every bounding-box pixel (-1 where uncovered) and compacts the list
    # (rasterize.py:33-53); here the covered pixels are counted and written straight into a
    # list of their own: the same fragments in the same order
    return _core.compact_fragments(H, W, pos, tri, prefix, rects, F)


def depth_test(B: int, resolution: Tuple[int, int], frag_pix: torch.Tensor, frag_attrs: torch.Tensor) -> torch.Tensor:
    """Nearest fragment per pixel (``rasterize.py:55-95``): (B, H, W, 4) float32, zeros where empty."""
    if not (frag_pix.is_cuda and frag_attrs.is_cuda):
        raise ValueError("Input tensors must be on CUDA.")
    if frag_pix.dtype != torch.int32:
        raise ValueError("frag_pix must be int32.")
    if frag_attrs.dtype != torch.float32:
        raise ValueError("frag_attrs must be float32.")
    if frag_pix.ndim != 2 or frag_pix.shape[1] != 3:
        raise ValueError("frag_pix must have shape (N, 3).")
    if frag_attrs.ndim != 2 or frag_attrs.shape[1] != 4:
        raise ValueError("frag_attrs must have shape (N, 4).")
    if frag_pix.shape[0] != frag_attrs.shape[0]:
        raise ValueError("frag_pix and frag_attrs must match in length.")
    H, W = resolution
    rast = torch.zeros((B, H, W, 4), dtype=torch.float32, device=frag_pix.device)
    _core.depth_test(H, W, frag_pix.contiguous(), frag_attrs.contiguous(), rast)
    return rast


def rasterize_fused(resolution: Tuple[int, int], pos: torch.Tensor, tri: torch.Tensor,
                    tri2cluster: Optional[torch.Tensor] = None, num_clusters: int = 0, want_rast: bool = True,
                    rast: Optional[torch.Tensor] = None, bitset: Optional[torch.Tensor] = None,
                    workspace: Optional[torch.Tensor] = None):
    """One pass of compute_fragments + depth_test (+ cluster_mask_from_fragments when
    ``tri2cluster`` is given) with no fragment list and no host synchronisation.
    Returns (rast or None, bitset or None); outputs may be passed in to reuse memory."""
    if not (pos.is_cuda and tri.is_cuda):
        raise ValueError("Input tensors must be on CUDA.")
    if pos.dtype != torch.float32 or pos.ndim != 3 or pos.shape[-1] != 4:
        raise ValueError("pos must be float32 (B, V, 4).")
    if tri.dtype != torch.int32 or tri.ndim != 2 or tri.shape[1] != 3:
        raise ValueError("tri must be int32 (T, 3).")
    H, W = resolution
    B, V = pos.shape[0], pos.shape[1]
    dev = pos.device
    p, t = pos.contiguous(), tri.contiguous()
    S = 0
    if tri2cluster is not None:
        S = (int(num_clusters) + 31) // 32
        if S <= 0:
            raise ValueError("num_clusters must be positive with tri2cluster.")
        tri2cluster = tri2cluster.contiguous()
        if bitset is None:
            bitset = torch.empty((B, H, W, S), dtype=torch.int32, device=dev)
    if want_rast and rast is None:
        rast = torch.empty((B, H, W, 4), dtype=torch.float32, device=dev)
    if not want_rast:
        rast = None
    need = _lib.lib().s2c_rasterize_fused_workspace_size(B, H, W, t.shape[0])
    if workspace is None or workspace.numel() < need:
        workspace = _lib.workspace(need, dev)
    _lib.call("s2c_rasterize_fused", B, H, W, V, _lib.ptr(p), t.shape[0], _lib.ptr(t), _lib.ptr(tri2cluster),
              0 if tri2cluster is None else tri2cluster.shape[0], S, _lib.ptr(bitset), _lib.ptr(rast),
              _lib.ptr(workspace), workspace.numel(), _lib.stream_of(p))
    return rast, bitset


def rasterize(resolution: Tuple[int, int], pos: torch.Tensor, tri: torch.Tensor) -> torch.Tensor:
    """``compute_fragments`` then ``depth_test`` (``rasterize.py:97-116``), computed by the
    fused single pass (the same rast as the two ops)."""
    return rasterize_fused(resolution, pos, tri)[0]


def barycentric_derivatives(rast: torch.Tensor, pos: torch.Tensor, tri: torch.Tensor) -> torch.Tensor:
    """d(b0, b1)/d(x, y) in pixel units, (B, H, W, 4) = (db0/dx, db0/dy, db1/dx, db1/dy), of the
    triangle covering each pixel of ``rast``; zeros where empty.  Not in the reference."""
    if not (rast.is_cuda and pos.is_cuda and tri.is_cuda):
        raise ValueError("All inputs must be CUDA tensors.")
    if rast.ndim != 4 or rast.shape[-1] != 4 or pos.ndim != 3 or pos.shape[-1] != 4 or tri.ndim != 2:
        raise ValueError("rast must be (B, H, W, 4), pos (B, V, 4) and tri (T, 3).")
    if rast.shape[0] > pos.shape[0]:
        raise ValueError("pos must hold every view of rast.")
    r = rast.contiguous()
    db = torch.empty_like(r)
    B, H, W, _ = r.shape
    p = pos.contiguous()
    t = tri.contiguous()
    _lib.call("s2c_barycentric_derivatives", B, H, W, p.shape[1], _lib.ptr(p), t.shape[0], _lib.ptr(t), _lib.ptr(r),
              _lib.ptr(db), _lib.stream_of(r))
    return db


def rasterize_with_derivatives(resolution: Tuple[int, int], pos: torch.Tensor, tri: torch.Tensor):
    """``rasterize`` plus ``barycentric_derivatives``: (rast, rast_db)."""
    rast = rasterize(resolution, pos, tri)
    return rast, barycentric_derivatives(rast, pos, tri)


class InterpolateTriangleAttributes(torch.autograd.Function):
    """``rasterize.py:119-147``: image = b0 a0 + b1 a1 + (1 - b0 - b1) a2; the backward
    scatters grad * b_i to the vertex attributes."""

    @staticmethod
    def forward(ctx, rast: torch.Tensor, attr: torch.Tensor, tri: torch.Tensor) -> torch.Tensor:
        if not (rast.is_cuda and attr.is_cuda and tri.is_cuda):
            raise ValueError("All inputs must be CUDA tensors.")
        B, H, W, _ = rast.shape
        V, C = attr.shape
        image = torch.zeros((B, H, W, C), dtype=attr.dtype, device=attr.device)
        _core.interpolate_triangle_attributes(rast.contiguous(), attr.contiguous(), tri.contiguous(), image)
        ctx.save_for_backward(rast, tri, attr)
        return image

    @staticmethod
    def backward(ctx, grad_output: torch.Tensor):
        rast, tri, attr = ctx.saved_tensors
        d_attr = torch.zeros_like(attr)
        _core.backward_interpolate_triangle_attributes(rast.contiguous(), grad_output.contiguous(), tri.contiguous(),
                                                       d_attr)
        return None, d_attr, None


def interpolate_triangle_attributes(rast: torch.Tensor, attr: torch.Tensor, tri: torch.Tensor) -> torch.Tensor:
    """Differentiable barycentric interpolation of per-vertex attributes (``rasterize.py:150-167``)."""
    return InterpolateTriangleAttributes.apply(rast, attr, tri)


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
