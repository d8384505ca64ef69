"""Antialiased cluster-bitset loss (the reference's ``pystrns2cards/antialias.py``).

The loss value is a constant 1 or, with ``count_xor_error``, the number of mismatching
(pixel, cluster) bits; the learning signal is the hand-written gradient ``d_pos`` of the
card vertices' clip positions, computed at the silhouette/boundary edges of the card mesh
from a Gaussian-windowed bitset-vs-target difference (``antialias.cu:121-279``).
"""
from __future__ import annotations

from typing import Any, Tuple

import weakref

import torch

from . import _core
from .dda import dda_compute_fragments


def mark_discontinuity_edges(
    resolution: Tuple[int, int],
    pos: torch.Tensor,
    tri: torch.Tensor,
    edges: torch.Tensor,
    edge2tri: torch.Tensor,
) -> Tuple[torch.Tensor, torch.Tensor]:
    """Silhouette and boundary edges per view (``antialias.py:8-52``).

    Returns ``prim_ids`` (N,) int32 (b*E + e of the marked edges, in increasing order) and
    ``normals`` (B*E, 2) float32 oriented edge normals for all edges.
    """
    H, W = resolution
    dev = pos.device
    B = pos.shape[0]
    E = edges.shape[0]
    prim_ids = torch.full((B * E,), -1, dtype=torch.int32, device=dev)
    normals = torch.zeros((B * E, 2), dtype=torch.float32, device=dev)
    _core.mark_discontinuity_edges(H, W, tri.contiguous(), edges.contiguous(), edge2tri.contiguous(), pos.contiguous(),
                                   prim_ids, normals)
    out = torch.empty_like(prim_ids)
    n = _core.compact_valid_ints(prim_ids, out)
    return out[:n], normals


class _AntialiasedClusterBitsetLossFn(torch.autograd.Function):
    """``antialias.py:55-64``: passes the loss value through; the gradient w.r.t. ``pos`` is
    ``grad_output * d_pos``."""

    @staticmethod
    def forward(ctx: Any, loss_value: torch.Tensor, pos: torch.Tensor, d_pos: torch.Tensor) -> torch.Tensor:
        ctx.save_for_backward(d_pos)
        return loss_value

    @staticmethod
    def backward(ctx: Any, grad_output: torch.Tensor):
        (d_pos,) = ctx.saved_tensors
        return None, grad_output * d_pos, None


class _TargetPlanesCache:
    """Cluster planes of target bitsets.  A fitting loop passes the same target to the loss
    every iteration (``3_fitting.py``), so its transpose is kept while that tensor object is
    alive and unmodified: an entry holds a weak reference to the tensor and its version
    counter and data pointer, and is used only when all three still match."""

    def __init__(self, capacity: int = 4):
        self.capacity = capacity
        self._entries = []   # (weakref, version, data_ptr, planes, stream that wrote them)

    def planes(self, target: torch.Tensor) -> torch.Tensor:
        live = []
        hit = None
        for ref, ver, dp, pl, st in self._entries:
            t = ref()
            if t is None:
                continue
            live.append((ref, ver, dp, pl, st))
            if t is target and ver == target._version and dp == target.data_ptr():
                hit = (pl, st)
        self._entries = live
        cur = torch.cuda.current_stream(target.device)
        if hit is not None:
            if hit[1] != cur:
                # planes written on another stream: wait for them, and tell the caching
                # allocator that this stream reads them too, so that dropping the entry
                # later cannot hand the block out while this stream's kernels still read it
                cur.wait_stream(hit[1])
                hit[0].record_stream(cur)
            return hit[0]
        pl = _core.bitset_to_planes(target)
        self._entries.append((weakref.ref(target), target._version, target.data_ptr(), pl, cur))
        self._entries = self._entries[-self.capacity:]
        return pl

    def clear(self):
        self._entries = []


target_planes_cache = _TargetPlanesCache()


def antialiased_cluster_bitset_grad(
    bitset: torch.Tensor,
    target_bitset: torch.Tensor,
    pos: torch.Tensor,
    tri: torch.Tensor,
    edges: torch.Tensor,
    edge2tri: torch.Tensor,
    edge2cluster: torch.Tensor,
    kernel_radius: float = 7.0,
    rho: float = 1.0,
    fused: bool = True,
) -> torch.Tensor:
    """``d_pos`` (B, V, 4) of ``antialiased_cluster_bitset_loss`` (``antialias.py:100-122``).

    ``fused`` (default): one pass per (view, edge) without a fragment list or host
    synchronisation.  ``fused=False``: the reference's sequence of ops
    (mark_discontinuity_edges, dda_compute_fragments, backward_antialiased_cluster_bitset).
    """
    _, H, W, S = target_bitset.shape
    if not fused:
        prim_ids, normals = mark_discontinuity_edges((H, W), pos, tri, edges, edge2tri)
        frag_pix, frag_attrs = dda_compute_fragments((H, W), pos.contiguous(), edges.contiguous(), prim_ids)
        d_pos = torch.zeros_like(pos)
        _core.backward_antialiased_cluster_bitset(frag_pix, frag_attrs, bitset.contiguous(),
                                                  target_bitset.contiguous(), pos.contiguous(), edges.contiguous(),
                                                  normals, edge2cluster.contiguous(), d_pos, kernel_radius, rho)
        return d_pos
    # the bitset's cluster planes each call, the target's from the cache (same result as
    # the bitset entry point, which transposes both)
    bits = bitset.contiguous()
    if tuple(target_bitset.shape) != tuple(bits.shape) or target_bitset.dtype != bits.dtype:
        raise RuntimeError("antialiased_cluster_bitset_grad: bitset, target_bitset and pos views must match.")
    tplanes = target_planes_cache.planes(target_bitset if target_bitset.is_contiguous()
                                         else target_bitset.contiguous())
    return _core.antialiased_cluster_bitset_grad_planes(_core.bitset_to_planes(bits), tplanes, tuple(bits.shape),
                                                        pos.contiguous(), tri.contiguous(), edges.contiguous(),
                                                        edge2tri.contiguous(), edge2cluster.contiguous(),
                                                        kernel_radius, rho)


def antialiased_cluster_bitset_loss(
    bitset: torch.Tensor,
    target_bitset: torch.Tensor,
    pos: torch.Tensor,
    tri: torch.Tensor,
    edges: torch.Tensor,
    edge2tri: torch.Tensor,
    edge2cluster: torch.Tensor,
    kernel_radius: float = 7.0,
    rho: float = 1.0,
    count_xor_error: bool = False,
) -> torch.Tensor:
    """Scalar loss whose backward hands ``grad_output * d_pos`` to ``pos`` (``antialias.py:66-130``)."""
    device = bitset.device
    for t in (target_bitset, pos, tri, edges, edge2tri, edge2cluster):
        assert t.device == device
    d_pos = antialiased_cluster_bitset_grad(bitset, target_bitset, pos, tri, edges, edge2tri, edge2cluster,
                                            kernel_radius, rho)
    if count_xor_error:
        loss_value = _core.xor_popcount(bitset.contiguous(), target_bitset.contiguous()).to(pos.dtype)[0]
    else:
        loss_value = torch.ones([], dtype=pos.dtype, device=device)
    return _AntialiasedClusterBitsetLossFn.apply(loss_value, pos, d_pos)
