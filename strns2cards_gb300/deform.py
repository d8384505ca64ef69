"""Card deformation operators: Laplacian smoothing of card vertices and linear blend
skinning of strand vertices to card guide points.

``card_laplacian_smooth`` runs ``steps`` Jacobi steps p <- p - lam * D^-1 L p of the
uniform Laplacian L = D - A of the card quad edges (the L of ``optimizer.py:70-99``, built
from ``h_edges + w_edges`` as ``3_fitting.py:319`` does), for every card at once.

``LBSBinding`` binds strand vertices to their 4 nearest guides with weights
softmax(-d^2 / tau); ``lbs`` evaluates y = sum_k w_k (A_k x + t_k) with per-guide affine
maps ``M (G, 3, 4) = [A | t]`` and is differentiable in ``M`` (and in ``x`` with the
weights held at their bound values).
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr, workspace


def vertex_adjacency(num_verts: int, edges: np.ndarray):
    """CSR (offsets (V + 1,), adj) int32 numpy arrays of an undirected edge list."""
    e = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
    off = np.empty(num_verts + 1, np.int32)
    adj = np.empty(max(2 * e.shape[0], 1), np.int32)
    n = _lib.i64_out()
    call("s2c_build_vertex_adjacency", int(num_verts), e.shape[0], e.ctypes.data, off.ctypes.data, adj.ctypes.data,
         ctypes.byref(n))
    return off, adj[:int(n.value)].copy()


class CardLaplacian:
    """Device CSR of one card's quad-edge topology, shared by every card."""

    def __init__(self, verts_per_card: int, quad_edges: np.ndarray, device="cuda"):
        off, adj = vertex_adjacency(verts_per_card, quad_edges)
        self.verts_per_card = int(verts_per_card)
        self.offsets = torch.from_numpy(off).to(device)
        self.adj = torch.from_numpy(adj if adj.size else np.zeros(1, np.int32)).to(device)
        self.num_adj = int(adj.shape[0])

    def __call__(self, verts: torch.Tensor, lam: float = 0.5, steps: int = 10,
                 out: Optional[torch.Tensor] = None) -> torch.Tensor:
        if not verts.is_cuda or verts.dtype != torch.float32 or verts.shape[-1] != 3:
            raise ValueError("card_laplacian_smooth: verts must be a float32 CUDA tensor (..., 3).")
        v = verts.contiguous()
        n = v.numel() // 3
        if n % self.verts_per_card:
            raise ValueError("card_laplacian_smooth: vertex count is not a multiple of verts_per_card.")
        out = torch.empty_like(v) if out is None else out
        call("s2c_card_laplacian_smooth", n // self.verts_per_card, self.verts_per_card, ptr(self.offsets),
             ptr(self.adj), self.num_adj, ptr(v), ptr(out), float(lam), int(steps), _lib.stream_of(v))
        return out


def card_laplacian_smooth(verts: torch.Tensor, quad_edges: np.ndarray, verts_per_card: int, lam: float = 0.5,
                          steps: int = 10) -> torch.Tensor:
    """Smooth every card (vertices ``(num_cards * verts_per_card, 3)``, cards contiguous;
    ``quad_edges`` local to one card)."""
    return CardLaplacian(verts_per_card, quad_edges, verts.device)(verts, lam, steps)


class LBSBinding:
    """4-nearest-guide binding: ``idx (Nv, 4)``, ``w (Nv, 4)`` and the per-guide inverse lists."""

    def __init__(self, x: torch.Tensor, guides: torch.Tensor, tau: float = 0.01):
        if not (x.is_cuda and guides.is_cuda):
            raise ValueError("LBSBinding: tensors must be on CUDA.")
        x = x.reshape(-1, 3).contiguous().float()
        g = guides.reshape(-1, 3).contiguous().float()
        Nv, G = x.shape[0], g.shape[0]
        dev = x.device
        self.num_verts, self.num_guides, self.tau = Nv, G, float(tau)
        self.idx = torch.empty((Nv, 4), dtype=torch.int32, device=dev)
        self.w = torch.empty((Nv, 4), dtype=torch.float32, device=dev)
        self.offsets = torch.empty(G + 1, dtype=torch.int32, device=dev)
        self.entries = torch.empty(max(4 * Nv, 1), dtype=torch.int32, device=dev)
        ws = workspace(_lib.lib().s2c_lbs_bind_workspace_size(Nv, G), dev)
        call("s2c_lbs_bind", Nv, ptr(x), G, ptr(g), float(tau), ptr(self.idx), ptr(self.w), ptr(self.offsets),
             ptr(self.entries), ptr(ws), ws.numel(), _lib.stream_of(x))


class _LBSFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, M, binding: LBSBinding):
        y = torch.empty_like(x)
        call("s2c_lbs_forward", binding.num_verts, ptr(x), ptr(binding.idx), ptr(binding.w), binding.num_guides,
             ptr(M), ptr(y), _lib.stream_of(x))
        ctx.binding = binding
        ctx.save_for_backward(x, M)
        return y

    @staticmethod
    def backward(ctx, gy):
        x, M = ctx.saved_tensors
        b = ctx.binding
        gy = gy.contiguous()
        dM = torch.empty_like(M) if ctx.needs_input_grad[1] else None
        dx = torch.empty_like(x) if ctx.needs_input_grad[0] else None
        call("s2c_lbs_backward", b.num_verts, ptr(x), ptr(b.idx), ptr(b.w), b.num_guides, ptr(M), ptr(b.offsets),
             ptr(b.entries), ptr(gy), ptr(dM), ptr(dx), _lib.stream_of(gy))
        return dx, dM, None


def lbs(x: torch.Tensor, M: torch.Tensor, binding: LBSBinding) -> torch.Tensor:
    """y (Nv, 3) = sum over the 4 bound guides of w_k (A_k x + t_k); ``M`` (G, 3, 4)."""
    if not (x.is_cuda and M.is_cuda):
        raise ValueError("lbs: tensors must be on CUDA.")
    x = x.reshape(-1, 3).contiguous()
    if x.shape[0] != binding.num_verts or tuple(M.shape) != (binding.num_guides, 3, 4):
        raise ValueError("lbs: x must be (Nv, 3) and M (G, 3, 4) as bound.")
    return _LBSFn.apply(x, M.contiguous(), binding)
