"""Software-MSAA texture render of a wisp's tube mesh (the per-wisp sample loop of the
reference's ``render_texture``, ``texture_utils.py:106-288``).

The reference rasterises the mesh 64 times, once per jitter of an 8 x 8 grid over two
pixels, interpolates the vertex attribute (tangents) each time and accumulates
``rgb * valid``, ``valid`` and ``weight * valid`` with Mitchell-Netravali weights: about
five launches per sample.  Here the 64 jitters are the views of one fused raster launch
and one resolve kernel interpolates and accumulates all samples per pixel, in the same
order with the same FP32 operations, so the sums are identical to the loop's.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from .rasterize import interpolate_triangle_attributes, rasterize, rasterize_fused


def mitchell_netravali(x, B=1.0 / 3.0, C=1.0 / 3.0):
    """The reference's filter (texture_utils.py:182-195)."""
    ax = np.abs(x)
    x2, x3 = ax ** 2, ax ** 3
    c1 = ax < 1
    c2 = (ax >= 1) & (ax < 2)
    return (((12 - 9 * B - 6 * C) * x3 + (-18 + 12 * B + 6 * C) * x2 + (6 - 2 * B)) * c1 +
            ((-B - 6 * C) * x3 + (6 * B + 30 * C) * x2 + (-12 * B - 48 * C) * ax + (8 * B + 24 * C)) * c2) / 6.0


def msaa_pattern(grid_res: int = 8, span: float = 2.0) -> Tuple[List[Tuple[float, float]], List[float]]:
    """Sample offsets (pixels) and normalised weights (texture_utils.py:199-211)."""
    g = span * ((np.arange(grid_res) + 0.5) / grid_res - 0.5)
    offsets = [(dx, dy) for dy in g for dx in g]
    w = np.array([mitchell_netravali(dx) * mitchell_netravali(dy) for dx, dy in offsets])
    w /= w.sum()
    return offsets, w.tolist()


def _jittered(pos: torch.Tensor, offsets: Sequence[Tuple[float, float]], H: int, W: int) -> torch.Tensor:
    # the reference adds the NDC offset (a Python float, applied in float32) to x and y
    off = torch.tensor([[dx * 2.0 / W, dy * 2.0 / H] for dx, dy in offsets], dtype=torch.float32, device=pos.device)
    S, V = len(offsets), pos.shape[0]
    out = torch.empty((S, V, 4), dtype=torch.float32, device=pos.device)
    out[..., :2] = pos[None, :, :2] + off[:, None, :]
    out[..., 2] = pos[None, :, 2]
    out[..., 3] = 1.0
    return out


def msaa_render(resolution: Tuple[int, int], pos: torch.Tensor, tri: torch.Tensor, attr: torch.Tensor,
                offsets: Sequence[Tuple[float, float]], weights: Sequence[float]):
    """(acc_rgb (H, W, C), valid_count (H, W), acc_alpha (H, W)) of the sample loop, batched:
    one fused raster over all jitters and one resolve launch."""
    if not (pos.is_cuda and tri.is_cuda and attr.is_cuda):
        raise ValueError("msaa_render: tensors must be on CUDA.")
    H, W = resolution
    p = pos.float().reshape(-1, 3).contiguous()
    t = tri.contiguous()
    a = attr.float().contiguous()
    rast, _ = rasterize_fused((H, W), _jittered(p, offsets, H, W), t)
    C = a.shape[1]
    acc = torch.empty((H, W, C), dtype=torch.float32, device=p.device)
    cnt = torch.empty((H, W), dtype=torch.float32, device=p.device)
    alpha = torch.empty((H, W), dtype=torch.float32, device=p.device)
    w = torch.tensor(weights, dtype=torch.float32, device=p.device)
    _lib.call("s2c_msaa_resolve", len(offsets), H, W, C, _lib.ptr(rast), a.shape[0], _lib.ptr(a), t.shape[0],
              _lib.ptr(t), _lib.ptr(w), _lib.ptr(acc), _lib.ptr(cnt), _lib.ptr(alpha), _lib.stream_of(p))
    return acc, cnt, alpha


def msaa_render_loop(resolution: Tuple[int, int], pos: torch.Tensor, tri: torch.Tensor, attr: torch.Tensor,
                     offsets: Sequence[Tuple[float, float]], weights: Sequence[float]):
    """The reference's per-sample loop (texture_utils.py:213-226) over the drop-in ops."""
    H, W = resolution
    acc = torch.zeros((H, W, attr.shape[1]), device=pos.device)
    cnt = torch.zeros((H, W), device=pos.device)
    alpha = 0
    for i, (dx, dy) in enumerate(offsets):
        pj = pos.clone()
        pj[:, 0] += dx * 2.0 / W
        pj[:, 1] += dy * 2.0 / H
        ph = torch.cat([pj, torch.ones_like(pos[:, :1])], dim=-1)
        rast = rasterize((H, W), ph[None], tri)
        rgb = interpolate_triangle_attributes(rast, attr, tri)[0]
        valid = (rast[0, ..., -1] > 0).float()
        acc += rgb * valid[..., None]
        cnt += valid
        alpha = alpha + weights[i] * valid
    return acc, cnt, alpha


def resolve_patch(acc: torch.Tensor, cnt: torch.Tensor):
    """Mean attribute of the valid samples, (0, 1, 0) where none (texture_utils.py:228-233),
    mapped to [0, 1] as 0.5 (rgb + 1)."""
    rgb = acc / cnt.clamp(min=1)[..., None]
    rgb[cnt <= 0] = torch.tensor([0.0, 1.0, 0.0], device=acc.device)
    return 0.5 * (rgb + 1.0)
