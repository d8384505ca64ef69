"""Strand curve operators with the reference's ``pystrns2cards.curve_utils`` signatures:
``compute_arclength``, ``smooth_strands``, ``skinning`` (``curve_utils.py:167-240``), the
frame helpers ``minimal_rotation``, ``tangent_frame``, ``compute_bishop_frame``,
``compute_aligned_strands``, ``compute_alignment_rotation`` (``:9-165, 243-308``), the wisp
aligners ``align_wisps`` / ``align_wisp`` (``:376-607``) and ``strands_to_tube`` (``:310-374``).

``smooth_strands`` and ``skinning`` run as one launch each: the kernel computes the
arclength of the strands it stages instead of reading a separately computed tensor.
The rotation-minimising frame is one thread per strand walking the double-reflection
recurrence (the reference loops over the points in Python); its alignment rotations and
canonical handles come out of the same pass.  ``align_wisps`` is two launches for all
wisps together -- the per-wisp frames (one CTA per wisp, a 3x3 eigen-solve in place of the
host SVD), then smoothing, rotation, frames + canonical handles and skinning fused, one
warp per strand -- with no host synchronisation (the reference runs a Python loop over
wisps with a host SVD each, and a Python loop over the points for the frames).
"""
from __future__ import annotations

from typing import List, Tuple

import numpy as np
import torch

from . import _core

# the wisp target frame of align_wisps (curve_utils.py:502-504)
WISP_T_DST = (0.0, 1.0, 0.0)
WISP_N_DST = (0.0, 0.0, -1.0)
WISP_B_DST = (-1.0, 0.0, 0.0)


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


def _check_strands(strands: torch.Tensor, name: str):
    if not strands.is_cuda:
        raise ValueError(f"{name}: Input tensor must be on CUDA.")
    if strands.ndim != 3 or strands.shape[-1] != 3:
        raise ValueError(f"{name}: strands must have shape (N, V, 3)")
    return strands.float().contiguous()


def _t_dst(T_dst: torch.Tensor, name: str) -> Tuple[float, float, float]:
    if T_dst.ndim != 2 or tuple(T_dst.shape) != (1, 3):
        raise ValueError(f"{name}: T_dst must have shape (1, 3)")
    return tuple(float(x) for x in T_dst.detach().reshape(3).cpu().tolist())


def minimal_rotation(T_src: torch.Tensor, T_dst: torch.Tensor) -> torch.Tensor:
    """Rotation matrices (*, 3, 3) taking T_src onto T_dst (Rodrigues; identity when
    parallel, diag(-1, -1, 1) when antiparallel), ``curve_utils.py:9-74``.  Elementwise
    tensor arithmetic on the inputs' device."""
    s = T_src.float()
    d = T_dst.float().expand_as(s)
    s = s / s.norm(dim=-1, keepdim=True).clamp(min=1e-8)
    d = d / d.norm(dim=-1, keepdim=True).clamp(min=1e-8)
    ax = torch.cross(s, d, dim=-1)
    sn = ax.norm(dim=-1)
    cs = (s * d).sum(-1).clamp(-1.0, 1.0)
    ax = ax / sn.clamp(min=1e-8)[..., None]
    x, y, z = ax.unbind(-1)
    o = torch.zeros_like(x)
    K = torch.stack([o, -z, y, z, o, -x, -y, x, o], -1).reshape(*ax.shape[:-1], 3, 3)
    eye = torch.eye(3, device=s.device, dtype=s.dtype)
    R = eye + sn[..., None, None] * K + (1.0 - cs)[..., None, None] * (K @ K)
    R = torch.where((cs > 1 - 1e-6)[..., None, None], eye, R)
    flip = torch.diag(torch.tensor([-1.0, -1.0, 1.0], device=s.device))
    return torch.where((cs < -1 + 1e-6)[..., None, None], flip, R)


def tangent_frame(tangent: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
    """(normal, binormal) of the branch-free orthonormal basis around ``tangent``
    (``curve_utils.py:76-102``)."""
    t = tangent / tangent.norm(dim=-1, keepdim=True).clamp(min=1e-8)
    x, y, z = t.unbind(-1)
    sign = torch.where(z < 0, -1.0, 1.0).to(t.dtype)
    a = -1.0 / (sign + z)
    b = x * y * a
    return (torch.stack([1.0 + sign * x * x * a, sign * b, -sign * x], -1),
            torch.stack([b, sign + y * y * a, -y], -1))


def compute_bishop_frame(strands: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """Rotation-minimising frame (T, N, B), each (N, S, 3), by double reflection
    (``curve_utils.py:104-165``); one thread per strand."""
    s = _check_strands(strands, "compute_bishop_frame")
    T, N, B = torch.empty_like(s), torch.empty_like(s), torch.empty_like(s)
    _core.strand_frames(s, T=T, N=N, B=B)
    return T, N, B


def compute_aligned_strands(strands: torch.Tensor, roots: torch.Tensor, T_dst: torch.Tensor) -> torch.Tensor:
    """Strands straightened along T_dst from the given roots: arclength * T_dst + root
    (``curve_utils.py:243-271``)."""
    s = _check_strands(strands, "compute_aligned_strands")
    if roots.ndim != 2 or roots.shape[-1] != 3:
        raise ValueError("roots must have shape (N, 3)")
    td = _t_dst(T_dst, "compute_aligned_strands")
    r = roots.float()
    if r.stride(-1) != 1:
        r = r.contiguous()
    out = torch.empty_like(s)
    _core.strand_frames(s, t_dst=td, roots=r, canon=out)
    return out


def compute_alignment_rotation(strands: torch.Tensor, T_dst: torch.Tensor) -> torch.Tensor:
    """Per-point rotations (N, V, 3, 3) taking each point's Bishop frame to the root frame
    turned onto T_dst (``curve_utils.py:273-308``)."""
    s = _check_strands(strands, "compute_alignment_rotation")
    td = _t_dst(T_dst, "compute_alignment_rotation")
    R = torch.empty((*s.shape[:2], 3, 3), dtype=torch.float32, device=s.device)
    _core.strand_frames(s, t_dst=td, R=R)
    return R


def align_wisps(wisps: List, beta: float) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """Align every wisp to the canonical orientation (``curve_utils.py:481-607``).

    ``wisps``: list of (N_i, V, 3) arrays (numpy or torch), one per wisp.  Returns the
    aligned strands (N, V, 3), the smoothed strands before alignment (N, V, 3) and the
    global index of each wisp's longest strand (int64), on the GPU.  The per-wisp frame
    takes the least-variance axis of the wisp's centred roots from an FP32 Jacobi eigen-solve
    of their second moment (the reference's host SVD gives the same axis up to sign, and the
    frame fixes the sign); below 3 strands the axes are the identity's, as there."""
    dev = torch.device("cuda")
    parts, sizes = [], []
    for w in wisps:
        x = w if isinstance(w, torch.Tensor) else torch.from_numpy(np.asarray(w))
        if x.ndim != 3 or x.shape[-1] != 3:
            raise ValueError("Input tensor must have shape (N, V, 3)")
        if x.shape[0] == 0:
            raise RuntimeError("align_wisps: a wisp has no strands")
        parts.append(x)
        sizes.append(int(x.shape[0]))
    if not parts:
        raise RuntimeError("align_wisps: no wisps")
    V = int(parts[0].shape[1])
    if any(int(x.shape[1]) != V for x in parts):
        raise RuntimeError("align_wisps: wisps differ in points per strand")
    strands = torch.cat([x.to(dev, dtype=torch.float32, non_blocking=True) for x in parts], 0).contiguous()
    return align_wisps_packed(strands, torch.tensor(sizes, dtype=torch.int64), beta)


def align_wisps_packed(strands: torch.Tensor, wisp_sizes: torch.Tensor, beta: float):
    """``align_wisps`` on strands already on the device, wisp w being the next
    ``wisp_sizes[w]`` strands (a host tensor or sequence of sizes, all > 0).  Two launches:
    the per-wisp frames, then smoothing, rotation, frames and skinning of every strand
    fused (strands longer than the fused kernel stages take the same steps one launch
    each, with the same results)."""
    s = _check_strands(strands, "align_wisps")
    S, V, _ = s.shape
    sizes = torch.as_tensor(wisp_sizes, dtype=torch.int64).cpu()
    K = int(sizes.numel())
    if K == 0 or int(sizes.min()) <= 0 or int(sizes.sum()) != S:
        raise RuntimeError("align_wisps: wisp sizes must be positive and add up to the strands")
    if V < 2:
        raise RuntimeError("align_wisps: strands need at least 2 points")
    dev = s.device
    offs = torch.zeros(K + 1, dtype=torch.int32)
    offs[1:] = torch.cumsum(sizes, 0).to(torch.int32)
    offs = offs.pin_memory().to(dev, non_blocking=True)
    Rg = torch.empty((K, 3, 3), dtype=torch.float32, device=dev)
    centre = torch.empty((K, 3), dtype=torch.float32, device=dev)
    longest = torch.empty(K, dtype=torch.int32, device=dev)
    _core.wisp_frames(offs, s, WISP_T_DST, WISP_N_DST, WISP_B_DST, Rg, centre, longest)
    if V <= _core.align_strands_max_points():
        handles_orig, aligned = torch.empty_like(s), torch.empty_like(s)
        _core.align_strands(s, offs, Rg, centre, WISP_T_DST, beta, handles_orig, aligned)
    else:
        aligned, handles_orig = _align_strands_unfused(s, offs, Rg, centre, beta)
    return aligned, handles_orig, longest.to(torch.int64)


def _align_strands_unfused(s, offs, Rg, centre, beta):
    """The steps of the fused align_strands as separate launches: smoothing, rotation into
    the wisp frames, frames + canonical handles of the rotated handles, skinning."""
    S, V, _ = s.shape
    handles_orig = smooth_strands(s, beta)
    s_rot, h_rot = torch.empty_like(s), torch.empty_like(s)
    _core.wisp_rotate(offs, Rg, centre, s, handles_orig, s_rot, h_rot)
    canon = torch.empty_like(s)
    R_local = torch.empty((S, V, 3, 3), dtype=torch.float32, device=s.device)
    _core.strand_frames(h_rot, t_dst=WISP_T_DST, R=R_local, roots=s_rot[:, 0], canon=canon)
    aligned = torch.empty_like(s)
    _core.skinning(s_rot, None, h_rot, canon, R_local, aligned, beta)
    return aligned, handles_orig


def align_wisp(strands: torch.Tensor, beta: float) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """Align one wisp (``curve_utils.py:376-479``): root-centred strands turned so that the
    longest smoothed strand's root direction, projected off the roots' principal axis,
    maps to (0, -1, 0); returns the aligned strands, the smoothed strands in the aligned
    frame and the index of the longest strand.  The principal axis comes from an FP64
    eigen-solve of the roots' second moment on the device (the reference: host SVD; the
    projection does not depend on the axis' sign)."""
    s = _check_strands(strands, "align_wisp")
    S, V, _ = s.shape
    if S == 0 or V < 3:
        raise RuntimeError("align_wisp: need at least one strand of 3 points")
    s = s - s[:, 0].mean(0, keepdim=True)
    r = s[:, 0].double()
    if S >= 2:
        evals, evecs = torch.linalg.eigh(r.T @ r)
        pa = evecs[:, 2].float()
    else:
        pa = torch.tensor([1.0, 0.0, 0.0], device=s.device)
    lengths = (s[:, 1:] - s[:, :-1]).norm(dim=2).sum(1)
    li = torch.argmax(lengths)
    handles = smooth_strands(s, beta)
    g = handles[li]
    t0, t1 = g[1] - g[0], g[2] - g[1]
    t0 = t0 - torch.dot(t0, pa) * pa
    t1 = t1 - torch.dot(t1, pa) * pa
    t0 = t0 / t0.norm()
    t1 = t1 / t1.norm()
    b0 = torch.cross(t0, t1, dim=-1)
    b0 = b0 / b0.norm()
    n0 = torch.cross(b0, t0, dim=-1)
    n0 = n0 / n0.norm()
    ok = torch.isfinite(n0).all() & torch.isfinite(b0).all()
    nf, bf = tangent_frame(t0[None])
    n0 = torch.where(ok, n0, nf[0])
    b0 = torch.where(ok, b0, bf[0])
    Rsrc = torch.stack([t0, n0, b0], -1)
    Rdst = torch.tensor([[0.0, 0.0, 1.0], [-1.0, 0.0, 0.0], [0.0, -1.0, 0.0]], device=s.device)
    Rg = Rdst @ Rsrc.T
    s = (s.reshape(-1, 3) @ Rg.T).reshape(S, V, 3).contiguous()
    handles = (handles.reshape(-1, 3) @ Rg.T).reshape(S, V, 3).contiguous()
    td = (0.0, -1.0, 0.0)
    canon = torch.empty_like(s)
    R_local = torch.empty((S, V, 3, 3), dtype=torch.float32, device=s.device)
    _core.strand_frames(handles, t_dst=td, R=R_local, roots=s[:, 0], canon=canon)
    aligned = torch.empty_like(s)
    _core.skinning(s, None, handles, canon, R_local, aligned, beta)
    return aligned, handles, li


def strands_to_tube(strands, radius=1.0, n_circle=8, attr=None):
    """Open tube mesh around every strand with the rotation-minimising frame
    (``curve_utils.py:310-374``): verts (N*S*n_circle, 3), faces (M, 3) int32 and, given
    ``attr`` (N, S, C), the per-vertex attributes.  numpy in, numpy out, as the reference;
    the frame is computed on the GPU."""
    st = np.asarray(strands)
    assert st.ndim == 3 and st.shape[2] == 3, f"Expected (N, S, 3), got {st.shape}"
    N, S, _ = st.shape
    x = torch.from_numpy(np.ascontiguousarray(st, dtype=np.float32)).cuda()
    _, Nn, Bn = compute_bishop_frame(x)
    th = np.linspace(0, 2 * np.pi, n_circle, endpoint=False)
    c = torch.from_numpy(np.cos(th)).to(x.device)
    sn = torch.from_numpy(np.sin(th)).to(x.device)
    dirs = c[None, None, :, None] * Nn[:, :, None, :].double() + sn[None, None, :, None] * Bn[:, :, None, :].double()
    verts = torch.from_numpy(np.asarray(st, np.float64)).to(x.device)[:, :, None, :] + radius * dirs
    verts = verts.reshape(N * S * n_circle, 3).cpu().numpy()
    idx = np.arange(S * n_circle).reshape(S, n_circle)
    a, b = idx[:-1], np.roll(idx[:-1], -1, axis=1)
    cc, d = idx[1:], np.roll(idx[1:], -1, axis=1)
    faces = np.stack([np.stack([a, cc, d], -1), np.stack([a, d, b], -1)], 0).reshape(-1, 3)
    faces = (faces[None] + (np.arange(N) * S * n_circle)[:, None, None]).reshape(-1, 3).astype(np.int32)
    if attr is None:
        return verts, faces
    attr = np.asarray(attr)
    assert attr.shape[:2] == (N, S), f"Expected attr shape (N, S, C), got {attr.shape}"
    return verts, faces, np.repeat(attr[:, :, None, :], n_circle, axis=2).reshape(N * S * n_circle, -1)
