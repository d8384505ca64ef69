"""Drop-in for the reference's compiled ``pystrns2cards._core`` module.

Each function keeps the name, argument order, dtype/shape contract and return value of
the corresponding ``m.def`` in ``pystrns2cards/src/pystrns2cards.cpp`` and forwards to
the C ABI of libs2c.so (include/s2c.h) on the tensor's current CUDA stream.  Argument
type errors raise TypeError (as nanobind does), validation failures RuntimeError, like
the reference's ``std::runtime_error``.  Temporaries come from the torch caching
allocator as workspace; the C side never allocates.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import call, ptr, workspace

_f32, _i32 = torch.float32, torch.int32


def _arr(t, dtype, ndim=None, last=None, name="array"):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name}: expected a torch.Tensor, got {type(t).__name__}")
    if t.dtype != dtype:
        raise TypeError(f"{name}: expected dtype {dtype}, got {t.dtype}")
    if ndim is not None and t.ndim != ndim:
        raise TypeError(f"{name}: expected {ndim} dimensions, got {t.ndim}")
    if last is not None and t.shape[-1] != last:
        raise TypeError(f"{name}: expected last dimension {last}, got {t.shape[-1]}")
    if not t.is_contiguous():
        raise TypeError(f"{name}: expected a C-contiguous tensor")
    return t


def _cuda(*ts, msg="All tensors must be CUDA tensors."):
    for t in ts:
        if t is not None and not t.is_cuda:
            raise RuntimeError(msg)


def _stream(t):
    return _lib.stream_of(t)


def print_version():
    print(f"strns2cards_gb300 C ABI version {_lib.lib().s2c_version()}")


# ---- DDA (pystrns2cards.cpp:531-611) -------------------------------------------------
def dda_compute_span(edge_ids, H, W, pos, edges, frag_prefix_sum, frag_slopes, frag_spans) -> int:
    _arr(edge_ids, _i32, 1, name="edge_ids")
    _arr(pos, _f32, 3, 4, "pos")
    _arr(edges, _i32, 2, 2, "edges")
    _arr(frag_prefix_sum, _i32, 1, name="frag_prefix_sum")
    _arr(frag_slopes, _f32, 2, 2, "frag_slopes")
    _arr(frag_spans, _f32, 2, 4, "frag_spans")
    _cuda(edge_ids, pos, edges, frag_prefix_sum, frag_slopes, frag_spans)
    P = edge_ids.shape[0]
    B, V, _ = pos.shape
    E = edges.shape[0]
    if frag_prefix_sum.shape[0] != P or frag_slopes.shape[0] != P or frag_spans.shape[0] != P:
        raise RuntimeError("Invalid output tensor shapes for frag_prefix_sum, frag_slopes, or frag_spans.")
    L = _lib.lib()
    ws = workspace(L.s2c_dda_compute_span_workspace_size(P), pos.device)
    n = _lib.i64_out()
    call("s2c_dda_compute_span", P, ptr(edge_ids), int(H), int(W), B, V, ptr(pos), E, ptr(edges),
         ptr(frag_prefix_sum), ptr(frag_slopes), ptr(frag_spans), ptr(ws), ws.numel(), ctypes.byref(n),
         _stream(pos))
    return int(n.value)


def dda_compute_fragments(frag_prefix_sum, edge_ids, frag_slopes, frag_spans, H, W, pos, edges, frag_pix,
                          frag_attrs) -> None:
    _arr(frag_prefix_sum, _i32, 1, name="frag_prefix_sum")
    _arr(edge_ids, _i32, 1, name="edge_ids")
    _arr(frag_slopes, _f32, 2, 2, "frag_slopes")
    _arr(frag_spans, _f32, 2, 4, "frag_spans")
    _arr(pos, _f32, 3, 4, "pos")
    _arr(edges, _i32, 2, 2, "edges")
    _arr(frag_pix, _i32, 2, 3, "frag_pix")
    _arr(frag_attrs, _f32, 2, 4, "frag_attrs")
    _cuda(frag_prefix_sum, edge_ids, frag_slopes, frag_spans, pos, edges, frag_pix, frag_attrs)
    F = frag_pix.shape[0]
    P = edge_ids.shape[0]
    if (frag_prefix_sum.shape[0] != P or frag_slopes.shape[0] != P or frag_spans.shape[0] != P
            or frag_attrs.shape[0] != F):
        raise RuntimeError("Invalid shape for input or output arrays.")
    B, V, _ = pos.shape
    call("s2c_dda_compute_fragments", P, F, ptr(frag_prefix_sum), ptr(edge_ids), ptr(frag_slopes), ptr(frag_spans),
         int(H), int(W), B, V, ptr(pos), edges.shape[0], ptr(edges), ptr(frag_pix), ptr(frag_attrs), _stream(pos))


def dda_compact_fragments(frag_prefix_sum, edge_ids, frag_slopes, frag_spans, H, W, pos, edges, num_steps):
    """The compacted DDA fragment list (``filter_valid_fragments`` of ``dda_compute_fragments``'s
    raw list, same order and values) in two passes without the raw list: (frag_pix, frag_attrs)."""
    _arr(frag_prefix_sum, _i32, 1, name="frag_prefix_sum")
    _arr(edge_ids, _i32, 1, name="edge_ids")
    _arr(frag_slopes, _f32, 2, 2, "frag_slopes")
    _arr(frag_spans, _f32, 2, 4, "frag_spans")
    _arr(pos, _f32, 3, 4, "pos")
    _arr(edges, _i32, 2, 2, "edges")
    _cuda(frag_prefix_sum, edge_ids, frag_slopes, frag_spans, pos, edges)
    P = edge_ids.shape[0]
    if frag_prefix_sum.shape[0] != P or frag_slopes.shape[0] != P or frag_spans.shape[0] != P:
        raise RuntimeError("Invalid shape for input arrays.")
    B, V, _ = pos.shape
    F = int(num_steps)
    ws = workspace(_lib.lib().s2c_dda_count_fragments_workspace_size(F), pos.device)
    args = (P, F, ptr(frag_prefix_sum), ptr(edge_ids), ptr(frag_slopes), ptr(frag_spans), int(H), int(W), B, V,
            ptr(pos), edges.shape[0], ptr(edges), ptr(ws), ws.numel())
    n = _lib.i64_out()
    call("s2c_dda_count_fragments", *args, ctypes.byref(n), _stream(pos))
    N = int(n.value)
    frag_pix = torch.empty((N, 3), dtype=torch.int32, device=pos.device)
    frag_attrs = torch.empty((N, 4), dtype=torch.float32, device=pos.device)
    if N:
        call("s2c_dda_write_fragments", *args, ptr(frag_pix), ptr(frag_attrs), _stream(pos))
    return frag_pix, frag_attrs


# ---- fragments (pystrns2cards.cpp:358-392, 440-478) ----------------------------------
def filter_valid_fragments(frag_pix, frag_attrs, frag_pix_out, frag_attrs_out) -> int:
    for t, d, last, nm in ((frag_pix, _i32, 3, "frag_pix"), (frag_attrs, _f32, 4, "frag_attrs"),
                           (frag_pix_out, _i32, 3, "frag_pix_out"), (frag_attrs_out, _f32, 4, "frag_attrs_out")):
        _arr(t, d, 2, last, nm)
    _cuda(frag_pix, frag_attrs, frag_pix_out, frag_attrs_out, msg="All tensors must be CUDA tensors (device_id >= 0).")
    F = frag_pix.shape[0]
    if frag_attrs.shape[0] != F or frag_pix_out.shape[0] != F or frag_attrs_out.shape[0] != F:
        raise RuntimeError("Mismatch in fragment counts between input/output tensors.")
    if F == 0:
        return 0
    L = _lib.lib()
    ws = workspace(L.s2c_filter_valid_fragments_workspace_size(F), frag_pix.device)
    n = _lib.i64_out()
    call("s2c_filter_valid_fragments", F, ptr(frag_pix), ptr(frag_attrs), ptr(frag_pix_out), ptr(frag_attrs_out),
         ptr(ws), ws.numel(), ctypes.byref(n), _stream(frag_pix))
    return int(n.value)


def cluster_mask_from_fragments(frag_pix, frag_attrs, prim2cluster, bitset) -> None:
    _arr(frag_pix, _i32, 2, 3, "frag_pix")
    _arr(frag_attrs, _f32, 2, 4, "frag_attrs")
    _arr(prim2cluster, _i32, 1, name="prim2cluster")
    _arr(bitset, _i32, 4, name="bitset")
    _cuda(frag_pix, frag_attrs, prim2cluster, bitset, msg="All tensors must be CUDA tensors (device_id >= 0).")
    F = frag_pix.shape[0]
    if frag_attrs.shape[0] != F:
        raise RuntimeError("frag_pix and frag_attrs must have the same number of fragments.")
    B, H, W, S = bitset.shape
    call("s2c_cluster_mask_from_fragments", F, ptr(frag_pix), ptr(frag_attrs), ptr(prim2cluster),
         prim2cluster.shape[0], B, H, W, S, ptr(bitset), _stream(bitset))


# ---- triangles (pystrns2cards.cpp:245-438) --------------------------------------------
def compute_triangle_rects(H, W, pos, tri, triangle_rects, frag_prefix_sum) -> int:
    _arr(pos, _f32, 3, 4, "pos")
    _arr(tri, _i32, 2, 3, "tri")
    _arr(triangle_rects, _i32, 2, 4, "triangle_rects")
    _arr(frag_prefix_sum, _i32, 1, name="frag_prefix_sum")
    _cuda(pos, tri, triangle_rects, frag_prefix_sum, msg="All tensors must be CUDA tensors (device_id >= 0).")
    B, V, _ = pos.shape
    T = tri.shape[0]
    if triangle_rects.shape[0] != B * T:
        raise RuntimeError("`triangle_rects` must have shape [B * T, 4].")
    if frag_prefix_sum.shape[0] != B * T:
        raise RuntimeError("`frag_prefix_sum` must have shape [B * T].")
    L = _lib.lib()
    ws = workspace(L.s2c_compute_triangle_rects_workspace_size(B, T), pos.device)
    n = _lib.i64_out()
    call("s2c_compute_triangle_rects", int(H), int(W), B, V, ptr(pos), T, ptr(tri), ptr(triangle_rects),
         ptr(frag_prefix_sum), ptr(ws), ws.numel(), ctypes.byref(n), _stream(pos))
    return int(n.value)


def compute_fragments(H, W, pos, tri, frag_prefix_sum, triangle_rects, frag_pix, frag_attrs) -> None:
    _arr(pos, _f32, 3, 4, "pos")
    _arr(tri, _i32, 2, 3, "tri")
    _arr(frag_prefix_sum, _i32, 1, name="frag_prefix_sum")
    _arr(triangle_rects, _i32, 2, 4, "triangle_rects")
    _arr(frag_pix, _i32, 2, 3, "frag_pix")
    _arr(frag_attrs, _f32, 2, 4, "frag_attrs")
    _cuda(pos, tri, frag_prefix_sum, triangle_rects, frag_pix, frag_attrs,
          msg="All tensors must be CUDA tensors (device_id >= 0).")
    B, V, _ = pos.shape
    T = tri.shape[0]
    F = frag_pix.shape[0]
    if frag_attrs.shape[0] != F or frag_prefix_sum.shape[0] != B * T:
        raise RuntimeError("Mismatch in fragment count or prefix sum length.")
    call("s2c_compute_fragments", int(H), int(W), B, V, ptr(pos), T, ptr(tri), ptr(frag_prefix_sum),
         ptr(triangle_rects), F, ptr(frag_pix), ptr(frag_attrs), _stream(pos))


def compact_fragments(H, W, pos, tri, frag_prefix_sum, triangle_rects, num_bbox_pixels):
    """The compacted fragment list (``filter_valid_fragments`` of ``compute_fragments``'s raw
    list, same order and values) in two passes without the raw list: (frag_pix, frag_attrs)."""
    _arr(pos, _f32, 3, 4, "pos")
    _arr(tri, _i32, 2, 3, "tri")
    _arr(frag_prefix_sum, _i32, 1, name="frag_prefix_sum")
    _arr(triangle_rects, _i32, 2, 4, "triangle_rects")
    _cuda(pos, tri, frag_prefix_sum, triangle_rects, msg="All tensors must be CUDA tensors (device_id >= 0).")
    B, V, _ = pos.shape
    T = tri.shape[0]
    if frag_prefix_sum.shape[0] != B * T or triangle_rects.shape[0] != B * T:
        raise RuntimeError("Mismatch in prefix sum or rectangle count.")
    F = int(num_bbox_pixels)
    ws = workspace(_lib.lib().s2c_count_fragments_workspace_size(F), pos.device)
    n = _lib.i64_out()
    args = (int(H), int(W), B, V, ptr(pos), T, ptr(tri), ptr(frag_prefix_sum), ptr(triangle_rects), F, ptr(ws),
            ws.numel())
    call("s2c_count_fragments", *args, ctypes.byref(n), _stream(pos))
    N = int(n.value)
    frag_pix = torch.empty((N, 3), dtype=torch.int32, device=pos.device)
    frag_attrs = torch.empty((N, 4), dtype=torch.float32, device=pos.device)
    if N:
        call("s2c_write_fragments", *args, ptr(frag_pix), ptr(frag_attrs), _stream(pos))
    return frag_pix, frag_attrs


def depth_test(H, W, frag_pix, frag_attrs, rast_out) -> None:
    _arr(frag_pix, _i32, 2, 3, "frag_pix")
    _arr(frag_attrs, _f32, 2, 4, "frag_attrs")
    _arr(rast_out, _f32, 4, 4, "rast_out")
    _cuda(frag_pix, frag_attrs, rast_out, msg="All tensors must be on a CUDA device (device_id >= 0)")
    F = frag_pix.shape[0]
    B = rast_out.shape[0]
    if frag_attrs.shape[0] != F:
        raise RuntimeError("frag_attrs must match frag_pix in size.")
    if rast_out.shape[1] != H or rast_out.shape[2] != W:
        raise RuntimeError("rast_out must have shape (B, H, W, 4).")
    L = _lib.lib()
    ws = workspace(L.s2c_depth_test_workspace_size(B, int(H), int(W)), rast_out.device)
    call("s2c_depth_test", B, int(H), int(W), F, ptr(frag_pix), ptr(frag_attrs), ptr(rast_out), ptr(ws), ws.numel(),
         _stream(rast_out))


def interpolate_triangle_attributes(rast, attr, tri, image) -> None:
    _arr(rast, _f32, 4, 4, "rast")
    _arr(attr, _f32, 2, name="attr")
    _arr(tri, _i32, 2, 3, "tri")
    _arr(image, _f32, 4, name="image")
    _cuda(rast, attr, tri, image, msg="All tensors must be on a CUDA device")
    B, H, W, _ = rast.shape
    V, C = attr.shape
    call("s2c_interpolate_triangle_attributes", B, H, W, C, ptr(rast), V, ptr(attr), tri.shape[0], ptr(tri), ptr(image),
         _stream(rast))


def backward_interpolate_triangle_attributes(rast, d_image, tri, d_attr) -> None:
    _arr(rast, _f32, 4, 4, "rast")
    _arr(d_image, _f32, 4, name="d_image")
    _arr(tri, _i32, 2, 3, "tri")
    _arr(d_attr, _f32, 2, name="d_attr")
    _cuda(rast, d_image, tri, d_attr, msg="All tensors must be on a CUDA device")
    B, H, W, _ = rast.shape
    V, C = d_attr.shape
    # FP64 sums of the exact FP32 products, rounded once into d_attr
    acc = torch.empty(V * C, dtype=torch.float64, device=d_attr.device)
    call("s2c_backward_interpolate_triangle_attributes", B, H, W, C, ptr(rast), ptr(d_image), tri.shape[0], ptr(tri), V,
         ptr(d_attr), ptr(acc), _stream(rast))


def dda_interpolate_attributes(rast_dda, attr, edges, image) -> None:
    _arr(rast_dda, _f32, 4, 4, "rast_dda")
    _arr(attr, _f32, 2, name="attr")
    _arr(edges, _i32, 2, 2, "edges")
    _arr(image, _f32, 4, name="image")
    _cuda(rast_dda, attr, edges, image, msg="All arrays must be CUDA tensors.")
    B, H, W, _ = rast_dda.shape
    V, C = attr.shape
    if tuple(image.shape) != (B, H, W, C):
        raise RuntimeError("image must have shape [B, H, W, C]")
    call("s2c_dda_interpolate_attributes", B, H, W, C, ptr(rast_dda), V, ptr(attr), edges.shape[0], ptr(edges),
         ptr(image), _stream(rast_dda))


def backward_dda_interpolate_attributes(rast_dda, d_image, edges, d_attr) -> None:
    _arr(rast_dda, _f32, 4, 4, "rast_dda")
    _arr(d_image, _f32, 4, name="d_image")
    _arr(edges, _i32, 2, 2, "edges")
    _arr(d_attr, _f32, 2, name="d_attr")
    _cuda(rast_dda, d_image, edges, d_attr, msg="All tensors must be on CUDA.")
    B, H, W, _ = rast_dda.shape
    C = d_image.shape[3]
    if tuple(d_image.shape[:3]) != (B, H, W):
        raise RuntimeError("`d_image` must have shape [B, H, W, C] matching rast_dda")
    if d_attr.shape[1] != C:
        raise RuntimeError("`d_attr` must have shape [V, C] where C matches d_image.shape(3)")
    acc = torch.empty(d_attr.shape[0] * C, dtype=torch.float64, device=d_attr.device)
    call("s2c_backward_dda_interpolate_attributes", B, H, W, C, ptr(rast_dda), ptr(d_image), edges.shape[0], ptr(edges),
         d_attr.shape[0], ptr(d_attr), ptr(acc), _stream(rast_dda))


# ---- bitsets (pystrns2cards.cpp:480-529) ---------------------------------------------
def accumulate_bitset_rgb(bitset, cluster_rgb, accum_color) -> None:
    _arr(bitset, _i32, 4, name="bitset")
    _arr(cluster_rgb, _f32, 2, 3, "cluster_rgb")
    _arr(accum_color, _f32, 4, 3, "accum_color")
    _cuda(bitset, cluster_rgb, accum_color, msg="All tensors must be on CUDA")
    B, H, W, S = bitset.shape
    K = cluster_rgb.shape[0]
    if S * 32 < K:
        raise RuntimeError("Too few slots for the number of clusters.")
    call("s2c_accumulate_bitset_rgb", B * H * W, S, ptr(bitset), K, ptr(cluster_rgb), ptr(accum_color),
         _stream(bitset))


def popcount_bitset(bitset, count_image) -> None:
    _arr(bitset, _i32, 4, name="bitset")
    _arr(count_image, _f32, 3, name="count_image")
    _cuda(bitset, count_image, msg="All tensors must be on CUDA")
    B, H, W, S = bitset.shape
    if tuple(count_image.shape) != (B, H, W):
        raise RuntimeError("count_image must have shape [B, H, W]")
    call("s2c_popcount_bitset", B * H * W, S, ptr(bitset), ptr(count_image), _stream(bitset))


# ---- antialias (pystrns2cards.cpp:682-772) --------------------------------------------
def mark_discontinuity_edges(H, W, tri, edges, edge2tri, pos, prim_ids, normals) -> None:
    _arr(tri, _i32, 2, 3, "tri")
    _arr(edges, _i32, 2, 2, "edges")
    _arr(edge2tri, _i32, 2, 2, "edge2tri")
    _arr(pos, _f32, 3, 4, "pos")
    _arr(prim_ids, _i32, 1, name="prim_ids")
    _arr(normals, _f32, 2, 2, "normals")
    _cuda(tri, edges, edge2tri, pos, prim_ids, normals, msg="mark_discontinuity_edges: all input tensors must be CUDA.")
    B, V, _ = pos.shape
    E = edges.shape[0]
    if edge2tri.shape[0] != E:
        raise RuntimeError("mark_discontinuity_edges: edge2tri must have the same number of edges.")
    if prim_ids.shape[0] != B * E:
        raise RuntimeError("mark_discontinuity_edges: prim_ids must have shape (B * E).")
    if normals.shape[0] != B * E:
        raise RuntimeError("mark_discontinuity_edges: normals must have shape (B * E, 2).")
    call("s2c_mark_discontinuity_edges", int(H), int(W), B, V, ptr(pos), tri.shape[0], ptr(tri), E, ptr(edges),
         ptr(edge2tri), ptr(prim_ids), ptr(normals), _stream(pos))


def backward_antialiased_cluster_bitset(frag_pix, frag_attrs_dda, bitset, target_bitset, pos, edges, normals,
                                        edge2cluster, d_pos, kernel_radius, rho) -> None:
    _arr(frag_pix, _i32, 2, 3, "frag_pix")
    _arr(frag_attrs_dda, _f32, 2, 4, "frag_attrs_dda")
    _arr(bitset, _i32, 4, name="bitset")
    _arr(target_bitset, _i32, 4, name="target_bitset")
    _arr(pos, _f32, 3, 4, "pos")
    _arr(edges, _i32, 2, 2, "edges")
    _arr(normals, _f32, 2, 2, "normals")
    _arr(edge2cluster, _i32, 1, name="edge2cluster")
    _arr(d_pos, _f32, 3, 4, "d_pos")
    _cuda(frag_pix, frag_attrs_dda, bitset, target_bitset, pos, edges, normals, edge2cluster, d_pos,
          msg="backward_antialiased_bitset: all input tensors must be CUDA.")
    F = frag_pix.shape[0]
    B, H, W, S = bitset.shape
    V = pos.shape[1]
    E = edges.shape[0]
    if frag_attrs_dda.shape[0] != F:
        raise RuntimeError("backward_antialiased_bitset: frag_pix and frag_attrs_dda must match in number of fragments.")
    if tuple(target_bitset.shape) != (B, H, W, S):
        raise RuntimeError("backward_antialiased_bitset: target_bitset must match bitset shape.")
    if d_pos.shape[0] != B or d_pos.shape[1] != V:
        raise RuntimeError("backward_antialiased_bitset: d_pos must match pos shape.")
    if edge2cluster.shape[0] < E or normals.shape[0] < B * E or pos.shape[0] < B:
        raise RuntimeError("backward_antialiased_bitset: edge2cluster / normals / pos too short.")
    # contributions summed in FP64 in a workspace, then added into d_pos once
    need = _lib.lib().s2c_backward_antialiased_cluster_bitset_workspace_size(B, V)
    ws = workspace(need, pos.device)
    call("s2c_backward_antialiased_cluster_bitset_f64", F, ptr(frag_pix), ptr(frag_attrs_dda), B, H, W, S,
         ptr(bitset), ptr(target_bitset), V, ptr(pos), E, ptr(edges), ptr(normals), ptr(edge2cluster), ptr(d_pos),
         float(kernel_radius), float(rho), ptr(ws), ws.numel(), _stream(pos))


def antialiased_cluster_bitset_grad_planes(bitset_planes, target_planes, shape, pos, tri, edges, edge2tri,
                                           edge2cluster, kernel_radius, rho, d_pos=None, ws=None) -> torch.Tensor:
    """The fused gradient from cluster planes (``bitset_to_planes``) of the bitset and the
    target; ``shape`` = (B, H, W, S) of the bitsets."""
    B, H, W, S = shape
    _arr(pos, _f32, 3, 4, "pos")
    _arr(tri, _i32, 2, 3, "tri")
    _arr(edges, _i32, 2, 2, "edges")
    _arr(edge2tri, _i32, 2, 2, "edge2tri")
    _arr(edge2cluster, _i32, 1, name="edge2cluster")
    _cuda(bitset_planes, target_planes, pos, tri, edges, edge2tri, edge2cluster)
    pshape = (B, 32 * S, H, (W + 31) // 32)
    for t, nm in ((bitset_planes, "bitset_planes"), (target_planes, "target_planes")):
        if tuple(t.shape) != pshape or t.dtype != _i32 or not t.is_contiguous():
            raise RuntimeError(f"antialiased_cluster_bitset_grad_planes: {nm} must be contiguous int32 {pshape}.")
    if pos.shape[0] != B:
        raise RuntimeError("antialiased_cluster_bitset_grad: bitset, target_bitset and pos views must match.")
    if edge2tri.shape[0] != edges.shape[0] or edge2cluster.shape[0] < edges.shape[0]:
        raise RuntimeError("antialiased_cluster_bitset_grad: edge2tri / edge2cluster must cover every edge.")
    V = pos.shape[1]
    if d_pos is None:
        d_pos = torch.zeros_like(pos)
    need = _lib.lib().s2c_antialiased_cluster_bitset_grad_planes_workspace_size(B, V, edges.shape[0])
    if ws is None or ws.numel() < need:
        ws = workspace(need, pos.device)
    call("s2c_antialiased_cluster_bitset_grad_planes", B, H, W, S, ptr(bitset_planes), ptr(target_planes), V,
         ptr(pos), tri.shape[0], ptr(tri), edges.shape[0], ptr(edges), ptr(edge2tri), ptr(edge2cluster), ptr(d_pos),
         float(kernel_radius), float(rho), ptr(ws), ws.numel(), _stream(pos))
    return d_pos


def antialiased_cluster_bitset_grad(bitset, target_bitset, pos, tri, edges, edge2tri, edge2cluster, kernel_radius,
                                    rho, d_pos=None, ws=None) -> torch.Tensor:
    """Fused silhouette marking + edge DDA + edge gradient; returns d_pos (B, V, 4), added
    into ``d_pos`` when given."""
    _arr(bitset, _i32, 4, name="bitset")
    _arr(target_bitset, _i32, 4, name="target_bitset")
    _arr(pos, _f32, 3, 4, "pos")
    _arr(tri, _i32, 2, 3, "tri")
    _arr(edges, _i32, 2, 2, "edges")
    _arr(edge2tri, _i32, 2, 2, "edge2tri")
    _arr(edge2cluster, _i32, 1, name="edge2cluster")
    _cuda(bitset, target_bitset, pos, tri, edges, edge2tri, edge2cluster)
    B, H, W, S = bitset.shape
    if tuple(target_bitset.shape) != (B, H, W, S) or pos.shape[0] != B:
        raise RuntimeError("antialiased_cluster_bitset_grad: bitset, target_bitset and pos views must match.")
    if edge2tri.shape[0] != edges.shape[0] or edge2cluster.shape[0] < edges.shape[0]:
        raise RuntimeError("antialiased_cluster_bitset_grad: edge2tri / edge2cluster must cover every edge.")
    V = pos.shape[1]
    if d_pos is None:
        d_pos = torch.zeros_like(pos)
    need = _lib.lib().s2c_antialiased_cluster_bitset_grad_workspace_size(B, V, H, W, S, edges.shape[0])
    if ws is None or ws.numel() < need:
        ws = workspace(need, pos.device)
    call("s2c_antialiased_cluster_bitset_grad", B, H, W, S, ptr(bitset), ptr(target_bitset), V, ptr(pos),
         tri.shape[0], ptr(tri), edges.shape[0], ptr(edges), ptr(edge2tri), ptr(edge2cluster), ptr(d_pos),
         float(kernel_radius), float(rho), ptr(ws), ws.numel(), _stream(pos))
    return d_pos


# ---- compaction (pystrns2cards.cpp:774-786) ------------------------------------------
def compact_valid_ints(input, output) -> int:
    _arr(input, _i32, 1, name="input")
    _arr(output, _i32, 1, name="output")
    _cuda(input, output, msg="compact_valid_ints: both input and output must be CUDA tensors.")
    if input.shape[0] != output.shape[0]:
        raise RuntimeError("compact_valid_ints: input and output must have the same size.")
    N = input.shape[0]
    if N == 0:
        return 0
    L = _lib.lib()
    ws = workspace(L.s2c_compact_valid_ints_workspace_size(N), input.device)
    n = _lib.i64_out()
    call("s2c_compact_valid_ints", N, ptr(input), ptr(output), ptr(ws), ws.numel(), ctypes.byref(n), _stream(input))
    return int(n.value)


# ---- fused entries (no reference counterpart) ----------------------------------------
def xor_popcount(a, b) -> torch.Tensor:
    """Device uint64 (as int64) total of popc(a ^ b) over two equal-shape int32 bitsets."""
    _arr(a, _i32, name="a")
    _arr(b, _i32, name="b")
    _cuda(a, b)
    if a.shape != b.shape:
        raise RuntimeError("xor_popcount: bitsets must have the same shape.")
    out = torch.empty(1, dtype=torch.int64, device=a.device)
    call("s2c_xor_popcount", a.numel(), ptr(a), ptr(b), ptr(out), _stream(a))
    return out


def cluster_iou_counts(a, b, K) -> tuple:
    _arr(a, _i32, 4, name="a")
    _arr(b, _i32, 4, name="b")
    _cuda(a, b)
    if a.shape != b.shape:
        raise RuntimeError("cluster_iou_counts: bitsets must have the same shape.")
    B, H, W, S = a.shape
    inter = torch.empty(K, dtype=torch.int64, device=a.device)
    uni = torch.empty(K, dtype=torch.int64, device=a.device)
    call("s2c_cluster_iou_counts", B * H * W, S, int(K), ptr(a), ptr(b), ptr(inter), ptr(uni), _stream(a))
    return inter, uni

def dda_cluster_bitset(pos, edges, prim2cluster, bitset, edge_ids=None, ws=None) -> torch.Tensor:
    """Fused DDA -> cluster bitset into ``bitset`` (B, H, W, S), fully overwritten."""
    _arr(pos, _f32, 3, 4, "pos")
    _arr(edges, _i32, 2, 2, "edges")
    _arr(prim2cluster, _i32, 1, name="prim2cluster")
    _arr(bitset, _i32, 4, name="bitset")
    if edge_ids is not None:
        _arr(edge_ids, _i32, 1, name="edge_ids")
    _cuda(pos, edges, prim2cluster, bitset, edge_ids)
    B, V, _ = pos.shape
    E = edges.shape[0]
    if prim2cluster.shape[0] < E:
        raise RuntimeError("prim2cluster must have one entry per edge.")
    if bitset.shape[0] != B:
        raise RuntimeError("bitset must have one image per view of pos.")
    _, H, W, S = bitset.shape
    P = B * E if edge_ids is None else edge_ids.shape[0]
    L = _lib.lib()
    need = L.s2c_dda_cluster_bitset_workspace_size(P, B, H, W, S)
    if ws is None or ws.numel() < need:
        ws = workspace(need, pos.device)
    call("s2c_dda_cluster_bitset", P, ptr(edge_ids), H, W, B, V, ptr(pos), E, ptr(edges), ptr(prim2cluster), S,
         ptr(bitset), ptr(ws), ws.numel(), _stream(pos))
    return bitset


def rasterize_fused_planes(pos, tri, tri2cluster, cluster_count, H, W, planes=None, rast=None, ws=None):
    """Fused card raster into cluster planes (B, 32 S, H, ceil(W / 32)) int32 (and rast when
    given); returns planes."""
    _arr(pos, _f32, 3, 4, "pos")
    _arr(tri, _i32, 2, 3, "tri")
    _arr(tri2cluster, _i32, 1, name="tri2cluster")
    _cuda(pos, tri, tri2cluster)
    B, V = pos.shape[0], pos.shape[1]
    S = (int(cluster_count) + 31) // 32
    shape = (B, 32 * S, H, (W + 31) // 32)
    if planes is None:
        planes = torch.empty(shape, dtype=torch.int32, device=pos.device)
    elif tuple(planes.shape) != shape or not planes.is_contiguous():
        raise RuntimeError("rasterize_fused_planes: planes must be contiguous " + str(shape))
    need = _lib.lib().s2c_rasterize_fused_workspace_size(B, H, W, tri.shape[0])
    if ws is None or ws.numel() < need:
        ws = workspace(need, pos.device)
    call("s2c_rasterize_fused_planes", B, H, W, V, ptr(pos), tri.shape[0], ptr(tri), ptr(tri2cluster),
         tri2cluster.shape[0], S, ptr(planes), ptr(rast), ptr(ws), ws.numel(), _stream(pos))
    return planes


def cluster_iou_counts_planes(a_planes, b_planes, shape, K) -> tuple:
    """Per-cluster (inter, union) pixel counts from cluster planes; ``shape`` = (B, H, W, S)."""
    B, H, W, S = shape
    _cuda(a_planes, b_planes)
    if a_planes.shape != b_planes.shape:
        raise RuntimeError("cluster_iou_counts_planes: planes must have the same shape.")
    inter = torch.empty(K, dtype=torch.int64, device=a_planes.device)
    uni = torch.empty(K, dtype=torch.int64, device=a_planes.device)
    call("s2c_cluster_iou_counts_planes", B, H, W, S, int(K), ptr(a_planes), ptr(b_planes), ptr(inter), ptr(uni),
         _stream(a_planes))
    return inter, uni


def rasterize_fused_planes_onto(pos, tri, tri2cluster, cluster_count, H, W, planes, rects=None, ws=None):
    """The fused card raster ORed onto ``planes`` (not cleared: zeros wherever it can set a
    bit, e.g. after ``planes_clear_rects`` with the previous pass's rectangles); returns the
    per-(view, plane) word rectangles (B, 32 S, 4) int32 of every bit it can set."""
    _arr(pos, _f32, 3, 4, "pos")
    _arr(tri, _i32, 2, 3, "tri")
    _arr(tri2cluster, _i32, 1, name="tri2cluster")
    _cuda(pos, tri, tri2cluster, planes)
    B, V = pos.shape[0], pos.shape[1]
    S = (int(cluster_count) + 31) // 32
    shape = (B, 32 * S, H, (W + 31) // 32)
    if tuple(planes.shape) != shape or not planes.is_contiguous() or planes.dtype != _i32:
        raise RuntimeError("rasterize_fused_planes_onto: planes must be contiguous int32 " + str(shape))
    if rects is None:
        rects = torch.empty((B, 32 * S, 4), dtype=torch.int32, device=pos.device)
    elif tuple(rects.shape) != (B, 32 * S, 4) or rects.dtype != _i32 or not rects.is_contiguous():
        raise RuntimeError(f"rasterize_fused_planes_onto: rects must be contiguous int32 {(B, 32 * S, 4)}")
    need = _lib.lib().s2c_rasterize_fused_workspace_size(B, H, W, tri.shape[0])
    if ws is None or ws.numel() < need:
        ws = workspace(need, pos.device)
    call("s2c_rasterize_fused_planes_onto", B, H, W, V, ptr(pos), tri.shape[0], ptr(tri), ptr(tri2cluster),
         tri2cluster.shape[0], S, ptr(planes), ptr(rects), ptr(ws), ws.numel(), _stream(pos))
    return rects


def _plane_rects_arg(planes, rects, shape, name):
    B, H, W, S = shape
    want = (B, 32 * S, H, (W + 31) // 32)
    if tuple(planes.shape) != want or not planes.is_contiguous():
        raise RuntimeError(f"{name}: planes must be contiguous {want}")
    if rects is not None and (tuple(rects.shape) != (B, 32 * S, 4) or rects.dtype != _i32 or
                              not rects.is_contiguous()):
        raise RuntimeError(f"{name}: rects must be contiguous int32 {(B, 32 * S, 4)}")


def planes_clear_rects(planes, rects, shape) -> None:
    """Zero each (view, plane)'s word rectangle (y0, y1, q0, q1); ``shape`` = (B, H, W, S)."""
    _cuda(planes, rects)
    _plane_rects_arg(planes, rects, shape, "planes_clear_rects")
    B, H, W, S = shape
    call("s2c_planes_clear_rects", B, H, W, S, ptr(planes), ptr(rects), _stream(planes))


def planes_bounds(planes, shape, rects=None) -> torch.Tensor:
    """The smallest word rectangle (y0, y1, q0, q1) holding every non-zero word of each
    (view, plane); (B, 32 S, 4) int32."""
    _cuda(planes)
    B, H, W, S = shape
    if rects is None:
        rects = torch.empty((B, 32 * S, 4), dtype=torch.int32, device=planes.device)
    _plane_rects_arg(planes, rects, shape, "planes_bounds")
    call("s2c_planes_bounds", B, H, W, S, ptr(planes), ptr(rects), _stream(planes))
    return rects


def cluster_iou_counts_planes_rects(a_planes, b_planes, a_rects, b_rects, shape, K) -> tuple:
    """Per-cluster (inter, union) counts and the XOR-popcount total, counting only inside each
    plane's rectangles (exact when every set bit lies inside its plane's rectangle)."""
    _cuda(a_planes, b_planes, a_rects, b_rects)
    for pl, r in ((a_planes, a_rects), (b_planes, b_rects)):
        _plane_rects_arg(pl, r, shape, "cluster_iou_counts_planes_rects")
    B, H, W, S = shape
    out = torch.empty(2 * K + 1, dtype=torch.int64, device=a_planes.device)
    call("s2c_cluster_iou_counts_planes_rects", B, H, W, S, int(K), ptr(a_planes), ptr(b_planes), ptr(a_rects),
         ptr(b_rects), ptr(out), ptr(out[K:]), ptr(out[2 * K:]), _stream(a_planes))
    return out[:K], out[K:2 * K], out[2 * K]


def bitset_to_planes(bitset, planes=None) -> torch.Tensor:
    """Cluster planes (B, 32 S, H, ceil(W / 32)) int32 of a bitset (B, H, W, S)."""
    _arr(bitset, _i32, 4, name="bitset")
    _cuda(bitset)
    B, H, W, S = bitset.shape
    shape = (B, 32 * S, H, (W + 31) // 32)
    if planes is None:
        planes = torch.empty(shape, dtype=torch.int32, device=bitset.device)
    elif tuple(planes.shape) != shape or planes.dtype != _i32 or not planes.is_contiguous():
        raise RuntimeError("bitset_to_planes: planes must be contiguous int32 " + str(shape))
    call("s2c_bitset_to_planes", B, H, W, S, ptr(bitset), ptr(planes), _stream(bitset))
    return planes


def dda_cluster_bitset_stats(ws) -> tuple:
    e, o = _lib.i64_out(), _lib.i64_out()
    call("s2c_dda_cluster_bitset_stats", ptr(ws), ws.numel(), ctypes.byref(e), ctypes.byref(o))
    return int(e.value), int(o.value)


# ---- mesh topology (pystrns2cards.cpp:208-243) -----------------------------------------
def build_edges_from_triangles(tri):
    """Host: unique edges (E, 2) and edge->triangle map (E, 2) of an int32 (T, 3) numpy array,
    edges sorted by (min, max) vertex (the reference's order is its hash map's)."""
    import numpy as np
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    T = int(tri.shape[0])
    edges = np.empty((max(3 * T, 1), 2), np.int32)
    e2t = np.empty((max(3 * T, 1), 2), np.int32)
    n = _lib.i64_out()
    call("s2c_build_edges_from_triangles", T, tri.ctypes.data, edges.ctypes.data, e2t.ctypes.data, ctypes.byref(n))
    E = int(n.value)
    return edges[:E].copy(), e2t[:E].copy()


def build_edges_device(tri, num_verts: int, edges=None, edge2tri=None, counts=None):
    """Device: (edges (3T, 2), edge2tri (3T, 2), counts int64 (2,) = [num_edges, num_bad]) of a
    CUDA int32 (T, 3) triangle tensor; the first num_edges rows are the edges.  No host
    synchronisation."""
    _arr(tri, _i32, 2, 3, "tri")
    _cuda(tri, msg="build_edges_device: tri must be CUDA.")
    T = tri.shape[0]
    dev = tri.device
    if edges is None:
        edges = torch.empty((max(3 * T, 1), 2), dtype=_i32, device=dev)
    if edge2tri is None:
        edge2tri = torch.empty((max(3 * T, 1), 2), dtype=_i32, device=dev)
    if counts is None:
        counts = torch.zeros(2, dtype=torch.int64, device=dev)
    ws = workspace(_lib.lib().s2c_build_edges_device_workspace_size(T, int(num_verts)), dev)
    call("s2c_build_edges_device", T, ptr(tri), int(num_verts), ptr(edges), ptr(edge2tri), ptr(counts),
         counts.data_ptr() + 8, ptr(ws), ws.numel(), _stream(tri))
    return edges, edge2tri, counts


# ---- strand curves (pystrns2cards.cpp:841-915) -----------------------------------------
def compute_arclength(strands, arclength) -> None:
    _arr(strands, _f32, 3, 3, "strands")
    _arr(arclength, _f32, 2, name="arclength")
    _cuda(strands, arclength, msg="compute_arclength: All input tensors must be CUDA.")
    N, V, _ = strands.shape
    if tuple(arclength.shape) != (N, V):
        raise RuntimeError("compute_arclength: arclength must match (num_strands, num_points).")
    call("s2c_compute_arclength", N, V, ptr(strands), ptr(arclength), _stream(strands))


def smooth_strands(strands, arclength, smoothed_strands, beta) -> None:
    """``arclength`` may be None: the kernel then computes it itself."""
    _arr(strands, _f32, 3, 3, "strands")
    _arr(smoothed_strands, _f32, 3, 3, "smoothed_strands")
    if arclength is not None:
        _arr(arclength, _f32, 2, name="arclength")
    _cuda(strands, arclength, smoothed_strands, msg="smooth_strands: All input tensors must be CUDA.")
    N, V, _ = strands.shape
    if arclength is not None and tuple(arclength.shape) != (N, V):
        raise RuntimeError("smooth_strands: arclength must match (num_strands, num_points).")
    if tuple(smoothed_strands.shape) != (N, V, 3):
        raise RuntimeError("smooth_strands: smoothed_strands must match (num_strands, num_points, 3).")
    call("s2c_smooth_strands", N, V, ptr(strands), ptr(arclength), ptr(smoothed_strands), float(beta),
         _stream(strands))


def skinning(strands, arclength, handle_strands, canonical_handles, R, skinned_strands, beta) -> None:
    """``arclength`` may be None: the kernel then computes it itself."""
    _arr(strands, _f32, 3, 3, "strands")
    _arr(handle_strands, _f32, 3, 3, "handle_strands")
    _arr(canonical_handles, _f32, 3, 3, "canonical_handles")
    _arr(R, _f32, 4, 3, "R")
    _arr(skinned_strands, _f32, 3, 3, "skinned_strands")
    if arclength is not None:
        _arr(arclength, _f32, 2, name="arclength")
    _cuda(strands, arclength, handle_strands, canonical_handles, R, skinned_strands,
          msg="skinning: All input tensors must be CUDA.")
    N, V, _ = strands.shape
    if arclength is not None and tuple(arclength.shape) != (N, V):
        raise RuntimeError("skinning: arclength must match (num_strands, num_points).")
    if tuple(handle_strands.shape) != (N, V, 3):
        raise RuntimeError("skinning: handle_strands must match (num_strands, num_points, 3).")
    if tuple(canonical_handles.shape) != (N, V, 3):
        raise RuntimeError("skinning: canonical_handles must match (num_strands, num_points, 3).")
    if tuple(R.shape) != (N, V, 3, 3):
        raise RuntimeError("skinning: R must match (num_strands, num_points, 3, 3).")
    if tuple(skinned_strands.shape) != (N, V, 3):
        raise RuntimeError("skinning: skinned_strands must match (num_strands, num_points, 3).")
    call("s2c_skinning", N, V, ptr(strands), ptr(arclength), ptr(handle_strands), ptr(canonical_handles), ptr(R),
         ptr(skinned_strands), float(beta), _stream(strands))


# ---- strand frames and wisp alignment (curve_utils.py:104-165, 243-308, 481-607) ----------
def _vec3(v):
    v = [float(x) for x in (v.tolist() if hasattr(v, "tolist") else v)]
    if len(v) != 3:
        raise RuntimeError("expected a 3-vector")
    return (ctypes.c_float * 3)(*v)


def strand_frames(strands, t_dst=None, T=None, N=None, B=None, R=None, roots=None, canon=None) -> None:
    """Bishop frames (T, N, B), alignment rotations R and canonical handles ``canon`` of
    strands (S, V, 3) in one launch; every output optional.  ``roots`` is an (S, 3) tensor or
    a strided view of one point per strand (e.g. ``x[:, 0]`` of an (S, V, 3) tensor)."""
    _arr(strands, _f32, 3, 3, "strands")
    S, V, _ = strands.shape
    for t, nm in ((T, "T"), (N, "N"), (B, "B"), (canon, "canon")):
        if t is not None:
            _arr(t, _f32, 3, 3, nm)
            if tuple(t.shape) != (S, V, 3):
                raise RuntimeError(f"strand_frames: {nm} must match (num_strands, num_points, 3).")
    if R is not None:
        _arr(R, _f32, 4, 3, "R")
        if tuple(R.shape) != (S, V, 3, 3):
            raise RuntimeError("strand_frames: R must match (num_strands, num_points, 3, 3).")
    stride = 3
    if roots is not None:
        if not isinstance(roots, torch.Tensor) or roots.dtype != _f32 or roots.ndim != 2 or tuple(roots.shape) != (S, 3):
            raise RuntimeError("strand_frames: roots must be float32 (num_strands, 3).")
        if roots.stride(1) != 1 or (S > 1 and roots.stride(0) < 3):
            raise RuntimeError("strand_frames: roots must be rows of 3 contiguous floats.")
        stride = roots.stride(0) if S > 1 else 3
    if (R is not None or canon is not None) and t_dst is None:
        raise RuntimeError("strand_frames: R and canon need t_dst.")
    _cuda(strands, T, N, B, R, roots, canon, msg="strand_frames: All input tensors must be CUDA.")
    call("s2c_strand_frames", S, V, ptr(strands), _vec3(t_dst) if t_dst is not None else None, ptr(T), ptr(N), ptr(B),
         ptr(R), ptr(roots), stride, ptr(canon), _stream(strands))


def wisp_frames(offsets, strands, t_dst, n_dst, b_dst, R_global, centre, longest) -> None:
    """Per-wisp centre, longest strand and global rotation (``align_wisps``'s loop body)."""
    _arr(offsets, _i32, 1, name="offsets")
    _arr(strands, _f32, 3, 3, "strands")
    _arr(R_global, _f32, 3, 3, "R_global")
    _arr(centre, _f32, 2, 3, "centre")
    _arr(longest, _i32, 1, name="longest")
    _cuda(offsets, strands, R_global, centre, longest, msg="wisp_frames: All input tensors must be CUDA.")
    K = offsets.shape[0] - 1
    if K < 0 or R_global.shape[0] != K or centre.shape[0] != K or longest.shape[0] != K:
        raise RuntimeError("wisp_frames: outputs must hold one row per wisp.")
    S, V, _ = strands.shape
    if V < 2:
        raise RuntimeError("wisp_frames: strands need at least 2 points.")
    call("s2c_wisp_frames", K, ptr(offsets), S, V, ptr(strands), _vec3(t_dst), _vec3(n_dst), _vec3(b_dst),
         ptr(R_global), ptr(centre), ptr(longest), _stream(strands))


def wisp_rotate(offsets, R_global, centre, a, b, a_out, b_out) -> None:
    """a_out = R (a - c), b_out = R (b - c) with the frame of each strand's wisp (wisp w = the
    strands offsets[w] .. offsets[w+1]-1)."""
    for t, nm in ((a, "a"), (b, "b"), (a_out, "a_out"), (b_out, "b_out")):
        _arr(t, _f32, 3, 3, nm)
    _arr(offsets, _i32, 1, name="offsets")
    _arr(R_global, _f32, 3, 3, "R_global")
    _arr(centre, _f32, 2, 3, "centre")
    _cuda(offsets, R_global, centre, a, b, a_out, b_out, msg="wisp_rotate: All input tensors must be CUDA.")
    S, V, _ = a.shape
    K = offsets.shape[0] - 1
    if any(tuple(t.shape) != (S, V, 3) for t in (b, a_out, b_out)) or K < 0 or R_global.shape[0] != K \
            or centre.shape[0] != K:
        raise RuntimeError("wisp_rotate: shapes do not match.")
    call("s2c_wisp_rotate", K, ptr(offsets), S, V, ptr(R_global), ptr(centre), ptr(a), ptr(b), ptr(a_out), ptr(b_out),
         _stream(a))


def align_strands_max_points() -> int:
    return int(_lib.lib().s2c_align_strands_max_points())


def align_strands(strands, offsets, R_global, centre, t_dst, beta, handles, aligned) -> None:
    """Smoothing, wisp rotation, frames and skinning of every strand in one launch (the part
    of align_wisps after its per-wisp frames)."""
    _arr(strands, _f32, 3, 3, "strands")
    _arr(offsets, _i32, 1, name="offsets")
    _arr(R_global, _f32, 3, 3, "R_global")
    _arr(centre, _f32, 2, 3, "centre")
    _arr(handles, _f32, 3, 3, "handles")
    _arr(aligned, _f32, 3, 3, "aligned")
    _cuda(strands, offsets, R_global, centre, handles, aligned, msg="align_strands: All input tensors must be CUDA.")
    S, V, _ = strands.shape
    K = offsets.shape[0] - 1
    if K < 0 or R_global.shape[0] != K or centre.shape[0] != K or tuple(handles.shape) != (S, V, 3) \
            or tuple(aligned.shape) != (S, V, 3):
        raise RuntimeError("align_strands: shapes do not match.")
    call("s2c_align_strands", S, V, ptr(strands), K, ptr(offsets), ptr(R_global), ptr(centre), _vec3(t_dst),
         float(beta), ptr(handles), ptr(aligned), _stream(strands))


# ---- strand ingest (pystrns2cards.cpp:788-839) -----------------------------------------
def load_strands(filepath):
    """Host: (num_samples int32 (N, 1), points float32 (P, 3)) of a .bin/.data/.hair file."""
    import numpy as np
    h = ctypes.c_void_p()
    n, p = _lib.i64_out(), _lib.i64_out()
    call("s2c_load_strands", str(filepath).encode(), ctypes.byref(h), ctypes.byref(n), ctypes.byref(p),
         exc=ValueError)
    counts = np.empty((int(n.value), 1), np.int32)
    points = np.empty((int(p.value), 3), np.float32)
    call("s2c_strands_take", h, counts.ctypes.data, points.ctypes.data)
    return counts, points


def resample_strands_by_arclength(num_samples, points, target_num_samples):
    """Host: (N, target, 3) float32 of ragged strands resampled uniformly in arclength."""
    import numpy as np
    ns = np.ascontiguousarray(num_samples, dtype=np.int32).ravel()
    pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
    if int(ns.sum()) != pts.shape[0]:
        raise RuntimeError("resample_strands_by_arclength: num_samples do not add up to the points.")
    out = np.empty((ns.shape[0], int(target_num_samples), 3), np.float32)
    call("s2c_resample_strands_by_arclength_host", ns.shape[0], ns.ctypes.data, pts.ctypes.data,
         int(target_num_samples), out.ctypes.data)
    return out


def resample_strands_by_arclength_device(num_samples, points, target_num_samples, out=None):
    """Device: the same from CUDA tensors num_samples int32 (N,) and points float32 (P, 3)."""
    _arr(num_samples, _i32, 1, name="num_samples")
    _arr(points, _f32, 2, 3, "points")
    _cuda(num_samples, points)
    N, P, T = num_samples.shape[0], points.shape[0], int(target_num_samples)
    if out is None:
        out = torch.empty((N, T, 3), dtype=_f32, device=points.device)
    ws = workspace(_lib.lib().s2c_resample_strands_workspace_size(N, P), points.device)
    call("s2c_resample_strands_by_arclength", N, ptr(num_samples), ptr(points), P, T, ptr(out), ptr(ws), ws.numel(),
         _stream(points))
    return out
