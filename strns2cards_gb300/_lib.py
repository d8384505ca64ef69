"""ctypes binding of libs2c.so (the C ABI declared in include/s2c.h).

The library is built in-tree (strns2cards_gb300/build.py).  There is no CPU fallback:
if the library is missing or cannot be loaded, every op raises RuntimeError.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libs2c.so")

c_i = ctypes.c_int
c_i64 = ctypes.c_int64
c_sz = ctypes.c_size_t
c_f = ctypes.c_float
vp = ctypes.c_void_p
i64p = ctypes.POINTER(ctypes.c_int64)

S2C_OK, S2C_ERR_INVALID, S2C_ERR_CUDA, S2C_ERR_WORKSPACE, S2C_ERR_TIMEOUT = 0, 1, 2, 3, 4

# name: (argtypes, restype)
SIGNATURES = {
    "s2c_version": ([], c_i),
    "s2c_last_error": ([], ctypes.c_char_p),
    "s2c_dda_compute_span_workspace_size": ([c_i64], c_sz),
    "s2c_dda_compute_span": ([c_i64, vp, c_i, c_i, c_i, c_i, vp, c_i, vp, vp, vp, vp, vp, c_sz, i64p, vp], c_i),
    "s2c_dda_compute_fragments": ([c_i64, c_i64, vp, vp, vp, vp, c_i, c_i, c_i, c_i, vp, c_i, vp, vp, vp, vp], c_i),
    "s2c_filter_valid_fragments_workspace_size": ([c_i64], c_sz),
    "s2c_filter_valid_fragments": ([c_i64, vp, vp, vp, vp, vp, c_sz, i64p, vp], c_i),
    "s2c_cluster_mask_from_fragments": ([c_i64, vp, vp, vp, c_i64, c_i, c_i, c_i, c_i, vp, vp], c_i),
    "s2c_dda_cluster_bitset_workspace_size": ([c_i64, c_i, c_i, c_i, c_i], c_sz),
    "s2c_dda_cluster_bitset": ([c_i64, vp, c_i, c_i, c_i, c_i, vp, c_i, vp, vp, c_i, vp, vp, c_sz, vp], c_i),
    "s2c_dda_cluster_bitset_stats": ([vp, c_sz, i64p, i64p], c_i),
    "s2c_dda_cluster_bitset_noalloc": ([c_i64, vp, c_i, c_i, c_i, c_i, vp, c_i, vp, vp, c_i, vp, vp], c_i),
    "s2c_fit_smem_bytes": ([c_i, c_i, c_i, c_i, c_i], c_sz),
    "s2c_fit_workspace_size": ([c_i, c_i, c_i], c_sz),
    "s2c_fit_iteration": ([c_i, c_i, c_i, c_i, vp, vp, c_i, vp, vp, vp, c_i, vp, c_i, vp, c_i, vp, vp, vp, vp, c_i,
                           vp, c_i, c_i, vp, c_f, c_f, c_i, c_f, c_f, c_i, c_i, c_i, vp, c_sz, vp], c_i),
    "s2c_compute_triangle_rects_workspace_size": ([c_i, c_i], c_sz),
    "s2c_compute_triangle_rects": ([c_i, c_i, c_i, c_i, vp, c_i, vp, vp, vp, vp, c_sz, i64p, vp], c_i),
    "s2c_compute_fragments": ([c_i, c_i, c_i, c_i, vp, c_i, vp, vp, vp, c_i64, vp, vp, vp], c_i),
    "s2c_dda_count_fragments_workspace_size": ([c_i64], c_sz),
    "s2c_dda_count_fragments": ([c_i64, c_i64, vp, vp, vp, vp, c_i, c_i, c_i, c_i, vp, c_i, vp, vp, c_sz, i64p, vp], c_i),
    "s2c_dda_write_fragments": ([c_i64, c_i64, vp, vp, vp, vp, c_i, c_i, c_i, c_i, vp, c_i, vp, vp, c_sz, vp, vp, vp],
                                c_i),
    "s2c_count_fragments_workspace_size": ([c_i64], c_sz),
    "s2c_count_fragments": ([c_i, c_i, c_i, c_i, vp, c_i, vp, vp, vp, c_i64, vp, c_sz, i64p, vp], c_i),
    "s2c_write_fragments": ([c_i, c_i, c_i, c_i, vp, c_i, vp, vp, vp, c_i64, vp, c_sz, vp, vp, vp], c_i),
    "s2c_depth_test_workspace_size": ([c_i, c_i, c_i], c_sz),
    "s2c_depth_test": ([c_i, c_i, c_i, c_i64, vp, vp, vp, vp, c_sz, vp], c_i),
    "s2c_rasterize_fused_workspace_size": ([c_i, c_i, c_i, c_i], c_sz),
    "s2c_rasterize_fused": ([c_i, c_i, c_i, c_i, vp, c_i, vp, vp, c_i, c_i, vp, vp, vp, c_sz, vp], c_i),
    "s2c_rasterize_fused_planes": ([c_i, c_i, c_i, c_i, vp, c_i, vp, vp, c_i, c_i, vp, vp, vp, c_sz, vp], c_i),
    "s2c_cluster_iou_counts_planes": ([c_i, c_i, c_i, c_i, c_i, vp, vp, vp, vp, vp], c_i),
    "s2c_rasterize_fused_planes_onto": ([c_i, c_i, c_i, c_i, vp, c_i, vp, vp, c_i, c_i, vp, vp, vp, c_sz, vp], c_i),
    "s2c_planes_clear_rects": ([c_i, c_i, c_i, c_i, vp, vp, vp], c_i),
    "s2c_planes_bounds": ([c_i, c_i, c_i, c_i, vp, vp, vp], c_i),
    "s2c_cluster_iou_counts_planes_rects": ([c_i, c_i, c_i, c_i, c_i, vp, vp, vp, vp, vp, vp, vp, vp], c_i),
    "s2c_msaa_resolve": ([c_i, c_i, c_i, c_i, vp, c_i, vp, c_i, vp, vp, vp, vp, vp, vp], c_i),
    "s2c_barycentric_derivatives": ([c_i, c_i, c_i, c_i, vp, c_i, vp, vp, vp, vp], c_i),
    "s2c_interpolate_triangle_attributes": ([c_i, c_i, c_i, c_i, vp, c_i, vp, c_i, vp, vp, vp], c_i),
    "s2c_backward_interpolate_triangle_attributes": ([c_i, c_i, c_i, c_i, vp, vp, c_i, vp, c_i, vp, vp, vp], c_i),
    "s2c_dda_interpolate_attributes": ([c_i, c_i, c_i, c_i, vp, c_i, vp, c_i, vp, vp, vp], c_i),
    "s2c_backward_dda_interpolate_attributes": ([c_i, c_i, c_i, c_i, vp, vp, c_i, vp, c_i, vp, vp, vp], c_i),
    "s2c_xor_popcount": ([c_i64, vp, vp, vp, vp], c_i),
    "s2c_cluster_iou_counts": ([c_i64, c_i, c_i, vp, vp, vp, vp, vp], c_i),
    "s2c_mark_discontinuity_edges": ([c_i, c_i, c_i, c_i, vp, c_i, vp, c_i, vp, vp, vp, vp, vp], c_i),
    "s2c_backward_antialiased_cluster_bitset": ([c_i64, vp, vp, c_i, c_i, c_i, c_i, vp, vp, c_i, vp, c_i, vp, vp, vp,
                                                 vp, c_f, c_f, vp], c_i),
    "s2c_backward_antialiased_cluster_bitset_workspace_size": ([c_i, c_i], c_sz),
    "s2c_backward_antialiased_cluster_bitset_f64": ([c_i64, vp, vp, c_i, c_i, c_i, c_i, vp, vp, c_i, vp, c_i, vp, vp,
                                                     vp, vp, c_f, c_f, vp, c_sz, vp], c_i),
    "s2c_antialiased_cluster_bitset_grad_workspace_size": ([c_i, c_i, c_i, c_i, c_i, c_i], c_sz),
    "s2c_antialiased_cluster_bitset_grad_planes_workspace_size": ([c_i, c_i, c_i], c_sz),
    "s2c_antialiased_cluster_bitset_grad_planes": ([c_i, c_i, c_i, c_i, vp, vp, c_i, vp, c_i, vp, c_i, vp, vp, vp,
                                                    vp, c_f, c_f, vp, c_sz, vp], c_i),
    "s2c_bitset_planes_size": ([c_i, c_i, c_i, c_i], c_sz),
    "s2c_bitset_to_planes": ([c_i, c_i, c_i, c_i, vp, vp, vp], c_i),
    "s2c_antialiased_cluster_bitset_grad": ([c_i, c_i, c_i, c_i, vp, vp, c_i, vp, c_i, vp, c_i, vp, vp, vp, vp, c_f,
                                             c_f, vp, c_sz, vp], c_i),
    "s2c_compact_valid_ints_workspace_size": ([c_i64], c_sz),
    "s2c_compact_valid_ints": ([c_i64, vp, vp, vp, c_sz, i64p, vp], c_i),
    "s2c_popcount_bitset": ([c_i64, c_i, vp, vp, vp], c_i),
    "s2c_accumulate_bitset_rgb": ([c_i64, c_i, vp, c_i, vp, vp, vp], c_i),
    "s2c_compute_arclength": ([c_i, c_i, vp, vp, vp], c_i),
    "s2c_smooth_strands": ([c_i, c_i, vp, vp, vp, c_f, vp], c_i),
    "s2c_skinning": ([c_i, c_i, vp, vp, vp, vp, vp, vp, c_f, vp], c_i),
    "s2c_strand_frames": ([c_i, c_i, vp, vp, vp, vp, vp, vp, vp, c_i64, vp, vp], c_i),
    "s2c_wisp_frames": ([c_i, vp, c_i64, c_i, vp, vp, vp, vp, vp, vp, vp, vp], c_i),
    "s2c_wisp_rotate": ([c_i, vp, c_i64, c_i, vp, vp, vp, vp, vp, vp, vp], c_i),
    "s2c_align_strands_max_points": ([], c_i),
    "s2c_build_edges_device_workspace_size": ([c_i, c_i], c_sz),
    "s2c_build_edges_device": ([c_i, vp, c_i, vp, vp, vp, vp, vp, c_sz, vp], c_i),
    "s2c_align_strands": ([c_i64, c_i, vp, c_i, vp, vp, vp, vp, c_f, vp, vp, vp], c_i),
    "s2c_build_edges_from_triangles": ([c_i, vp, vp, vp, i64p], c_i),
    "s2c_load_strands": ([ctypes.c_char_p, ctypes.POINTER(vp), i64p, i64p], c_i),
    "s2c_strands_take": ([vp, vp, vp], c_i),
    "s2c_resample_strands_by_arclength_host": ([c_i, vp, vp, c_i, vp], c_i),
    "s2c_resample_strands_workspace_size": ([c_i, c_i64], c_sz),
    "s2c_resample_strands_by_arclength": ([c_i, vp, vp, c_i64, c_i, vp, vp, c_sz, vp], c_i),
    "s2c_build_vertex_adjacency": ([c_i, c_i, vp, vp, vp, i64p], c_i),
    "s2c_card_laplacian_smooth": ([c_i, c_i, vp, vp, c_i, vp, vp, c_f, c_i, vp], c_i),
    "s2c_lbs_bind_workspace_size": ([c_i64, c_i], c_sz),
    "s2c_lbs_bind": ([c_i64, vp, c_i, vp, c_f, vp, vp, vp, vp, vp, c_sz, vp], c_i),
    "s2c_lbs_forward": ([c_i64, vp, vp, vp, c_i, vp, vp, vp], c_i),
    "s2c_lbs_backward": ([c_i64, vp, vp, vp, c_i, vp, vp, vp, vp, vp, vp, vp], c_i),
}

_lib = None
_lock = threading.Lock()


class S2CError(RuntimeError):
    pass


def lib() -> ctypes.CDLL:
    """Load libs2c.so once; raise if it was not built (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m strns2cards_gb300.build` "
                "(or __graft_entry__.build()); there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name, None)
            if fn is None:
                raise RuntimeError(f"{LIB_PATH} does not export {name}; rebuild it")
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(status: int, what: str, exc=RuntimeError):
    if status == S2C_OK:
        return
    msg = lib().s2c_last_error().decode(errors="replace")
    if status == S2C_ERR_INVALID:
        raise exc(f"{what}: {msg}")
    raise S2CError(f"{what}: status {status}: {msg}")


def call(name: str, *args, exc=RuntimeError):
    check(getattr(lib(), name)(*args), name, exc)


def ptr(t) -> int | None:
    if t is None:
        return None
    return t.data_ptr()


def stream_of(t: torch.Tensor) -> int:
    return torch.cuda.current_stream(t.device).cuda_stream


def workspace(nbytes: int, device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


def i64_out():
    return ctypes.c_int64(0)
