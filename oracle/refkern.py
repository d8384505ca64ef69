"""Launcher for the reference's own CUDA kernels (test infrastructure only).

``oracle/build_ref.sh`` compiles the reference sources ``pystrns2cards/src/*.cu``
unmodified with nvcc into device-only cubins under ``oracle/_ref/`` (sm_103a; the cubins
are host-architecture independent, so the copy built on an x86 host runs on the Arm GPU
host). This module loads those cubins with the CUDA driver API through ctypes and
re-creates the reference's Python-level call sequences (``dda.py``, ``rasterize.py``,
``antialias.py``, ``bitset_utils.py``, ``curve_utils.py``) around them:

* the kernels and their launch shapes (256 threads, ``GET_BLOCKS``, ``cuda_common.cuh:25-26``)
  are the reference's;
* ``thrust::inclusive_scan`` (``dda.cu:111``, ``rasterize.cu:77``) is replaced by
  ``torch.cumsum`` in int32, an exact integer scan with the same result;
* the legacy default stream is used, as in the reference.

Nothing in the product imports this module: it only produces golden vectors and serves
as a second checker in the GPU tests when the cubins are present.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import torch

REF_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref")
_UNITS = ["dda", "rasterize", "antialias", "bitset_utils", "compact_utils", "curve_utils"]
# unique length-prefixed pieces of the Itanium-mangled kernel names
_KERNELS = {
    "dda_compute_span_kernel": ("dda", "23dda_compute_span_kernel"),
    "dda_compute_fragments_kernel": ("dda", "28dda_compute_fragments_kernel"),
    "dda_interpolate_attributes_kernel": ("dda", "33dda_interpolate_attributes_kernel"),
    "backward_dda_interpolate_attributes_kernel": ("dda", "42backward_dda_interpolate_attributes_kernel"),
    "compute_triangle_rects_kernel": ("rasterize", "29compute_triangle_rects_kernel"),
    "compute_fragments_kernel": ("rasterize", "24compute_fragments_kernel"),
    "depth_test_kernel": ("rasterize", "17depth_test_kernel"),
    "gather_depth_test_kernel": ("rasterize", "24gather_depth_test_kernel"),
    "fill_ll_max": ("rasterize", "11fill_ll_max"),
    "filter_valid_fragments_kernel": ("rasterize", "29filter_valid_fragments_kernel"),
    "interpolate_triangle_attributes_kernel": ("rasterize", "38interpolate_triangle_attributes_kernel"),
    "backward_interpolate_triangle_attributes_kernel": ("rasterize", "47backward_interpolate_triangle_attributes_kernel"),
    "cluster_mask_from_fragments_kernel": ("rasterize", "34cluster_mask_from_fragments_kernel"),
    "mark_discontinuity_edges_kernel": ("antialias", "31mark_discontinuity_edges_kernel"),
    "backward_antialiased_cluster_bitset_kernel": ("antialias", "42backward_antialiased_cluster_bitset_kernel"),
    "accumulate_bitset_rgb_kernel": ("bitset_utils", "28accumulate_bitset_rgb_kernel"),
    "popcount_bitset_kernel": ("bitset_utils", "22popcount_bitset_kernel"),
    "compact_valid_ints_kernel": ("compact_utils", "25compact_valid_ints_kernel"),
    "smooth_strands_kernel": ("curve_utils", "21smooth_strands_kernel"),
    "skinning_kernel": ("curve_utils", "15skinning_kernel"),
}
TPB = 256


def available() -> bool:
    return all(os.path.exists(os.path.join(REF_DIR, u + ".cubin")) for u in _UNITS)


class _I(ctypes.c_int):
    pass


def _blocks(n: int) -> int:
    return (n + TPB - 1) // TPB


class RefKernels:
    def __init__(self):
        if not available():
            raise FileNotFoundError(f"reference cubins missing under {REF_DIR}")
        torch.cuda.init()
        torch.empty(1, device="cuda")  # make the primary context current on this thread
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.cu.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        self.mods = {}
        for u in _UNITS:
            m = ctypes.c_void_p()
            self._ck(self.cu.cuModuleLoad(ctypes.byref(m), os.path.join(REF_DIR, u + ".cubin").encode()), "cuModuleLoad " + u)
            self.mods[u] = m
        self.funcs = {}
        for name, (unit, key) in _KERNELS.items():
            self.funcs[name] = self._find(self.mods[unit], key)

    def _ck(self, rc, what):
        if rc != 0:
            s = ctypes.c_char_p()
            self.cu.cuGetErrorString(rc, ctypes.byref(s))
            raise RuntimeError(f"{what}: CUDA driver error {rc} ({s.value})")

    def _find(self, mod, key):
        n = ctypes.c_uint()
        self._ck(self.cu.cuModuleGetFunctionCount(ctypes.byref(n), mod), "cuModuleGetFunctionCount")
        arr = (ctypes.c_void_p * n.value)()
        self._ck(self.cu.cuModuleEnumerateFunctions(arr, n, mod), "cuModuleEnumerateFunctions")
        for f in arr:
            nm = ctypes.c_char_p()
            self._ck(self.cu.cuFuncGetName(ctypes.byref(nm), ctypes.c_void_p(f)), "cuFuncGetName")
            s = nm.value.decode()
            if key in s and "device_stub" not in s:
                return ctypes.c_void_p(f)
        raise KeyError(key)

    def launch(self, name, n_threads, args, smem=0):
        if n_threads <= 0:
            return
        vals = []
        for a in args:
            if isinstance(a, torch.Tensor):
                vals.append(ctypes.c_uint64(a.data_ptr()))
            elif isinstance(a, float):
                vals.append(ctypes.c_float(a))
            elif isinstance(a, int):
                vals.append(ctypes.c_int(a))
            elif a is None:
                vals.append(ctypes.c_uint64(0))
            else:
                raise TypeError(type(a))
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        self._ck(self.cu.cuLaunchKernel(self.funcs[name], _blocks(n_threads), 1, 1, TPB, 1, 1,
                                        smem, None, params, None), "cuLaunchKernel " + name)

    def sync(self):
        torch.cuda.synchronize()

    # ---- dda.py --------------------------------------------------------------------
    def dda_compute_fragments(self, H, W, pos, edges, edge_ids: Optional[torch.Tensor] = None):
        """``dda.py:5-76`` over the reference kernels."""
        B, V, _ = pos.shape
        E = edges.shape[0]
        dev = pos.device
        if edge_ids is None:
            edge_ids = torch.arange(B * E, dtype=torch.int32, device=dev)
        P = edge_ids.shape[0]
        counts = torch.empty(P, dtype=torch.int32, device=dev)
        slopes = torch.empty((P, 2), dtype=torch.float32, device=dev)
        spans = torch.empty((P, 4), dtype=torch.float32, device=dev)
        self.launch("dda_compute_span_kernel", P, [P, edge_ids, H, W, V, pos, E, edges, counts, slopes, spans])
        prefix = torch.cumsum(counts, 0, dtype=torch.int32) if P else counts
        F = int(prefix[-1].item()) if P else 0
        frag_pix = torch.full((F, 3), -1, dtype=torch.int32, device=dev)
        frag_attrs = torch.empty((F, 4), dtype=torch.float32, device=dev)
        self.launch("dda_compute_fragments_kernel", F, [P, F, prefix, edge_ids, slopes, spans, H, W, V, pos,
                                                        E, edges, frag_pix, frag_attrs])
        out = self.filter_valid_fragments(frag_pix, frag_attrs)
        return out, (counts, slopes, spans, prefix, frag_pix, frag_attrs)

    def filter_valid_fragments(self, frag_pix, frag_attrs):
        F = frag_pix.shape[0]
        if F == 0:
            return frag_pix[:0].clone(), frag_attrs[:0].clone()
        po = torch.empty_like(frag_pix)
        ao = torch.empty_like(frag_attrs)
        ctr = torch.zeros(1, dtype=torch.int32, device=frag_pix.device)
        self.launch("filter_valid_fragments_kernel", F, [F, frag_pix, frag_attrs, po, ao, ctr], smem=4 * (TPB + 1))
        n = int(ctr.item())
        return po[:n], ao[:n]

    # ---- rasterize.py --------------------------------------------------------------
    def compute_fragments(self, H, W, pos, tri):
        """``rasterize.py:6-53`` over the reference kernels."""
        B, V, _ = pos.shape
        T = tri.shape[0]
        dev = pos.device
        rects = torch.empty((B * T, 4), dtype=torch.int32, device=dev)
        counts = torch.empty(B * T, dtype=torch.int32, device=dev)
        self.launch("compute_triangle_rects_kernel", B * T, [H, W, B, V, pos, T, tri, rects, counts])
        prefix = torch.cumsum(counts, 0, dtype=torch.int32)
        F = int(prefix[-1].item()) if B * T else 0
        frag_pix = torch.full((F, 3), -1, dtype=torch.int32, device=dev)
        frag_attrs = torch.empty((F, 4), dtype=torch.float32, device=dev)
        self.launch("compute_fragments_kernel", F, [H, W, V, pos, T, tri, B * T, F, prefix, rects, frag_pix, frag_attrs])
        return self.filter_valid_fragments(frag_pix, frag_attrs), (rects, counts)

    def depth_test(self, B, H, W, frag_pix, frag_attrs):
        """``rasterize.py:55-95`` / ``rasterize.cu:258-278``."""
        total = B * H * W
        rast = torch.zeros((B, H, W, 4), dtype=torch.float32, device=frag_pix.device)
        zb = torch.empty(total, dtype=torch.int64, device=frag_pix.device)
        self.launch("fill_ll_max", total, [zb, total])
        self.launch("depth_test_kernel", frag_pix.shape[0], [frag_pix.shape[0], frag_pix, frag_attrs, H, W, zb])
        self.launch("gather_depth_test_kernel", total, [B, H, W, zb, frag_attrs, rast])
        return rast

    def interpolate(self, rast, attr, tri):
        B, H, W, _ = rast.shape
        C = attr.shape[1]
        img = torch.zeros((B, H, W, C), dtype=torch.float32, device=rast.device)
        self.launch("interpolate_triangle_attributes_kernel", B * H * W, [B, H, W, rast, C, attr, tri, img])
        return img

    def interpolate_backward(self, rast, d_img, tri, V):
        B, H, W, _ = rast.shape
        C = d_img.shape[3]
        d_attr = torch.zeros((V, C), dtype=torch.float32, device=rast.device)
        self.launch("backward_interpolate_triangle_attributes_kernel", B * H * W, [B, H, W, rast, C, d_img, tri, d_attr])
        return d_attr

    def dda_interpolate(self, rast, attr, edges):
        B, H, W, _ = rast.shape
        C = attr.shape[1]
        img = torch.zeros((B, H, W, C), dtype=torch.float32, device=rast.device)
        self.launch("dda_interpolate_attributes_kernel", B * H * W, [B, H, W, rast, C, attr, edges, img])
        return img

    def dda_interpolate_backward(self, rast, d_img, edges, V):
        B, H, W, _ = rast.shape
        C = d_img.shape[3]
        d_attr = torch.zeros((V, C), dtype=torch.float32, device=rast.device)
        self.launch("backward_dda_interpolate_attributes_kernel", B * H * W, [B, H, W, rast, C, d_img, edges, d_attr])
        return d_attr

    def cluster_mask_from_fragments(self, H, W, frag_pix, frag_attrs, prim2cluster, cluster_count=None):
        """``rasterize.py:170-214``."""
        B = int(frag_pix[:, 0].max().item()) + 1
        K = cluster_count if cluster_count is not None else int(prim2cluster.max().item()) + 1
        S = (K + 31) // 32
        bitset = torch.zeros((B, H, W, S), dtype=torch.int32, device=frag_pix.device)
        F = frag_pix.shape[0]
        if F:
            self.launch("cluster_mask_from_fragments_kernel", F, [F, frag_pix, frag_attrs, prim2cluster, H, W, S, bitset])
        return bitset

    # ---- antialias.py --------------------------------------------------------------
    def mark_discontinuity_edges(self, H, W, pos, tri, edges, edge2tri):
        """``antialias.py:8-52``: raw (uncompacted) ids, compacted ids and normals."""
        B, V, _ = pos.shape
        E = edges.shape[0]
        ids = torch.full((B * E,), -1, dtype=torch.int32, device=pos.device)
        normals = torch.zeros((B * E, 2), dtype=torch.float32, device=pos.device)
        self.launch("mark_discontinuity_edges_kernel", B * E, [H, W, B, V, pos, tri, E, edges, edge2tri, ids, normals])
        out = torch.empty_like(ids)
        ctr = torch.zeros(1, dtype=torch.int32, device=pos.device)
        self.launch("compact_valid_ints_kernel", B * E, [B * E, ids, out, ctr], smem=4 * (TPB + 1))
        n = int(ctr.item())
        return ids, out[:n], normals

    def backward_antialiased(self, frag_pix, frag_attrs, bitset, target, pos, edges, normals, edge2cluster,
                             kernel_radius, rho):
        B, H, W, S = bitset.shape
        V = pos.shape[1]
        E = edges.shape[0]
        d_pos = torch.zeros_like(pos)
        F = frag_pix.shape[0]
        self.launch("backward_antialiased_cluster_bitset_kernel", F,
                    [F, frag_pix, frag_attrs, H, W, S, bitset, target, V, pos, E, edges, normals, edge2cluster,
                     d_pos, float(kernel_radius), float(rho)])
        return d_pos

    def antialiased_loss_grad(self, bitset, target, pos, tri, edges, edge2tri, edge2cluster, kernel_radius=7.0, rho=1.0):
        """``antialias.py:66-130`` up to ``d_pos`` (the gradient the loss hands back)."""
        _, H, W, _ = target.shape
        _, prim_ids, normals = self.mark_discontinuity_edges(H, W, pos, tri, edges, edge2tri)
        (fp, fa), _ = self.dda_compute_fragments(H, W, pos, edges, prim_ids)
        return self.backward_antialiased(fp, fa, bitset, target, pos, edges, normals, edge2cluster, kernel_radius, rho)

    # ---- bitset_utils.py -----------------------------------------------------------
    def popcount(self, bitset):
        B, H, W, S = bitset.shape
        out = torch.zeros((B, H, W), dtype=torch.float32, device=bitset.device)
        self.launch("popcount_bitset_kernel", B * H * W, [B, H, W, S, bitset, out])
        return out

    def accumulate_rgb(self, bitset, rgb):
        B, H, W, S = bitset.shape
        out = torch.zeros((B, H, W, 3), dtype=torch.float32, device=bitset.device)
        self.launch("accumulate_bitset_rgb_kernel", B * H * W, [B, H, W, S, bitset, rgb, out])
        return out

    # ---- curve_utils.py ------------------------------------------------------------
    def smooth_strands(self, strands, arclength, beta):
        N, V, _ = strands.shape
        out = torch.zeros_like(strands)
        self.launch("smooth_strands_kernel", N, [N, V, strands, arclength, out, float(beta)])
        return out

    def skinning(self, strands, arclength, handles, canonical, R, beta):
        N, V, _ = strands.shape
        out = torch.zeros_like(strands)
        self.launch("skinning_kernel", N, [N, V, strands, arclength, handles, canonical, R, out, float(beta)])
        return out
