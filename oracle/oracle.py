"""numpy front end of the CPU oracle (test infrastructure only).

Mirrors the reference's Python-level ops (``pystrns2cards/{dda,rasterize,antialias,
bitset_utils,curve_utils}.py``) on numpy arrays over ``liboracle.so`` (s2c_oracle.c).
Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

i32p = ctypes.POINTER(ctypes.c_int32)
f32p = ctypes.POINTER(ctypes.c_float)
f64p = ctypes.POINTER(ctypes.c_double)
I64 = ctypes.c_int64
I = ctypes.c_int
F = ctypes.c_float

_SIGS = {
    "or_version": ([], I),
    "or_set_model": ([I], None),
    "or_get_model": ([], I),
    "or_set_threads": ([I], None),
    "or_dda_span": ([I64, i32p, I, I, I, f32p, I, i32p, i32p, f32p, f32p], None),
    "or_dda_fragments": ([I64, i32p, i32p, f32p, f32p, I, I, I, f32p, I, i32p, i32p, f32p], None),
    "or_dda_cluster_bitset": ([I, I, I, I, f32p, I, i32p, i32p, I64, i32p, I, i32p], None),
    "or_tri_rects": ([I, I, I, I, f32p, I, i32p, i32p, i32p], None),
    "or_tri_fragments": ([I, I, I, I, f32p, I, i32p, i32p, i32p, i32p, f32p], None),
    "or_filter_valid": ([I64, i32p, f32p, i32p, f32p], I64),
    "or_depth_test": ([I, I, I, I64, i32p, f32p, f32p], None),
    "or_cluster_mask": ([I64, i32p, f32p, i32p, I, I, I, i32p], None),
    "or_interpolate": ([I, I, I, f32p, I, f32p, i32p, f64p], None),
    "or_interpolate_backward": ([I, I, I, f32p, I, f32p, i32p, f64p], None),
    "or_dda_interpolate": ([I, I, I, f32p, I, f32p, i32p, f64p], None),
    "or_dda_interpolate_backward": ([I, I, I, f32p, I, f32p, i32p, f64p], None),
    "or_mark_edges": ([I, I, I, I, f32p, i32p, I, i32p, i32p, i32p, f32p], None),
    "or_compact_ints": ([I64, i32p, i32p], I64),
    "or_aa_backward": ([I64, i32p, f32p, I, I, I, i32p, i32p, I, f32p, I, i32p, f32p, i32p, f64p, F, F, f64p], None),
    "or_popcount": ([I64, I, i32p, f32p], None),
    "or_accumulate_rgb": ([I64, I, i32p, f32p, f32p], None),
    "or_smooth_strands": ([I, I, f32p, f32p, f64p, F], None),
    "or_skinning": ([I, I, f32p, f32p, f32p, f32p, f32p, f64p, F], None),
    "or_knn4": ([ctypes.c_int64, f32p, I, f32p, i32p, f32p], None),
}

# arithmetic-model flags (s2c_oracle.h)
FMA_DDA_SPAN, FMA_DDA_STEP, FMA_DDA_PERSP, FMA_DDA_Z = 1, 2, 4, 8
FMA_TRI_RECT, FMA_TRI_Q, FMA_TRI_A, FMA_TRI_A_ALT, FMA_TRI_Z, FMA_AA = 16, 32, 64, 128, 256, 512


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        src = os.path.join(HERE, "s2c_oracle.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            subprocess.run(["make", "-s", "-C", HERE], check=True)
        L = ctypes.CDLL(path)
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = L
    return _LIB


def _p(a: Optional[np.ndarray], ptype):
    if a is None:
        return ctypes.cast(None, ptype)
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be contiguous"
    return a.ctypes.data_as(ptype)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def set_model(flags: int = -1):
    lib().or_set_model(int(flags))


def get_model() -> int:
    return int(lib().or_get_model())


def set_threads(n: int):
    lib().or_set_threads(int(n))


# ---- dda.py ------------------------------------------------------------------------
def dda_span(H, W, pos, edges, edge_ids=None):
    pos, edges = _f32(pos), _i32(edges)
    B, V, _ = pos.shape
    E = edges.shape[0]
    ids = None if edge_ids is None else _i32(edge_ids)
    P = B * E if ids is None else ids.shape[0]
    counts = np.empty(P, np.int32)
    slopes = np.empty((P, 2), np.float32)
    spans = np.empty((P, 4), np.float32)
    lib().or_dda_span(P, _p(ids, i32p), H, W, V, _p(pos, f32p), E, _p(edges, i32p),
                      _p(counts, i32p), _p(slopes, f32p), _p(spans, f32p))
    return counts, slopes, spans


def dda_compute_fragments(H, W, pos, edges, edge_ids=None, raw=False):
    """``dda.py:5-76``; fragments in prim order (the order an in-order compaction gives)."""
    pos, edges = _f32(pos), _i32(edges)
    B, V, _ = pos.shape
    E = edges.shape[0]
    ids = None if edge_ids is None else _i32(edge_ids)
    counts, slopes, spans = dda_span(H, W, pos, edges, ids)
    prefix = np.cumsum(counts, dtype=np.int64).astype(np.int32)
    Ft = int(prefix[-1]) if prefix.shape[0] else 0
    pix = np.full((Ft, 3), -1, np.int32)
    attrs = np.zeros((Ft, 4), np.float32)
    lib().or_dda_fragments(counts.shape[0], _p(prefix, i32p), _p(ids, i32p), _p(slopes, f32p),
                           _p(spans, f32p), H, W, V, _p(pos, f32p), E, _p(edges, i32p),
                           _p(pix, i32p), _p(attrs, f32p))
    po = np.empty_like(pix)
    ao = np.empty_like(attrs)
    n = lib().or_filter_valid(Ft, _p(pix, i32p), _p(attrs, f32p), _p(po, i32p), _p(ao, f32p))
    if raw:
        return po[:n], ao[:n], dict(counts=counts, slopes=slopes, spans=spans, prefix=prefix,
                                    raw_pix=pix, raw_attrs=attrs)
    return po[:n], ao[:n]


def dda_cluster_bitset(H, W, pos, edges, prim2cluster, K, edge_ids=None):
    pos, edges, p2c = _f32(pos), _i32(edges), _i32(prim2cluster)
    B, V, _ = pos.shape
    E = edges.shape[0]
    S = (K + 31) // 32
    ids = None if edge_ids is None else _i32(edge_ids)
    P = B * E if ids is None else ids.shape[0]
    bits = np.empty((B, H, W, S), np.int32)
    lib().or_dda_cluster_bitset(B, H, W, V, _p(pos, f32p), E, _p(edges, i32p), _p(ids, i32p), P,
                                _p(p2c, i32p), S, _p(bits, i32p))
    return bits


def cluster_mask_from_fragments(H, W, frag_pix, frag_attrs, prim2cluster, cluster_count=None, B=None):
    """``rasterize.py:170-214`` (B inferred from the fragments unless given)."""
    fp, fa, p2c = _i32(frag_pix), _f32(frag_attrs), _i32(prim2cluster)
    if B is None:
        B = int(fp[:, 0].max()) + 1
    K = cluster_count if cluster_count is not None else int(p2c.max()) + 1
    S = (K + 31) // 32
    bits = np.zeros((B, H, W, S), np.int32)
    lib().or_cluster_mask(fp.shape[0], _p(fp, i32p), _p(fa, f32p), _p(p2c, i32p), H, W, S, _p(bits, i32p))
    return bits


# ---- rasterize.py --------------------------------------------------------------------
def tri_rects(H, W, pos, tri):
    pos, tri = _f32(pos), _i32(tri)
    B, V, _ = pos.shape
    T = tri.shape[0]
    rects = np.empty((B * T, 4), np.int32)
    counts = np.empty(B * T, np.int32)
    lib().or_tri_rects(H, W, B, V, _p(pos, f32p), T, _p(tri, i32p), _p(rects, i32p), _p(counts, i32p))
    return rects, counts


def compute_fragments(H, W, pos, tri, raw=False):
    """``rasterize.py:6-53``; fragments in (view, triangle, row-major pixel) order."""
    pos, tri = _f32(pos), _i32(tri)
    B, V, _ = pos.shape
    T = tri.shape[0]
    rects, counts = tri_rects(H, W, pos, tri)
    prefix = np.cumsum(counts, dtype=np.int64).astype(np.int32)
    Ft = int(prefix[-1]) if prefix.shape[0] else 0
    pix = np.full((Ft, 3), -1, np.int32)
    attrs = np.zeros((Ft, 4), np.float32)
    lib().or_tri_fragments(H, W, B, V, _p(pos, f32p), T, _p(tri, i32p), _p(rects, i32p),
                           _p(prefix, i32p), _p(pix, i32p), _p(attrs, f32p))
    po = np.empty_like(pix)
    ao = np.empty_like(attrs)
    n = lib().or_filter_valid(Ft, _p(pix, i32p), _p(attrs, f32p), _p(po, i32p), _p(ao, f32p))
    if raw:
        return po[:n], ao[:n], dict(rects=rects, counts=counts)
    return po[:n], ao[:n]


def depth_test(B, H, W, frag_pix, frag_attrs):
    fp, fa = _i32(frag_pix), _f32(frag_attrs)
    rast = np.empty((B, H, W, 4), np.float32)
    lib().or_depth_test(B, H, W, fp.shape[0], _p(fp, i32p), _p(fa, f32p), _p(rast, f32p))
    return rast


def rasterize(H, W, pos, tri):
    fp, fa = compute_fragments(H, W, pos, tri)
    return depth_test(pos.shape[0], H, W, fp, fa)


def interpolate(rast, attr, tri):
    rast, attr, tri = _f32(rast), _f32(attr), _i32(tri)
    B, H, W, _ = rast.shape
    C = attr.shape[1]
    img = np.empty((B, H, W, C), np.float64)
    lib().or_interpolate(B, H, W, _p(rast, f32p), C, _p(attr, f32p), _p(tri, i32p), _p(img, f64p))
    return img


def interpolate_backward(rast, d_image, tri, V):
    rast, g, tri = _f32(rast), _f32(d_image), _i32(tri)
    B, H, W, _ = rast.shape
    C = g.shape[3]
    d = np.zeros((V, C), np.float64)
    lib().or_interpolate_backward(B, H, W, _p(rast, f32p), C, _p(g, f32p), _p(tri, i32p), _p(d, f64p))
    return d


def dda_interpolate(rast, attr, edges):
    rast, attr, edges = _f32(rast), _f32(attr), _i32(edges)
    B, H, W, _ = rast.shape
    C = attr.shape[1]
    img = np.empty((B, H, W, C), np.float64)
    lib().or_dda_interpolate(B, H, W, _p(rast, f32p), C, _p(attr, f32p), _p(edges, i32p), _p(img, f64p))
    return img


def dda_interpolate_backward(rast, d_image, edges, V):
    rast, g, edges = _f32(rast), _f32(d_image), _i32(edges)
    B, H, W, _ = rast.shape
    C = g.shape[3]
    d = np.zeros((V, C), np.float64)
    lib().or_dda_interpolate_backward(B, H, W, _p(rast, f32p), C, _p(g, f32p), _p(edges, i32p), _p(d, f64p))
    return d


# ---- antialias.py --------------------------------------------------------------------
def mark_discontinuity_edges(H, W, pos, tri, edges, edge2tri, raw=False):
    """``antialias.py:8-52``: (compacted prim ids in index order, normals (B*E, 2))."""
    pos, tri, edges, e2t = _f32(pos), _i32(tri), _i32(edges), _i32(edge2tri)
    B, V, _ = pos.shape
    E = edges.shape[0]
    ids = np.full(B * E, -1, np.int32)
    normals = np.zeros((B * E, 2), np.float32)
    lib().or_mark_edges(H, W, B, V, _p(pos, f32p), _p(tri, i32p), E, _p(edges, i32p), _p(e2t, i32p),
                        _p(ids, i32p), _p(normals, f32p))
    out = np.empty_like(ids)
    n = lib().or_compact_ints(ids.shape[0], _p(ids, i32p), _p(out, i32p))
    if raw:
        return out[:n], normals, ids
    return out[:n], normals


def aa_backward(frag_pix, frag_attrs, bitset, target, pos, edges, normals, edge2cluster,
                kernel_radius=7.0, rho=1.0, return_dc=False):
    fp, fa = _i32(frag_pix), _f32(frag_attrs)
    bits, tgt = _i32(bitset), _i32(target)
    pos, edges, normals, e2c = _f32(pos), _i32(edges), _f32(normals), _i32(edge2cluster)
    B, H, W, S = bits.shape
    V = pos.shape[1]
    E = edges.shape[0]
    d = np.zeros(pos.shape, np.float64)
    dc = np.zeros(fp.shape[0], np.float64)
    lib().or_aa_backward(fp.shape[0], _p(fp, i32p), _p(fa, f32p), H, W, S, _p(bits, i32p), _p(tgt, i32p),
                         V, _p(pos, f32p), E, _p(edges, i32p), _p(normals, f32p), _p(e2c, i32p),
                         _p(d, f64p), float(kernel_radius), float(rho), _p(dc, f64p))
    return (d, dc) if return_dc else d


def antialias_grad(bitset, target, pos, tri, edges, edge2tri, edge2cluster, kernel_radius=7.0, rho=1.0):
    """``antialias.py:66-130`` up to ``d_pos`` (FP64)."""
    _, H, W, _ = target.shape
    ids, normals = mark_discontinuity_edges(H, W, pos, tri, edges, edge2tri)
    fp, fa = dda_compute_fragments(H, W, pos, edges, ids)
    return aa_backward(fp, fa, bitset, target, pos, edges, normals, edge2cluster, kernel_radius, rho)


# ---- bitset_utils.py -----------------------------------------------------------------
def popcount_bitset(bitset):
    b = _i32(bitset)
    out = np.empty(b.shape[:3], np.float32)
    lib().or_popcount(int(np.prod(b.shape[:3])), b.shape[3], _p(b, i32p), _p(out, f32p))
    return out


def accumulate_bitset_rgb(bitset, rgb):
    b, c = _i32(bitset), _f32(rgb)
    out = np.empty(b.shape[:3] + (3,), np.float32)
    lib().or_accumulate_rgb(int(np.prod(b.shape[:3])), b.shape[3], _p(b, i32p), _p(c, f32p), _p(out, f32p))
    return out


# ---- curve_utils.py ------------------------------------------------------------------
def smooth_strands(strands, arclength, beta):
    s, a = _f32(strands), _f32(arclength)
    N, V, _ = s.shape
    out = np.zeros(s.shape, np.float64)
    lib().or_smooth_strands(N, V, _p(s, f32p), _p(a, f32p), _p(out, f64p), float(beta))
    return out


def skinning(strands, arclength, handles, canonical, R, beta):
    s, a, h, c, r = _f32(strands), _f32(arclength), _f32(handles), _f32(canonical), _f32(R)
    N, V, _ = s.shape
    out = np.zeros(s.shape, np.float64)
    lib().or_skinning(N, V, _p(s, f32p), _p(a, f32p), _p(h, f32p), _p(c, f32p), _p(r, f32p),
                      _p(out, f64p), float(beta))
    return out


def sort_frags(pix, attrs):
    """Canonical order (batch, prim id, h, w) used by the golden fixtures."""
    if pix.shape[0] == 0:
        return pix, attrs
    key = np.lexsort((pix[:, 2], pix[:, 1], attrs[:, 3], pix[:, 0]))
    return pix[key], attrs[key]


# ---- mesh topology: mesh_utils.cpp:36-95 (edge set and first-two-triangle adjacency),
# in the fixed (min, max)-sorted edge order
def build_edges_from_triangles(tri: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    if not isinstance(tri, np.ndarray):
        raise TypeError("Input must be a NumPy ndarray.")
    if tri.dtype != np.int32:
        raise TypeError("Triangle indices must be int32.")
    if tri.ndim != 2 or tri.shape[1] != 3:
        raise ValueError("Input triangle array must have shape (T, 3).")
    T = tri.shape[0]
    if T == 0:
        return np.zeros((0, 2), np.int32), np.zeros((0, 2), np.int32)
    t64 = tri.astype(np.int64)
    a = np.stack([t64[:, 0], t64[:, 1], t64[:, 2]], 1).reshape(-1)
    b = np.stack([t64[:, 1], t64[:, 2], t64[:, 0]], 1).reshape(-1)
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    owner = np.repeat(np.arange(T, dtype=np.int64), 3)
    order = np.lexsort((owner, hi, lo))
    lo, hi, owner = lo[order], hi[order], owner[order]
    first = np.ones(lo.shape[0], dtype=bool)
    first[1:] = (lo[1:] != lo[:-1]) | (hi[1:] != hi[:-1])
    starts = np.nonzero(first)[0]
    edges = np.stack([lo[starts], hi[starts]], 1).astype(np.int32)
    e2t = np.full((starts.shape[0], 2), -1, dtype=np.int32)
    e2t[:, 0] = owner[starts]
    nxt = starts + 1
    has2 = nxt < lo.shape[0]
    has2[has2] = ~first[nxt[has2]]
    e2t[has2, 1] = owner[nxt[has2]]
    return edges, e2t


# ---- card Laplacian smoothing: p <- p - lam * D^-1 L p with the uniform Laplacian of
# optimizer.py:70-99 (unique neighbour pairs, a self-loop counted once), FP64
def card_laplacian_smooth(verts, quad_edges, verts_per_card, lam=0.5, steps=10):
    nv = int(verts_per_card)
    e = np.asarray(quad_edges, np.int64).reshape(-1, 2)
    pairs = np.unique(np.concatenate([e, e[:, ::-1]], 0), axis=0) if e.size else np.zeros((0, 2), np.int64)
    deg = np.bincount(pairs[:, 0], minlength=nv).astype(np.float64)
    p = np.asarray(verts, np.float64).reshape(-1, nv, 3).copy()
    has = deg > 0
    for _ in range(int(steps)):
        s = np.zeros_like(p)
        np.add.at(s, (slice(None), pairs[:, 0]), p[:, pairs[:, 1]])
        mean = s[:, has] / deg[has][None, :, None]
        p[:, has] = p[:, has] - lam * (p[:, has] - mean)
    return p.reshape(-1, 3)


# ---- linear blend skinning to the 4 nearest guides: binding (exact FP32 selection, FP64
# weights), forward and gradients in FP64
def lbs_bind(x, guides, tau=0.01):
    xs, g = _f32(np.asarray(x).reshape(-1, 3)), _f32(np.asarray(guides).reshape(-1, 3))
    Nv, G = xs.shape[0], g.shape[0]
    idx = np.empty((Nv, 4), np.int32)
    d2 = np.empty((Nv, 4), np.float32)
    lib().or_knn4(Nv, _p(xs, f32p), G, _p(g, f32p), _p(idx, ctypes.POINTER(ctypes.c_int32)), _p(d2, f32p))
    ok = idx >= 0
    d = d2.astype(np.float64)
    e = np.where(ok, np.exp(-(np.where(ok, d, d[:, :1]) - d[:, :1]) / float(tau)), 0.0)
    w = e / np.maximum(e.sum(1, keepdims=True), 1e-300)
    return idx, w


def lbs_forward(x, idx, w, M, chunk=1 << 19):
    """y_v = sum_k w_vk (A_k x_v + t_k) in FP64, in chunks of vertices."""
    x = np.asarray(x, np.float64).reshape(-1, 3)
    M = np.asarray(M, np.float64)
    idx = np.asarray(idx)
    w = np.asarray(w, np.float64)
    y = np.zeros((x.shape[0], 3), np.float64)
    for a in range(0, x.shape[0], chunk):
        b = min(a + chunk, x.shape[0])
        xh = np.concatenate([x[a:b], np.ones((b - a, 1))], 1)
        ok = idx[a:b] >= 0
        Mi = M[np.where(ok, idx[a:b], 0)]                       # (n, 4, 3, 4)
        yk = np.einsum("vkrc,vc->vkr", Mi, xh)
        y[a:b] = np.einsum("vk,vkr->vr", np.where(ok, w[a:b], 0.0), yk)
    return y


def lbs_backward(x, idx, w, M, gy, chunk=1 << 19):
    """dM_g = sum over bindings (v, k) to guide g of w_vk gy_v [x_v; 1]^T, and
    dx_v = sum_k w_vk A_k^T gy_v, in FP64 (chunks of vertices; per-guide sums by bincount)."""
    x = np.asarray(x, np.float64).reshape(-1, 3)
    M = np.asarray(M, np.float64)
    gy = np.asarray(gy, np.float64).reshape(-1, 3)
    idx = np.asarray(idx)
    w = np.asarray(w, np.float64)
    G = M.shape[0]
    dM = np.zeros_like(M)
    dx = np.zeros((x.shape[0], 3), np.float64)
    for a in range(0, x.shape[0], chunk):
        b = min(a + chunk, x.shape[0])
        xh = np.concatenate([x[a:b], np.ones((b - a, 1))], 1)
        ok = idx[a:b] >= 0
        wz = np.where(ok, w[a:b], 0.0)
        ii = np.where(ok, idx[a:b], 0).reshape(-1)
        for r in range(3):
            for c in range(4):
                dM[:, r, c] += np.bincount(ii, weights=(wz * (gy[a:b, r] * xh[:, c])[:, None]).reshape(-1),
                                           minlength=G)
        A = M[np.where(ok, idx[a:b], 0)][..., :3]                # (n, 4, 3, 3)
        dx[a:b] = np.einsum("vk,vkrc,vr->vc", wz, A, gy[a:b])
    return dM, dx


# ---- barycentric derivatives (new output): the forward's clip-space edge functions
# (rasterize.cu:144-156) at the pixel centre, differentiated in FP64
def barycentric_derivatives(rast, pos, tri, with_mag=False, chunk=1 << 20):
    """d(b0, b1)/d(x, y) in FP64 (out[..., 0:2] = db0/dx, db0/dy; out[..., 2:4] = db1/dx,
    db1/dy).  With ``with_mag``, also a first-order condition scale per element: the error
    that one unit roundoff in every input and intermediate of the formula would cause,
    propagated with absolute values (sums and products add their terms' magnitudes; a
    quotient n / d adds |n| / |d| times the relative error of d)."""
    rast = np.asarray(rast, np.float32)
    B, H, W, _ = rast.shape
    out = np.zeros((B, H, W, 4), np.float64)
    mag = np.zeros((B, H, W, 4), np.float64) if with_mag else None
    t = rast[..., 3].astype(np.int64) - 1
    bs, ys, xs = np.nonzero(t >= 0)
    pos64 = np.asarray(pos, np.float64)
    tri = np.asarray(tri)
    j, k = [1, 2, 0], [2, 0, 1]
    for c0 in range(0, bs.shape[0], chunk):
        b, y, x = bs[c0:c0 + chunk], ys[c0:c0 + chunk], xs[c0:c0 + chunk]
        tt = t[b, y, x]
        # pixel centre in NDC, in FP32 as the forward computes it
        px = (np.float32(-1) + (np.float32(2) * (x.astype(np.float32) + np.float32(0.5))) / np.float32(W)).astype(np.float64)
        py = (np.float32(-1) + (np.float32(2) * (y.astype(np.float32) + np.float32(0.5))) / np.float32(H)).astype(np.float64)
        P = pos64[b[:, None], tri[tt]]                                               # (n, 3, 4)
        qx = P[..., 0] - px[:, None] * P[..., 3]
        qy = -P[..., 1] - py[:, None] * P[..., 3]
        A = qx[:, j] * qy[:, k] - qy[:, j] * qx[:, k]                               # (n, 3)
        dAx = P[:, j, 3] * P[:, k, 1] - P[:, k, 3] * P[:, j, 1]
        dAy = P[:, j, 3] * P[:, k, 0] - P[:, k, 3] * P[:, j, 0]
        S = A.sum(1)
        ok = S != 0
        Ss = np.where(ok, S, 1.0)
        bb = A / Ss[:, None]
        sxy = (2.0 / W, 2.0 / H)
        if with_mag:
            mqx = np.abs(P[..., 0]) + np.abs(px[:, None] * P[..., 3])
            mqy = np.abs(P[..., 1]) + np.abs(py[:, None] * P[..., 3])
            mA = mqx[:, j] * mqy[:, k] + mqy[:, j] * mqx[:, k]
            mS = mA.sum(1)
            mdx = np.abs(P[:, j, 3] * P[:, k, 1]) + np.abs(P[:, k, 3] * P[:, j, 1])
            mdy = np.abs(P[:, j, 3] * P[:, k, 0]) + np.abs(P[:, k, 3] * P[:, j, 0])
        for i in range(2):
            for d, (dA, sc) in enumerate(((dAx, sxy[0]), (dAy, sxy[1]))):
                sd = dA.sum(1)
                N = dA[:, i] - bb[:, i] * sd
                out[b, y, x, 2 * i + d] = np.where(ok, N / Ss * sc, 0.0)
                if with_mag:
                    md = (mdx if d == 0 else mdy)
                    # |bb_i| times its relative error (A_i / S): mag(A_i) / |S| + |bb_i| mag(S) / |S|
                    mN = md[:, i] + np.abs(bb[:, i]) * md.sum(1) + np.abs(sd) * (mA[:, i] + np.abs(bb[:, i]) * mS) / np.abs(Ss)
                    mag[b, y, x, 2 * i + d] = np.where(ok, (mN / np.abs(Ss) + np.abs(N) * mS / Ss ** 2) * sc, 0.0)
    return (out, mag) if with_mag else out


# ---- strand frames and wisp alignment (curve_utils.py:9-165, 243-308, 481-607), FP64 numpy
def tangent_frame(t):
    """curve_utils.py:76-102: branch-free orthonormal (normal, binormal) around t."""
    t = np.asarray(t, np.float64)
    t = t / np.maximum(np.linalg.norm(t, axis=-1, keepdims=True), 1e-8)
    x, y, z = t[..., 0], t[..., 1], t[..., 2]
    sign = np.where(z > 0, 1.0, np.where(z < 0, -1.0, 1.0))
    a = -1.0 / (sign + z)
    b = x * y * a
    n = np.stack([1.0 + sign * x * x * a, sign * b, -sign * x], -1)
    bn = np.stack([b, sign + y * y * a, -y], -1)
    return n, bn


def minimal_rotation(src, dst):
    """curve_utils.py:9-74: Rodrigues rotation taking src onto dst; identity when parallel
    (cos > 1 - 1e-6), diag(-1, -1, 1) when antiparallel (cos < -1 + 1e-6)."""
    s = np.asarray(src, np.float64)
    d = np.broadcast_to(np.asarray(dst, np.float64), s.shape)
    s = s / np.maximum(np.linalg.norm(s, axis=-1, keepdims=True), 1e-8)
    d = d / np.maximum(np.linalg.norm(d, axis=-1, keepdims=True), 1e-8)
    ax = np.cross(s, d)
    sn = np.linalg.norm(ax, axis=-1)
    cs = np.clip((s * d).sum(-1), -1.0, 1.0)
    ax = ax / np.maximum(sn, 1e-8)[..., None]
    K = np.zeros(s.shape[:-1] + (3, 3))
    K[..., 0, 1], K[..., 0, 2] = -ax[..., 2], ax[..., 1]
    K[..., 1, 0], K[..., 1, 2] = ax[..., 2], -ax[..., 0]
    K[..., 2, 0], K[..., 2, 1] = -ax[..., 1], ax[..., 0]
    R = np.eye(3) + sn[..., None, None] * K + (1.0 - cs)[..., None, None] * (K @ K)
    R = np.where((cs > 1 - 1e-6)[..., None, None], np.eye(3), R)
    return np.where((cs < -1 + 1e-6)[..., None, None], np.diag([-1.0, -1.0, 1.0]), R)


def bishop_frame(strands):
    """curve_utils.py:104-165: double-reflection rotation-minimising frame (T, N, B)."""
    p = np.asarray(strands, np.float64)
    d = p[:, 1:] - p[:, :-1]
    T = np.zeros_like(p)
    T[:, :-1] += d
    T[:, 1:] += d
    T = T / np.maximum(np.linalg.norm(T, axis=-1, keepdims=True), 1e-8)
    N = np.zeros_like(p)
    B = np.zeros_like(p)
    N[:, 0], B[:, 0] = tangent_frame(T[:, 0])

    def dot(a, b):
        return (a * b).sum(-1, keepdims=True)

    for i in range(1, p.shape[1]):
        v1 = p[:, i] - p[:, i - 1]
        c1 = np.maximum(dot(v1, v1), 1e-8)
        nL = N[:, i - 1] - 2 * (dot(v1, N[:, i - 1]) / c1) * v1
        tL = T[:, i - 1] - 2 * (dot(v1, T[:, i - 1]) / c1) * v1
        v2 = T[:, i] - tL
        c2 = np.maximum(dot(v2, v2), 1e-8)
        n1 = nL - 2 * (dot(v2, nL) / c2) * v2
        n1 = n1 / np.maximum(np.linalg.norm(n1, axis=-1, keepdims=True), 1e-8)
        b1 = np.cross(T[:, i], n1)
        B[:, i] = b1 / np.maximum(np.linalg.norm(b1, axis=-1, keepdims=True), 1e-8)
        N[:, i] = n1
    return T, N, B


def alignment_rotation(strands, t_dst):
    """curve_utils.py:273-308: R = [t_dst n_dst b_dst][T N B]^T per point, (n_dst, b_dst) the
    root frame turned by the minimal rotation of the root tangent onto t_dst."""
    T, N, B = bishop_frame(strands)
    td = np.broadcast_to(np.asarray(t_dst, np.float64).reshape(3), T.shape)
    Ra = minimal_rotation(T[:, 0], td[:, 0])
    nd = np.einsum("sij,sj->si", Ra, N[:, 0])
    bd = np.einsum("sij,sj->si", Ra, B[:, 0])
    Rdst = np.stack([td, np.broadcast_to(nd[:, None], T.shape), np.broadcast_to(bd[:, None], T.shape)], -1)
    Rsrc = np.stack([T, N, B], -1)
    return Rdst @ np.swapaxes(Rsrc, -1, -2)


def aligned_strands(strands, roots, t_dst):
    """curve_utils.py:243-271: arclength * t_dst + root."""
    p = np.asarray(strands, np.float64)
    arc = np.concatenate([np.zeros((p.shape[0], 1)), np.cumsum(np.linalg.norm(p[:, 1:] - p[:, :-1], axis=-1), 1)], 1)
    return arc[..., None] * np.asarray(t_dst, np.float64).reshape(1, 1, 3) + np.asarray(roots, np.float64)[:, None]


WISP_T_DST = np.array([0.0, 1.0, 0.0])
WISP_N_DST = np.array([0.0, 0.0, -1.0])
WISP_B_DST = np.array([-1.0, 0.0, 0.0])


def wisp_frame(strands):
    """The loop body of align_wisps (curve_utils.py:521-568) for one wisp's float32 strands:
    (R_global, root centre, index of the longest strand), with the same numpy SVD call."""
    p = np.asarray(strands, np.float32).astype(np.float64)
    lengths = np.linalg.norm(p[:, 1:] - p[:, :-1], axis=-1).sum(1)
    centre = p[:, 0].mean(0)
    q = p - centre
    roots = q[:, 0]
    try:
        _, _, Vt = np.linalg.svd(roots, full_matrices=False)
        axes = Vt[:3] if Vt.shape == (3, 3) and np.all(np.isfinite(Vt[:3])) else np.eye(3)
    except np.linalg.LinAlgError:
        axes = np.eye(3)
    least, second = axes[2], axes[1]
    li = int(np.argmax(lengths))
    g = q[li]
    view = g[0] - g[1]
    view = view / max(np.linalg.norm(view), 1e-8)
    down = g[-1] - g[0]
    down = down / max(np.linalg.norm(down), 1e-8)
    sg = np.sign(least @ view)
    nsrc = least * (1.0 if sg == 0 else sg)
    tsrc = down - (down @ nsrc) * nsrc
    with np.errstate(invalid="ignore", divide="ignore"):
        tsrc = tsrc / np.linalg.norm(tsrc)
    if not np.all(np.isfinite(tsrc)):
        tsrc = second
    bsrc = np.cross(tsrc, nsrc)
    Rsrc = np.stack([tsrc, nsrc, bsrc], -1)
    Rdst = np.stack([WISP_T_DST, WISP_N_DST, WISP_B_DST], -1)
    return Rdst @ Rsrc.T, centre, li


def align_wisps(wisps, beta):
    """curve_utils.py:481-607 with the stages' float32 hand-offs: (aligned strands, smoothed
    strands before alignment, global index of each wisp's longest strand)."""
    arrs = [np.asarray(w, np.float32) for w in wisps]
    strands = np.concatenate(arrs, 0)
    arc = np.concatenate([np.zeros((strands.shape[0], 1), np.float32),
                          np.cumsum(np.linalg.norm(strands[:, 1:] - strands[:, :-1], axis=-1), 1)], 1)
    handles = smooth_strands(strands, arc, beta).astype(np.float32)
    s_rot, h_rot, longest = [], [], []
    off = 0
    for w in arrs:
        R, c, li = wisp_frame(w)
        s_rot.append((w.astype(np.float64) - c) @ R.T)
        h_rot.append((handles[off:off + w.shape[0]].astype(np.float64) - c) @ R.T)
        longest.append(off + li)
        off += w.shape[0]
    s_rot = np.concatenate(s_rot).astype(np.float32)
    h_rot = np.concatenate(h_rot).astype(np.float32)
    canon = aligned_strands(h_rot, s_rot[:, 0], WISP_T_DST).astype(np.float32)
    Rl = alignment_rotation(h_rot, WISP_T_DST).astype(np.float32)
    arc_s = np.concatenate([np.zeros((s_rot.shape[0], 1), np.float32),
                            np.cumsum(np.linalg.norm(s_rot[:, 1:] - s_rot[:, :-1], axis=-1), 1)], 1)
    out = skinning(s_rot, arc_s, h_rot, canon, Rl, beta)
    return out, handles, np.asarray(longest, np.int64)


def align_wisp(strands, beta):
    """curve_utils.py:376-479 (one wisp): (aligned strands, smoothed strands in the aligned
    frame, index of the longest strand), FP64 between float32 hand-offs."""
    p = np.asarray(strands, np.float32).astype(np.float64)
    p = p - p[:, 0].mean(0)
    _, _, Vt = np.linalg.svd(p[:, 0], full_matrices=False)
    pa = Vt[0] if np.all(np.isfinite(Vt[0])) else np.array([1.0, 0.0, 0.0])
    li = int(np.argmax(np.linalg.norm(p[:, 1:] - p[:, :-1], axis=-1).sum(1)))
    p32 = p.astype(np.float32)
    arc = np.concatenate([np.zeros((p.shape[0], 1), np.float32),
                          np.cumsum(np.linalg.norm(p32[:, 1:] - p32[:, :-1], axis=-1), 1)], 1)
    h = smooth_strands(p32, arc, beta)
    g = h[li]
    t0, t1 = g[1] - g[0], g[2] - g[1]
    t0 = t0 - (t0 @ pa) * pa
    t1 = t1 - (t1 @ pa) * pa
    t0, t1 = t0 / np.linalg.norm(t0), t1 / np.linalg.norm(t1)
    b0 = np.cross(t0, t1)
    b0 = b0 / np.linalg.norm(b0)
    n0 = np.cross(b0, t0)
    n0 = n0 / np.linalg.norm(n0)
    if not (np.all(np.isfinite(n0)) and np.all(np.isfinite(b0))):
        n0, b0 = tangent_frame(t0)
    Rsrc = np.stack([t0, n0, b0], -1)
    Rdst = np.stack([[0.0, -1.0, 0.0], [0.0, 0.0, -1.0], [1.0, 0.0, 0.0]], -1)
    Rg = Rdst @ Rsrc.T
    s_rot = (p @ Rg.T).astype(np.float32)
    h_rot = (h @ Rg.T).astype(np.float32)
    td = np.array([0.0, -1.0, 0.0])
    canon = aligned_strands(h_rot, s_rot[:, 0], td).astype(np.float32)
    Rl = alignment_rotation(h_rot, td).astype(np.float32)
    arc_s = np.concatenate([np.zeros((p.shape[0], 1), np.float32),
                            np.cumsum(np.linalg.norm(s_rot[:, 1:] - s_rot[:, :-1], axis=-1), 1)], 1)
    return skinning(s_rot, arc_s, h_rot, canon, Rl, beta), h_rot, li


# ---- condition scales of the float outputs -------------------------------------------
# Every float output on this path is a sum of products (weights and barycentrics are
# non-negative).  FP32 evaluation, here or in the reference, is accurate relative to the
# sum of the terms' magnitudes, which equals |value| only where no terms cancel.  Each
# function below evaluates the same FP64 formula on absolute values: per output element,
# sum |term|, where a factor that the formula itself forms by a subtraction (b2 = 1 - b0 -
# b1, t0 = 1 - t1) counts with the magnitude it was formed from.  The parity tests bound
# |got - FP64| by 1e-5 x max(|FP64 value|, this scale).
def _covered(rast, prim_count):
    r = np.asarray(rast, np.float32).reshape(-1, 4)
    t = r[:, 3].astype(np.int64) - 1
    ok = (t >= 0) & (t < prim_count)
    return np.nonzero(ok)[0], r[ok].astype(np.float64), t[ok]


def interpolate_mag(rast, attr, tri):
    """|b0 a0| + |b1 a1| + (1 + |b0| + |b1|) |a2| (rasterize.cu:367-400): b2 = 1 - b0 - b1 is
    itself a rounded difference, so its term is scaled by what it was computed from."""
    rast = np.asarray(rast, np.float32)
    a = np.abs(np.asarray(attr, np.float64))
    tri = np.asarray(tri, np.int64)
    B, H, W, _ = rast.shape
    out = np.zeros((B * H * W, a.shape[1]), np.float64)
    p, r, t = _covered(rast, tri.shape[0])
    v = tri[t]
    b0, b1 = np.abs(r[:, :1]), np.abs(r[:, 1:2])
    out[p] = b0 * a[v[:, 0]] + b1 * a[v[:, 1]] + (1.0 + b0 + b1) * a[v[:, 2]]
    return out.reshape(B, H, W, -1)


def _scatter_mag(V, C, idx_w):
    d = np.zeros((V, C), np.float64)
    for vi, w in idx_w:
        for c in range(C):
            d[:, c] += np.bincount(vi, weights=w[:, c], minlength=V)
    return d


def interpolate_backward_mag(rast, d_image, tri, V):
    """sum over pixels of |g| b0, |g| b1 and |g| (1 + b0 + b1) into the three vertices"""
    rast = np.asarray(rast, np.float32)
    tri = np.asarray(tri, np.int64)
    g = np.abs(np.asarray(d_image, np.float64)).reshape(-1, np.asarray(d_image).shape[-1])
    p, r, t = _covered(rast, tri.shape[0])
    v, gp = tri[t], g[p]
    b0, b1 = np.abs(r[:, :1]), np.abs(r[:, 1:2])
    return _scatter_mag(int(V), g.shape[1], [(v[:, 0], gp * b0), (v[:, 1], gp * b1), (v[:, 2], gp * (1.0 + b0 + b1))])


def dda_interpolate_mag(rast, attr, edges):
    """(1 + |t1|) |a0| + |t1| |a1| (dda.cu:258-298; t0 = 1 - t1 rounded)"""
    rast = np.asarray(rast, np.float32)
    a = np.abs(np.asarray(attr, np.float64))
    edges = np.asarray(edges, np.int64)
    B, H, W, _ = rast.shape
    out = np.zeros((B * H * W, a.shape[1]), np.float64)
    p, r, e = _covered(rast, edges.shape[0])
    v = edges[e]
    t1 = np.abs(r[:, 1:2])
    out[p] = (1.0 + t1) * a[v[:, 0]] + t1 * a[v[:, 1]]
    return out.reshape(B, H, W, -1)


def dda_interpolate_backward_mag(rast, d_image, edges, V):
    rast = np.asarray(rast, np.float32)
    edges = np.asarray(edges, np.int64)
    g = np.abs(np.asarray(d_image, np.float64)).reshape(-1, np.asarray(d_image).shape[-1])
    p, r, e = _covered(rast, edges.shape[0])
    v, gp = edges[e], g[p]
    t1 = np.abs(r[:, 1:2])
    return _scatter_mag(int(V), g.shape[1], [(v[:, 0], gp * (1.0 + t1)), (v[:, 1], gp * t1)])


def smooth_strands_mag(strands, arclength, beta):
    """sum_j w_j |x_j| / sum_j w_j (curve_utils.cu:24-68; w_j > 0)"""
    return smooth_strands(np.abs(np.asarray(strands, np.float32)), arclength, beta)


def skinning_mag(strands, arclength, handles, canonical, R, beta):
    """sum_j w_j (|R_j| (|x_i| + |h_j|) + |c_j|) / sum_j w_j (curve_utils.cu:70-131)"""
    a32 = lambda a: np.abs(np.asarray(a, np.float32))
    return skinning(a32(strands), arclength, -a32(handles), a32(canonical), a32(R), beta)


def card_laplacian_smooth_mag(verts, quad_edges, verts_per_card, lam=0.5, steps=10):
    """p <- (1 - lam) p + lam mean(neighbours) has non-negative coefficients for lam in
    [0, 1]: the same iteration on |p|"""
    return card_laplacian_smooth(np.abs(np.asarray(verts, np.float64)), quad_edges, verts_per_card, lam, steps)


def lbs_forward_mag(x, idx, w, M):
    return lbs_forward(np.abs(np.asarray(x, np.float64)), idx, w, np.abs(np.asarray(M, np.float64)))


def lbs_backward_mag(x, idx, w, M, gy):
    return lbs_backward(np.abs(np.asarray(x, np.float64)), idx, w, np.abs(np.asarray(M, np.float64)),
                        np.abs(np.asarray(gy, np.float64)))
