"""Seeded synthetic hair, cluster and card workloads.

The reference pipeline reads CT2Hair-derived grooms from disk (``3_fitting.py:204-233``).
Those files are not available, so every benchmark and test in this package runs on
synthetic hair with the shapes of the published workloads:

* roots uniform on the upper (y >= 0) half of the unit sphere, sorted in 3-D Morton order
  before strand indices (and therefore cluster ids ``strand_idx // per_cluster``) are
  assigned, so each cluster is spatially compact;
* each strand steps 0.05 per segment along a direction that turns linearly from the root
  normal toward -y by 90 degrees over the strand, plus Gaussian jitter sigma = 0.005;
* orthographic views built like ``build_ortho_cameras`` (``3_fitting.py:62-152``):
  uniform XY scale with a margin, Z mapped to [-0.5, 0.5], w = 1;
* one card per cluster: a grid strip (``texture_utils.py:525-599`` topology) that follows
  the cluster's mean strand and spans the spread of its roots.

All positions are quantised to multiples of 2**-20 so that the inputs are identical on
x86 and Arm hosts even where libm's sin/cos differ in the last bit.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

_Q = 2.0 ** -20


def _quantise(a: np.ndarray) -> np.ndarray:
    return (np.round(a / _Q) * _Q).astype(np.float32)


def _morton3(q: np.ndarray) -> np.ndarray:
    """Interleave the bits of three 10-bit integer coordinates (N, 3) -> (N,) uint32."""
    def spread(v):
        v = v.astype(np.uint32) & np.uint32(0x3FF)
        v = (v | (v << np.uint32(16))) & np.uint32(0x030000FF)
        v = (v | (v << np.uint32(8))) & np.uint32(0x0300F00F)
        v = (v | (v << np.uint32(4))) & np.uint32(0x030C30C3)
        v = (v | (v << np.uint32(2))) & np.uint32(0x09249249)
        return v
    return spread(q[:, 0]) | (spread(q[:, 1]) << np.uint32(1)) | (spread(q[:, 2]) << np.uint32(2))


def make_strands(num_strands: int, num_verts: int, seed: int = 0,
                 step: float = 0.05, jitter: float = 0.005) -> np.ndarray:
    """Return (N, V, 3) float32 strands (see the module docstring for the model)."""
    rng = np.random.default_rng(seed)
    roots = rng.standard_normal((num_strands, 3))
    roots /= np.linalg.norm(roots, axis=1, keepdims=True)
    roots[:, 1] = np.abs(roots[:, 1])
    # spatially coherent strand order
    q = np.clip(((roots + 1.0) * 0.5 * 1023.0).astype(np.int64), 0, 1023)
    order = np.argsort(_morton3(q), kind="stable")
    roots = roots[order]

    n = roots
    down = np.array([0.0, -1.0, 0.0])
    u = down[None, :] - (n @ down)[:, None] * n
    un = np.linalg.norm(u, axis=1, keepdims=True)
    fallback = np.array([1.0, 0.0, 0.0])
    bad = un[:, 0] < 1e-6
    if np.any(bad):
        fb = fallback[None, :] - (n[bad] @ fallback)[:, None] * n[bad]
        u[bad] = fb
        un[bad] = np.linalg.norm(fb, axis=1, keepdims=True)
    u = u / un

    nseg = max(num_verts - 1, 1)
    theta = (0.5 * math.pi) * np.arange(nseg) / max(nseg - 1, 1)
    dirs = np.cos(theta)[None, :, None] * n[:, None, :] + np.sin(theta)[None, :, None] * u[:, None, :]
    pts = np.empty((num_strands, num_verts, 3), dtype=np.float64)
    pts[:, 0] = roots
    if num_verts > 1:
        pts[:, 1:] = roots[:, None, :] + step * np.cumsum(dirs, axis=1)
    pts += jitter * rng.standard_normal(pts.shape)
    return _quantise(pts)


def strand_edges(num_strands: int, num_verts: int) -> np.ndarray:
    """Polyline edges (N*(V-1), 2) int32 for strands stored back to back."""
    base = (np.arange(num_strands, dtype=np.int64) * num_verts)[:, None]
    j = np.arange(num_verts - 1, dtype=np.int64)[None, :]
    e0 = (base + j).reshape(-1)
    return np.stack([e0, e0 + 1], axis=1).astype(np.int32)


def ortho_cameras(points: np.ndarray, margin: float = 0.3, num_views: int = 1) -> np.ndarray:
    """(num_views, 4, 4) float32 orthographic MVPs following ``3_fitting.py:62-152``.

    View 0 looks down -z (the front view); views 1..12 are the reference's diagonal,
    face and edge directions of the bounding box.
    """
    p = points.reshape(-1, 3).astype(np.float64)
    mn, mx = p.min(0), p.max(0)
    center = 0.5 * (mn + mx)
    ex, ey, ez = 0.5 * (mx - mn)
    dirs = [(0.0, 0.0, ez),
            (ex, ey, ez), (-ex, ey, ez), (ex, -ey, ez), (ex, ey, -ez),
            (ex, 0.0, 0.0), (0.0, ey, 0.0),
            (ex, ey, 0.0), (ex, -ey, 0.0), (ex, 0.0, ez), (ex, 0.0, -ez),
            (0.0, ey, ez), (0.0, ey, -ez)]
    out = []
    for vp in dirs[:num_views]:
        vp = np.asarray(vp, dtype=np.float64)
        direction = -vp / np.linalg.norm(vp)
        up = np.array([0.0, 1.0, 0.0])
        if abs(direction @ up) > 0.9:
            up = np.array([1.0, 0.0, 0.0])
        right = np.cross(up, direction)
        right /= np.linalg.norm(right)
        up = np.cross(direction, right)
        R = np.stack([right, up, direction], axis=1)
        view = np.eye(4)
        view[:3, :3] = R.T
        view[:3, 3] = -R.T @ center
        cam = (p - center) @ R
        cmin, cmax = cam.min(0), cam.max(0)
        ext = cmax - cmin
        s_xy = 2.0 * (1.0 - margin) / max(ext[0], ext[1])
        s_z = 1.0 / ext[2]
        proj = np.eye(4)
        proj[0, 0] = proj[1, 1] = s_xy
        proj[2, 2] = s_z
        proj[:2, 3] = -(cmin[:2] + cmax[:2]) / 2 * s_xy
        proj[2, 3] = -(cmin[2] + cmax[2]) / 2 * s_z
        out.append(proj @ view)
    return np.stack(out).astype(np.float32)


def project(points: np.ndarray, mvp: np.ndarray) -> np.ndarray:
    """Homogeneous clip positions (B, V, 4) float32 of (V, 3) points under (B, 4, 4) MVPs."""
    p = points.reshape(-1, 3).astype(np.float64)
    ph = np.concatenate([p, np.ones((p.shape[0], 1))], axis=1)
    out = np.einsum("vk,bjk->bvj", ph, mvp.astype(np.float64))
    return np.ascontiguousarray(out.astype(np.float32))


def grid_strip(rows: int, cols: int):
    """Topology of a (rows x cols)-vertex grid strip, rows = polylines, cols = points.

    Follows ``wisp_to_grid_mesh`` (``texture_utils.py:525-599``): vertex ``i*cols+j``,
    triangles (i0,i1,i2),(i0,i2,i3) per quad, h_edges along polylines, w_edges across.
    """
    i = np.arange(rows - 1)[:, None]
    j = np.arange(cols - 1)[None, :]
    i0 = (i * cols + j).reshape(-1)
    i1 = ((i + 1) * cols + j).reshape(-1)
    i2 = ((i + 1) * cols + j + 1).reshape(-1)
    i3 = (i * cols + j + 1).reshape(-1)
    faces = np.stack([np.stack([i0, i1, i2], 1), np.stack([i0, i2, i3], 1)], 1).reshape(-1, 3)
    quads = np.stack([i0, i1, i2, i3], 1)
    hi = np.arange(rows)[:, None] * cols + np.arange(cols - 1)[None, :]
    h_edges = np.stack([hi.reshape(-1), hi.reshape(-1) + 1], 1)
    wi = np.arange(rows - 1)[:, None] * cols + np.arange(cols)[None, :]
    w_edges = np.stack([wi.reshape(-1), wi.reshape(-1) + cols], 1)
    return (faces.astype(np.int32), quads.astype(np.int32),
            h_edges.astype(np.int32), w_edges.astype(np.int32))


@dataclass
class Cards:
    verts: np.ndarray      # (Vc, 3) float32
    tri: np.ndarray        # (T, 3) int32
    quads: np.ndarray      # (Q, 4) int32
    h_edges: np.ndarray    # (He, 2) int32
    w_edges: np.ndarray    # (We, 2) int32
    tri2cluster: np.ndarray  # (T,) int32
    vert2cluster: np.ndarray  # (Vc,) int32


def make_cards(strands: np.ndarray, per_cluster: int, quads_along: int, quads_across: int,
               width_scale: float = 2.0, num_cards: int = 0) -> Cards:
    """One grid strip per cluster that follows the cluster's mean strand.  Clusters are
    runs of ``per_cluster`` consecutive strands, or, with ``num_cards`` > 0, the balanced
    split strand k -> card k * num_cards // N."""
    N, V, _ = strands.shape
    if num_cards > 0:
        K = int(num_cards)
        starts = (np.arange(K + 1) * N + K - 1) // K              # first strand s with s*K//N == k
    else:
        K = (N + per_cluster - 1) // per_cluster
        starts = np.minimum(np.arange(K + 1) * per_cluster, N)
    cols = quads_along + 1
    rows = quads_across + 1
    faces, quads, h_e, w_e = grid_strip(rows, cols)
    nv = rows * cols
    verts = np.empty((K, nv, 3), dtype=np.float64)
    src = np.linspace(0.0, V - 1, cols)
    lo = np.floor(src).astype(np.int64)
    hi = np.minimum(lo + 1, V - 1)
    fr = (src - lo)[:, None]
    for k in range(K):
        cl = strands[starts[k]:starts[k + 1]].astype(np.float64)
        mean = cl.mean(0)
        centre = (1.0 - fr) * mean[lo] + fr * mean[hi]           # (cols, 3)
        tangent = mean[-1] - mean[0]
        tangent /= max(np.linalg.norm(tangent), 1e-9)
        spread = cl[:, 0] - cl[:, 0].mean(0)
        side = np.cross(tangent, np.array([0.0, 0.0, 1.0]))
        if np.linalg.norm(side) < 1e-6:
            side = np.array([1.0, 0.0, 0.0])
        side /= np.linalg.norm(side)
        half = max(width_scale * float(np.sqrt((spread ** 2).sum(1).mean())), 0.02)
        offs = np.linspace(-half, half, rows)
        verts[k] = (centre[None, :, :] + offs[:, None, None] * side[None, None, :]).reshape(nv, 3)
    vbase = (np.arange(K) * nv)[:, None, None]
    tri = (faces[None] + vbase).reshape(-1, 3)
    qd = (quads[None] + vbase).reshape(-1, 4)
    he = (h_e[None] + vbase).reshape(-1, 2)
    we = (w_e[None] + vbase).reshape(-1, 2)
    t2c = np.repeat(np.arange(K), faces.shape[0])
    v2c = np.repeat(np.arange(K), nv)
    return Cards(_quantise(verts.reshape(-1, 3)), tri.astype(np.int32), qd.astype(np.int32),
                 he.astype(np.int32), we.astype(np.int32), t2c.astype(np.int32), v2c.astype(np.int32))


@dataclass
class StrandScene:
    strands: np.ndarray     # (N, V, 3)
    pos: np.ndarray         # (B, N*V, 4) clip positions
    edges: np.ndarray       # (E, 2)
    edge2cluster: np.ndarray  # (E,)
    num_clusters: int
    mvp: np.ndarray         # (B, 4, 4)


def strand_scene(num_strands: int, num_verts: int, per_cluster: int, num_views: int = 1,
                 seed: int = 0, margin: float = 0.3) -> StrandScene:
    strands = make_strands(num_strands, num_verts, seed=seed)
    mvp = ortho_cameras(strands, margin=margin, num_views=num_views)
    pos = project(strands, mvp)
    edges = strand_edges(num_strands, num_verts)
    e2c = (np.arange(edges.shape[0]) // (num_verts - 1) // per_cluster).astype(np.int32)
    K = (num_strands + per_cluster - 1) // per_cluster
    return StrandScene(strands, pos, edges, e2c, K, mvp)


# Named workloads (sizes of the published configurations)
CONFIG_SMALL = dict(num_strands=1024, num_verts=32, per_cluster=16, H=256, W=256)
CONFIG_FULL = dict(num_strands=50_000, num_verts=100, per_cluster=25, H=1024, W=1024)


def tube_mesh(strands: np.ndarray, radius: float, n_circle: int = 8):
    """Open tube around every strand (n_circle vertices per point), the topology of the
    reference's ``strands_to_tube`` (curve_utils.py:310-374) with a simple frame: verts
    (N*S*n, 3), faces (M, 3) int32, per-vertex unit tangents (N*S*n, 3)."""
    N, S, _ = strands.shape
    st = strands.astype(np.float64)
    tan = np.zeros_like(st)
    d = np.diff(st, axis=1)
    tan[:, :-1] += d
    tan[:, 1:] += d
    tan /= np.maximum(np.linalg.norm(tan, axis=2, keepdims=True), 1e-12)
    ref = np.where(np.abs(tan[..., 2:3]) < 0.9, np.array([0.0, 0.0, 1.0]), np.array([1.0, 0.0, 0.0]))
    nrm = np.cross(tan, ref)
    nrm /= np.maximum(np.linalg.norm(nrm, axis=2, keepdims=True), 1e-12)
    bin_ = np.cross(tan, nrm)
    th = np.linspace(0, 2 * np.pi, n_circle, endpoint=False)
    dirs = np.cos(th)[None, None, :, None] * nrm[:, :, None, :] + np.sin(th)[None, None, :, None] * bin_[:, :, None, :]
    verts = (st[:, :, None, :] + radius * dirs).reshape(N * S * n_circle, 3)
    idx = np.arange(S * n_circle).reshape(S, n_circle)
    a, b = idx[:-1], np.roll(idx[:-1], -1, axis=1)
    c, e = idx[1:], np.roll(idx[1:], -1, axis=1)
    faces = np.stack([np.stack([a, c, e], -1), np.stack([a, e, b], -1)], 0).reshape(-1, 3)
    faces = (faces[None] + (np.arange(N) * S * n_circle)[:, None, None]).reshape(-1, 3).astype(np.int32)
    attr = np.repeat(tan[:, :, None, :], n_circle, axis=2).reshape(-1, 3)
    return verts.astype(np.float32), faces, attr.astype(np.float32)


def wisp_patch(num_strands: int, num_verts: int, n_circle: int = 8, seed: int = 0):
    """A wisp of neighbouring strands as a tube mesh in NDC ([-0.9, 0.9] on x and y, z scaled
    by 0.2 as the reference does to avoid depth clipping)."""
    st = make_strands(num_strands, num_verts, seed=seed)
    lo, hi = st.reshape(-1, 3).min(0), st.reshape(-1, 3).max(0)
    scale = 1.8 / np.maximum(hi - lo, 1e-6)
    ndc = (st - (lo + hi) / 2) * scale
    ndc[..., 2] *= 0.2
    return tube_mesh(ndc.astype(np.float32), radius=0.004, n_circle=n_circle)


def make_wisps(num_strands: int, num_verts: int, num_wisps: int, seed: int = 0):
    """Strands grouped into wisps: the generator's strands (Morton order, so neighbours share
    a wisp) with lengths scaled per strand by a factor in [0.6, 1.0] about the root, cut into
    ``num_wisps`` contiguous groups of random positive sizes.  Returns (strands (N, V, 3)
    float32, sizes (num_wisps,) int64)."""
    rng = np.random.default_rng(seed + 101)
    st = make_strands(num_strands, num_verts, seed=seed).astype(np.float64)
    f = rng.uniform(0.6, 1.0, size=(num_strands, 1, 1))
    st = st[:, :1] + f * (st - st[:, :1])
    K = max(1, min(num_wisps, num_strands))
    cuts = np.sort(rng.choice(np.arange(1, num_strands), size=K - 1, replace=False)) if K > 1 else np.array([], int)
    sizes = np.diff(np.concatenate([[0], cuts, [num_strands]])).astype(np.int64)
    return _quantise(st), sizes
