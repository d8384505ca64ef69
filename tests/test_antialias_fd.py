"""Central finite differences of the antialias backward (h = 1e-3, 64 random vertices,
seed 0), on the FP64 oracle whose formulas the GPU kernels match to 1e-5.

The backward is hand-written: per silhouette fragment f of edge (v0, v1) at parameter t it
adds dc_f times the derivative of the edge point's screen position along the edge normal
n_f.  With the window sums dc_f, the parameters t_f and the normals frozen, that is the
gradient of the surrogate L(pos) = sum_f dc_f (n_f . s_f(pos)), s_f the screen position of
t0 p0 + t1 p1.  Its x and y components must equal central differences of L; its w component
equals MINUS the central difference: antialias.cu:268 adds +(dx px + dy py) / pw^2 where the
derivative of the same expression is -(dx px + dy py) / pw^2 (the sign is reproduced for
parity; orthographic views, w = 1, never move w)."""
import numpy as np

from conftest import golden
from oracle import oracle as O


def _surrogate(pos, fp, fa, normals, dc, edges, H, W):
    b = fp[:, 0]
    e = fa[:, 3].astype(np.int64) - 1
    t1 = fa[:, 1].astype(np.float64)
    t0 = 1.0 - t1
    P = t0[:, None] * pos[b, edges[e, 0]] + t1[:, None] * pos[b, edges[e, 1]]
    sx = 0.5 * W * (1.0 + P[:, 0] / P[:, 3])
    sy = 0.5 * H * (1.0 - P[:, 1] / P[:, 3])
    n = normals.reshape(pos.shape[0], -1, 2)[b, e]
    return float(np.sum(dc * (n[:, 0] * sx + n[:, 1] * sy)))


def test_antialias_backward_matches_central_differences():
    a = golden("antialias.npz")
    H, W = int(a["H"]), int(a["W"])
    pos = a["pos"].astype(np.float32).copy()
    # a perspective-like view: scale each vertex by its own w
    w = (1.0 + 0.25 * np.sin(np.arange(pos.shape[1]) * 0.37)).astype(np.float32)
    pos[..., :3] *= w[None, :, None]
    pos[..., 3] = w[None, :]
    ids, normals = O.mark_discontinuity_edges(H, W, pos, a["tri"], a["edges"], a["edge2tri"])
    fp, fa = O.dda_compute_fragments(H, W, pos, a["edges"], ids)
    grad, dc = O.aa_backward(fp, fa, a["bitset"], a["target"], pos, a["edges"], normals, a["edge2cluster"],
                             7.0, 0.5, return_dc=True)
    assert np.count_nonzero(dc) > 10
    p64 = pos.astype(np.float64)
    edges = a["edges"].astype(np.int64)
    live = np.nonzero(np.abs(grad).sum(-1) > 0)
    rng = np.random.default_rng(0)
    pick = rng.choice(len(live[0]), size=min(64, len(live[0])), replace=False)
    h = 1e-3
    scale = np.abs(grad).max()
    for k in pick:
        bv, v = live[0][k], live[1][k]
        for comp in (0, 1, 3):
            pp, pm = p64.copy(), p64.copy()
            pp[bv, v, comp] += h
            pm[bv, v, comp] -= h
            fd = (_surrogate(pp, fp, fa, normals, dc, edges, H, W) - _surrogate(pm, fp, fa, normals, dc, edges, H, W)) / (2 * h)
            want = -fd if comp == 3 else fd
            assert abs(grad[bv, v, comp] - want) <= 1e-5 * scale, (bv, v, comp, grad[bv, v, comp], want)
