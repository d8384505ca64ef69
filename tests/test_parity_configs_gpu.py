"""Elementwise float parity at the published workload shapes.

Every float output of the triangle / line / curve / deformation operators, computed on the
GPU at the sizes of the published configurations, against an FP64 evaluation of the same
formula, element by element (``parity.py``):

    |got - FP64| <= 1e-5 x max(|FP64|, sum|terms|)

Per output, the scale ``sum|terms|`` is:

* rast barycentric derivatives (du/dx, du/dy, dv/dx, dv/dy): the formula's first-order
  condition scale (``oracle.barycentric_derivatives(with_mag=True)``);
* interpolated image, triangles and lines: sum_i |b_i a_i|;
* d_attr, triangles and lines: sum over pixels |b_i g| (the products are summed in FP64
  and rounded once; the reference's float atomics round at every addition);
* smoothed strands: sum_j w_j |x_j| / sum_j w_j;  skinned strands: sum_j w_j (|R_j|
  (|x_i| + |h_j|) + |c_j|) / sum_j w_j;
* card Laplacian (10 Jacobi steps, lambda = 0.5): the same iteration on |p|;
* LBS y, dM, dx: the same sums on |x|, |M|, |gy|.

Where no term cancels the scale equals |FP64| and the bound is the plain 1e-5 relative one.
Shapes: config 1 = 1,024 x 32 strands, 256x256, 64 cards (8 x 2 quads); config 2 =
50,000 x 100 strands, 1024x1024, 2,048 cards (16 x 4 quads); config 3 = 256 cards of 32 x 4
quads (Laplacian); config 4 = 100,000 x 64 strands, 2048x2048, 4,096 cards (16 x 4 quads),
LBS of all 6.4 M strand vertices to the cards' 69,632 centre-line guides.  Attributes and
upstream gradients are N(0, 1) with seed 0.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from parity import assert_rel

pytestmark = pytest.mark.gpu
TOL = 1e-5

CONFIGS = {
    "config1": dict(strands=(1024, 32), res=256, per_cluster=16, cards=0, quads=(8, 2)),
    "config2": dict(strands=(50_000, 100), res=1024, per_cluster=25, cards=2048, quads=(16, 4)),
    "config4": dict(strands=(100_000, 64), res=2048, per_cluster=25, cards=4096, quads=(16, 4)),
}
_scenes = {}


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    yield lib_built
    _scenes.clear()


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def np_(t):
    return t.detach().cpu().numpy()


def scene(name):
    if name not in _scenes:
        from strns2cards_gb300 import synthetic as syn
        c = CONFIGS[name]
        N, V = c["strands"]
        strands = syn.make_strands(N, V, seed=0)
        mvp = syn.ortho_cameras(strands, margin=0.3, num_views=1)
        cards = syn.make_cards(strands, c["per_cluster"], *c["quads"], num_cards=c["cards"])
        _scenes[name] = dict(strands=strands.astype(np.float32), mvp=mvp, cards=cards, H=c["res"],
                             spos=syn.project(strands.reshape(-1, 3), mvp).astype(np.float32),
                             sedges=syn.strand_edges(N, V),
                             cpos=syn.project(cards.verts, mvp).astype(np.float32))
    return _scenes[name]


def n01(shape, seed=0):
    return torch.randn(shape, generator=torch.Generator().manual_seed(seed)).numpy()


@pytest.mark.parametrize("cfg", ["config1", "config2", "config4"])
def test_triangle_interpolation_and_derivatives(cfg):
    import strns2cards_gb300 as s2c
    sc = scene(cfg)
    H, cpos, tri = sc["H"], sc["cpos"], sc["cards"].tri
    V = cpos.shape[1]
    rast_t, db = s2c.rasterize_with_derivatives((H, H), cu(cpos), cu(tri))
    rast = np_(rast_t)
    assert (rast[..., 3] > 0).sum() > 0.02 * H * H
    ref, mag = O.barycentric_derivatives(rast, cpos, tri, with_mag=True)
    assert_rel(np_(db), ref, mag, TOL, f"{cfg} barycentric derivatives")
    attr = np.random.default_rng(0).normal(size=(V, 3)).astype(np.float32)
    grad = n01((1, H, H, 3))
    a = cu(attr).requires_grad_(True)
    img = s2c.interpolate_triangle_attributes(rast_t, a, cu(tri))
    assert_rel(np_(img), O.interpolate(rast, attr, tri), O.interpolate_mag(rast, attr, tri), TOL, f"{cfg} image")
    img.backward(cu(grad))
    assert_rel(np_(a.grad), O.interpolate_backward(rast, grad, tri, V), O.interpolate_backward_mag(rast, grad, tri, V),
               TOL, f"{cfg} d_attr")


@pytest.mark.parametrize("cfg", ["config1", "config2", "config4"])
def test_line_interpolation(cfg):
    import strns2cards_gb300 as s2c
    sc = scene(cfg)
    H, pos, edges = sc["H"], sc["spos"], sc["sedges"]
    V = pos.shape[1]
    fp, fa = s2c.dda_compute_fragments((H, H), cu(pos), cu(edges))
    rast_t = s2c.depth_test(1, (H, H), fp, fa)
    del fp, fa
    rast = np_(rast_t)
    assert (rast[..., 3] > 0).sum() > 0.01 * H * H
    attr = np.random.default_rng(0).normal(size=(V, 3)).astype(np.float32)
    grad = n01((1, H, H, 3))
    a = cu(attr).requires_grad_(True)
    img = s2c.dda_interpolate_attributes(rast_t, a, cu(edges))
    assert_rel(np_(img), O.dda_interpolate(rast, attr, edges), O.dda_interpolate_mag(rast, attr, edges), TOL,
               f"{cfg} line image")
    img.backward(cu(grad))
    assert_rel(np_(a.grad), O.dda_interpolate_backward(rast, grad, edges, V),
               O.dda_interpolate_backward_mag(rast, grad, edges, V), TOL, f"{cfg} line d_attr")


@pytest.mark.parametrize("cfg", ["config1", "config2", "config4"])
def test_smoothing_and_skinning(cfg):
    import strns2cards_gb300 as s2c
    st = scene(cfg)["strands"]
    beta = 0.05
    rng = np.random.default_rng(0)
    hs = (st + rng.normal(scale=0.01, size=st.shape)).astype(np.float32)
    ch = (st + rng.normal(scale=0.02, size=st.shape)).astype(np.float32)
    Q, _ = np.linalg.qr(rng.normal(size=st.shape[:2] + (3, 3)))
    R = Q.astype(np.float32)
    x = cu(st)
    arc = np_(s2c.compute_arclength(x))
    sm = s2c.smooth_strands(x, beta)
    assert_rel(np_(sm), O.smooth_strands(st, arc, beta), O.smooth_strands_mag(st, arc, beta), TOL, f"{cfg} smoothed")
    sk = s2c.skinning(x, cu(hs), cu(ch), cu(R), beta)
    assert_rel(np_(sk), O.skinning(st, arc, hs, ch, R, beta), O.skinning_mag(st, arc, hs, ch, R, beta), TOL,
               f"{cfg} skinned")


@pytest.mark.parametrize("cards,qa,qx", [(256, 32, 4), (2048, 16, 4), (4096, 16, 4)])
def test_card_laplacian_on_card_meshes(cards, qa, qx):
    """The cards of config 3 (256 x 32 x 4 quads), config 2 and config 4 (16 x 4 quads),
    smoothed 10 steps with lambda = 0.5 from their generated positions."""
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    strands = scene("config4")["strands"] if cards == 4096 else syn.make_strands(max(cards * 25, 6400), 64, seed=0)
    cm = syn.make_cards(strands, 0, qa, qx, num_cards=cards)
    _, _, h, w = syn.grid_strip(qx + 1, qa + 1)          # one card's quad edges, as make_cards lays them out
    qe = np.concatenate([h, w], 0)
    nv = (qx + 1) * (qa + 1)
    p = cm.verts.astype(np.float32)
    got = np_(s2c.card_laplacian_smooth(cu(p), qe, nv, 0.5, 10))
    assert_rel(got, O.card_laplacian_smooth(p, qe, nv, 0.5, 10), O.card_laplacian_smooth_mag(p, qe, nv, 0.5, 10), TOL,
               f"Laplacian {cards} cards")


def test_lbs_config4():
    import strns2cards_gb300 as s2c
    sc = scene("config4")
    x = sc["strands"].reshape(-1, 3)
    g = np.ascontiguousarray(sc["cards"].verts.reshape(-1, 5, 17, 3)[:, 2].reshape(-1, 3), dtype=np.float32)
    G = g.shape[0]
    assert x.shape[0] == 6_400_000 and G == 69_632
    b = s2c.LBSBinding(cu(x), cu(g), tau=0.01)
    idx, w = np_(b.idx), np_(b.w)
    # binding: a random sample of vertices against the brute-force exact-FP32 selection
    pick = np.random.default_rng(1).choice(x.shape[0], 4096, replace=False)
    oidx, ow = O.lbs_bind(x[pick], g, 0.01)
    assert np.array_equal(idx[pick], oidx)
    assert np.abs(w[pick] - ow).max() <= 1e-6
    rng = np.random.default_rng(0)
    M = (np.tile(np.eye(3, 4), (G, 1, 1)) + rng.normal(scale=0.05, size=(G, 3, 4))).astype(np.float32)
    gy = n01((x.shape[0], 3))
    Mt = cu(M).requires_grad_(True)
    xt = cu(x).requires_grad_(True)
    y = s2c.lbs(xt, Mt, b)
    assert_rel(np_(y), O.lbs_forward(x, idx, w, M), O.lbs_forward_mag(x, idx, w, M), TOL, "LBS y")
    y.backward(cu(gy))
    dM, dx = O.lbs_backward(x, idx, w, M, gy)
    mM, mx = O.lbs_backward_mag(x, idx, w, M, gy)
    assert_rel(np_(Mt.grad), dM, mM, TOL, "LBS dM")
    assert_rel(np_(xt.grad), dx, mx, TOL, "LBS dx")
