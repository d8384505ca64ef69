"""Cluster planes cleared and counted inside rectangles.

* ``rasterize_fused_planes_onto`` ORs the card raster onto kept planes and reports, per
  (view, plane), a word rectangle holding every bit it can set: over iterations with moving
  cards, clearing the previous rectangles and rastering onto the planes gives exactly the
  planes of the clearing raster (``rasterize_fused_planes``), and no set bit lies outside its
  rectangle.
* ``planes_bounds`` is the tightest rectangle of each plane's non-zero words (numpy).
* ``planes_clear_rects`` zeroes exactly the rectangles.
* ``cluster_iou_counts_planes_rects`` equals the whole-plane per-cluster counts and the
  whole-plane XOR popcount whenever the rectangles hold every set bit."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def cards(seed, B=2, H=96, W=200, K=70):
    from strns2cards_gb300 import synthetic as syn
    rng = np.random.default_rng(seed)
    strands = syn.make_strands(400, 16, seed=seed)
    mvp = syn.ortho_cameras(strands, margin=0.3, num_views=B)
    c = syn.make_cards(strands, 0, 8, 2, num_cards=K)
    pos = syn.project(c.verts, mvp).astype(np.float32)
    return pos, c.tri, c.tri2cluster.astype(np.int32), rng


def np_bounds(planes):
    B, Kp, H, WQ = planes.shape
    out = np.zeros((B, Kp, 4), np.int32)
    for b in range(B):
        for c in range(Kp):
            ys, qs = np.nonzero(planes[b, c])
            out[b, c] = (ys.min(), ys.max() + 1, qs.min(), qs.max() + 1) if ys.size else (H, 0, WQ, 0)
    return out


def inside(planes, rects):
    B, Kp, H, WQ = planes.shape
    mask = np.zeros(planes.shape, bool)
    for b in range(B):
        for c in range(Kp):
            y0, y1, q0, q1 = (int(v) for v in rects[b, c])
            y0, y1, q0, q1 = max(y0, 0), min(y1, H), max(q0, 0), min(q1, WQ)
            if y0 < y1 and q0 < q1:
                mask[b, c, y0:y1, q0:q1] = True
    return mask


def test_raster_onto_planes_over_iterations_equals_clearing_raster():
    from strns2cards_gb300 import _core
    pos, tri, t2c, rng = cards(1)
    B, H, W, K = pos.shape[0], 96, 200, 70
    S = (K + 31) // 32
    shape = (B, H, W, S)
    planes = torch.zeros((B, 32 * S, H, (W + 31) // 32), dtype=torch.int32, device="cuda")
    rects = torch.tensor([H, 0, (W + 31) // 32, 0], dtype=torch.int32, device="cuda").repeat(B, 32 * S, 1)
    p = pos.copy()
    t, t2 = torch.from_numpy(tri).cuda(), torch.from_numpy(t2c).cuda()
    for it in range(4):
        pc = torch.from_numpy(p).cuda()
        _core.planes_clear_rects(planes, rects, shape)
        _core.rasterize_fused_planes_onto(pc, t, t2, K, H, W, planes, rects=rects)
        full = _core.rasterize_fused_planes(pc, t, t2, K, H, W)
        torch.cuda.synchronize()
        assert torch.equal(planes, full), it
        pl, r = planes.cpu().numpy(), rects.cpu().numpy()
        assert not (pl[~inside(pl, r)] != 0).any()
        assert (r[..., 1] > r[..., 0]).sum() > 0
        p[..., :2] += rng.normal(scale=0.03, size=p[..., :2].shape).astype(np.float32)   # the cards move


@pytest.mark.parametrize("H,W", [(37, 150), (40, 128)])   # plane words not / a multiple of 4
def test_planes_bounds_and_clear_rects(H, W):
    from strns2cards_gb300 import _core
    rng = np.random.default_rng(3 + H)
    B, S = 2, 2
    WQ = (W + 31) // 32
    pl = np.zeros((B, 32 * S, H, WQ), np.uint32)
    for b in range(B):
        for c in range(0, 32 * S, 3):                      # a third of the planes hold a few words
            n = rng.integers(1, 6)
            pl[b, c, rng.integers(0, H, n), rng.integers(0, WQ, n)] = rng.integers(1, 2 ** 32, n, dtype=np.uint64)
    planes = torch.from_numpy(pl.view(np.int32)).cuda()
    got = _core.planes_bounds(planes, (B, H, W, S)).cpu().numpy()
    assert np.array_equal(got, np_bounds(pl))
    rects = np.zeros((B, 32 * S, 4), np.int32)
    rects[..., 0] = rng.integers(-3, H, rects.shape[:2])
    rects[..., 1] = rects[..., 0] + rng.integers(-2, 12, rects.shape[:2])
    rects[..., 2] = rng.integers(-1, WQ + 1, rects.shape[:2])
    rects[..., 3] = rects[..., 2] + rng.integers(-1, 4, rects.shape[:2])
    full = torch.from_numpy(rng.integers(-2 ** 31, 2 ** 31 - 1, pl.shape, dtype=np.int64).astype(np.int32)).cuda()
    before = full.cpu().numpy()
    _core.planes_clear_rects(full, torch.from_numpy(rects).cuda(), (B, H, W, S))
    after = full.cpu().numpy()
    m = inside(pl, rects)
    assert (after[m] == 0).all() and np.array_equal(after[~m], before[~m])


def test_iou_counts_in_rectangles_equal_whole_planes():
    from strns2cards_gb300 import _core
    rng = np.random.default_rng(5)
    B, H, W, S, K = 2, 40, 100, 2, 50
    WQ = (W + 31) // 32
    a = np.zeros((B, 32 * S, H, WQ), np.uint32)
    bb = np.zeros_like(a)
    for arr in (a, bb):
        for b in range(B):
            for c in range(32 * S):
                if rng.random() < 0.7:
                    y0, x0 = rng.integers(0, H - 8), rng.integers(0, WQ - 1)
                    blk = rng.integers(0, 2 ** 32, (rng.integers(1, 8), rng.integers(1, 2)), dtype=np.uint64)
                    arr[b, c, y0:y0 + blk.shape[0], x0:x0 + blk.shape[1]] = blk
    ta, tb = (torch.from_numpy(x.view(np.int32)).cuda() for x in (a, bb))
    shape = (B, H, W, S)
    ra, rb = _core.planes_bounds(ta, shape), _core.planes_bounds(tb, shape)
    inter, uni, xor = _core.cluster_iou_counts_planes_rects(ta, tb, ra, rb, shape, K)
    fi, fu = _core.cluster_iou_counts_planes(ta, tb, shape, K)
    assert torch.equal(inter, fi) and torch.equal(uni, fu)
    assert int(xor) == int(_core.xor_popcount(ta, tb))
    # looser (but still covering) rectangles count the same
    big = torch.tensor([0, H, 0, WQ], dtype=torch.int32, device="cuda").repeat(B, 32 * S, 1)
    i2, u2, x2 = _core.cluster_iou_counts_planes_rects(ta, tb, big, rb, shape, K)
    assert torch.equal(i2, fi) and torch.equal(u2, fu) and int(x2) == int(xor)
