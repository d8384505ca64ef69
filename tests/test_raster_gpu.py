"""GPU parity of the triangle path and attribute interpolation.

Coverage, barycentrics, depth and triangle ids are bit-identical to the reference's golden
vectors and to the oracle.  Float outputs are checked element by element (``parity.py``):

* interpolated image (a6 / a7 forward): |got - FP64| <= 1e-5 x max(|FP64|, sum_i |b_i a_i|);
* d_attr (a6 / a7 backward; FP64 sums of the exact FP32 products, rounded once): the
  same with sum over pixels |b_i g| as the scale;
* barycentric derivatives: 1e-5 x max(|FP64|, the formula's first-order condition scale);
* against the reference's own golden outputs (also FP32, with its own rounding): 2e-5,
  the sum of both sides' bounds.
"""
import hashlib
import json
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN, golden
from oracle import oracle as O
from parity import assert_rel

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def np_(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("name", ["tri_cards", "tri_random"])
def test_compute_fragments_and_rasterize_match_golden(name):
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import _core
    d = golden(name + ".npz")
    H, W = int(d["H"]), int(d["W"])
    pos, tri = cu(d["pos"]), cu(d["tri"])
    B, T = d["pos"].shape[0], d["tri"].shape[0]
    rects = torch.empty((B * T, 4), dtype=torch.int32, device="cuda")
    prefix = torch.empty(B * T, dtype=torch.int32, device="cuda")
    F = _core.compute_triangle_rects(H, W, pos, tri, rects, prefix)
    assert np.array_equal(np_(rects), d["rects"])
    assert F == int(d["rect_counts"].sum())
    fp, fa = s2c.compute_fragments((H, W), pos, tri)
    op, oa = O.compute_fragments(H, W, d["pos"], d["tri"])
    assert np.array_equal(np_(fp), op) and np.array_equal(np_(fa), oa)
    sp, sa = O.sort_frags(np_(fp), np_(fa))
    assert np.array_equal(sp, d["frag_pix"]) and np.array_equal(sa, d["frag_attrs"])
    rast = s2c.rasterize((H, W), pos, tri)
    assert np.array_equal(np_(rast), d["rast"])
    if "bitset" in d:
        m = s2c.cluster_mask_from_fragments((H, W), fp, fa, cu(d["tri2cluster"]), int(d["K"]))
        assert np.array_equal(np_(m), d["bitset"])


def test_rasterize_random_perspective_matches_oracle():
    import strns2cards_gb300 as s2c
    rng = np.random.default_rng(21)
    V, T, B = 400, 300, 3
    pos = rng.uniform(-1.2, 1.2, size=(B, V, 4)).astype(np.float32)
    pos[..., 3] = rng.uniform(0.5, 1.5, size=(B, V))
    pos[..., 2] *= pos[..., 3] * 0.7
    tri = rng.integers(0, V, size=(T, 3)).astype(np.int32)
    H, W = 90, 110
    got = np_(s2c.rasterize((H, W), cu(pos), cu(tri)))
    assert np.array_equal(got, O.rasterize(H, W, pos, tri))


def test_fullsize_card_raster_matches_reference():
    """2,000 cards (256,000 triangles) over 1024x1024: fragment count and cluster bitset equal
    the reference's (sha256); triangle ids equal the oracle's (exact depth ties resolve to the
    first fragment here, while the reference's choice depends on scheduling)."""
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    ref = json.load(open(os.path.join(GOLDEN, "fullsize_ref.json")))["tri_full"]
    sc = syn.strand_scene(50_000, 100, per_cluster=25, num_views=1, seed=0)
    cards = syn.make_cards(sc.strands, 25, 16, 4)
    cpos = syn.project(cards.verts, sc.mvp)
    fp, fa = s2c.compute_fragments((1024, 1024), cu(cpos), cu(cards.tri))
    assert fp.shape[0] == ref["num_frags"]
    bits = s2c.cluster_mask_from_fragments((1024, 1024), fp, fa, cu(cards.tri2cluster), 2048)
    assert hashlib.sha256(np_(bits).tobytes()).hexdigest() == ref["bitset_sha256"]
    rast = np_(s2c.depth_test(1, (1024, 1024), fp, fa))
    ofp, ofa = O.compute_fragments(1024, 1024, cpos, cards.tri)
    orast = O.depth_test(1, 1024, 1024, ofp, ofa)
    assert np.array_equal(rast, orast)
    assert int((rast[..., 3] > 0).sum()) == ref["covered"]
    # the fused single pass gives the same rast and bitset
    frast, fbits = s2c.rasterize_fused((1024, 1024), cu(cpos), cu(cards.tri), cu(cards.tri2cluster), 2048)
    assert hashlib.sha256(np_(fbits).tobytes()).hexdigest() == ref["bitset_sha256"]
    assert np.array_equal(np_(frast), rast)


def test_triangle_interpolation_forward_backward():
    import strns2cards_gb300 as s2c
    d = golden("interp.npz")
    rast, attr, tri, grad = cu(d["rast"]), cu(d["attr"]).requires_grad_(True), cu(d["tri"]), cu(d["grad"])
    img = s2c.interpolate_triangle_attributes(rast, attr, tri)
    mag = O.interpolate_mag(d["rast"], d["attr"], d["tri"])
    assert_rel(np_(img), O.interpolate(d["rast"], d["attr"], d["tri"]), mag, TOL, "image")
    assert_rel(np_(img), d["image"], mag, 2 * TOL, "image vs the reference")
    img.backward(grad)
    V = d["attr"].shape[0]
    ref = O.interpolate_backward(d["rast"], d["grad"], d["tri"], V)
    gmag = O.interpolate_backward_mag(d["rast"], d["grad"], d["tri"], V)
    assert_rel(np_(attr.grad), ref, gmag, TOL, "d_attr")
    assert_rel(np_(attr.grad), d["d_attr"], gmag, 2 * TOL, "d_attr vs the reference")
    # without an FP64 accumulator the entry adds with float atomics, as the reference
    from strns2cards_gb300 import _lib
    B, H, W, _ = d["rast"].shape
    C = d["attr"].shape[1]
    d32 = torch.zeros((V, C), dtype=torch.float32, device="cuda")
    _lib.call("s2c_backward_interpolate_triangle_attributes", B, H, W, C, rast.data_ptr(), grad.data_ptr(),
              d["tri"].shape[0], tri.data_ptr(), V, d32.data_ptr(), None, torch.cuda.current_stream().cuda_stream)
    assert_rel(np_(d32), ref, gmag, TOL, "d_attr (float atomics)")


def test_dda_interpolation_forward_backward():
    import strns2cards_gb300 as s2c
    d = golden("interp.npz")
    rast, attr, edges, grad = cu(d["rast_dda"]), cu(d["attr_dda"]).requires_grad_(True), cu(d["edges"]), cu(d["grad_dda"])
    img = s2c.dda_interpolate_attributes(rast, attr, edges)
    mag = O.dda_interpolate_mag(d["rast_dda"], d["attr_dda"], d["edges"])
    assert_rel(np_(img), O.dda_interpolate(d["rast_dda"], d["attr_dda"], d["edges"]), mag, TOL, "line image")
    assert_rel(np_(img), d["image_dda"], mag, 2 * TOL, "line image vs the reference")
    img.backward(grad)
    V = d["attr_dda"].shape[0]
    ref = O.dda_interpolate_backward(d["rast_dda"], d["grad_dda"], d["edges"], V)
    gmag = O.dda_interpolate_backward_mag(d["rast_dda"], d["grad_dda"], d["edges"], V)
    assert_rel(np_(attr.grad), ref, gmag, TOL, "line d_attr")
    assert_rel(np_(attr.grad), d["d_attr_dda"], gmag, 2 * TOL, "line d_attr vs the reference")


def tie_pixels(fp, fa, B, H, W):
    """Pixels whose nearest depth is shared by two or more fragments."""
    pix = (fp[:, 0].astype(np.int64) * H + fp[:, 1]) * W + fp[:, 2]
    zb = (fa[:, 2] + np.float32(2)).astype(np.float32).view(np.int32)
    order = np.lexsort((zb, pix))
    ps, zs = pix[order], zb[order]
    first = np.ones(len(ps), bool)
    first[1:] = ps[1:] != ps[:-1]
    st = np.nonzero(first)[0]
    nx = st + 1
    ok = nx < len(ps)
    tie = np.zeros(len(st), bool)
    tie[ok] = (ps[nx[ok]] == ps[st[ok]]) & (zs[nx[ok]] == zs[st[ok]])
    mask = np.zeros(B * H * W, bool)
    mask[ps[st[tie]]] = True
    return mask.reshape(B, H, W)


def test_depth_test_of_line_fragments():
    """texture_utils.py renders lines with dda_compute_fragments + depth_test.  Exact against
    the oracle; against the reference everywhere except exact depth ties (joint pixels of
    consecutive segments), where the reference's pick depends on scheduling."""
    import strns2cards_gb300 as s2c
    d = golden("dda_strands.npz")
    B, H, W = d["pos"].shape[0], int(d["H"]), int(d["W"])
    fp, fa = s2c.dda_compute_fragments((H, W), cu(d["pos"]), cu(d["edges"]))
    rast = np_(s2c.depth_test(B, (H, W), fp, fa))
    ofp, ofa = O.dda_compute_fragments(H, W, d["pos"], d["edges"])
    assert np.array_equal(rast, O.depth_test(B, H, W, ofp, ofa))
    ref = golden("interp.npz")["rast_dda"]
    ties = tie_pixels(ofp, ofa, B, H, W)
    assert np.array_equal(rast[~ties], ref[~ties])
    assert np.array_equal(rast[ties][:, 2], ref[ties][:, 2])  # same depth at the ties


@pytest.mark.parametrize("name", ["tri_cards", "tri_random"])
def test_barycentric_derivatives(name):
    """db/dxy against the FP64 oracle (elementwise, with the formula's condition scale), and
    against a difference of the reference's own barycentrics across neighbouring pixels of
    the same triangle."""
    import strns2cards_gb300 as s2c
    d = golden(name + ".npz")
    H, W = int(d["H"]), int(d["W"])
    rast, db = s2c.rasterize_with_derivatives((H, W), cu(d["pos"]), cu(d["tri"]))
    got = np_(db)
    ref, mag = O.barycentric_derivatives(np_(rast), d["pos"], d["tri"], with_mag=True)
    assert_rel(got, ref, mag, TOL, "barycentric derivatives")
    assert np.array_equal(np.any(got != 0, -1), np.any(ref != 0, -1) | np.any(got != 0, -1))
    # b is affine in NDC for orthographic views (w = 1): the golden barycentrics one pixel
    # apart differ by exactly db/dx
    r = d["rast"]
    if np.allclose(d["pos"][..., 3], 1.0):
        same = (r[:, :, 1:, 3] == r[:, :, :-1, 3]) & (r[:, :, 1:, 3] > 0)
        fd = (r[:, :, 1:, 0] - r[:, :, :-1, 0]).astype(np.float64)
        an = ref[:, :, :-1, 0]
        assert np.abs(fd[same] - an[same]).max() <= 1e-3 * max(np.abs(an[same]).max(), 1e-6)


def test_barycentric_derivatives_perspective():
    import strns2cards_gb300 as s2c
    rng = np.random.default_rng(22)
    V, T, B = 300, 200, 2
    pos = rng.uniform(-1.2, 1.2, size=(B, V, 4)).astype(np.float32)
    pos[..., 3] = rng.uniform(0.5, 1.5, size=(B, V))
    pos[..., 2] *= pos[..., 3] * 0.7
    tri = rng.integers(0, V, size=(T, 3)).astype(np.int32)
    rast, db = s2c.rasterize_with_derivatives((70, 90), cu(pos), cu(tri))
    ref, mag = O.barycentric_derivatives(np_(rast), pos, tri, with_mag=True)
    assert_rel(np_(db), ref, mag, TOL, "barycentric derivatives (perspective)")


@pytest.mark.parametrize("name", ["tri_cards", "tri_random"])
def test_rasterize_fused_matches_list_path(name):
    import strns2cards_gb300 as s2c
    d = golden(name + ".npz")
    H, W = int(d["H"]), int(d["W"])
    pos, tri = cu(d["pos"]), cu(d["tri"])
    fp, fa = s2c.compute_fragments((H, W), pos, tri)
    rast = s2c.depth_test(d["pos"].shape[0], (H, W), fp, fa)
    t2c = cu(d["tri2cluster"]) if "tri2cluster" in d else torch.zeros(d["tri"].shape[0], dtype=torch.int32, device="cuda")
    K = int(d["K"]) if "K" in d else 1
    frast, fbits = s2c.rasterize_fused((H, W), pos, tri, t2c, K)
    assert torch.equal(frast, rast)
    B = d["pos"].shape[0]
    ref_bits = torch.zeros((B, H, W, (K + 31) // 32), dtype=torch.int32, device="cuda")
    from strns2cards_gb300 import _core
    if fp.shape[0]:
        _core.cluster_mask_from_fragments(fp, fa, t2c, ref_bits)
    assert torch.equal(fbits, ref_bits)
    # bitset only, rast only
    r2, b2 = s2c.rasterize_fused((H, W), pos, tri, t2c, K, want_rast=False)
    assert r2 is None and torch.equal(b2, ref_bits)


def test_rasterize_fused_ties_and_perspective():
    """Coincident triangles (exact depth ties: the lower triangle id wins, as the list path)
    and perspective views with triangles behind the camera."""
    import strns2cards_gb300 as s2c
    rng = np.random.default_rng(31)
    V, T, B = 200, 300, 3
    pos = rng.uniform(-1.2, 1.2, size=(B, V, 4)).astype(np.float32)
    pos[..., 3] = rng.uniform(-0.2, 1.5, size=(B, V))
    pos[..., 2] *= np.abs(pos[..., 3]) * 0.7
    tri = rng.integers(0, V, size=(T, 3)).astype(np.int32)
    tri[T // 2:] = tri[:T - T // 2]                    # duplicates: exact ties
    t2c = rng.integers(0, 40, size=T).astype(np.int32)
    H, W = 64, 96
    fr, fb = s2c.rasterize_fused((H, W), cu(pos), cu(tri), cu(t2c), 40)
    orast = O.rasterize(H, W, pos, tri)
    assert np.array_equal(np_(fr), orast)
    ofp, ofa = O.compute_fragments(H, W, pos, tri)
    assert np.array_equal(np_(fb), O.cluster_mask_from_fragments(H, W, ofp, ofa, t2c, 40, B=B))


def test_raster_into_planes_and_plane_iou():
    """The fused raster writing cluster planes gives the planes of the bitset it writes, and
    the per-cluster counts from planes equal those from the bitsets."""
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import _core
    d = golden("tri_cards.npz")
    H, W, K = int(d["H"]), int(d["W"]), int(d["K"])
    pos, tri, t2c = cu(d["pos"]), cu(d["tri"]), cu(d["tri2cluster"])
    rast, bits = s2c.rasterize_fused((H, W), pos, tri, t2c, K)
    rast2 = torch.empty_like(rast)
    planes = _core.rasterize_fused_planes(pos, tri, t2c, K, H, W, rast=rast2)
    assert torch.equal(planes, _core.bitset_to_planes(bits)) and torch.equal(rast2, rast)
    other = torch.roll(bits, 3, dims=2).contiguous()
    op = _core.bitset_to_planes(other)
    i1, u1 = _core.cluster_iou_counts(bits, other, K)
    i2, u2 = _core.cluster_iou_counts_planes(planes, op, tuple(bits.shape), K)
    assert torch.equal(i1, i2) and torch.equal(u1, u2)
    assert int(_core.xor_popcount(planes, op)) == int(_core.xor_popcount(bits, other))


def test_rasterize_fused_rows_on_hard_triangles():
    """The fused raster tests only the columns of each bounding-box row that the triangle's
    projection can reach (with a pixel of margin); triangles that are collinear, zero-area,
    sub-pixel, slivers, far larger than the view, in perspective or with a corner behind
    the camera must still give the list path's rast and bitset exactly."""
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import _core
    rng = np.random.default_rng(77)
    B, H, W = 2, 97, 131
    groups = []
    n = 120
    base = rng.uniform(-1.1, 1.1, size=(n, 3, 4))
    base[..., 3] = 1.0
    groups.append(base)                                                  # ordinary
    col = base.copy()
    t = rng.uniform(0, 1, size=(n, 1))
    col[:, 2, :2] = col[:, 0, :2] + t * (col[:, 1, :2] - col[:, 0, :2])   # collinear corners
    groups.append(col)
    tiny = base.copy()
    tiny[:, 1:, :2] = tiny[:, :1, :2] + rng.normal(scale=1e-3, size=(n, 2, 2))   # sub-pixel
    groups.append(tiny)
    sliver = base.copy()
    sliver[:, 2, :2] = 0.5 * (sliver[:, 0, :2] + sliver[:, 1, :2]) + rng.normal(scale=2e-4, size=(n, 2))
    groups.append(sliver)
    same = base.copy()
    same[:, 1] = same[:, 0]                                             # two equal corners
    groups.append(same)
    huge = base.copy()
    huge[..., :2] *= 50.0                                               # far beyond the view
    groups.append(huge)
    persp = base.copy()
    persp[..., 3] = rng.uniform(0.05, 2.0, size=(n, 3))
    persp[..., :2] *= persp[..., 3:4]
    groups.append(persp)
    behind = persp.copy()
    behind[::3, 1, 3] = -0.3                                            # a corner behind the camera
    groups.append(behind)
    tris = np.concatenate(groups, 0)                                    # (T, 3, 4)
    tris[..., 2] = rng.uniform(-0.9, 0.9, size=tris.shape[:2]) * np.abs(tris[..., 3])
    T = tris.shape[0]
    pos = np.stack([tris.reshape(-1, 4), (tris * [[[1.0, -1.0, 1.0, 1.0]]]).reshape(-1, 4)]).astype(np.float32)
    tri = np.arange(3 * T, dtype=np.int32).reshape(T, 3)
    t2c = (np.arange(T) % 70).astype(np.int32)
    fp, fa = s2c.compute_fragments((H, W), cu(pos), cu(tri))
    rast = s2c.depth_test(B, (H, W), fp, fa)
    ref_bits = torch.zeros((B, H, W, 3), dtype=torch.int32, device="cuda")
    _core.cluster_mask_from_fragments(fp, fa, cu(t2c), ref_bits)
    frast, fbits = s2c.rasterize_fused((H, W), cu(pos), cu(tri), cu(t2c), 70)
    assert torch.equal(fbits, ref_bits)
    assert torch.equal(frast, rast)
    assert int((rast[..., 3] > 0).sum()) > 1000


@pytest.mark.parametrize("seed", [3, 4])
def test_compacted_fragments_equal_the_filtered_raw_list(seed):
    """``compute_fragments`` writes the covered pixels straight into their own list (a coverage
    bit per bounding-box pixel, a scan, a write pass); it must equal the reference's way --
    the raw list of every bounding-box pixel (-1 where uncovered) compacted by
    ``filter_valid_fragments`` -- value for value and in order, including triangles with
    empty, off-screen, degenerate and huge boxes, several views and an empty input."""
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import _core
    rng = np.random.default_rng(seed)
    B, H, W, V, T = 3, 83, 150, 500, 700
    pos = rng.uniform(-1.3, 1.3, size=(B, V, 4)).astype(np.float32)
    pos[..., 3] = rng.uniform(0.4, 1.6, size=(B, V))
    pos[..., :2] *= pos[..., 3:4]
    pos[..., 2] = rng.uniform(-0.8, 0.8, size=(B, V)) * pos[..., 3]
    pos[:, :40, :2] *= 40.0                                    # far beyond the view
    tri = rng.integers(0, V, size=(T, 3)).astype(np.int32)
    tri[:50, 1] = tri[:50, 0]                                  # degenerate
    tri[50:60] = rng.integers(0, 40, size=(10, 3))             # huge boxes
    p, t = cu(pos), cu(tri)
    rects = torch.empty((B * T, 4), dtype=torch.int32, device="cuda")
    prefix = torch.empty(B * T, dtype=torch.int32, device="cuda")
    F = _core.compute_triangle_rects(H, W, p, t, rects, prefix)
    raw_p = torch.full((F, 3), -1, dtype=torch.int32, device="cuda")
    raw_a = torch.empty((F, 4), dtype=torch.float32, device="cuda")
    _core.compute_fragments(H, W, p, t, prefix, rects, raw_p, raw_a)
    out_p, out_a = torch.empty_like(raw_p), torch.empty_like(raw_a)
    n = _core.filter_valid_fragments(raw_p, raw_a, out_p, out_a)
    fp, fa = s2c.compute_fragments((H, W), p, t)
    assert fp.shape[0] == n > 1000
    assert torch.equal(fp, out_p[:n]) and torch.equal(fa, out_a[:n])
    ep, ea = s2c.compute_fragments((H, W), p, t[:0])
    assert ep.shape == (0, 3) and ea.shape == (0, 4)
