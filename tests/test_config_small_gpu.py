"""The small published configuration end to end on the GPU against the oracle: 1,024
strands x 32 vertices (the generator), one orthographic 256x256 view, 64 clusters
(cluster = strand_idx // 16), and 64 cards (one per cluster, 8 x 2 quads).

- DDA raster of all 31,744 segments into the cluster bitset: bit-exact;
- card raster (rast = b0, b1, z, triangle id + 1) and the cards' cluster bitset: triangle
  ids, coverage and bits exact, b0 / b1 / z equal to the oracle's FP32 mirror;
- attribute interpolation forward and backward with an N(0, 1) upstream image gradient
  (seed 0): elementwise against FP64, |got - FP64| <= 1e-5 x max(|FP64|, sum|terms|);
- antialias forward (XOR-popcount loss) exact and backward d_pos within 1e-5 elementwise
  (floor 1e-3 of the max-norm) of the FP64 oracle, the same non-zero pattern.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from parity import assert_rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def np_(t):
    return t.detach().cpu().numpy()


@pytest.fixture(scope="module")
def scene():
    from strns2cards_gb300 import synthetic as syn
    c = syn.CONFIG_SMALL
    sc = syn.strand_scene(c["num_strands"], c["num_verts"], per_cluster=c["per_cluster"], num_views=1, seed=0)
    cards = syn.make_cards(sc.strands, c["per_cluster"], 8, 2)
    cpos = syn.project(cards.verts, sc.mvp).astype(np.float32)
    return sc, cards, cpos, c["H"], c["W"]


def test_small_config_shapes(scene):
    sc, cards, cpos, H, W = scene
    assert sc.edges.shape[0] == 31_744 and sc.num_clusters == 64
    assert cards.tri.shape[0] == 64 * 32 and cpos.shape[1] == 64 * 27


def test_small_config_dda_bitset(scene):
    import strns2cards_gb300 as s2c
    sc, _, _, H, W = scene
    ref = O.dda_cluster_bitset(H, W, sc.pos, sc.edges, sc.edge2cluster, sc.num_clusters)
    got = np_(s2c.dda_cluster_bitset((H, W), cu(sc.pos), cu(sc.edges), cu(sc.edge2cluster), sc.num_clusters))
    assert np.array_equal(got, ref)
    # and through the reference's op sequence (fragment list, then the mask)
    fp, fa = s2c.dda_compute_fragments((H, W), cu(sc.pos), cu(sc.edges))
    got2 = np_(s2c.cluster_mask_from_fragments((H, W), fp, fa, cu(sc.edge2cluster), sc.num_clusters))
    assert np.array_equal(got2, ref)


def test_small_config_card_raster_and_interpolation(scene):
    import strns2cards_gb300 as s2c
    _, cards, cpos, H, W = scene
    tri = cards.tri.astype(np.int32)
    rast = np_(s2c.rasterize((H, W), cu(cpos), cu(tri)))
    ref = O.rasterize(H, W, cpos, tri)
    assert np.array_equal(rast[..., 3], ref[..., 3])
    assert np.array_equal(rast[..., :3], ref[..., :3])
    attr = np.random.default_rng(0).normal(size=(cpos.shape[1], 3)).astype(np.float32)
    img = np_(s2c.interpolate_triangle_attributes(cu(rast), cu(attr), cu(tri)))
    assert_rel(img, O.interpolate(rast, attr, tri), O.interpolate_mag(rast, attr, tri), 1e-5, "image")
    grad = torch.randn((1, H, W, 3), generator=torch.Generator().manual_seed(0)).numpy()
    a = cu(attr).requires_grad_(True)
    out = s2c.interpolate_triangle_attributes(cu(rast), a, cu(tri))
    out.backward(cu(grad))
    V = cpos.shape[1]
    assert_rel(np_(a.grad), O.interpolate_backward(rast, grad, tri, V), O.interpolate_backward_mag(rast, grad, tri, V),
               1e-5, "d_attr")


def test_small_config_antialias(scene):
    import strns2cards_gb300 as s2c
    sc, cards, cpos, H, W = scene
    tri = cards.tri.astype(np.int32)
    t2c = cards.tri2cluster.astype(np.int32)
    target = s2c.dda_cluster_bitset((H, W), cu(sc.pos), cu(sc.edges), cu(sc.edge2cluster), sc.num_clusters)
    fp, fa = s2c.compute_fragments((H, W), cu(cpos), cu(tri))
    bits = s2c.cluster_mask_from_fragments((H, W), fp, fa, cu(t2c), sc.num_clusters)
    edges, e2t = s2c.build_edges_from_triangles(tri)
    e2c = t2c[e2t[:, 0]].astype(np.int32)
    pos = cu(cpos).requires_grad_(True)
    loss = s2c.antialiased_cluster_bitset_loss(bits, target, pos, cu(tri), cu(edges), cu(e2t), cu(e2c),
                                               kernel_radius=7.0, rho=0.5, count_xor_error=True)
    xor = int(np.unpackbits((np_(bits) ^ np_(target)).view(np.uint8)).sum())
    assert int(loss.detach()) == xor
    loss.backward()
    got = np_(pos.grad).astype(np.float64)
    ora = O.antialias_grad(np_(bits), np_(target), cpos, tri, edges, e2t, e2c, 7.0, 0.5)
    floor = 1e-3 * np.abs(ora).max()
    assert np.all(np.abs(got - ora) <= 1e-5 * np.maximum(np.abs(ora), floor))
    assert np.array_equal(got != 0, ora != 0)
