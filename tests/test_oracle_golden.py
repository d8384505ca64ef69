"""The CPU oracle against the golden vectors produced by the reference's own kernels.

These pin the oracle: every integer output and every FP32 span / t1 / z / barycentric /
normal value must be bit-identical to the reference; FP64-evaluated outputs (gradients,
interpolation, curves) must agree within the reference's own FP32 error, stated per test.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden
from oracle import oracle as O


def nan_equal(a, b):
    return np.array_equal(a, b) or bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


@pytest.mark.parametrize("name", ["dda_strands", "dda_edgecases", "dda_edge_ids"])
def test_dda_fragments_bit_exact(name):
    d = golden(name + ".npz")
    ids = d["edge_ids"] if "edge_ids" in d else None
    fp, fa, raw = O.dda_compute_fragments(int(d["H"]), int(d["W"]), d["pos"], d["edges"], ids, raw=True)
    m = raw["counts"] > 0
    assert np.array_equal(raw["counts"], d["span_counts"])
    assert nan_equal(raw["slopes"][m], d["span_slopes"][m])
    assert nan_equal(raw["spans"][m], d["span_spans"][m])
    # pre-compaction fragment arrays (-1 = rejected), element for element
    assert np.array_equal(raw["raw_pix"], d["raw_pix"])
    ok = d["raw_pix"][:, 0] >= 0
    assert np.array_equal(raw["raw_attrs"][ok], d["raw_attrs"][ok])
    fp, fa = O.sort_frags(fp, fa)
    assert np.array_equal(fp, d["frag_pix"]) and np.array_equal(fa, d["frag_attrs"])


@pytest.mark.parametrize("name", ["dda_strands", "dda_edgecases", "dda_edge_ids"])
def test_dda_bitsets_bit_exact(name):
    d = golden(name + ".npz")
    ids = d["edge_ids"] if "edge_ids" in d else None
    H, W, K = int(d["H"]), int(d["W"]), int(d["K"])
    ref = d["bitset"]
    fp, fa = O.dda_compute_fragments(H, W, d["pos"], d["edges"], ids)
    got = O.cluster_mask_from_fragments(H, W, fp, fa, d["edge2cluster"], K, B=ref.shape[0])
    assert np.array_equal(got, ref)
    fused = O.dda_cluster_bitset(H, W, d["pos"], d["edges"], d["edge2cluster"], K, ids)
    assert np.array_equal(fused[: ref.shape[0]], ref)
    assert not fused[ref.shape[0]:].any()


@pytest.mark.parametrize("name", ["tri_cards", "tri_random"])
def test_triangle_fragments_and_rast_bit_exact(name):
    d = golden(name + ".npz")
    H, W = int(d["H"]), int(d["W"])
    fp, fa, raw = O.compute_fragments(H, W, d["pos"], d["tri"], raw=True)
    assert np.array_equal(raw["rects"], d["rects"]) and np.array_equal(raw["counts"], d["rect_counts"])
    s_fp, s_fa = O.sort_frags(fp, fa)
    assert np.array_equal(s_fp, d["frag_pix"]) and np.array_equal(s_fa, d["frag_attrs"])
    rast = O.depth_test(d["pos"].shape[0], H, W, fp, fa)
    assert np.array_equal(rast, d["rast"])
    if "bitset" in d:
        got = O.cluster_mask_from_fragments(H, W, fp, fa, d["tri2cluster"], int(d["K"]), B=d["bitset"].shape[0])
        assert np.array_equal(got, d["bitset"])


def test_silhouette_edges_bit_exact():
    a = golden("antialias.npz")
    ids, normals, raw = O.mark_discontinuity_edges(int(a["H"]), int(a["W"]), a["pos"], a["tri"], a["edges"],
                                                   a["edge2tri"], raw=True)
    assert np.array_equal(raw, a["raw_prim_ids"])
    assert np.array_equal(normals, a["normals"])
    fp, fa = O.sort_frags(*O.dda_compute_fragments(int(a["H"]), int(a["W"]), a["pos"], a["edges"], ids))
    assert np.array_equal(fp, a["sil_frag_pix"]) and np.array_equal(fa, a["sil_frag_attrs"])


@pytest.mark.parametrize("tag,kr,rho", [("r7", 7.0, 0.5), ("r3", 3.5, 1.0)])
def test_antialias_gradient_matches_reference(tag, kr, rho):
    """The reference sums 225 __expf-weighted taps in FP32 with atomics; it agrees with
    the FP64 evaluation of the same formula to 1e-5 of max(|g|, 1e-3 max|g|)."""
    a = golden("antialias.npz")
    g = O.antialias_grad(a["bitset"], a["target"], a["pos"], a["tri"], a["edges"], a["edge2tri"],
                         a["edge2cluster"], kr, rho)
    ref = a["d_pos_" + tag].astype(np.float64)
    assert np.array_equal(g != 0, ref != 0)
    scale = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    assert (np.abs(g - ref) / scale).max() < 1e-5


def test_interpolation_matches_reference():
    d = golden("interp.npz")
    img = O.interpolate(d["rast"], d["attr"], d["tri"])
    assert np.abs(img - d["image"]).max() < 1e-5 * max(1.0, np.abs(d["image"]).max())
    da = O.interpolate_backward(d["rast"], d["grad"], d["tri"], d["attr"].shape[0])
    assert np.abs(da - d["d_attr"]).max() < 1e-5 * np.abs(d["d_attr"]).max()
    img = O.dda_interpolate(d["rast_dda"], d["attr_dda"], d["edges"])
    assert np.abs(img - d["image_dda"]).max() < 1e-5 * max(1.0, np.abs(d["image_dda"]).max())
    da = O.dda_interpolate_backward(d["rast_dda"], d["grad_dda"], d["edges"], d["attr_dda"].shape[0])
    assert np.abs(da - d["d_attr_dda"]).max() < 1e-5 * np.abs(d["d_attr_dda"]).max()


def test_curves_match_reference():
    d = golden("curves.npz")
    sm = O.smooth_strands(d["strands"], d["arclength"], float(d["beta"]))
    assert (np.abs(sm - d["smoothed"]) / np.maximum(np.abs(d["smoothed"]), 1e-3)).max() < 1e-5
    sk = O.skinning(d["strands"], d["arclength"], d["handles"], d["canonical"], d["R"], float(d["beta"]))
    assert (np.abs(sk - d["skinned"]) / np.maximum(np.abs(d["skinned"]), 1e-3)).max() < 1e-5


def test_bitset_utils_bit_exact():
    d = golden("bitset_utils.npz")
    assert np.array_equal(O.popcount_bitset(d["bitset"]), d["popcount"])
    assert np.array_equal(O.accumulate_bitset_rgb(d["bitset"], d["rgb"]), d["accum"])


def test_fullsize_dda_bitset_checksum():
    """50,000 x 100 strands (4.95M segments), 1024x1024, 2048 clusters: the oracle's bitset
    has the sha256 of the reference's (tests/golden/fullsize_ref.json)."""
    import hashlib
    from strns2cards_gb300 import synthetic as syn
    ref = json.load(open(os.path.join(GOLDEN, "fullsize_ref.json")))["dda_full"]
    sc = syn.strand_scene(50_000, 100, per_cluster=25, num_views=1, seed=0)
    bits = O.dda_cluster_bitset(1024, 1024, sc.pos, sc.edges, sc.edge2cluster, 2048)
    assert hashlib.sha256(bits.tobytes()).hexdigest() == ref["bitset_sha256"]
