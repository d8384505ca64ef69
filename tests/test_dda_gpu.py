"""GPU parity of the DDA path: drop-in fragments and the fused segment -> bitset kernel.

Integer outputs (fragment pixels, bitsets) must be bit-identical to the reference's
golden vectors and to the oracle; FP32 fragment attributes are bit-identical too.
"""
import hashlib
import json
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN, golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def np_(t):
    return t.detach().cpu().numpy()


DDA_CASES = ["dda_strands", "dda_edgecases", "dda_edge_ids"]


@pytest.mark.parametrize("name", DDA_CASES)
def test_dda_compute_fragments_matches_golden(name):
    import strns2cards_gb300 as s2c
    d = golden(name + ".npz")
    ids = cu(d["edge_ids"]) if "edge_ids" in d else None
    fp, fa = s2c.dda_compute_fragments((int(d["H"]), int(d["W"])), cu(d["pos"]), cu(d["edges"]), ids)
    fp, fa = np_(fp), np_(fa)
    # in-order compaction: same order as the oracle
    op, oa = O.dda_compute_fragments(int(d["H"]), int(d["W"]), d["pos"], d["edges"], d.get("edge_ids"))
    assert np.array_equal(fp, op) and np.array_equal(fa, oa)
    sp, sa = O.sort_frags(fp, fa)
    assert np.array_equal(sp, d["frag_pix"]) and np.array_equal(sa, d["frag_attrs"])


@pytest.mark.parametrize("name", DDA_CASES)
def test_core_span_outputs_match_golden(name):
    from strns2cards_gb300 import _core
    d = golden(name + ".npz")
    pos, edges = cu(d["pos"]), cu(d["edges"])
    B, E = d["pos"].shape[0], d["edges"].shape[0]
    ids = cu(d["edge_ids"]) if "edge_ids" in d else torch.arange(B * E, dtype=torch.int32, device="cuda")
    P = ids.shape[0]
    prefix = torch.empty(P, dtype=torch.int32, device="cuda")
    slopes = torch.empty((P, 2), dtype=torch.float32, device="cuda")
    spans = torch.empty((P, 4), dtype=torch.float32, device="cuda")
    F = _core.dda_compute_span(ids, int(d["H"]), int(d["W"]), pos, edges, prefix, slopes, spans)
    counts = np.diff(np.concatenate([[0], np_(prefix).astype(np.int64)]))
    assert F == int(d["span_counts"].sum())
    assert np.array_equal(counts, d["span_counts"])
    m = counts > 0
    for got, ref in ((np_(slopes)[m], d["span_slopes"][m]), (np_(spans)[m], d["span_spans"][m])):
        assert np.all((got == ref) | (np.isnan(got) & np.isnan(ref)))
    # raw (pre-compaction) fragments, element for element
    fp = torch.full((F, 3), -1, dtype=torch.int32, device="cuda")
    fa = torch.empty((F, 4), dtype=torch.float32, device="cuda")
    _core.dda_compute_fragments(prefix, ids, slopes, spans, int(d["H"]), int(d["W"]), pos, edges, fp, fa)
    assert np.array_equal(np_(fp), d["raw_pix"])
    ok = d["raw_pix"][:, 0] >= 0
    assert np.array_equal(np_(fa)[ok], d["raw_attrs"][ok])


@pytest.mark.parametrize("name", DDA_CASES)
def test_cluster_mask_and_fused_bitset_match_golden(name):
    import strns2cards_gb300 as s2c
    d = golden(name + ".npz")
    H, W, K = int(d["H"]), int(d["W"]), int(d["K"])
    ref = d["bitset"]
    ids = cu(d["edge_ids"]) if "edge_ids" in d else None
    pos, edges, e2c = cu(d["pos"]), cu(d["edges"]), cu(d["edge2cluster"])
    fp, fa = s2c.dda_compute_fragments((H, W), pos, edges, ids)
    m = s2c.cluster_mask_from_fragments((H, W), fp, fa, e2c, K)
    assert np.array_equal(np_(m), ref)
    fused = np_(s2c.dda_cluster_bitset((H, W), pos, edges, e2c, K, edge_ids=ids))
    assert np.array_equal(fused[: ref.shape[0]], ref) and not fused[ref.shape[0]:].any()


def _persp(points, B, seed):
    rng = np.random.default_rng(seed)
    p = points.reshape(-1, 3).astype(np.float64)
    c = 0.5 * (p.min(0) + p.max(0))
    q = (p - c) / (p.max(0) - p.min(0)).max()
    out = []
    for _ in range(B):
        a = rng.uniform(-0.7, 0.7)
        R = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
        r = q @ R.T
        w = 1.2 + 0.8 * r[:, 2]
        out.append(np.stack([1.4 * r[:, 0], 1.4 * r[:, 1], 0.95 * r[:, 2] * w, w], 1))
    return np.stack(out).astype(np.float32)


@pytest.mark.parametrize("H,W,K,views,seed", [
    (256, 256, 64, 1, 0),      # the small published workload
    (97, 131, 33, 3, 1),       # odd sizes, S = 2
    (200, 160, 100, 2, 2),     # S = 4
    (128, 96, 1, 2, 3),        # S = 1
    (64, 64, 2048, 1, 4),      # S = 64
    (150, 150, 4000, 1, 5),    # S = 125 (not a multiple of 4)
])
def test_fused_bitset_matches_oracle(H, W, K, views, seed):
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    n = 1024 if K < 2048 else 2048
    st = syn.make_strands(n, 32, seed=seed)
    pos = np.concatenate([syn.project(st, syn.ortho_cameras(st, 0.3, 1)), _persp(st, views - 1, seed)], 0) \
        if views > 1 else syn.project(st, syn.ortho_cameras(st, 0.3, 1))
    edges = syn.strand_edges(n, 32)
    rng = np.random.default_rng(seed)
    e2c = rng.integers(0, K, size=edges.shape[0]).astype(np.int32)
    ref = O.dda_cluster_bitset(H, W, pos, edges, e2c, K)
    got = np_(s2c.dda_cluster_bitset((H, W), cu(pos), cu(edges), cu(e2c), K))
    assert np.array_equal(got, ref)


def _call_fused_raw(pos, edges, e2c, K, H, W, ws_bytes, edge_ids=None):
    from strns2cards_gb300 import _lib
    from strns2cards_gb300._lib import ptr
    B, V, _ = pos.shape
    E = edges.shape[0]
    S = (K + 31) // 32
    P = B * E if edge_ids is None else edge_ids.shape[0]
    out = torch.full((B, H, W, S), -7, dtype=torch.int32, device="cuda")
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    _lib.call("s2c_dda_cluster_bitset", P, ptr(edge_ids), H, W, B, V, ptr(pos), E, ptr(edges), ptr(e2c), S,
              ptr(out), ptr(ws), ws.numel(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return out, ws


def test_fused_bitset_with_tiny_workspace_uses_fallback_and_stays_exact():
    from strns2cards_gb300 import _core, _lib
    from strns2cards_gb300 import synthetic as syn
    sc = syn.strand_scene(1024, 32, per_cluster=16, num_views=2, seed=7)
    H = W = 256
    P = sc.edges.shape[0] * 2
    full = _lib.lib().s2c_dda_cluster_bitset_workspace_size(P, 2, H, W, 2)
    fixed = full - (2 * P + (1 << 16)) * 8
    out, ws = _call_fused_raw(cu(sc.pos), cu(sc.edges), cu(sc.edge2cluster), 64, H, W, fixed + 40 * 1024)
    n_ent, n_over = _core.dda_cluster_bitset_stats(ws)
    assert n_over > 0
    assert np.array_equal(np_(out), O.dda_cluster_bitset(H, W, sc.pos, sc.edges, sc.edge2cluster, 64))


def test_fused_bitset_many_chunks_in_one_tile_stays_exact():
    """147 chunks of 2048 segments all landing in one 8x8 tile (long record list, heavy tile)."""
    from strns2cards_gb300 import _core, _lib
    rng = np.random.default_rng(3)
    n = 300_000
    p0 = rng.uniform(-0.9, 0.9, size=(n, 2))
    p1 = p0 + rng.uniform(-0.3, 0.3, size=(n, 2))
    pos = np.zeros((1, 2 * n, 4), np.float32)
    pos[0, 0::2, :2] = p0
    pos[0, 1::2, :2] = p1
    pos[0, :, 3] = 1.0
    edges = np.arange(2 * n, dtype=np.int32).reshape(n, 2)
    e2c = rng.integers(0, 40, size=n).astype(np.int32)
    H = W = 8
    need = _lib.lib().s2c_dda_cluster_bitset_workspace_size(n, 1, H, W, 2)
    out, ws = _call_fused_raw(cu(pos), cu(edges), cu(e2c), 40, H, W, need)
    n_ent, n_over = _core.dda_cluster_bitset_stats(ws)
    assert n_ent > 0
    assert np.array_equal(np_(out), O.dda_cluster_bitset(H, W, pos, edges, e2c, 40))


def test_fused_bitset_invalid_ids_are_skipped_not_read():
    import strns2cards_gb300 as s2c
    d = golden("dda_edgecases.npz")
    E = d["edges"].shape[0]
    ids = np.array([3, -1, 3, E + 5, 0, 2 ** 31 - 1, 17], dtype=np.int32)
    keep = ids[(ids >= 0) & (ids < E)]
    e2c = d["edge2cluster"]
    got = np_(s2c.dda_cluster_bitset((int(d["H"]), int(d["W"])), cu(d["pos"]), cu(d["edges"]), cu(e2c), 40,
                                     edge_ids=cu(ids)))
    ref = O.dda_cluster_bitset(int(d["H"]), int(d["W"]), d["pos"], d["edges"], e2c, 40, keep)
    assert np.array_equal(got, ref)


def test_fused_bitset_empty_input_zeroes_output():
    import strns2cards_gb300 as s2c
    pos = torch.zeros((2, 4, 4), dtype=torch.float32, device="cuda")
    edges = torch.zeros((0, 2), dtype=torch.int32, device="cuda")
    e2c = torch.zeros((0,), dtype=torch.int32, device="cuda")
    out = torch.full((2, 16, 24, 3), 5, dtype=torch.int32, device="cuda")
    s2c.dda_cluster_bitset((16, 24), pos, edges, e2c, 96, out=out)
    assert not out.any()


def test_fused_bitset_is_deterministic():
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    sc = syn.strand_scene(4096, 48, per_cluster=16, num_views=2, seed=11)
    args = ((512, 512), cu(sc.pos), cu(sc.edges), cu(sc.edge2cluster), 256)
    a = s2c.dda_cluster_bitset(*args)
    b = s2c.dda_cluster_bitset(*args)
    assert torch.equal(a, b)


def test_fullsize_fused_bitset_matches_reference_checksum():
    """4.95M segments into a 1024x1024x2048-cluster bitset (256 MiB): sha256 equal to the
    reference's composition, computed on the same input."""
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    ref = json.load(open(os.path.join(GOLDEN, "fullsize_ref.json")))["dda_full"]
    sc = syn.strand_scene(50_000, 100, per_cluster=25, num_views=1, seed=0)
    bits = s2c.dda_cluster_bitset((1024, 1024), cu(sc.pos), cu(sc.edges), cu(sc.edge2cluster), 2048)
    assert hashlib.sha256(np_(bits).tobytes()).hexdigest() == ref["bitset_sha256"]
    assert int(s2c.popcount_bitset(bits).sum().item()) == ref["popcount"]


def test_bitset_utils_match_golden():
    import strns2cards_gb300 as s2c
    d = golden("bitset_utils.npz")
    assert np.array_equal(np_(s2c.popcount_bitset(cu(d["bitset"]))), d["popcount"])
    assert np.array_equal(np_(s2c.accumulate_bitset_rgb(cu(d["bitset"]), cu(d["rgb"]))), d["accum"])


def test_compact_valid_ints_in_order():
    from strns2cards_gb300 import _core
    rng = np.random.default_rng(0)
    a = rng.integers(-3, 5, size=100_003).astype(np.int32)
    out = torch.empty(a.shape[0], dtype=torch.int32, device="cuda")
    n = _core.compact_valid_ints(cu(a), out)
    assert np.array_equal(np_(out[:n]), a[a >= 0])


@pytest.mark.parametrize("seed", [5, 6])
def test_compacted_dda_fragments_equal_the_filtered_raw_list(seed):
    """``dda_compute_fragments`` writes the accepted DDA steps straight into their own list;
    it must equal the raw list of every step (-1 where rejected: outside the image or the
    depth range) compacted by ``filter_valid_fragments``, in order -- with edge_ids selecting
    views, segments leaving the image, perspective, a vertex behind the camera and an empty
    selection."""
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import _core
    rng = np.random.default_rng(seed)
    B, V, E, H, W = 2, 900, 800, 70, 130
    pos = rng.uniform(-1.4, 1.4, size=(B, V, 4)).astype(np.float32)
    pos[..., 3] = rng.uniform(0.3, 1.7, size=(B, V))
    pos[..., :2] *= pos[..., 3:4]
    pos[..., 2] = rng.uniform(-1.3, 1.3, size=(B, V)) * pos[..., 3]     # some beyond the depth range
    pos[0, :20, 3] = -0.5                                                # behind the camera
    edges = np.stack([rng.integers(0, V, E), rng.integers(0, V, E)], 1).astype(np.int32)
    ids = rng.permutation(B * E)[: B * E - 137].astype(np.int32)
    p, e, i = cu(pos), cu(edges), cu(ids)
    P = ids.shape[0]
    prefix = torch.empty(P, dtype=torch.int32, device="cuda")
    slopes = torch.empty((P, 2), dtype=torch.float32, device="cuda")
    spans = torch.empty((P, 4), dtype=torch.float32, device="cuda")
    F = _core.dda_compute_span(i, H, W, p, e, prefix, slopes, spans)
    raw_p = torch.full((F, 3), -1, dtype=torch.int32, device="cuda")
    raw_a = torch.empty((F, 4), dtype=torch.float32, device="cuda")
    _core.dda_compute_fragments(prefix, i, slopes, spans, H, W, p, e, raw_p, raw_a)
    out_p, out_a = torch.empty_like(raw_p), torch.empty_like(raw_a)
    n = _core.filter_valid_fragments(raw_p, raw_a, out_p, out_a)
    fp, fa = s2c.dda_compute_fragments((H, W), p, e, i)
    assert F > n > 1000 and fp.shape[0] == n
    assert torch.equal(fp, out_p[:n]) and torch.equal(fa, out_a[:n])
    ep, ea = s2c.dda_compute_fragments((H, W), p, e, i[:0])
    assert ep.shape == (0, 3) and ea.shape == (0, 4)
