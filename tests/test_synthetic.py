"""Synthetic workloads are deterministic and identical across hosts."""
import hashlib
import json
import os

import numpy as np

from conftest import GOLDEN
from strns2cards_gb300 import synthetic as syn
from oracle.oracle import build_edges_from_triangles


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_fullsize_inputs_match_the_reference_run():
    ref = json.load(open(os.path.join(GOLDEN, "fullsize_ref.json")))
    sc = syn.strand_scene(50_000, 100, per_cluster=25, num_views=1, seed=0)
    assert sha(sc.pos) + ":" + sha(sc.edges) == ref["dda_full"]["input_sha256"]


def test_small_config_shapes():
    sc = syn.strand_scene(1024, 32, per_cluster=16, num_views=1, seed=0)
    assert sc.pos.shape == (1, 32768, 4) and sc.edges.shape == (31744, 2) and sc.num_clusters == 64
    cards = syn.make_cards(sc.strands, 16, 8, 2)
    assert cards.verts.shape == (64 * 27, 3) and cards.tri.shape == (64 * 32, 3)


def test_edge_topology_of_a_grid_strip():
    f, q, h, w = syn.grid_strip(3, 9)
    e, e2t = build_edges_from_triangles(f)
    assert e.shape[0] == len(h) + len(w) + q.shape[0]        # boundary/interior + one diagonal per quad
    assert (e[:, 0] < e[:, 1]).all()
    interior = (e2t[:, 1] >= 0).sum()
    assert interior == e.shape[0] - 2 * (8 + 2)              # boundary edges have one triangle
