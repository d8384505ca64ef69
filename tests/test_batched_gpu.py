"""Batched per-cluster fitting: one launch sequence over all clusters gives the clusters the
same iteration as independent per-cluster calls (card positions equal to 1e-5 of their
max-norm: the gradient's FP64 sums may round differently), and a CUDA-graph replay of the
iteration equals the eager launch sequence.  The persistent launch (one kernel per
iteration) gives the same iterations as the launch sequence, for every launch shape the
autotuner may choose (chunks of the largest clusters split over CTAs, one thread or one
warp per antialias fragment, 128 to 1024 threads), with empty clusters and frames whose
width is not a multiple of 32, reading the strands packed (each cluster's used vertices only);
the tuner's choice is cached per shape class."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def small_batch():
    from strns2cards_gb300.batched import synthetic_clusters
    return synthetic_clusters(num_clusters=6, verts=32, min_strands=10, max_strands=120, quads_along=16,
                              quads_across=4, H=256, W=64, seed=3)


def close(a, b, tol=1e-5):
    a, b = a.detach().cpu().double(), b.detach().cpu().double()
    return float((a - b).abs().max()) <= tol * max(float(b.abs().max()), 1e-30)


def test_batched_equals_per_cluster_and_graph_equals_eager():
    from strns2cards_gb300.batched import BatchedClusterFit, FitSchedule
    batch = small_batch()
    fa = BatchedClusterFit(batch)
    fb = BatchedClusterFit(batch)
    fb.prepare_plain()
    for _ in range(3):
        fa.eager_step()
        fb.plain_iteration()
    torch.cuda.synchronize()
    assert torch.equal(fa.target, fb.target)
    assert close(fa.cpos, fb.cpos)
    assert not torch.equal(fa.cpos, torch.from_numpy(batch.card_pos).cuda())   # the cards moved
    # graph replay == eager
    fc = BatchedClusterFit(batch)
    fd = BatchedClusterFit(batch)
    fc.capture()
    fc.cpos.copy_(torch.from_numpy(batch.card_pos).cuda())        # undo the capture warm-up
    for _ in range(3):
        fc.graph.replay()
        fd.eager_step()
    torch.cuda.synchronize()
    assert torch.equal(fc.pplanes, fd.pplanes) and close(fc.cpos, fd.cpos, 1e-6)
    sched = FitSchedule(BatchedClusterFit(batch), trials=2, search=True, cache=os.devnull)
    assert sched.best in ("persistent", "eager", "eager2", "graph", "graph2") and len(sched.results) > 4


def _persistent_vs_eager(batch, params, iters=3):
    from strns2cards_gb300.batched import BatchedClusterFit
    fa = BatchedClusterFit(batch)
    fb = BatchedClusterFit(batch)
    for _ in range(iters):
        fa.eager_step()
        fb.persistent_step(params)
    torch.cuda.synchronize()
    return fa, fb


@pytest.mark.parametrize("params", [dict(chunk=8192, threads=256, ctas_per_sm=2, aa_warp=0),
                                    dict(chunk=256, threads=128, ctas_per_sm=1, aa_warp=1),
                                    dict(chunk=1000, threads=512, ctas_per_sm=4, aa_warp=0),
                                    dict(chunk=64, threads=1024, ctas_per_sm=1, aa_warp=1)])
def test_persistent_iteration_equals_launch_sequence(params):
    batch = small_batch()
    fa, fb = _persistent_vs_eager(batch, params)
    assert close(fb.cpos, fa.cpos)
    assert not torch.equal(fb.cpos, torch.from_numpy(batch.card_pos).cuda())
    # the w column is never written
    assert torch.equal(fb.cpos[..., 3], torch.from_numpy(batch.card_pos[..., 3]).cuda())


def test_persistent_empty_cluster_and_ragged_width():
    from strns2cards_gb300.batched import synthetic_clusters
    batch = synthetic_clusters(num_clusters=5, verts=24, min_strands=8, max_strands=60, quads_along=8,
                               quads_across=2, H=96, W=100, seed=7)
    E = batch.strand_edges.shape[0]
    batch.edge_ids = batch.edge_ids[batch.edge_ids // E != 2]          # cluster 2 has no strands
    fa, fb = _persistent_vs_eager(batch, dict(chunk=300, threads=256, ctas_per_sm=2, aa_warp=1))
    assert close(fb.cpos, fa.cpos)
    # the persistent launch reads the strands packed: no rows for the empty cluster
    assert fb.voff_h[3] == fb.voff_h[2] and fb.spos_packed.shape[0] < batch.strand_pos.shape[0] * batch.strand_pos.shape[1]


def test_persistent_graph_replay_and_tuning_cache(tmp_path):
    from strns2cards_gb300.batched import BatchedClusterFit, FitSchedule
    batch = small_batch()
    fa = BatchedClusterFit(batch)
    fa.capture(persistent=True)
    fa.cpos.copy_(torch.from_numpy(batch.card_pos).cuda())           # undo the capture warm-up
    fb = BatchedClusterFit(batch)
    for _ in range(3):
        fa.graph.replay()
        fb.persistent_step()
    torch.cuda.synchronize()
    assert close(fa.cpos, fb.cpos, 1e-6)
    cache = str(tmp_path / "tune.json")
    fit = BatchedClusterFit(batch)
    start = fit.cpos.clone()
    s1 = FitSchedule(fit, trials=1, cache=cache)
    assert not s1.from_cache and torch.equal(fit.cpos, start)        # tuning leaves the cards as they were
    assert len(s1.table) == int(np.prod([len(v) for v in FitSchedule.SPACE.values()])) + 4
    s2 = FitSchedule(BatchedClusterFit(batch), trials=1, cache=cache)
    assert s2.from_cache and s2.best == s1.best and s2.best_params == s1.best_params
    fit.step()                                                         # the applied schedule runs
    torch.cuda.synchronize()
