"""Batched per-cluster fitting: one launch sequence over all clusters gives the clusters the
same iteration as independent per-cluster calls (card positions equal to 1e-5 of their
max-norm: the gradient's FP64 sums may round differently), and a CUDA-graph replay of the
iteration equals the eager launch sequence."""
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
    sched = FitSchedule(BatchedClusterFit(batch), trials=2)
    assert sched.best in ("eager", "eager2", "graph", "graph2") and len(sched.results) == 4
