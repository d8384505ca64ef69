"""Continuous-batching server: every job gives the same result alone (serial plain calls)
and in the mix (admitted by HBM budget, iterations of all active jobs overlapped on their
own streams) -- the first iteration's XOR loss and per-card IoU counts exactly, the final
card positions to 1e-5 of their max-norm (the gradient's FP64 sums may round differently
between runs) -- and a budget that holds one job at a time makes the others queue."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def jobs():
    from strns2cards_gb300.serving import synthetic_job
    spec = [(400, 16, 128, 64), (1500, 32, 256, 256), (700, 16, 192, 96), (2500, 32, 256, 1024)]
    return [synthetic_job(n, v, r, k, seed=7 + i, iterations=6, arrival=0.01 * i) for i, (n, v, r, k) in enumerate(spec)]


def close(a, b, tol=1e-5):
    return float(np.abs(a.astype(np.float64) - b).max()) <= tol * max(float(np.abs(b).max()), 1e-30)


def test_results_alone_equal_results_in_the_mix():
    from strns2cards_gb300.serving import serve, serve_serial
    reqs = jobs()
    alone = serve_serial(reqs, realtime=False)
    mixed = serve(reqs, budget_bytes=64 << 30, realtime=False)
    for a, m in zip(alone, mixed):
        assert a.loss[0] == m.loss[0] and len(a.loss) == len(m.loss) == 6
        # the first iteration reads only inputs: its per-card counts are exact
        assert np.array_equal(a.iou_first_inter, m.iou_first_inter)
        assert np.array_equal(a.iou_first_union, m.iou_first_union)
        assert a.iou_first_union.sum() > 0 and a.iou_first_inter.sum() > 0
        assert close(m.card_pos, a.card_pos)
        assert m.finished >= m.admitted >= 0
    assert any(a.loss[0] > 0 for a in alone)
    # a budget for one job at a time: later jobs wait for memory, results unchanged
    one = max(r.footprint() for r in reqs)
    queued = serve(reqs, budget_bytes=one, realtime=False)
    for a, q in zip(alone, queued):
        assert a.loss[0] == q.loss[0] and close(q.card_pos, a.card_pos)
    admits = sorted(q.admitted for q in queued)
    finishes = sorted(q.finished for q in queued)
    assert admits[1] >= finishes[0] - 1e-6        # the second admission waited for the first release


def test_footprint_bounds_the_allocator():
    """JobSpec.footprint() (the admission budget's unit) is at least what the allocator
    holds for an admitted job through its first iterations, and not wildly more."""
    from strns2cards_gb300.serving import _Active
    for spec in jobs():
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        base = torch.cuda.memory_allocated()
        torch.cuda.reset_peak_memory_stats()
        job = _Active(spec, torch.device("cuda"), torch.cuda.current_stream()).prepare()
        for _ in range(2):
            job.iterate()
        torch.cuda.synchronize()
        peak = torch.cuda.max_memory_allocated() - base
        assert peak <= spec.footprint(), (spec.name, peak, spec.footprint())
        del job


def test_plain_dropin_loop_gives_the_served_results():
    """The plain per-call baseline (the drop-in ops in the reference's fitting-loop order) and
    the served iteration (cluster planes in rectangles) are the same iteration: first XOR loss
    and per-card IoU counts exact, final cards to 1e-5 of their max-norm."""
    from strns2cards_gb300.serving import serve_serial, serve_serial_dropin, synthetic_job
    reqs = [synthetic_job(600, 16, 192, 96, seed=31, iterations=5), synthetic_job(900, 32, 128, 256, seed=32,
                                                                                  iterations=5)]
    served = serve_serial(reqs, realtime=False)
    plain = serve_serial_dropin(reqs)
    for a, b in zip(served, plain):
        assert a.loss[0] == b.loss[0] > 0 and len(b.loss) == 5
        assert np.array_equal(a.iou_first_inter, b.iou_first_inter)
        assert np.array_equal(a.iou_first_union, b.iou_first_union)
        assert close(b.card_pos, a.card_pos)
