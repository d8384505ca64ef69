"""GPU parity of the strand curve operators.

smooth_strands / skinning are float, checked element by element (``parity.py``): against
the FP64 oracle (same arclength) |got - FP64| <= 1e-5 x max(|FP64|, scale), the scale
being sum_j w_j |x_j| / sum_j w_j for smoothing and sum_j w_j (|R_j| (|x_i| + |h_j|) +
|c_j|) / sum_j w_j for skinning (coordinates of either sign cancel in the weighted sums);
against the reference's golden outputs 2e-5, the sum of both sides' bounds.  The in-kernel arclength equals the standalone
arclength kernel bit for bit, and the arclength agrees with an FP64 cumulative sum to 1e-6
relative.
"""
import numpy as np
import pytest
import torch

from conftest import golden
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


def arc64(x):
    d = np.linalg.norm(np.diff(x.astype(np.float64), axis=1), axis=2)
    return np.concatenate([np.zeros((x.shape[0], 1)), np.cumsum(d, axis=1)], axis=1)


def random_case(N, V, seed):
    from strns2cards_gb300 import synthetic as syn
    rng = np.random.default_rng(seed)
    st = syn.make_strands(N, V, seed=seed).astype(np.float32)
    hs = (st + rng.normal(scale=0.01, size=st.shape)).astype(np.float32)
    ch = (st + rng.normal(scale=0.02, size=st.shape)).astype(np.float32)
    Q, _ = np.linalg.qr(rng.normal(size=(N, V, 3, 3)))
    return st, hs, ch, Q.astype(np.float32)


def test_curves_match_golden():
    from strns2cards_gb300 import _core
    d = golden("curves.npz")
    st, arc, beta = cu(d["strands"]), cu(d["arclength"]), float(d["beta"])
    out = torch.empty_like(st)
    _core.smooth_strands(st, arc, out, beta)
    smag = O.smooth_strands_mag(d["strands"], d["arclength"], beta)
    assert_rel(np_(out), d["smoothed"], smag, 2 * TOL, "smoothed vs the reference")
    assert_rel(np_(out), O.smooth_strands(d["strands"], d["arclength"], beta), smag, TOL, "smoothed")
    sk = torch.empty_like(st)
    _core.skinning(st, arc, cu(d["handles"]), cu(d["canonical"]), cu(d["R"]), sk, beta)
    args = (d["strands"], d["arclength"], d["handles"], d["canonical"], d["R"], beta)
    kmag = O.skinning_mag(*args)
    assert_rel(np_(sk), d["skinned"], kmag, 2 * TOL, "skinned vs the reference")
    assert_rel(np_(sk), O.skinning(*args), kmag, TOL, "skinned")


@pytest.mark.parametrize("N,V,beta", [(3000, 100, 0.03), (517, 33, 0.2), (64, 1, 0.1), (5, 1000, 0.05),
                                      (40, 7, 1e-9)])
def test_curves_random_match_oracle(N, V, beta):
    """Several strands per CTA, a ragged tail group, single-point strands, strands too long
    to stage for skinning (global path), and a beta whose windows hold only the point itself."""
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import _core
    st, hs, ch, R = random_case(N, V, seed=N + V)
    x = cu(st)
    arc = s2c.compute_arclength(x)
    ref_arc = arc64(st)
    assert np.allclose(np_(arc), ref_arc, rtol=1e-6, atol=1e-6 * max(ref_arc.max(), 1e-30))
    a = np_(arc)
    sm = s2c.smooth_strands(x, beta)
    sm2 = torch.empty_like(x)
    _core.smooth_strands(x, arc, sm2, beta)
    assert torch.equal(sm, sm2)
    assert_rel(np_(sm), O.smooth_strands(st, a, beta), O.smooth_strands_mag(st, a, beta), TOL, "smoothed")
    sk = s2c.skinning(x, cu(hs), cu(ch), cu(R), beta)
    sk2 = torch.empty_like(x)
    _core.skinning(x, arc, cu(hs), cu(ch), cu(R), sk2, beta)
    assert torch.equal(sk, sk2)
    assert_rel(np_(sk), O.skinning(st, a, hs, ch, R, beta), O.skinning_mag(st, a, hs, ch, R, beta), TOL, "skinned")


def test_curves_empty_and_errors():
    import strns2cards_gb300 as s2c
    x = torch.zeros((0, 10, 3), device="cuda")
    assert s2c.smooth_strands(x, 0.1).shape == (0, 10, 3)
    with pytest.raises(ValueError):
        s2c.smooth_strands(torch.zeros((4, 10, 2), device="cuda"), 0.1)
    with pytest.raises(ValueError):
        s2c.smooth_strands(torch.zeros((4, 10, 3)), 0.1)
    with pytest.raises(ValueError):
        s2c.skinning(torch.zeros((4, 10, 3), device="cuda"), torch.zeros((4, 10, 3), device="cuda"),
                     torch.zeros((4, 10, 3), device="cuda"), torch.zeros((4, 10, 3), device="cuda"), 0.1)


def test_device_resampling_equals_host():
    """Ragged strands resampled on the device equal the host version bit for bit (the same
    FP32 operations in the same order), for strands a warp takes through shared memory and
    for strands longer than that (up to 1,500 points, a thread each); strands too short give
    NaN rows."""
    import strns2cards_gb300 as s2c
    rng = np.random.default_rng(9)
    counts = rng.integers(2, 300, size=5000).astype(np.int32)
    counts[::97] = rng.integers(380, 1500, size=counts[::97].shape[0])
    pts = np.cumsum(rng.normal(scale=0.02, size=(int(counts.sum()), 3)), 0).astype(np.float32)
    for T in (2, 33, 100):
        host = s2c.resample_strands_by_arclength(counts, pts, T)
        dev = s2c.resample_strands_by_arclength(cu(counts), cu(pts), T)
        assert np.array_equal(np_(dev), host)
    bad = counts.copy()
    bad[7] = 1
    bad[8] += 1
    out = np_(s2c.resample_strands_by_arclength(cu(bad), cu(pts), 10))
    assert np.isnan(out[7]).all()


@pytest.mark.parametrize("n", [16384, 16385, 40000])
def test_device_resampling_scan_sizes(n):
    """The strand offsets come from the device scan: one CTA up to 16,384 strands, the
    three-launch scan above; both give the host's offsets."""
    import strns2cards_gb300 as s2c
    rng = np.random.default_rng(n)
    counts = rng.integers(2, 12, size=n).astype(np.int32)
    pts = np.cumsum(rng.normal(scale=0.02, size=(int(counts.sum()), 3)), 0).astype(np.float32)
    host = s2c.resample_strands_by_arclength(counts, pts, 7)
    dev = s2c.resample_strands_by_arclength(cu(counts), cu(pts), 7)
    assert np.array_equal(np_(dev), host)
