"""GPU parity of the strand frames and the wisp alignment.

Float outputs against the reference's golden vectors (tests/golden/frames.npz: its torch
functions run on the CPU) and the FP64 oracle.  Tolerances, written per check:
- unit vectors and rotation entries: 1e-5 absolute on the 24-point golden strands, 1e-4
  on 64-point strands (the FP32 recurrence accumulates over the points, as the
  reference's does);
- canonical handles: 1e-5 of their max-norm;
- wisp frames: 1e-5 + 1e-6 x the conditioning lambda_max / (lambda_mid - lambda_min) of
  the roots' least-variance axis (an FP32 eigen-solve); centres 1e-6 of the extent;
  longest-strand indices exactly;
- aligned strands: 2e-4 of their max-norm (three FP32 stages -- smoothing, frames,
  skinning -- after the rotation).
"""
import numpy as np
import pytest
import torch

from conftest import golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def np_(t):
    return t.detach().cpu().numpy()


def maxdiff(a, b):
    return float(np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64)).max(initial=0.0))


def test_bishop_frame_matches_golden():
    import strns2cards_gb300 as s2c
    g = golden("frames.npz")
    T, N, B = s2c.compute_bishop_frame(cu(g["strands"]))
    for nm, a in (("T", T), ("N", N), ("B", B)):
        assert maxdiff(np_(a), g[nm]) <= 1e-5, nm


def test_alignment_rotation_and_aligned_strands_match_golden():
    import strns2cards_gb300 as s2c
    g = golden("frames.npz")
    R = s2c.compute_alignment_rotation(cu(g["strands"]), cu(g["t_dst"]))
    assert maxdiff(np_(R), g["R"]) <= 1e-5
    c = s2c.compute_aligned_strands(cu(g["strands"]), cu(g["roots"]), cu(g["t_dst2"]))
    assert maxdiff(np_(c), g["canon"]) <= 1e-5 * np.abs(g["canon"]).max()


def test_minimal_rotation_and_tangent_frame_match_golden():
    import strns2cards_gb300 as s2c
    g = golden("frames.npz")
    assert maxdiff(np_(s2c.minimal_rotation(cu(g["mr_src"]), cu(g["mr_dst"]))), g["mr"]) <= 1e-5
    n, b = s2c.tangent_frame(cu(g["tf_in"]))
    assert maxdiff(np_(n), g["tf_n"]) <= 1e-5 and maxdiff(np_(b), g["tf_b"]) <= 1e-5


def test_strands_to_tube_matches_golden():
    import strns2cards_gb300 as s2c
    g = golden("frames.npz")
    v, f, a = s2c.strands_to_tube(g["tube_strands"], radius=0.01, n_circle=5,
                                  attr=np.arange(18, dtype=np.float32).reshape(3, 6, 1))
    assert v.shape == g["tube_verts"].shape and maxdiff(v, g["tube_verts"]) <= 1e-6
    assert np.array_equal(f, g["tube_faces"]) and np.array_equal(a, g["tube_attr"])


def test_frames_long_strands_against_oracle():
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import _core
    from strns2cards_gb300 import synthetic as syn
    st = syn.make_strands(500, 64, seed=11).astype(np.float32)
    x = cu(st)
    S, V, _ = st.shape
    T, N, B, c = (torch.empty_like(x) for _ in range(4))
    R = torch.empty((S, V, 3, 3), device="cuda")
    roots = cu(np.random.default_rng(2).normal(size=(S, V, 3)).astype(np.float32))
    _core.strand_frames(x, t_dst=(0.0, 1.0, 0.0), T=T, N=N, B=B, R=R, roots=roots[:, 0], canon=c)
    oT, oN, oB = O.bishop_frame(st)
    assert maxdiff(np_(T), oT) <= 1e-5
    assert maxdiff(np_(N), oN) <= 1e-4 and maxdiff(np_(B), oB) <= 1e-4
    assert maxdiff(np_(R), O.alignment_rotation(st, [0.0, 1.0, 0.0])) <= 1e-4
    oc = O.aligned_strands(st, np_(roots[:, 0]), [0.0, 1.0, 0.0])
    assert maxdiff(np_(c), oc) <= 1e-5 * np.abs(oc).max()
    # each output alone equals the same output of the combined pass
    T2, N2, B2 = s2c.compute_bishop_frame(x)
    assert torch.equal(T2, T) and torch.equal(N2, N) and torch.equal(B2, B)
    assert torch.equal(s2c.compute_alignment_rotation(x, torch.tensor([[0.0, 1.0, 0.0]])), R)


def test_frames_of_strands_too_long_to_stage_against_oracle():
    # 3,500 points per strand do not fit the staged form's shared memory: one thread per
    # strand from global memory (1e-3 on unit vectors: 3,500 FP32 recurrence steps)
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    st = syn.make_strands(6, 3500, seed=3, step=0.002, jitter=2e-4).astype(np.float32)
    T, N, B = s2c.compute_bishop_frame(cu(st))
    oT, oN, oB = O.bishop_frame(st)
    assert maxdiff(np_(T), oT) <= 1e-5
    assert maxdiff(np_(N), oN) <= 1e-3 and maxdiff(np_(B), oB) <= 1e-3
    c = s2c.compute_aligned_strands(cu(st), cu(st[:, 0]), torch.tensor([[0.0, 1.0, 0.0]]))
    oc = O.aligned_strands(st, st[:, 0], [0.0, 1.0, 0.0])
    assert maxdiff(np_(c), oc) <= 1e-5 * np.abs(oc).max()


def _wisp_case(N, V, K, seed):
    from strns2cards_gb300 import synthetic as syn
    st, sizes = syn.make_wisps(N, V, K, seed=seed)
    return st, sizes


@pytest.mark.parametrize("N,V,K,seed", [(400, 24, 9, 0), (3000, 32, 64, 1), (40, 16, 20, 2)])
def test_wisp_frames_against_oracle(N, V, K, seed):
    from strns2cards_gb300 import _core, curve_utils as cv
    st, sizes = _wisp_case(N, V, K, seed)
    x = cu(st)
    offs = cu(np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32))
    Rg = torch.empty((K, 3, 3), device="cuda")
    cen = torch.empty((K, 3), device="cuda")
    li = torch.empty(K, dtype=torch.int32, device="cuda")
    _core.wisp_frames(offs, x, cv.WISP_T_DST, cv.WISP_N_DST, cv.WISP_B_DST, Rg, cen, li)
    off = 0
    ext = float(np.abs(st).max())
    for w, n in enumerate(sizes):
        R, c, l = O.wisp_frame(st[off:off + n])
        assert int(li[w]) == off + l
        assert maxdiff(np_(cen[w]), c) <= 1e-6 * ext
        # the FP32 eigen-solve resolves the least-variance axis to about
        # eps * lambda_max / (lambda_mid - lambda_min) (lambda = squared singular values)
        cond = 1.0
        if n >= 3:
            sv = np.linalg.svd(st[off:off + n, 0].astype(np.float64) - c, compute_uv=False) ** 2
            cond = sv[0] / max(sv[1] - sv[2], 1e-300)
        assert maxdiff(np_(Rg[w]), R) <= 1e-5 + 1e-6 * cond, (w, n, cond)
        off += n


def test_align_wisps_against_oracle():
    import strns2cards_gb300 as s2c
    st, sizes = _wisp_case(2000, 32, 37, 3)
    wisps = np.split(st, np.cumsum(sizes)[:-1])
    aligned, handles, longest = s2c.align_wisps(wisps, 0.05)
    oa, oh, ol = O.align_wisps(wisps, 0.05)
    assert np.array_equal(np_(longest), ol)
    assert maxdiff(np_(handles), oh) <= 1e-5 * np.abs(oh).max()
    assert maxdiff(np_(aligned), oa) <= 2e-4 * np.abs(oa).max()
    # the same wisps as device tensors with sizes give the same result bit for bit
    a2, h2, l2 = s2c.align_wisps_packed(cu(st), sizes, 0.05)
    assert torch.equal(a2, aligned) and torch.equal(h2, handles) and torch.equal(l2, longest)


def test_fused_align_strands_equals_the_unfused_steps_bit_for_bit():
    from strns2cards_gb300 import _core, curve_utils as cv
    st, sizes = _wisp_case(3000, 48, 61, 8)
    x = cu(st)
    K = len(sizes)
    offs = cu(np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32))
    Rg = torch.empty((K, 3, 3), device="cuda")
    cen = torch.empty((K, 3), device="cuda")
    li = torch.empty(K, dtype=torch.int32, device="cuda")
    _core.wisp_frames(offs, x, cv.WISP_T_DST, cv.WISP_N_DST, cv.WISP_B_DST, Rg, cen, li)
    h, a = torch.empty_like(x), torch.empty_like(x)
    _core.align_strands(x, offs, Rg, cen, cv.WISP_T_DST, 0.07, h, a)
    a2, h2 = cv._align_strands_unfused(x, offs, Rg, cen, 0.07)
    assert torch.equal(h, h2)
    assert torch.equal(a, a2)


def test_align_wisps_of_strands_too_long_to_fuse_against_oracle():
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import _core
    V = _core.align_strands_max_points() + 7
    st, sizes = _wisp_case(12, V, 3, 9)
    st = (st[:, :1] + 0.05 * (st - st[:, :1])).astype(np.float32)   # keep the strands a plausible length
    wisps = np.split(st, np.cumsum(sizes)[:-1])
    aligned, handles, longest = s2c.align_wisps(wisps, 0.002)
    oa, oh, ol = O.align_wisps(wisps, 0.002)
    assert np.array_equal(np_(longest), ol)
    assert maxdiff(np_(handles), oh) <= 1e-5 * np.abs(oh).max()
    assert maxdiff(np_(aligned), oa) <= 1e-3 * np.abs(oa).max()


def test_align_wisps_one_wisp_equals_alone_and_in_the_mix():
    import strns2cards_gb300 as s2c
    st, sizes = _wisp_case(600, 24, 11, 5)
    wisps = np.split(st, np.cumsum(sizes)[:-1])
    a_all, _, l_all = s2c.align_wisps(wisps, 0.05)
    off = int(sizes[:4].sum())
    a_one, _, l_one = s2c.align_wisps([wisps[4]], 0.05)
    assert torch.equal(a_one, a_all[off:off + sizes[4]])
    assert int(l_one[0]) + off == int(l_all[4])


def test_align_wisps_rejects_empty_wisps():
    import strns2cards_gb300 as s2c
    st, _ = _wisp_case(10, 8, 1, 0)
    with pytest.raises(RuntimeError):
        s2c.align_wisps([st[:5], st[:0], st[5:]], 0.05)


def test_align_wisp_against_oracle():
    import strns2cards_gb300 as s2c
    st, _ = _wisp_case(150, 32, 1, 6)
    a, h, li = s2c.align_wisp(cu(st), 0.05)
    oa, oh, ol = O.align_wisp(st, 0.05)
    assert int(li) == ol
    assert maxdiff(np_(h), oh) <= 1e-5 * np.abs(oh).max()
    assert maxdiff(np_(a), oa) <= 2e-4 * np.abs(oa).max()
