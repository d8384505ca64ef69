"""CPU checks of the strand-frame oracle: pinned against the reference's own torch
functions (``curve_utils.py``) run on the CPU (tests/golden/frames.npz, generated by
tests/golden/make_frames_golden.py), and properties of the per-wisp frame.

The reference computes in FP32 and the oracle in FP64, so they agree to FP32 rounding:
2e-6 absolute on unit vectors and rotation entries, 1e-6 relative on canonical handles.
"""
import numpy as np

from conftest import golden
from oracle import oracle as O
from strns2cards_gb300 import synthetic as syn


def test_bishop_frame_matches_reference():
    g = golden("frames.npz")
    T, N, B = O.bishop_frame(g["strands"])
    for nm, a in (("T", T), ("N", N), ("B", B)):
        assert np.abs(a - g[nm]).max() <= 2e-6, nm


def test_alignment_rotation_matches_reference():
    g = golden("frames.npz")
    R = O.alignment_rotation(g["strands"], g["t_dst"])
    assert np.abs(R - g["R"]).max() <= 2e-6


def test_aligned_strands_matches_reference():
    g = golden("frames.npz")
    c = O.aligned_strands(g["strands"], g["roots"], g["t_dst2"])
    assert np.abs(c - g["canon"]).max() <= 1e-6 * np.abs(g["canon"]).max()


def test_minimal_rotation_and_tangent_frame_match_reference():
    g = golden("frames.npz")
    assert np.abs(O.minimal_rotation(g["mr_src"], g["mr_dst"]) - g["mr"]).max() <= 2e-6
    n, b = O.tangent_frame(g["tf_in"])
    assert np.abs(n - g["tf_n"]).max() <= 2e-6 and np.abs(b - g["tf_b"]).max() <= 2e-6


def test_wisp_frame_is_a_rotation_taking_the_guide_frame_to_the_target():
    st, sizes = syn.make_wisps(300, 16, 7, seed=4)
    off = 0
    for n in sizes:
        w = st[off:off + n]
        off += n
        R, c, li = O.wisp_frame(w)
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-12) and np.isclose(np.linalg.det(R), 1.0)
        assert np.allclose(c, w[:, 0].astype(np.float64).mean(0))
        lengths = np.linalg.norm(np.diff(w.astype(np.float64), axis=1), axis=2).sum(1)
        assert li == int(np.argmax(lengths))
        # the guide's root-to-tip direction lands in the target's (t, b) plane, t >= 0 side
        g = w[li].astype(np.float64) - c
        down = (g[-1] - g[0]) / np.linalg.norm(g[-1] - g[0])
        d = R @ down
        if n >= 3:
            assert abs(d @ O.WISP_N_DST) < 1 - 1e-6
        assert d @ O.WISP_T_DST >= -1e-9


def test_wisp_frame_small_wisps_use_identity_axes():
    st, _ = syn.make_wisps(2, 8, 1, seed=1)
    R, c, li = O.wisp_frame(st)          # 2 strands: SVD gives 2 axes, the frame falls back to the identity's
    R1, _, _ = O.wisp_frame(st[:1])
    assert np.isfinite(R).all() and np.isfinite(R1).all()
    # least axis (0, 0, 1) signed by the view direction: N_src = +-z
    g = st[li].astype(np.float64) - c
    view = (g[0] - g[1]) / np.linalg.norm(g[0] - g[1])
    nsrc = np.array([0.0, 0.0, 1.0]) * (1.0 if view[2] >= 0 else -1.0)
    assert np.allclose(R @ nsrc, O.WISP_N_DST, atol=1e-12)
