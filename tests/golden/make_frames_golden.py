"""Golden vectors for the strand-frame helpers, made by running the reference's own
``pystrns2cards/curve_utils.py`` (pure torch on the CPU) in this container:

    python tests/golden/make_frames_golden.py --ref /root/reference --out tests/golden

The reference package's ``__init__`` imports its compiled ``_core``; the functions used
here (minimal_rotation, tangent_frame, compute_bishop_frame, compute_aligned_strands,
compute_alignment_rotation, strands_to_tube) do not call it, so the module is loaded on
its own with an empty stand-in for ``_core``.  Inputs are seeded synthetic strands plus
hand-made edge cases (straight strands along +-z and +-y, a hairpin, a repeated point).
"""
from __future__ import annotations

import argparse
import importlib.util
import os
import sys
import types

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from strns2cards_gb300 import synthetic as syn  # noqa: E402


def load_reference_curve_utils(ref_root: str):
    pkg_dir = os.path.join(ref_root, "pystrns2cards")
    pkg = types.ModuleType("pystrns2cards")
    pkg.__path__ = [pkg_dir]
    sys.modules["pystrns2cards"] = pkg
    sys.modules["pystrns2cards._core"] = types.ModuleType("pystrns2cards._core")
    spec = importlib.util.spec_from_file_location("pystrns2cards.curve_utils", os.path.join(pkg_dir, "curve_utils.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["pystrns2cards.curve_utils"] = mod
    spec.loader.exec_module(mod)
    return mod


def edge_strands(V: int) -> np.ndarray:
    t = np.linspace(0.0, 1.0, V)[:, None]
    out = [
        t * np.array([0.0, 0.0, 1.0]),                  # straight +z (tangent_frame sign +1)
        t * np.array([0.0, 0.0, -1.0]),                 # straight -z
        t * np.array([0.0, 1.0, 0.0]),                  # parallel to t_dst
        t * np.array([0.0, -1.0, 0.0]),                 # antiparallel to t_dst
        np.concatenate([t[: V // 2] * [1.0, 0.0, 0.2], (t[V // 2 - 1] - (t[: V - V // 2] - t[0]) * 0.9) * [1.0, 0.0, 0.2]
                        + [0.0, 0.05, 0.0]]),           # hairpin
    ]
    rep = np.cumsum(np.full((V, 3), 0.07), 0)
    rep[V // 3] = rep[V // 3 - 1]                       # a zero-length segment
    out.append(rep)
    return np.stack(out).astype(np.float32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--out", default=os.path.join(ROOT, "tests", "golden"))
    args = ap.parse_args()
    cu = load_reference_curve_utils(args.ref)
    V = 24
    st = np.concatenate([syn.make_strands(26, V, seed=7), edge_strands(V)]).astype(np.float32)
    rng = np.random.default_rng(3)
    x = torch.from_numpy(st)
    T, N, B = cu.compute_bishop_frame(x)
    t_dst = torch.tensor([[0.0, 1.0, 0.0]])
    R = cu.compute_alignment_rotation(x, t_dst)
    roots = torch.from_numpy(rng.normal(size=(st.shape[0], 3)).astype(np.float32))
    t_dst2 = torch.tensor([[0.3, -0.8, 0.2]])
    canon = cu.compute_aligned_strands(x, roots, t_dst2)
    src = rng.normal(size=(40, 3)).astype(np.float32)
    dst = rng.normal(size=(40, 3)).astype(np.float32)
    dst[:5] = src[:5] * 2.0                              # parallel
    dst[5:10] = -src[5:10]                               # antiparallel
    mr = cu.minimal_rotation(torch.from_numpy(src), torch.from_numpy(dst))
    tf_in = rng.normal(size=(30, 3)).astype(np.float32)
    tf_in[:4, 2] = 0.0                                   # sign(0) -> +1
    tn, tb = cu.tangent_frame(torch.from_numpy(tf_in))
    tube_st = syn.make_strands(3, 6, seed=2).astype(np.float32)
    tv, tfaces, tattr = cu.strands_to_tube(tube_st, radius=0.01, n_circle=5,
                                           attr=np.arange(18, dtype=np.float32).reshape(3, 6, 1))
    np.savez_compressed(
        os.path.join(args.out, "frames.npz"),
        strands=st, T=T.numpy(), N=N.numpy(), B=B.numpy(), t_dst=t_dst.numpy(), R=R.numpy(),
        roots=roots.numpy(), t_dst2=t_dst2.numpy(), canon=canon.numpy(),
        mr_src=src, mr_dst=dst, mr=mr.numpy(), tf_in=tf_in, tf_n=tn.numpy(), tf_b=tb.numpy(),
        tube_strands=tube_st, tube_verts=tv, tube_faces=tfaces, tube_attr=tattr)
    print("wrote", os.path.join(args.out, "frames.npz"), st.shape)


if __name__ == "__main__":
    main()
