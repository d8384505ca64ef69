"""The reference's own Python ops over this package's ``_core``.

``tests/golden/make_dropin_tape.py`` ran the reference's unmodified op modules
(``pystrns2cards/{dda,rasterize,antialias,bitset_utils,curve_utils}.py``) with their
``_core`` bound to the CPU oracle and recorded every ``_core`` call they made: name,
positional arguments (tensors with their contents before the call), return value and the
tensors each call wrote, plus each op's inputs and final outputs.

* replay: every recorded call is made through ``strns2cards_gb300._core`` with the same
  positional arguments as CUDA tensors, in the reference's order.  Return values must be
  equal; every tensor the reference's call wrote must come back equal -- bit for bit for
  integer, coverage, span, fragment, depth and normal outputs, and for the float sums
  (interpolation, the antialias gradient, colour sums, smoothing, skinning) within
  |got - ref| <= 2e-5 x max(|ref|, 1e-3 max|ref|) elementwise (the recorded values are the
  oracle's FP64 sums rounded to FP32); tensors the call did not write must be unchanged.
* ops: this package's op of the same name, on the same inputs, gives the reference op's
  final outputs under the same bounds.
"""
import json
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

FLOAT_CALLS = {"interpolate_triangle_attributes", "backward_interpolate_triangle_attributes",
               "dda_interpolate_attributes", "backward_dda_interpolate_attributes",
               "backward_antialiased_cluster_bitset", "accumulate_bitset_rgb", "smooth_strands", "skinning"}
FLOAT_OUTPUTS = {"image", "d_attr", "d_pos", "accum", "out"}


def _tape():
    with open(os.path.join(GOLDEN, "dropin_tape.json")) as f:
        cases = json.load(f)["cases"]
    return cases, np.load(os.path.join(GOLDEN, "dropin_tape.npz"))


CASES, ARR = _tape()


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def np_(t):
    return t.detach().cpu().numpy()


def assert_same(got, ref, floating, what):
    got, ref = np.asarray(got), np.asarray(ref)
    assert got.shape == ref.shape, (what, got.shape, ref.shape)
    if not floating:
        assert np.array_equal(got, ref), what
        return
    r = ref.astype(np.float64)
    scale = np.maximum(np.abs(r), 1e-3 * np.abs(r).max(initial=0.0))
    bad = ~(np.abs(got.astype(np.float64) - r) <= 2e-5 * scale + 1e-30)
    assert not bad.any(), f"{what}: {int(bad.sum())} of {bad.size} elements off"


@pytest.mark.parametrize("case", [c["case"] for c in CASES])
def test_reference_core_calls_replay(case):
    from strns2cards_gb300 import _core
    c = next(x for x in CASES if x["case"] == case)
    for k, call in enumerate(c["calls"]):
        args, pre = [], {}
        for i, a in enumerate(call["args"]):
            if "tensor" in a:
                pre[i] = ARR[a["tensor"]]
                t = cu(pre[i])
                assert str(t.dtype).replace("torch.", "") == a["dtype"]
                args.append(t)
            elif "int" in a:
                args.append(a["int"])
            else:
                args.append(a["float"])
        ret = getattr(_core, call["name"])(*args)
        torch.cuda.synchronize()
        what = f"{case} call {k} {call['name']}"
        assert ret == call["ret"], (what, ret, call["ret"])
        for i, t in enumerate(args):
            if not isinstance(t, torch.Tensor):
                continue
            if str(i) in call["wrote"]:
                assert_same(np_(t), ARR[call["wrote"][str(i)]], call["name"] in FLOAT_CALLS and t.is_floating_point(),
                            f"{what} arg {i}")
            else:
                assert np.array_equal(np_(t), pre[i]), f"{what}: arg {i} changed"


SCALARS = {"H", "W", "B", "K", "kernel_radius", "rho", "count_xor_error", "beta"}


def _inputs(c):
    return {k: (ARR[v].reshape(-1)[0] if k in SCALARS else ARR[v]) for k, v in c["inputs"].items()}


@pytest.mark.parametrize("case", [c["case"] for c in CASES])
def test_ops_give_the_reference_ops_outputs(case):
    import strns2cards_gb300 as s2c
    c = next(x for x in CASES if x["case"] == case)
    d = _inputs(c)
    hw = (int(d["H"]), int(d["W"])) if "H" in d else None
    op = c["op"]
    if op == "dda_compute_fragments":
        ids = cu(d["edge_ids"]) if "edge_ids" in d else None
        fp, fa = s2c.dda_compute_fragments(hw, cu(d["pos"]), cu(d["edges"]), ids)
        got = dict(frag_pix=fp, frag_attrs=fa)
    elif op == "cluster_mask_from_fragments":
        got = dict(bitset=s2c.cluster_mask_from_fragments(hw, cu(d["frag_pix"]), cu(d["frag_attrs"]),
                                                          cu(d["prim2cluster"]), int(d["K"])))
    elif op == "depth_test":
        got = dict(rast=s2c.depth_test(int(d["B"]), hw, cu(d["frag_pix"]), cu(d["frag_attrs"])))
    elif op == "dda_interpolate_attributes":
        a = cu(d["attr"]).requires_grad_(True)
        img = s2c.dda_interpolate_attributes(cu(d["rast"]), a, cu(d["edges"]))
        img.backward(cu(d["grad"]))
        got = dict(image=img, d_attr=a.grad)
    elif op == "interpolate_triangle_attributes":
        a = cu(d["attr"]).requires_grad_(True)
        img = s2c.interpolate_triangle_attributes(cu(d["rast"]), a, cu(d["tri"]))
        img.backward(cu(d["grad"]))
        got = dict(image=img, d_attr=a.grad)
    elif op == "popcount_bitset":
        got = dict(count=s2c.popcount_bitset(cu(d["bitset"])))
    elif op == "accumulate_bitset_rgb":
        got = dict(accum=s2c.accumulate_bitset_rgb(cu(d["bitset"]), cu(d["rgb"])))
    elif op == "compute_fragments":
        fp, fa = s2c.compute_fragments(hw, cu(d["pos"]), cu(d["tri"]))
        got = dict(frag_pix=fp, frag_attrs=fa)
    elif op == "rasterize":
        got = dict(rast=s2c.rasterize(hw, cu(d["pos"]), cu(d["tri"])))
    elif op == "mark_discontinuity_edges":
        ids, nrm = s2c.mark_discontinuity_edges(hw, cu(d["pos"]), cu(d["tri"]), cu(d["edges"]), cu(d["edge2tri"]))
        got = dict(prim_ids=ids, normals=nrm)
    elif op == "antialiased_cluster_bitset_loss":
        p = cu(d["pos"]).requires_grad_(True)
        loss = s2c.antialiased_cluster_bitset_loss(cu(d["bitset"]), cu(d["target"]), p, cu(d["tri"]), cu(d["edges"]),
                                                   cu(d["edge2tri"]), cu(d["edge2cluster"]), float(d["kernel_radius"]),
                                                   float(d["rho"]), bool(d["count_xor_error"]))
        loss.backward()
        got = dict(loss=loss.reshape(1), d_pos=p.grad)
    elif op == "smooth_strands":
        got = dict(out=s2c.smooth_strands(cu(d["strands"]), float(d["beta"])))
    elif op == "skinning":
        got = dict(out=s2c.skinning(cu(d["strands"]), cu(d["handles"]), cu(d["canonical"]), cu(d["R"]),
                                    float(d["beta"])))
    else:
        raise AssertionError(f"no op for {op}")
    assert set(got) == set(c["outputs"]), (set(got), set(c["outputs"]))
    for k, key in c["outputs"].items():
        assert_same(np_(got[k]), ARR[key], k in FLOAT_OUTPUTS, f"{case} {k}")
