"""The committed drop-in tape is what the reference's own op modules produce: where the
reference sources are present, regenerating it gives the same calls, arguments, return
values and arrays (the recorder runs the CPU oracle; no GPU needed)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

REF = os.environ.get("S2C_REFERENCE_ROOT", "/root/reference")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "pystrns2cards")), reason="reference sources not present")
def test_tape_regenerates_identically(tmp_path):
    subprocess.run([sys.executable, os.path.join(ROOT, "tests", "golden", "make_dropin_tape.py"), "--ref", REF,
                    "--out", str(tmp_path)], check=True, capture_output=True, timeout=600)
    with open(os.path.join(GOLDEN, "dropin_tape.json")) as f:
        want = json.load(f)
    with open(tmp_path / "dropin_tape.json") as f:
        got = json.load(f)
    assert got == want
    a, b = np.load(os.path.join(GOLDEN, "dropin_tape.npz")), np.load(tmp_path / "dropin_tape.npz")
    assert sorted(a.files) == sorted(b.files)
    for k in a.files:
        assert np.array_equal(a[k], b[k]), k


def test_tape_covers_every_core_call_of_the_ops():
    with open(os.path.join(GOLDEN, "dropin_tape.json")) as f:
        cases = json.load(f)["cases"]
    names = {c["name"] for case in cases for c in case["calls"]}
    assert names >= {"dda_compute_span", "dda_compute_fragments", "filter_valid_fragments", "compute_triangle_rects",
                     "compute_fragments", "depth_test", "interpolate_triangle_attributes",
                     "backward_interpolate_triangle_attributes", "dda_interpolate_attributes",
                     "backward_dda_interpolate_attributes", "cluster_mask_from_fragments", "mark_discontinuity_edges",
                     "compact_valid_ints", "backward_antialiased_cluster_bitset", "popcount_bitset",
                     "accumulate_bitset_rgb", "smooth_strands", "skinning"}
