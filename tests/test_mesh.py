"""Host edge builder of libs2c against the oracle's numpy statement and, when it was built
from the reference's sources (oracle/_ref/libref_mesh.so), the reference's own builder.
The reference's edge order is its hash map's, so it is compared after sorting rows by edge."""
import ctypes
import os

import numpy as np
import pytest

from conftest import ROOT
from oracle import oracle as O

REF_MESH = os.path.join(ROOT, "oracle", "_ref", "libref_mesh.so")


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def meshes():
    rng = np.random.default_rng(3)
    from strns2cards_gb300 import synthetic as syn
    f, _, _, _ = syn.grid_strip(5, 17)
    yield "grid", f.astype(np.int32)
    sc = syn.strand_scene(300, 16, per_cluster=10, num_views=1, seed=2)
    yield "cards", syn.make_cards(sc.strands, 10, 8, 2).tri
    yield "random", rng.integers(0, 50, size=(400, 3)).astype(np.int32)        # non-manifold, degenerate
    yield "one", np.array([[0, 1, 2]], np.int32)
    yield "empty", np.zeros((0, 3), np.int32)
    yield "repeated", np.array([[0, 1, 2], [2, 1, 0], [0, 1, 2], [3, 3, 3]], np.int32)


def ref_edges(tri):
    lib = ctypes.CDLL(REF_MESH)
    f = lib.ref_build_edges_from_triangles
    f.restype = ctypes.c_int64
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
    cap = max(3 * tri.shape[0], 1)
    e = np.empty((cap, 2), np.int32)
    t = np.empty((cap, 2), np.int32)
    n = f(tri.shape[0], tri.ctypes.data, e.ctypes.data, t.ctypes.data, cap)
    assert n >= 0
    e, t = e[:n], t[:n]
    order = np.lexsort((e[:, 1], e[:, 0]))
    return e[order], t[order]


@pytest.mark.parametrize("name,tri", list(meshes()), ids=[m[0] for m in meshes()])
def test_build_edges_matches_oracle_and_reference(name, tri):
    import strns2cards_gb300 as s2c
    e, t = s2c.build_edges_from_triangles(tri)
    oe, ot = O.build_edges_from_triangles(tri)
    assert e.dtype == np.int32 and t.dtype == np.int32 and e.shape == t.shape == (oe.shape[0], 2)
    assert np.array_equal(e, oe) and np.array_equal(t, ot)
    if os.path.exists(REF_MESH):
        re_, rt = ref_edges(tri)
        assert np.array_equal(e, re_) and np.array_equal(t, rt)


def test_build_edges_argument_errors():
    import strns2cards_gb300 as s2c
    with pytest.raises(TypeError):
        s2c.build_edges_from_triangles([[0, 1, 2]])
    with pytest.raises(TypeError):
        s2c.build_edges_from_triangles(np.zeros((2, 3), np.int64))
    with pytest.raises(ValueError):
        s2c.build_edges_from_triangles(np.zeros((2, 4), np.int32))
