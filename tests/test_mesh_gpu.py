"""The device edge builder against the host builder (itself checked against the oracle and
the reference's own builder in test_mesh.py): the same edges in the same order and the same
edge->triangle map, bit for bit, on grids, card meshes, random non-manifold and degenerate
triangle lists, repeated triangles, a high-degree fan and the empty list; half-edges with
out-of-range vertices are counted and left out."""
import numpy as np
import pytest
import torch

from test_mesh import meshes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def extra_meshes():
    rng = np.random.default_rng(8)
    yield "repeated", np.tile(np.array([[0, 1, 2], [2, 1, 3]], np.int32), (5, 1))
    fan = np.stack([np.zeros(3000, np.int32), np.arange(1, 3001), np.arange(2, 3002)], 1).astype(np.int32)
    yield "fan", fan                                           # one vertex in 3,000 triangles
    yield "big", rng.integers(0, 20000, size=(60000, 3)).astype(np.int32)


@pytest.mark.parametrize("name,tri", list(meshes()) + list(extra_meshes()), ids=lambda x: x if isinstance(x, str) else "")
def test_device_edges_equal_host_edges(name, tri):
    import strns2cards_gb300 as s2c
    he, ht = s2c.build_edges_from_triangles(tri)
    de, dt = s2c.build_edges_from_triangles(torch.from_numpy(tri).cuda())
    assert np.array_equal(de.cpu().numpy(), he), name
    assert np.array_equal(dt.cpu().numpy(), ht), name


def test_device_edges_count_out_of_range_vertices():
    import strns2cards_gb300 as s2c
    tri = np.array([[0, 1, 2], [2, 1, 7], [3, 0, 1]], np.int32)
    edges, e2t, counts = s2c.build_edges_from_triangles_device(torch.from_numpy(tri).cuda(), 4)
    E, bad = counts.tolist()
    assert bad == 2                                            # (1, 7) and (2, 7)
    he, ht = s2c.build_edges_from_triangles(tri[[0, 2]])
    # without the two bad half-edges: triangle 1 still contributes (1, 2)
    assert E == he.shape[0]
    assert np.array_equal(edges[:E].cpu().numpy(), he)
    with pytest.raises(ValueError):
        s2c.build_edges_from_triangles(torch.from_numpy(tri).cuda(), 4)
