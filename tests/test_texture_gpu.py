"""Software-MSAA texture render: the batched render (all jitters in one fused raster, one
resolve launch) equals the reference's per-sample loop over the drop-in ops bit for bit,
and its coverage counts equal the oracle's per-sample rasterisations exactly (the
accumulated attributes to 1e-5 of their max-norm, the weights' sum to 1e-6)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def np_(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("H,W,grid", [(48, 64, 8), (37, 29, 3)])
def test_msaa_batched_equals_loop_and_oracle(H, W, grid):
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    verts, faces, attr = syn.wisp_patch(24, 12, n_circle=6, seed=4)
    offsets, weights = s2c.msaa_pattern(grid)
    pos, tri, at = cu(verts), cu(faces), cu(attr)
    acc, cnt, alpha = s2c.msaa_render((H, W), pos, tri, at, offsets, weights)
    lacc, lcnt, lalpha = s2c.msaa_render_loop((H, W), pos, tri, at, offsets, weights)
    assert torch.equal(acc, lacc) and torch.equal(cnt, lcnt) and torch.equal(alpha, lalpha)
    assert float(cnt.max()) > 0
    # oracle: per-sample rasterisation and interpolation in the oracle, FP64 sums
    oacc = np.zeros((H, W, 3))
    ocnt = np.zeros((H, W))
    oal = np.zeros((H, W))
    for (dx, dy), w in zip(offsets, weights):
        pj = np.ones((1, verts.shape[0], 4), np.float32)
        pj[0, :, :3] = verts
        pj[0, :, 0] = (verts[:, 0] + np.float32(dx * 2.0 / W)).astype(np.float32)
        pj[0, :, 1] = (verts[:, 1] + np.float32(dy * 2.0 / H)).astype(np.float32)
        rast = O.rasterize(H, W, pj, faces)
        rgb = O.interpolate(rast, attr, faces)[0]
        v = (rast[0, ..., 3] > 0).astype(np.float64)
        oacc += rgb * v[..., None]
        ocnt += v
        oal += np.float32(w) * v
    assert np.array_equal(np_(cnt), ocnt)
    assert np.abs(np_(acc) - oacc).max() <= 1e-5 * max(np.abs(oacc).max(), 1e-30)
    assert np.abs(np_(alpha) - oal).max() <= 1e-6
    rgb = s2c.resolve_patch(acc, cnt)
    assert rgb.shape == (H, W, 3) and float(rgb.min()) >= 0.0
