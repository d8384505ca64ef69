"""GPU parity of the deformation operators.

Card Laplacian smoothing and LBS forward/backward are float, checked element by element
against the FP64 oracle (``parity.py``): |got - FP64| <= 1e-5 x max(|FP64|, scale), the
scale being the same formula on absolute values (Laplacian: the iteration on |p|; LBS y,
dM, dx: |x|, |M|, |gy| with the non-negative weights).  The LBS binding is exact: guide
indices equal the oracle's brute-force exact-FP32 selection, the inverse lists equal a
stable sort of the bound entries by guide; weights agree to 1e-6 absolute.
"""
import numpy as np
import pytest
import torch

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


@pytest.mark.parametrize("cards,qa,qx,steps", [(256, 32, 4, 10), (2048, 16, 4, 10), (3, 4, 1, 3), (7, 32, 4, 0)])
def test_card_laplacian_matches_oracle(cards, qa, qx, steps):
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    _, _, h, w = syn.grid_strip(qx + 1, qa + 1)
    qe = np.concatenate([h, w], 0)
    nv = (qx + 1) * (qa + 1)
    rng = np.random.default_rng(cards + steps)
    p = rng.normal(size=(cards * nv, 3)).astype(np.float32)
    got = s2c.card_laplacian_smooth(cu(p), qe, nv, 0.5, steps)
    ref = O.card_laplacian_smooth(p, qe, nv, 0.5, steps)
    if steps == 0:
        assert np.array_equal(np_(got), p)
    assert_rel(np_(got), ref, O.card_laplacian_smooth_mag(p, qe, nv, 0.5, steps), TOL, "Laplacian")
    lap = s2c.CardLaplacian(nv, qe)
    x = cu(p)
    lap(x, 0.5, steps, out=x)                          # in place
    assert torch.equal(x, got)


def guide_scene(n_strands, V, per_cluster, seed):
    from strns2cards_gb300 import synthetic as syn
    st = syn.make_strands(n_strands, V, seed=seed)
    cards = syn.make_cards(st, per_cluster, 16, 4)
    nv = 17 * 5
    g = cards.verts.reshape(-1, 5, 17, 3)[:, 2].reshape(-1, 3)      # centre line of every card
    return st.reshape(-1, 3).astype(np.float32), np.ascontiguousarray(g, dtype=np.float32)


@pytest.mark.parametrize("n,V,pc,seed", [(2000, 32, 20, 0), (300, 64, 4, 1)])
def test_lbs_bind_forward_backward(n, V, pc, seed):
    import strns2cards_gb300 as s2c
    x, g = guide_scene(n, V, pc, seed)
    rng = np.random.default_rng(seed)
    x[:5] = g[:5]                                     # on a guide
    x[5] = g[0] + 50.0                                # far outside the guide grid
    b = s2c.LBSBinding(cu(x), cu(g), tau=0.01)
    oidx, ow = O.lbs_bind(x, g, 0.01)
    idx = np_(b.idx)
    assert np.array_equal(idx, oidx)
    assert np.abs(np_(b.w) - ow).max() <= 1e-6
    # inverse lists: entries v*4+slot grouped by guide, ascending
    ent = np.arange(4 * x.shape[0])[oidx.reshape(-1) >= 0]
    order = np.argsort(oidx.reshape(-1)[ent], kind="stable")
    off = np.concatenate([[0], np.cumsum(np.bincount(oidx.reshape(-1)[ent], minlength=g.shape[0]))])
    assert np.array_equal(np_(b.offsets), off)
    assert np.array_equal(np_(b.entries)[:off[-1]], ent[order])
    M = (np.tile(np.eye(3, 4), (g.shape[0], 1, 1)) + rng.normal(scale=0.1, size=(g.shape[0], 3, 4))).astype(np.float32)
    Mt = cu(M).requires_grad_(True)
    xt = cu(x).requires_grad_(True)
    y = s2c.lbs(xt, Mt, b)
    w = np_(b.w)
    assert_rel(np_(y), O.lbs_forward(x, oidx, w, M), O.lbs_forward_mag(x, oidx, w, M), TOL, "LBS y")
    gy = torch.randn(y.shape, generator=torch.Generator().manual_seed(0)).cuda()
    y.backward(gy)
    dM, dx = O.lbs_backward(x, oidx, w, M, np_(gy))
    mM, mx = O.lbs_backward_mag(x, oidx, w, M, np_(gy))
    assert_rel(np_(Mt.grad), dM, mM, TOL, "LBS dM")
    assert_rel(np_(xt.grad), dx, mx, TOL, "LBS dx")
    # deterministic: a second backward gives the same bits
    Mt.grad = None
    xt.grad = None
    s2c.lbs(xt, Mt, b).backward(gy)
    dM2 = np_(Mt.grad)
    Mt.grad = None
    s2c.lbs(xt, Mt, b).backward(gy)
    assert np.array_equal(np_(Mt.grad), dM2)


def test_lbs_few_guides():
    import strns2cards_gb300 as s2c
    x = np.random.default_rng(5).normal(size=(100, 3)).astype(np.float32)
    g = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    b = s2c.LBSBinding(cu(x), cu(g))
    oidx, ow = O.lbs_bind(x, g, 0.01)
    assert np.array_equal(np_(b.idx), oidx) and (oidx[:, 3] == -1).all()
    assert np.abs(np_(b.w) - ow).max() <= 1e-6
