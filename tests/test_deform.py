"""CPU checks of the deformation host logic and oracle: the CSR adjacency equals the
uniform Laplacian's neighbour pairs (optimizer.py:70-99), the oracle's Jacobi smoothing
equals a sparse-matrix statement of p - lam D^-1 L p, the oracle's exact-FP32 4-NN equals a
numpy float32 brute force, and its FP64 LBS gradients equal torch FP64 autograd and
central finite differences (h = 1e-3, 64 random vertices, seed 0)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def test_vertex_adjacency_matches_unique_pairs():
    from strns2cards_gb300.deform import vertex_adjacency
    rng = np.random.default_rng(0)
    e = rng.integers(0, 30, size=(120, 2)).astype(np.int32)
    e[:3] = [[4, 4], [5, 6], [6, 5]]                 # self-loop, duplicate pair
    off, adj = vertex_adjacency(30, e)
    pairs = np.unique(np.concatenate([e, e[:, ::-1]], 0), axis=0)
    for v in range(30):
        assert sorted(adj[off[v]:off[v + 1]].tolist()) == sorted(pairs[pairs[:, 0] == v, 1].tolist())
    with pytest.raises(RuntimeError):
        vertex_adjacency(3, np.array([[0, 5]], np.int32))


def test_oracle_laplacian_is_jacobi_of_the_uniform_laplacian():
    from strns2cards_gb300 import synthetic as syn
    _, _, h, w = syn.grid_strip(5, 9)
    qe = np.concatenate([h, w], 0)
    nv = 45
    rng = np.random.default_rng(1)
    p0 = rng.normal(size=(3 * nv, 3))
    got = O.card_laplacian_smooth(p0, qe, nv, 0.5, 4)
    pairs = np.unique(np.concatenate([qe, qe[:, ::-1]], 0), axis=0)
    A = np.zeros((nv, nv))
    A[pairs[:, 0], pairs[:, 1]] = 1
    D = np.diag(A.sum(1))
    step = np.eye(nv) - 0.5 * np.linalg.inv(D) @ (D - A)
    ref = p0.reshape(3, nv, 3).copy()
    for _ in range(4):
        ref = np.einsum("ij,cjk->cik", step, ref)
    assert np.allclose(got, ref.reshape(-1, 3), rtol=1e-12, atol=1e-12)


def test_oracle_knn_matches_numpy_float32():
    rng = np.random.default_rng(2)
    x = rng.normal(size=(500, 3)).astype(np.float32)
    g = rng.normal(size=(300, 3)).astype(np.float32)
    g[7] = g[3]                                       # duplicate guide: tie to the lower index
    x[0] = g[3]
    idx, _ = O.lbs_bind(x, g)
    d = x[:, None, :] - g[None]
    d2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    order = np.lexsort((np.broadcast_to(np.arange(300), d2.shape), d2), axis=1)[:, :4]
    assert np.array_equal(idx, order.astype(np.int32))
    assert idx[0, 0] == 3 and idx[0, 1] == 7


def test_oracle_lbs_gradients_match_autograd_and_fd():
    rng = np.random.default_rng(0)
    x = rng.normal(size=(400, 3))
    g = rng.normal(size=(60, 3)).astype(np.float32)
    idx, w = O.lbs_bind(x.astype(np.float32), g)
    M = rng.normal(size=(60, 3, 4))
    gy = rng.normal(size=(400, 3))
    dM, dx = O.lbs_backward(x, idx, w, M, gy)
    xt = torch.tensor(x, requires_grad=True)
    Mt = torch.tensor(M, requires_grad=True)
    it, wt = torch.from_numpy(idx.astype(np.int64)), torch.from_numpy(w)
    xh = torch.cat([xt, torch.ones(400, 1, dtype=torch.float64)], 1)
    y = (wt[..., None] * torch.einsum("vkrc,vc->vkr", Mt[it], xh)).sum(1)
    assert np.allclose(y.detach().numpy(), O.lbs_forward(x, idx, w, M), rtol=1e-12, atol=1e-12)
    (y * torch.from_numpy(gy)).sum().backward()
    assert np.allclose(Mt.grad.numpy(), dM, rtol=1e-10, atol=1e-10)
    assert np.allclose(xt.grad.numpy(), dx, rtol=1e-10, atol=1e-10)
    # central differences on 64 random vertices (seed 0), weights held at their bound values
    h = 1e-3
    sel = np.random.default_rng(0).choice(400, 64, replace=False)
    for v in sel:
        for c in range(3):
            xp, xm = x.copy(), x.copy()
            xp[v, c] += h
            xm[v, c] -= h
            fd = ((O.lbs_forward(xp, idx, w, M) - O.lbs_forward(xm, idx, w, M)) * gy).sum() / (2 * h)
            assert abs(fd - dx[v, c]) <= 1e-7 * max(1.0, abs(dx[v, c]))
