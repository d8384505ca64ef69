"""s2c_dda_cluster_bitset_noalloc: the fused DDA -> bitset for callers that cannot
allocate device memory (for example a plugin hosted by an application that owns the
device memory pool and passes only input and output buffers).  Its scratch is a fixed
32 MiB array inside libs2c.so.

Checked through the C ABI against s2c_dda_cluster_bitset with a caller workspace, on two
calls in a row with different inputs (the shared scratch keeps the previous call's
contents, so the second call shows nothing stale leaks).  Bitsets are integer outputs and
must be identical.  This file is named to be collected last.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _args(sc, H, W, K, out):
    from strns2cards_gb300._lib import ptr
    pos, edges, e2c = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (sc.pos, sc.edges, sc.edge2cluster))
    B, V, _ = pos.shape
    E = edges.shape[0]
    keep = (pos, edges, e2c)
    return keep, (B * E, None, H, W, B, V, ptr(pos), E, ptr(edges), ptr(e2c), (K + 31) // 32, ptr(out))


def _run_pair(sc, H, W, K):
    from strns2cards_gb300 import _lib
    L = _lib.lib()
    S = (K + 31) // 32
    B = sc.pos.shape[0]
    stream = torch.cuda.current_stream().cuda_stream
    ref = torch.full((B, H, W, S), -1, dtype=torch.int32, device="cuda")
    got = torch.full((B, H, W, S), -1, dtype=torch.int32, device="cuda")
    keep, a = _args(sc, H, W, K, ref)
    ws = torch.empty(L.s2c_dda_cluster_bitset_workspace_size(a[0], B, H, W, S), dtype=torch.uint8, device="cuda")
    _lib.call("s2c_dda_cluster_bitset", *a, ws.data_ptr(), ws.numel(), stream)
    keep2, b = _args(sc, H, W, K, got)
    _lib.call("s2c_dda_cluster_bitset_noalloc", *b[:11], got.data_ptr(), stream)
    torch.cuda.synchronize()
    del keep, keep2
    return ref, got


def test_noalloc_matches_workspace_entry_on_two_calls(lib_built):
    from strns2cards_gb300 import synthetic as syn
    first = syn.strand_scene(1024, 32, per_cluster=16, num_views=2, seed=0)
    ref1, got1 = _run_pair(first, 256, 256, 64)
    assert torch.equal(ref1, got1)
    assert int(ref1.ne(0).sum()) > 0
    second = syn.strand_scene(3000, 40, per_cluster=10, num_views=1, seed=5)
    ref2, got2 = _run_pair(second, 320, 288, 300)
    assert torch.equal(ref2, got2)


def test_noalloc_matches_workspace_entry_at_its_size_limit(lib_built):
    # the largest strand scene (100-point strands, 1024x1024, K = 2048) whose scratch still
    # fits the fixed 32 MiB: the case where the entry pool is nearly full
    from strns2cards_gb300 import _lib
    from strns2cards_gb300 import synthetic as syn
    L = _lib.lib()
    limit = 32 << 20
    n_strands = 1
    while L.s2c_dda_cluster_bitset_workspace_size((2 * n_strands) * 99, 1, 1024, 1024, 64) <= limit:
        n_strands *= 2
    lo, hi = n_strands, 2 * n_strands
    while hi - lo > 1:
        mid = (lo + hi) // 2
        if L.s2c_dda_cluster_bitset_workspace_size(mid * 99, 1, 1024, 1024, 64) <= limit:
            lo = mid
        else:
            hi = mid
    assert L.s2c_dda_cluster_bitset_workspace_size((lo + 1) * 99, 1, 1024, 1024, 64) > limit
    sc = syn.strand_scene(lo, 100, per_cluster=25, num_views=1, seed=3)
    ref, got = _run_pair(sc, 1024, 1024, 2048)
    assert torch.equal(ref, got)
    assert int(ref.ne(0).sum()) > 100_000


def test_noalloc_rejects_problems_beyond_its_scratch(lib_built):
    from strns2cards_gb300 import _lib
    L = _lib.lib()
    out = torch.empty(16, dtype=torch.int32, device="cuda")
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    edges = torch.zeros(16, dtype=torch.int32, device="cuda")
    st = L.s2c_dda_cluster_bitset_noalloc(4_950_000, None, 1024, 1024, 1, 5_000_000, dummy.data_ptr(), 4_950_000,
                                          edges.data_ptr(), edges.data_ptr(), 64, out.data_ptr(),
                                          torch.cuda.current_stream().cuda_stream)
    assert st == _lib.S2C_ERR_INVALID
    assert b"fixed" in L.s2c_last_error()
