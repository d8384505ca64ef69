"""The C ABI library builds for this host, loads, and exports every declared entry."""
import os
import re
import subprocess

from conftest import ROOT


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "s2c.h")).read()
    return sorted(set(re.findall(r"^S2C_API [^(]*?\b(s2c_\w+)\s*\(", txt, flags=re.M)))


def test_header_declares_entries():
    syms = declared_symbols()
    assert "s2c_dda_cluster_bitset" in syms and len(syms) >= 10


def test_library_exports_every_declared_symbol(lib_built):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_built], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (s2c_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing


def test_ctypes_binding_covers_header(lib_built):
    from strns2cards_gb300 import _lib
    L = _lib.lib()
    assert L.s2c_version() >= 1
    assert L.s2c_last_error() is not None
    for s in declared_symbols():
        assert s in _lib.SIGNATURES, f"{s} has no ctypes signature"


def test_workspace_queries_are_pure_host(lib_built):
    from strns2cards_gb300 import _lib
    L = _lib.lib()
    assert L.s2c_dda_cluster_bitset_workspace_size(4_950_000, 1, 1024, 1024, 64) > 8 * 4_950_000
    assert L.s2c_dda_compute_span_workspace_size(1000) > 0
    assert L.s2c_filter_valid_fragments_workspace_size(0) > 0


def test_argument_errors_come_back_as_status_without_a_gpu(lib_built):
    """Invalid sizes and null pointers are rejected on the host before any CUDA call, with a
    status code and a message (the library never exits the process)."""
    import ctypes
    from strns2cards_gb300 import _lib
    L = _lib.lib()
    t3 = (ctypes.c_float * 3)(0.0, 1.0, 0.0)
    cases = [
        ("s2c_strand_frames", (-1, 4, None, None, None, None, None, None, None, 3, None, None)),
        ("s2c_strand_frames", (2, 4, None, None, None, None, None, None, None, 3, None, None)),   # null strands
        ("s2c_wisp_frames", (3, None, 10, 1, None, t3, t3, t3, None, None, None, None)),          # V < 2
        ("s2c_wisp_frames", (3, None, 10, 8, None, t3, t3, t3, None, None, None, None)),          # nulls
        ("s2c_wisp_rotate", (2, None, 10, 0, None, None, None, None, None, None, None)),          # V = 0
        ("s2c_align_strands", (10, L.s2c_align_strands_max_points() + 1, None, 1, None, None, None, t3, 0.05,
                               None, None, None)),                                                # too long to stage
        ("s2c_align_strands", (10, 1, None, 1, None, None, None, t3, 0.05, None, None, None)),    # V < 2
        ("s2c_build_edges_device", (-1, None, 4, None, None, None, None, None, 0, None)),
        ("s2c_build_edges_device", (5, None, 4, None, None, None, None, None, 0, None)),          # null counts
        ("s2c_resample_strands_by_arclength_host", (2, None, None, 1, None)),                     # target < 2
        # compacted fragment lists
        ("s2c_count_fragments", (0, 8, 1, 3, None, 1, None, None, None, 0, None, 0, None, None)),   # H = 0
        ("s2c_count_fragments", (8, 8, 1, 3, None, 1, None, None, None, 1 << 31, None, 0, None, None)),
        ("s2c_write_fragments", (8, 8, 1, 3, None, 1, None, None, None, 5, None, 0, None, None, None)),  # nulls
        ("s2c_dda_count_fragments", (4, 10, None, None, None, None, 0, 8, 1, 2, None, 1, None, None, 0, None,
                                     None)),                                                      # H = 0
        ("s2c_dda_write_fragments", (4, -1, None, None, None, None, 8, 8, 1, 2, None, 1, None, None, 0, None, None,
                                     None)),                                                      # F < 0
        # plane rectangles
        ("s2c_planes_clear_rects", (1, 8, 40, 1, None, None, None)),                              # nulls
        ("s2c_planes_clear_rects", (1, 8, 40, 1, ctypes.c_void_p(16), ctypes.c_void_p(20), None)),  # misaligned rects
        ("s2c_planes_bounds", (1, 8, 40, 0, ctypes.c_void_p(16), ctypes.c_void_p(16), None)),       # S = 0
        ("s2c_cluster_iou_counts_planes_rects", (1, 8, 40, 1, 33, None, None, None, None, None, None, None, None)),
        ("s2c_rasterize_fused_planes_onto", (1, 8, 8, 3, None, 1, None, None, 1, 1, None, ctypes.c_void_p(16), None,
                                             0, None)),                                           # null planes
    ]
    for name, args in cases:
        st = getattr(L, name)(*args)
        assert st == _lib.S2C_ERR_INVALID, (name, args, st)
        assert L.s2c_last_error(), name
    # empty problems are no-ops that succeed
    assert L.s2c_strand_frames(0, 4, None, None, None, None, None, None, None, 3, None, None) == 0
    assert L.s2c_wisp_frames(0, None, 0, 4, None, t3, t3, t3, None, None, None, None) == 0
    assert L.s2c_align_strands(0, 8, None, 0, None, None, None, t3, 0.05, None, None, None) == 0
    assert L.s2c_align_strands_max_points() >= 64
    assert L.s2c_build_edges_device_workspace_size(0, 0) > 0


def test_dda_cluster_bitset_argument_errors_without_a_gpu(lib_built):
    """The headline entry rejects bad arguments on the host, before any launch: sizes,
    slot count, null and misaligned pointers (INVALID), a short workspace (WORKSPACE), and
    a problem too large for the no-alloc variant's fixed scratch (INVALID).  The pointers
    below are aligned addresses that are never dereferenced."""
    from strns2cards_gb300 import _lib
    L = _lib.lib()
    pos, edges, p2c, bits, ws = 0x10000, 0x20000, 0x30000, 0x40000, 0x50000
    ok = dict(P=1000, ids=None, H=64, W=64, B=1, V=2000, pos=pos, E=1000, edges=edges, p2c=p2c, S=2, bits=bits,
              ws=ws, wsb=0)

    def call(**kw):
        a = dict(ok, **kw)
        return L.s2c_dda_cluster_bitset(a["P"], a["ids"], a["H"], a["W"], a["B"], a["V"], a["pos"], a["E"], a["edges"],
                                        a["p2c"], a["S"], a["bits"], a["ws"], a["wsb"], None)

    def call_noalloc(**kw):
        a = dict(ok, **kw)
        return L.s2c_dda_cluster_bitset_noalloc(a["P"], a["ids"], a["H"], a["W"], a["B"], a["V"], a["pos"], a["E"],
                                                a["edges"], a["p2c"], a["S"], a["bits"], None)

    # both entries reject the same bad arguments on the host, before any CUDA call (so
    # these run without a GPU and name the entry in the message)
    for kw in (dict(P=-1), dict(H=0), dict(W=40000), dict(B=0), dict(P=1001),    # P > B*E without edge ids
               dict(pos=None), dict(edges=None), dict(S=0), dict(S=2049), dict(bits=None),
               dict(bits=bits + 4), dict(pos=pos + 4), dict(edges=edges + 4), dict(p2c=None)):
        assert call(**kw) == _lib.S2C_ERR_INVALID, kw
        assert L.s2c_last_error(), kw
        assert call_noalloc(**kw) == _lib.S2C_ERR_INVALID, kw
        assert b"dda_cluster_bitset_noalloc" in L.s2c_last_error(), kw
    assert call() == _lib.S2C_ERR_WORKSPACE                                       # workspace of 0 bytes
    assert call(ws=None, wsb=1 << 30) == _lib.S2C_ERR_WORKSPACE
    assert L.s2c_dda_cluster_bitset_noalloc(5_000_000, None, 1024, 1024, 1, 5_050_000, pos, 5_000_000, edges, p2c, 64,
                                            bits, None) == _lib.S2C_ERR_INVALID
    assert b"fixed" in L.s2c_last_error()
