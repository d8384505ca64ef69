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
