"""Strand file ingest and arclength resampling on the host: libs2c against the reference's
own loader and resampler (hair_loader.cpp, compiled from the reference's sources into
oracle/_ref/libref_mesh.so by oracle/build_ref.sh) on files of every format written here --
identical strand counts, points and resampled points, bit for bit."""
import ctypes
import os

import numpy as np
import pytest

from conftest import ROOT

REF = os.path.join(ROOT, "oracle", "_ref", "libref_mesh.so")


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def _strands(seed=0, n=40):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        m = int(rng.integers(1, 30))
        s = np.cumsum(rng.normal(scale=0.05, size=(m, 3)), 0).astype(np.float32)
        out.append(s)
    out[3] = out[3][:1]                              # one-point strand
    if len(out[5]) > 3:
        out[5][2] = out[5][1]                        # duplicate consecutive point (.bin drops it)
    return out


def write_bin(path, strands):
    with open(path, "wb") as f:
        f.write(np.int32(len(strands)).tobytes())
        for s in strands:
            f.write(np.int32(len(s)).tobytes())
            rec = np.zeros((len(s), 7), np.float32)
            rec[:, :3] = s
            rec[:, 3:6] = 0.5
            rec[:, 6] = 7
            f.write(rec.tobytes())


def write_data(path, strands):
    with open(path, "wb") as f:
        f.write(np.int32(len(strands)).tobytes())
        for s in strands:
            f.write(np.int32(len(s)).tobytes())
            f.write(np.ascontiguousarray(s, np.float32).tobytes())


def write_hair(path, strands, default_seg=0):
    pts = np.concatenate(strands).astype(np.float32)
    with open(path, "wb") as f:
        f.write(b"HAIR")
        flags = 2 | (0 if default_seg else 1)
        hdr = [len(strands), pts.shape[0], flags] + ([default_seg] if default_seg else [])
        f.write(np.array(hdr, np.uint32).tobytes())
        f.write(np.zeros(128 - (3 if default_seg else 4), np.uint32).tobytes())
        if not default_seg:
            f.write(np.array([len(s) - 1 for s in strands], np.uint16).tobytes())
        f.write(pts.tobytes())


def write_zju(path, strands):
    pts = np.concatenate(strands).astype(np.float32)
    with open(path, "wb") as f:
        f.write(np.array([len(strands), pts.shape[0]], np.uint32).tobytes())
        f.write(np.array([len(s) for s in strands], np.uint16).tobytes())
        f.write(pts.tobytes())


def ref_load(path, kind):
    lib = ctypes.CDLL(REF)
    f = lib.ref_load_strands
    f.restype = ctypes.c_int64
    f.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]
    npts = ctypes.c_int64()
    ns = f(path.encode(), kind, None, None, ctypes.byref(npts))
    c = np.empty(ns, np.int32)
    p = np.empty((npts.value, 3), np.float32)
    f(path.encode(), kind, c.ctypes.data, p.ctypes.data, ctypes.byref(npts))
    return c, p


def ref_resample(counts, points, T):
    lib = ctypes.CDLL(REF)
    out = np.empty((len(counts), T, 3), np.float32)
    lib.ref_resample(ctypes.c_int(len(counts)), ctypes.c_void_p(counts.ctypes.data),
                     ctypes.c_void_p(points.ctypes.data), ctypes.c_int(T), ctypes.c_void_p(out.ctypes.data))
    return out


CASES = [("a.bin", write_bin, 0), ("a.data", write_data, 1), ("a.hair", write_hair, 2),
         ("b.hair", lambda p, s: write_hair(p, [x for x in s if len(x) == len(s[0])] or s[:1], default_seg=len(s[0]) - 1), 2),
         ("c.hair", write_zju, 2)]


@pytest.mark.parametrize("name,writer,kind", CASES, ids=[c[0] for c in CASES])
def test_load_and_resample_match_reference(tmp_path, name, writer, kind):
    import strns2cards_gb300 as s2c
    strands = [s for s in _strands() if len(s) >= 1]
    path = str(tmp_path / name)
    writer(path, strands)
    objs, counts, points = s2c.load_strands(path, return_raw=True)
    assert len(objs) == len(counts) and all(len(o) >= 2 for o in objs)
    if os.path.exists(REF):
        rc, rp = ref_load(path, kind)
        assert np.array_equal(counts, rc) and np.array_equal(points, rp)
    for T in (2, 7, 100):
        got = s2c.resample_strands_by_arclength(counts, points, T)
        assert got.shape == (len(counts), T, 3)
        if os.path.exists(REF):
            assert np.array_equal(got, ref_resample(counts.astype(np.int32), points, T))


def test_load_errors_and_missing_file(tmp_path):
    import strns2cards_gb300 as s2c
    with pytest.raises(ValueError):
        s2c.load_strands(str(tmp_path / "x.obj"))
    assert len(s2c.load_strands(str(tmp_path / "missing.bin"))) == 0
    path = str(tmp_path / "t.data")
    write_data(path, _strands())
    raw = open(path, "rb").read()
    open(path, "wb").write(raw[: len(raw) // 2])
    with pytest.raises(ValueError):
        s2c.load_strands(path)
