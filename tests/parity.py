"""Elementwise float parity against the FP64 oracle.

Every float output of the path is a sum of products.  Each element is held to

    |got - ref| <= tol * max(|ref|, mag)

where ``ref`` is the FP64 evaluation of the same formula and ``mag`` the element's
condition scale: the FP64 sum of its terms' magnitudes (the oracle's ``*_mag``
functions).  Where no term cancels, mag = |ref| and this is the plain relative bound;
where terms cancel (signed attributes, N(0, 1) gradients, coordinates near zero) no FP32
evaluation -- the reference's included -- is accurate relative to the small result, only
relative to what was summed.  Exact zeros must come out exactly zero.
"""
import numpy as np


def check_rel(got, ref, mag=None, tol=1e-5):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    scale = np.abs(ref) if mag is None else np.maximum(np.abs(ref), np.abs(np.asarray(mag, np.float64)))
    err = np.abs(got - ref)
    bad = ~(err <= tol * scale)          # NaN counts as a failure
    ratio = np.where(scale > 0, err / np.where(scale > 0, scale, 1.0), np.where(err > 0, np.inf, 0.0))
    return dict(ok=not bool(bad.any()), n=int(got.size), n_bad=int(bad.sum()),
                worst=float(np.nan_to_num(ratio, nan=np.inf).max(initial=0.0)),
                n_beyond_value=int((~(err <= tol * np.abs(ref))).sum()))


def assert_rel(got, ref, mag=None, tol=1e-5, what="output"):
    r = check_rel(got, ref, mag, tol)
    assert r["ok"], (f"{what}: {r['n_bad']} of {r['n']} elements beyond {tol:g} x max(|FP64|, sum|terms|); "
                     f"worst |got - ref| / scale = {r['worst']:.3g}")
    return r
