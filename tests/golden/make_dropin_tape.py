"""Drop-in tape: the reference's own Python ops, unmodified, driving a ``_core``.

The reference's op modules (``pystrns2cards/{dda,rasterize,antialias,bitset_utils,
curve_utils}.py``) are plain Python over its compiled ``_core``.  They cannot travel to the
GPU host, so their behaviour is recorded here and replayed there through
``strns2cards_gb300._core`` (``tests/test_dropin_tape_gpu.py``):

    python tests/golden/make_dropin_tape.py --ref /root/reference --out tests/golden

Recording: the modules are loaded from the reference sources as they are, with
``pystrns2cards._core`` bound to a recorder whose functions run the CPU oracle (pinned to
the reference's kernels) in place on the tensors the ops pass, and with a recording
context in which CPU tensors pass the ops' ``is_cuda`` checks and ``device='cuda'``
allocations land on the CPU.  For every op invocation the tape holds the op's inputs and
final outputs and, for every ``_core`` call it made, the call's name, its positional
arguments (tensors with their contents before the call; ints and floats as values), its
return value and the contents of every tensor the call wrote.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import sys
import types

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from strns2cards_gb300 import synthetic as syn  # noqa: E402

OPS = ("dda", "rasterize", "bitset_utils", "antialias", "curve_utils")


def _np(t):
    return t.detach().numpy()


# ---- the recorder: _core functions on CPU tensors, run by the oracle ----------------------
def _set(t, a):
    t.copy_(torch.from_numpy(np.ascontiguousarray(a)).to(t.dtype).reshape(t.shape))


def _add(t, a):
    t.add_(torch.from_numpy(np.ascontiguousarray(a)).to(t.dtype).reshape(t.shape))


def c_dda_compute_span(edge_ids, H, W, pos, edges, prefix, slopes, spans):
    counts, sl, sp = O.dda_span(H, W, _np(pos), _np(edges), _np(edge_ids))
    _set(prefix, np.cumsum(counts, dtype=np.int64).astype(np.int32))
    _set(slopes, sl)
    _set(spans, sp)
    return int(prefix[-1]) if prefix.numel() else 0


def c_dda_compute_fragments(prefix, edge_ids, slopes, spans, H, W, pos, edges, frag_pix, frag_attrs):
    p, ids, s1, s2 = _np(prefix), _np(edge_ids), _np(slopes), _np(spans)
    ps, es = np.ascontiguousarray(_np(pos)), np.ascontiguousarray(_np(edges))
    fp, fa = _np(frag_pix), _np(frag_attrs)
    O.lib().or_dda_fragments(p.shape[0], O._p(p, O.i32p), O._p(ids, O.i32p), O._p(s1, O.f32p), O._p(s2, O.f32p),
                             H, W, ps.shape[1], O._p(ps, O.f32p), es.shape[0], O._p(es, O.i32p),
                             O._p(fp, O.i32p), O._p(fa, O.f32p))


def c_filter_valid_fragments(frag_pix, frag_attrs, pix_out, attrs_out):
    fp, fa, po, ao = _np(frag_pix), _np(frag_attrs), _np(pix_out), _np(attrs_out)
    return int(O.lib().or_filter_valid(fp.shape[0], O._p(fp, O.i32p), O._p(fa, O.f32p), O._p(po, O.i32p),
                                       O._p(ao, O.f32p)))


def c_compute_triangle_rects(H, W, pos, tri, rects, prefix):
    r, counts = O.tri_rects(H, W, _np(pos), _np(tri))
    _set(rects, r)
    _set(prefix, np.cumsum(counts, dtype=np.int64).astype(np.int32))
    return int(prefix[-1]) if prefix.numel() else 0


def c_compute_fragments(H, W, pos, tri, prefix, rects, frag_pix, frag_attrs):
    ps, tr = np.ascontiguousarray(_np(pos)), np.ascontiguousarray(_np(tri))
    r, p, fp, fa = _np(rects), _np(prefix), _np(frag_pix), _np(frag_attrs)
    O.lib().or_tri_fragments(H, W, ps.shape[0], ps.shape[1], O._p(ps, O.f32p), tr.shape[0], O._p(tr, O.i32p),
                             O._p(r, O.i32p), O._p(p, O.i32p), O._p(fp, O.i32p), O._p(fa, O.f32p))


def c_depth_test(H, W, frag_pix, frag_attrs, rast):
    _set(rast, O.depth_test(rast.shape[0], H, W, _np(frag_pix), _np(frag_attrs)))


def c_interpolate_triangle_attributes(rast, attr, tri, image):
    _set(image, O.interpolate(_np(rast), _np(attr), _np(tri)))


def c_backward_interpolate_triangle_attributes(rast, d_image, tri, d_attr):
    _add(d_attr, O.interpolate_backward(_np(rast), _np(d_image), _np(tri), d_attr.shape[0]))


def c_dda_interpolate_attributes(rast, attr, edges, image):
    _set(image, O.dda_interpolate(_np(rast), _np(attr), _np(edges)))


def c_backward_dda_interpolate_attributes(rast, d_image, edges, d_attr):
    _add(d_attr, O.dda_interpolate_backward(_np(rast), _np(d_image), _np(edges), d_attr.shape[0]))


def c_cluster_mask_from_fragments(frag_pix, frag_attrs, prim2cluster, bitset):
    fp, fa, p2c, bits = _np(frag_pix), _np(frag_attrs), _np(prim2cluster), _np(bitset)
    B, H, W, S = bits.shape
    O.lib().or_cluster_mask(fp.shape[0], O._p(fp, O.i32p), O._p(fa, O.f32p), O._p(p2c, O.i32p), H, W, S,
                            O._p(bits, O.i32p))


def c_mark_discontinuity_edges(H, W, tri, edges, edge2tri, pos, prim_ids, normals):
    _, nrm, raw = O.mark_discontinuity_edges(H, W, _np(pos), _np(tri), _np(edges), _np(edge2tri), raw=True)
    _set(prim_ids, raw)
    _set(normals, nrm)


def c_compact_valid_ints(ids, out):
    a, o = _np(ids), _np(out)
    return int(O.lib().or_compact_ints(a.shape[0], O._p(a, O.i32p), O._p(o, O.i32p)))


def c_backward_antialiased_cluster_bitset(frag_pix, frag_attrs, bitset, target, pos, edges, normals, edge2cluster,
                                         d_pos, kernel_radius, rho):
    _add(d_pos, O.aa_backward(_np(frag_pix), _np(frag_attrs), _np(bitset), _np(target), _np(pos), _np(edges),
                              _np(normals), _np(edge2cluster), kernel_radius, rho))


def c_popcount_bitset(bitset, count):
    _set(count, O.popcount_bitset(_np(bitset)))


def c_accumulate_bitset_rgb(bitset, rgb, accum):
    _set(accum, O.accumulate_bitset_rgb(_np(bitset), _np(rgb)))


def c_smooth_strands(strands, arclength, out, beta):
    _set(out, O.smooth_strands(_np(strands), _np(arclength), beta))


def c_skinning(strands, arclength, handles, canonical, R, out, beta):
    _set(out, O.skinning(_np(strands), _np(arclength), _np(handles), _np(canonical), _np(R), beta))


class Tape:
    def __init__(self):
        self.arrays = {}
        self.cases = []
        self.calls = None

    def put(self, key, a):
        self.arrays[key] = np.ascontiguousarray(a)
        return key

    def recorder(self):
        core = types.ModuleType("pystrns2cards._core")
        for name, fn in list(globals().items()):
            if name.startswith("c_") and callable(fn):
                setattr(core, name[2:], self._wrap(name[2:], fn))
        return core

    def _wrap(self, name, fn):
        def call(*args):
            if self.calls is None:       # outside an op invocation: run, keep nothing
                return fn(*args)
            k = len(self.calls)
            pre = {}
            spec = []
            for i, a in enumerate(args):
                if isinstance(a, torch.Tensor):
                    pre[i] = a.detach().clone()
                    spec.append({"tensor": self.put(f"{self.case}/{k}/{i}/in", pre[i].numpy()),
                                 "dtype": str(a.dtype).replace("torch.", "")})
                elif isinstance(a, (bool, int, np.integer)):
                    spec.append({"int": int(a)})
                else:
                    spec.append({"float": float(a)})
            ret = fn(*args)
            wrote = {}
            for i, a in enumerate(args):
                if isinstance(a, torch.Tensor) and not torch.equal(a.detach(), pre[i]):
                    wrote[str(i)] = self.put(f"{self.case}/{k}/{i}/out", a.detach().numpy())
            self.calls.append({"name": name, "args": spec, "ret": ret, "wrote": wrote})
            return ret
        return call

    def run(self, case, op, fn, inputs, outputs_of):
        """Record the op invocation ``fn()`` (on ``inputs``); outputs_of(result) -> dict of
        tensors to keep; returns the result."""
        self.case = case
        self.calls = []
        res = fn()
        outs = {k: self.put(f"{case}/result/{k}", _np(v)) for k, v in outputs_of(res).items()}
        self.cases.append({"case": case, "op": op, "inputs": {k: self.put(f"{case}/input/{k}", v)
                                                              for k, v in inputs.items()},
                           "outputs": outs, "calls": self.calls})
        self.calls = None          # calls made outside an op invocation are not kept
        return res


class _CpuTorch:
    """``torch`` for the reference modules while recording: device='cuda' allocations land
    on the CPU, and uninitialised allocations (empty, empty_like) are zero-filled so that
    the recorded inputs of every call are reproducible; everything else is torch itself."""

    def __getattr__(self, name):
        obj = getattr(torch, {"empty": "zeros", "empty_like": "zeros_like"}.get(name, name))
        if name in ("zeros", "full", "empty", "ones", "arange", "zeros_like", "empty_like", "ones_like", "tensor"):
            def alloc(*a, **kw):
                if "device" in kw and str(kw["device"]).startswith("cuda"):
                    kw["device"] = "cpu"
                return obj(*a, **kw)
            return alloc
        return obj


def load_reference_ops(ref_root, core):
    pkg_dir = os.path.join(ref_root, "pystrns2cards")
    pkg = types.ModuleType("pystrns2cards")
    pkg.__path__ = [pkg_dir]
    sys.modules["pystrns2cards"] = pkg
    sys.modules["pystrns2cards._core"] = core
    pkg._core = core
    mods = {}
    for name in OPS:
        spec = importlib.util.spec_from_file_location(f"pystrns2cards.{name}", os.path.join(pkg_dir, f"{name}.py"))
        mod = importlib.util.module_from_spec(spec)
        sys.modules[f"pystrns2cards.{name}"] = mod
        spec.loader.exec_module(mod)
        mod.torch = _CpuTorch()
        setattr(pkg, name, mod)
        mods[name] = mod
    return mods


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--out", default=os.path.join(ROOT, "tests", "golden"))
    args = ap.parse_args()
    tape = Tape()
    R = load_reference_ops(args.ref, tape.recorder())
    O.set_threads(1)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a))  # noqa: E731
    is_cuda = torch.Tensor.is_cuda
    torch.Tensor.is_cuda = property(lambda self: True)    # CPU tensors pass the ops' CUDA checks
    try:
        # strands: 24 x 12 points, 2 views of 40 x 48 px, 40 clusters (2 slots)
        sc = syn.strand_scene(24, 12, per_cluster=1, num_views=2, seed=11)
        H, W = 40, 48
        pos, edges, e2c = sc.pos.astype(np.float32), sc.edges, sc.edge2cluster
        E = edges.shape[0]
        ids = np.sort(np.random.default_rng(1).choice(2 * E, E, replace=False)).astype(np.int32)
        fp, fa = tape.run("dda_all", "dda_compute_fragments", lambda: R["dda"].dda_compute_fragments((H, W), t(pos), t(edges)),
                 dict(pos=pos, edges=edges, H=np.int32(H), W=np.int32(W)), lambda r: dict(frag_pix=r[0], frag_attrs=r[1]))
        tape.run("dda_ids", "dda_compute_fragments",
                 lambda: R["dda"].dda_compute_fragments((H, W), t(pos), t(edges), t(ids)),
                 dict(pos=pos, edges=edges, edge_ids=ids, H=np.int32(H), W=np.int32(W)),
                 lambda r: dict(frag_pix=r[0], frag_attrs=r[1]))
        target = tape.run("mask_dda", "cluster_mask_from_fragments",
                 lambda: R["rasterize"].cluster_mask_from_fragments((H, W), fp, fa, t(e2c), 40),
                 dict(frag_pix=_np(fp), frag_attrs=_np(fa), prim2cluster=e2c, H=np.int32(H), W=np.int32(W),
                      K=np.int32(40)), lambda r: dict(bitset=r))
        rast_dda = tape.run("depth_dda", "depth_test", lambda: R["rasterize"].depth_test(2, (H, W), fp, fa),
                 dict(frag_pix=_np(fp), frag_attrs=_np(fa), B=np.int32(2), H=np.int32(H), W=np.int32(W)),
                 lambda r: dict(rast=r))
        rng = np.random.default_rng(2)
        attr = rng.normal(size=(pos.shape[1], 3)).astype(np.float32)
        g_img = rng.normal(size=(2, H, W, 3)).astype(np.float32)

        def dda_interp():
            a = t(attr).clone().requires_grad_(True)
            img = R["dda"].dda_interpolate_attributes(rast_dda, a, t(edges))
            img.backward(t(g_img))
            return img, a.grad
        tape.run("dda_interp", "dda_interpolate_attributes", dda_interp,
                 dict(rast=_np(rast_dda), attr=attr, edges=edges, grad=g_img),
                 lambda r: dict(image=r[0], d_attr=r[1]))
        rgb = rng.uniform(size=(40, 3)).astype(np.float32)
        tape.run("popcount", "popcount_bitset", lambda: R["bitset_utils"].popcount_bitset(target),
                 dict(bitset=_np(target)), lambda r: dict(count=r))
        tape.run("rgb", "accumulate_bitset_rgb", lambda: R["bitset_utils"].accumulate_bitset_rgb(target, t(rgb)),
                 dict(bitset=_np(target), rgb=rgb), lambda r: dict(accum=r))
        # cards: one 4 x 1-quad strip per 4 strands over the same views
        cards = syn.make_cards(sc.strands, 4, 4, 1)
        cpos = syn.project(cards.verts, sc.mvp).astype(np.float32)
        tri, t2c = cards.tri, cards.tri2cluster
        tfp, tfa = tape.run("tri_frags", "compute_fragments", lambda: R["rasterize"].compute_fragments((H, W), t(cpos), t(tri)),
                 dict(pos=cpos, tri=tri, H=np.int32(H), W=np.int32(W)), lambda r: dict(frag_pix=r[0], frag_attrs=r[1]))
        rast = tape.run("rasterize", "rasterize", lambda: R["rasterize"].rasterize((H, W), t(cpos), t(tri)),
                 dict(pos=cpos, tri=tri, H=np.int32(H), W=np.int32(W)), lambda r: dict(rast=r))
        cattr = rng.normal(size=(cpos.shape[1], 3)).astype(np.float32)

        def tri_interp():
            a = t(cattr).clone().requires_grad_(True)
            img = R["rasterize"].interpolate_triangle_attributes(rast, a, t(tri))
            img.backward(t(g_img))
            return img, a.grad
        tape.run("tri_interp", "interpolate_triangle_attributes", tri_interp,
                 dict(rast=_np(rast), attr=cattr, tri=tri, grad=g_img), lambda r: dict(image=r[0], d_attr=r[1]))
        bits = tape.run("mask_tri", "cluster_mask_from_fragments",
                 lambda: R["rasterize"].cluster_mask_from_fragments((H, W), tfp, tfa, t(t2c), 40),
                 dict(frag_pix=_np(tfp), frag_attrs=_np(tfa), prim2cluster=t2c, H=np.int32(H), W=np.int32(W),
                      K=np.int32(40)), lambda r: dict(bitset=r))
        # antialias: the cards' bitset against the strands', loss with the XOR count, backward
        cedges, ce2t = O.build_edges_from_triangles(tri)
        ce2c = t2c[ce2t[:, 0]].astype(np.int32)
        tape.run("mark", "mark_discontinuity_edges",
                 lambda: R["antialias"].mark_discontinuity_edges((H, W), t(cpos), t(tri), t(cedges), t(ce2t)),
                 dict(pos=cpos, tri=tri, edges=cedges, edge2tri=ce2t, H=np.int32(H), W=np.int32(W)),
                 lambda r: dict(prim_ids=r[0], normals=r[1]))
        for kr, rho, xor in ((7.0, 0.5, True), (3.5, 1.0, False)):
            def aa_loss(kr=kr, rho=rho, xor=xor):
                p = t(cpos).clone().requires_grad_(True)
                loss = R["antialias"].antialiased_cluster_bitset_loss(bits, target, p, t(tri), t(cedges), t(ce2t),
                                                                       t(ce2c), kr, rho, xor)
                loss.backward()
                return loss, p.grad
            tape.run(f"aa_r{kr}_x{int(xor)}", "antialiased_cluster_bitset_loss", aa_loss,
                     dict(bitset=_np(bits), target=_np(target), pos=cpos, tri=tri, edges=cedges, edge2tri=ce2t,
                          edge2cluster=ce2c, kernel_radius=np.float32(kr), rho=np.float32(rho),
                          count_xor_error=np.int32(xor)),
                     lambda r: dict(loss=r[0].reshape(1), d_pos=r[1]))
        # curves: 16 strands x 20 points
        st = syn.make_strands(16, 20, seed=5).astype(np.float32)
        hs = (st + rng.normal(scale=0.01, size=st.shape)).astype(np.float32)
        ch = (st + rng.normal(scale=0.02, size=st.shape)).astype(np.float32)
        Q, _ = np.linalg.qr(rng.normal(size=(16, 20, 3, 3)))
        Rm = Q.astype(np.float32)
        tape.run("smooth", "smooth_strands", lambda: R["curve_utils"].smooth_strands(t(st), 0.1),
                 dict(strands=st, beta=np.float32(0.1)), lambda r: dict(out=r))
        tape.run("skin", "skinning", lambda: R["curve_utils"].skinning(t(st), t(hs), t(ch), t(Rm), 0.1),
                 dict(strands=st, handles=hs, canonical=ch, R=Rm, beta=np.float32(0.1)), lambda r: dict(out=r))
    finally:
        torch.Tensor.is_cuda = is_cuda
    np.savez_compressed(os.path.join(args.out, "dropin_tape.npz"), **tape.arrays)
    with open(os.path.join(args.out, "dropin_tape.json"), "w") as f:
        json.dump({"cases": tape.cases}, f, indent=1)
    print(f"{len(tape.cases)} op invocations, {sum(len(c['calls']) for c in tape.cases)} _core calls, "
          f"{len(tape.arrays)} arrays")


if __name__ == "__main__":
    main()
