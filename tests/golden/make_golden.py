"""Generate golden vectors by running the reference's own CUDA kernels.

Run on a GPU host after ``oracle/build_ref.sh`` has produced ``oracle/_ref/*.cubin``:

    python tests/golden/make_golden.py --out tests/golden            # committed fixtures
    python tests/golden/make_golden.py --out DIR --battery           # large cases, not committed

Every fixture holds its own inputs (seeded, generated by ``strns2cards_gb300.synthetic``
or written out below) together with the reference outputs, so the CPU oracle can be
checked against them on any host without a GPU.  Fragment lists from the reference come
out in a nondeterministic order (``rasterize.cu:315-324``), so they are stored sorted.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.refkern import RefKernels  # noqa: E402
from strns2cards_gb300 import synthetic as syn  # noqa: E402
from oracle.oracle import build_edges_from_triangles  # noqa: E402


def sort_frags(pix: np.ndarray, attrs: np.ndarray):
    """Sort (F,3) int + (F,4) float fragments by (batch, prim id, h, w)."""
    if pix.shape[0] == 0:
        return pix, attrs
    key = np.lexsort((pix[:, 2], pix[:, 1], attrs[:, 3], pix[:, 0]))
    return pix[key], attrs[key]


def t(a, dtype=None):
    x = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        x = x.to(dtype)
    return x.cuda()


def n(x):
    return x.detach().cpu().numpy()


def perspective_pos(points: np.ndarray, B: int, seed: int) -> np.ndarray:
    """Clip positions under simple perspective cameras (w varies per vertex)."""
    rng = np.random.default_rng(seed)
    p = points.reshape(-1, 3).astype(np.float64)
    c = 0.5 * (p.min(0) + p.max(0))
    ext = (p.max(0) - p.min(0)).max()
    out = []
    for b in range(B):
        q = (p - c) / ext
        ang = rng.uniform(-0.6, 0.6)
        R = np.array([[np.cos(ang), 0, np.sin(ang)], [0, 1, 0], [-np.sin(ang), 0, np.cos(ang)]])
        q = q @ R.T
        w = 1.2 + 0.8 * q[:, 2]
        x = 1.3 * q[:, 0]
        y = 1.3 * q[:, 1]
        z = 0.9 * q[:, 2] * w
        out.append(np.stack([x, y, z, w], 1))
    return syn._quantise(np.stack(out)).astype(np.float32)


def edge_case_segments():
    """Hand-made segments in pixel space of a 16x24 (H x W) image, returned in clip space."""
    H, W = 16, 24
    segs = []

    def px(x, y, z=0.0, w=1.0):
        # pixel -> clip: x = 0.5*(xn+1)*W, y = 0.5*(1-yn)*H
        xn = 2.0 * x / W - 1.0
        yn = 1.0 - 2.0 * y / H
        return [xn * w, yn * w, z * w, w]

    segs += [(px(2.0, 3.5), px(20.0, 3.5)),          # horizontal through pixel centres
             (px(2.0, 5.0), px(20.0, 5.0)),          # horizontal on a pixel boundary
             (px(6.5, 1.0), px(6.5, 14.0)),          # vertical through centres
             (px(8.0, 1.0), px(8.0, 14.0)),          # vertical on a boundary
             (px(1.0, 1.0), px(13.0, 13.0)),         # 45 deg through corners
             (px(13.0, 13.0), px(1.0, 1.0)),         # reversed
             (px(3.3, 7.7), px(3.3, 7.7)),           # zero length
             (px(-5.0, 4.2), px(10.0, 9.1)),         # starts off-screen left
             (px(15.0, -3.0), px(18.0, 12.0)),       # starts above
             (px(10.0, 8.0), px(40.0, 11.0)),        # leaves on the right
             (px(-8.0, -8.0), px(-2.0, -1.0)),       # fully off-screen
             (px(2.0, 10.0, 0.5), px(22.0, 12.0, 1.5)),   # z leaves [-1,1] halfway
             (px(2.0, 12.0, 1.5), px(22.0, 14.0, 1.2)),   # z out of range
             (px(4.25, 2.0, 0.0, 0.5), px(19.75, 9.0, 0.3, 2.0)),  # perspective w
             (px(4.0, 2.0, 0.0, -1.0), px(19.0, 9.0, 0.0, 1.0)),   # negative w at one end
             (px(5.0, 5.0), [0.3, 0.2, 0.0, 0.0]),   # w = 0 (infinite)
             ([float("nan"), 0.0, 0.0, 1.0], px(9.0, 9.0)),  # NaN
             (px(0.0, 0.0), px(24.0, 16.0)),         # corner to corner
             (px(23.9, 0.2), px(0.1, 15.8)),         # anti-diagonal
             (px(7.2, 4.6), px(7.9, 4.9)),           # inside one pixel
             (px(11.5, 2.0), px(12.5, 14.0)),        # steep
             (px(1.0, 6.5), px(23.0, 7.5)),          # shallow
             (px(0.5, 15.5), px(0.5, 15.5 - 1e-3)),  # tiny vertical at the border
             (px(24.0, 3.0), px(24.0, 9.0)),         # vertical on the right edge x = W
             (px(3.0, 16.0), px(20.0, 16.0)),        # horizontal on the bottom edge y = H
             (px(2.0, 2.0), px(22.0, 13.0)),
             (px(5.5, 0.5), px(17.5, 12.5)),         # slope 1 through centres
             ]
    pos = np.array([v for s in segs for v in s], dtype=np.float32)[None]
    edges = np.arange(pos.shape[1], dtype=np.int32).reshape(-1, 2)
    return H, W, pos, edges


def dda_case(rk, H, W, pos, edges, e2c, K, edge_ids=None):
    pos_t, edges_t = t(pos), t(edges)
    ids_t = None if edge_ids is None else t(edge_ids)
    (fp, fa), (counts, slopes, spans, prefix, raw_pix, raw_attrs) = rk.dda_compute_fragments(H, W, pos_t, edges_t, ids_t)
    fp_n, fa_n = sort_frags(n(fp), n(fa))
    out = dict(H=H, W=W, pos=pos, edges=edges, K=K,
               span_counts=n(counts), span_slopes=n(slopes), span_spans=n(spans),
               raw_pix=n(raw_pix), raw_attrs=n(raw_attrs),
               frag_pix=fp_n, frag_attrs=fa_n)
    if edge_ids is not None:
        out["edge_ids"] = edge_ids
    if e2c is not None and fp.shape[0] > 0:
        out["edge2cluster"] = e2c
        out["bitset"] = n(rk.cluster_mask_from_fragments(H, W, fp, fa, t(e2c), K))
    return out


def tri_case(rk, H, W, pos, tri, t2c, K):
    pos_t, tri_t = t(pos), t(tri)
    (fp, fa), (rects, counts) = rk.compute_fragments(H, W, pos_t, tri_t)
    B = pos.shape[0]
    rast = rk.depth_test(B, H, W, fp, fa)
    fp_n, fa_n = sort_frags(n(fp), n(fa))
    out = dict(H=H, W=W, pos=pos, tri=tri, K=K, rects=n(rects), rect_counts=n(counts),
               frag_pix=fp_n, frag_attrs=fa_n, rast=n(rast))
    if t2c is not None and fp.shape[0] > 0:
        out["tri2cluster"] = t2c
        out["bitset"] = n(rk.cluster_mask_from_fragments(H, W, fp, fa, t(t2c), K))
    return out, (fp, fa, rast)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--battery", action="store_true")
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    rk = RefKernels()
    save = lambda name, d: np.savez_compressed(os.path.join(args.out, name), **d)  # noqa: E731

    if not args.battery:
        # A. strands, three views (two orthographic, one perspective), non-square image
        sc = syn.strand_scene(192, 24, per_cluster=8, num_views=2, seed=3)
        pos = np.concatenate([sc.pos, perspective_pos(sc.strands, 1, seed=4)], 0)
        save("dda_strands.npz", dda_case(rk, 96, 128, pos, sc.edges, sc.edge2cluster, 64))
        # B. hand-made edge cases, plus a repeated / partial edge_ids list
        H, W, p, e = edge_case_segments()
        save("dda_edgecases.npz", dda_case(rk, H, W, p, e, np.arange(e.shape[0], dtype=np.int32) % 40, 40))
        ids = np.array([3, 3, 0, 17, 25, 8, 26, 1], dtype=np.int32)
        save("dda_edge_ids.npz", dda_case(rk, H, W, p, e, np.arange(e.shape[0], dtype=np.int32) % 40, 40, ids))
        # C. cards of the same scene, three views
        cards = syn.make_cards(sc.strands, 8, 8, 2)
        cpos = np.concatenate([syn.project(cards.verts, sc.mvp), perspective_pos(cards.verts, 1, seed=4)], 0)
        tc, (fp, fa, rast) = tri_case(rk, 96, 128, cpos, cards.tri, cards.tri2cluster, 64)
        save("tri_cards.npz", tc)
        # C'. random triangles under perspective, including large and degenerate ones
        rng = np.random.default_rng(11)
        rv = rng.uniform(-1.3, 1.3, size=(2, 150, 4)).astype(np.float32)
        rv[..., 3] = rng.uniform(0.4, 1.6, size=(2, 150)).astype(np.float32)
        rv[..., 2] *= rv[..., 3] * 0.8
        rt = rng.integers(0, 150, size=(60, 3)).astype(np.int32)
        rt[5] = [7, 7, 9]  # degenerate
        tr, _ = tri_case(rk, 64, 80, syn._quantise(rv), rt, None, 1)
        save("tri_random.npz", tr)
        # D. antialiased bitset backward: card bitset vs strand target
        tgt = dda_case(rk, 96, 128, syn.project(sc.strands, sc.mvp).astype(np.float32),
                       sc.edges, sc.edge2cluster, 64)["bitset"]
        cpos2 = syn.project(cards.verts, sc.mvp)
        (fp2, fa2), _ = rk.compute_fragments(96, 128, t(cpos2), t(cards.tri))
        bits = n(rk.cluster_mask_from_fragments(96, 128, fp2, fa2, t(cards.tri2cluster), 64))
        edges_c, e2t = build_edges_from_triangles(cards.tri)
        e2cl = cards.tri2cluster[e2t[:, 0]].astype(np.int32)
        raw_ids, ids_c, normals = rk.mark_discontinuity_edges(96, 128, t(cpos2), t(cards.tri), t(edges_c), t(e2t))
        (sp, sa), _ = rk.dda_compute_fragments(96, 128, t(cpos2), t(edges_c), ids_c)
        aa = dict(H=96, W=128, pos=cpos2, tri=cards.tri, edges=edges_c, edge2tri=e2t, edge2cluster=e2cl,
                  bitset=bits, target=tgt, raw_prim_ids=n(raw_ids), normals=n(normals),
                  sil_frag_pix=sort_frags(n(sp), n(sa))[0], sil_frag_attrs=sort_frags(n(sp), n(sa))[1])
        for tag, kr, rho in (("r7", 7.0, 0.5), ("r3", 3.5, 1.0)):
            aa["d_pos_" + tag] = n(rk.backward_antialiased(sp, sa, t(bits), t(tgt), t(cpos2), t(edges_c), normals,
                                                           t(e2cl), kr, rho))
        save("antialias.npz", aa)
        # E. attribute interpolation (triangles and lines), forward and backward
        g = torch.Generator().manual_seed(0)
        V = cpos.shape[1]
        attr = torch.randn((V, 3), generator=g).numpy().astype(np.float32)
        grad = torch.randn(rast.shape[:3] + (3,), generator=g).numpy().astype(np.float32)
        img = n(rk.interpolate(rast, t(attr), t(cards.tri)))
        d_attr = n(rk.interpolate_backward(rast, t(grad), t(cards.tri), V))
        (lp, la), _ = rk.dda_compute_fragments(96, 128, t(pos), t(sc.edges))
        rast_l = rk.depth_test(pos.shape[0], 96, 128, lp, la)
        Vl = pos.shape[1]
        attr_l = torch.randn((Vl, 2), generator=g).numpy().astype(np.float32)
        grad_l = torch.randn(tuple(rast_l.shape[:3]) + (2,), generator=g).numpy().astype(np.float32)
        save("interp.npz", dict(rast=n(rast), tri=cards.tri, attr=attr, image=img, grad=grad, d_attr=d_attr,
                                rast_dda=n(rast_l), edges=sc.edges, attr_dda=attr_l,
                                image_dda=n(rk.dda_interpolate(rast_l, t(attr_l), t(sc.edges))),
                                grad_dda=grad_l,
                                d_attr_dda=n(rk.dda_interpolate_backward(rast_l, t(grad_l), t(sc.edges), Vl))))
        # F. strand smoothing and skinning
        st = syn.make_strands(16, 40, seed=5)
        st_t = t(st)
        d = torch.linalg.norm(st_t[:, 1:] - st_t[:, :-1], dim=2)
        arc = torch.cat([torch.zeros((16, 1), device="cuda"), torch.cumsum(d, 1)], 1).contiguous()
        rng = np.random.default_rng(6)
        hs = (st + rng.normal(0, 0.01, st.shape)).astype(np.float32)
        ch = (st + rng.normal(0, 0.05, st.shape)).astype(np.float32)
        A = rng.normal(size=(16, 40, 3, 3))
        Q, _ = np.linalg.qr(A)
        R = Q.astype(np.float32)
        save("curves.npz", dict(strands=st, arclength=n(arc), beta=np.float32(0.12),
                                smoothed=n(rk.smooth_strands(st_t, arc, 0.12)),
                                handles=hs, canonical=ch, R=R,
                                skinned=n(rk.skinning(st_t, arc, t(hs), t(ch), t(R), 0.12))))
        # G. popcount / rgb accumulation
        rb = rng.integers(-2 ** 31, 2 ** 31 - 1, size=(2, 8, 12, 3), dtype=np.int64).astype(np.int32)
        rb[0, :3] = 0
        rgb = rng.uniform(0, 1, size=(96, 3)).astype(np.float32)
        save("bitset_utils.npz", dict(bitset=rb, rgb=rgb, popcount=n(rk.popcount(t(rb))),
                                      accum=n(rk.accumulate_rgb(t(rb), t(rgb)))))
        print("golden fixtures written to", args.out)
        return

    # ---- battery: larger cases for pinning the FP32 arithmetic, plus full-size checksums
    drop = ("raw_attrs", "raw_pix")
    sc = syn.strand_scene(1024, 32, per_cluster=16, num_views=6, seed=0)
    d = dda_case(rk, 256, 256, sc.pos, sc.edges, sc.edge2cluster, 64)
    save("bat_dda_cfg1.npz", {k: v for k, v in d.items() if k not in drop})
    pp = perspective_pos(sc.strands, 2, seed=9)
    d = dda_case(rk, 256, 320, pp, sc.edges, sc.edge2cluster, 64)
    save("bat_dda_persp.npz", {k: v for k, v in d.items() if k not in drop})
    cards = syn.make_cards(sc.strands, 16, 8, 2)
    cpos = syn.project(cards.verts, sc.mvp)
    tc, _ = tri_case(rk, 256, 256, cpos, cards.tri, cards.tri2cluster, 64)
    save("bat_tri_cfg1.npz", tc)
    tc, _ = tri_case(rk, 200, 240, perspective_pos(cards.verts, 2, seed=10), cards.tri, cards.tri2cluster, 64)
    save("bat_tri_persp.npz", tc)
    # full-size single view: checksums only
    sums = {}
    full = syn.strand_scene(50_000, 100, per_cluster=25, num_views=1, seed=0)
    (fp, fa), _ = rk.dda_compute_fragments(1024, 1024, t(full.pos), t(full.edges))
    bits = rk.cluster_mask_from_fragments(1024, 1024, fp, fa, t(full.edge2cluster), 2048)
    sums["dda_full"] = dict(num_frags=int(fp.shape[0]), bitset_sha256=sha(n(bits)),
                            popcount=int(n(rk.popcount(bits)).sum()), shape=list(bits.shape),
                            input_sha256=sha(full.pos) + ":" + sha(full.edges))
    del fp, fa, bits
    fc = syn.make_cards(full.strands, 25, 16, 4)
    fcpos = syn.project(fc.verts, full.mvp)
    (fp, fa), _ = rk.compute_fragments(1024, 1024, t(fcpos), t(fc.tri))
    rast = rk.depth_test(1, 1024, 1024, fp, fa)
    bits = rk.cluster_mask_from_fragments(1024, 1024, fp, fa, t(fc.tri2cluster), 2048)
    r = n(rast)
    sums["tri_full"] = dict(num_frags=int(fp.shape[0]), bitset_sha256=sha(n(bits)),
                            triangle_id_sha256=sha(r[..., 3].copy()), covered=int((r[..., 3] > 0).sum()),
                            input_sha256=sha(fcpos) + ":" + sha(fc.tri))
    with open(os.path.join(args.out, "fullsize_ref.json"), "w") as f:
        json.dump(sums, f, indent=1)
    print(json.dumps(sums, indent=1))


if __name__ == "__main__":
    main()
