"""Batched per-cluster card fitting: every cluster of a model is one view of one batch.

The reference fits cards cluster by cluster (``3_fitting.py``: per cluster, a local
orthographic frame, the strands' target bitset, the card raster, the antialiased-bitset
gradient and a Laplacian-preconditioned step).  Here all clusters advance together: the
clusters are the views ``b`` of single launches --

* strands: vertices padded per cluster to ``(C, Vmax, 4)``; each cluster's own segments are
  selected by ``edge_ids = b * E + e``, so padding is never read;
* cards: ``(C, Vc, 4)`` with one shared grid topology;
* one iteration = target coverage (DDA), card raster, antialiased-bitset gradient, a
  gradient step on the card vertices and ``laplacian_steps`` Jacobi Laplacian steps.

Two ways to run an iteration:

* ``persistent`` (``s2c_fit_iteration``): one launch.  CTAs take (cluster, segment chunk)
  items from a queue, largest clusters first, rasterise their strand segments into a
  one-bit target plane in shared memory, and the CTA that completes a cluster's coverage
  runs the rest of that cluster's iteration in shared memory;
* the launch sequence over all clusters (fused DDA -> bitset, fused card raster into
  cluster planes, antialias backward from planes, the step, the Laplacian), eager or as a
  CUDA graph, on one or two streams.

``FitSchedule`` is the autotuner: on the first iterations it times the persistent launch
over its parameters -- segments per coverage chunk (the segment-bin size), threads per CTA,
CTAs per SM, and threads per antialias fragment (one thread, or a warp over the window
rows) -- and the launch sequences, keeps the fastest, and caches the choice in a JSON file
keyed by the problem's shape class.  ``plain_iteration`` runs the same work as one call
sequence per cluster, the per-call path this batching replaces.
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import dataclass
from typing import Dict, List, Optional

import numpy as np
import torch

from . import _core, _lib
from .dda import dda_cluster_bitset
from .deform import CardLaplacian
from .mesh import build_edges_from_triangles
from .rasterize import rasterize_fused


@dataclass
class ClusterBatch:
    """Host description of C clusters in their local frames (clip space, w = 1)."""
    strand_pos: np.ndarray      # (C, Vmax, 4) float32, padded
    strand_edges: np.ndarray    # (E, 2) int32, shared (strand polylines of the largest cluster)
    edge_ids: np.ndarray        # (P,) int32, b * E + e of each cluster's own segments
    card_pos: np.ndarray        # (C, Vc, 4) float32
    card_tri: np.ndarray        # (Tc, 3) int32, shared
    card_edges: np.ndarray      # (Ec, 2) int32, shared
    card_e2t: np.ndarray        # (Ec, 2) int32
    quad_edges: np.ndarray      # (Qe, 2) int32, local to one card
    H: int
    W: int


def synthetic_clusters(num_clusters=256, verts=64, min_strands=20, max_strands=2000, quads_along=32,
                       quads_across=4, H=512, W=128, seed=0) -> ClusterBatch:
    """Clusters of log-uniform size in [min_strands, max_strands] (seed 0), each framed by
    its own orthographic camera onto (W, H) = (128, 512), one 32 x 4-quad card each."""
    from . import synthetic as syn
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(min_strands), np.log(max_strands), size=num_clusters)).astype(np.int64)
    nmax = int(counts.max())
    Vmax = nmax * verts
    strand_pos = np.zeros((num_clusters, Vmax, 4), np.float32)
    strand_pos[..., 3] = 1.0
    E_one = verts - 1
    edges = syn.strand_edges(nmax, verts)
    edge_ids: List[np.ndarray] = []
    faces, _, he, we = syn.grid_strip(quads_across + 1, quads_along + 1)
    nv = (quads_across + 1) * (quads_along + 1)
    card_pos = np.zeros((num_clusters, nv, 4), np.float32)
    for c in range(num_clusters):
        st = syn.make_strands(int(counts[c]), verts, seed=seed + 1 + c)
        lo, hi = st.reshape(-1, 3).min(0), st.reshape(-1, 3).max(0)
        ctr, half = (lo + hi) / 2, np.maximum((hi - lo) / 2, 1e-6) * 1.15
        loc = (st.reshape(-1, 3) - ctr) / half                         # local frame in [-1/1.15, 1/1.15]
        strand_pos[c, :loc.shape[0], :3] = loc.astype(np.float32)
        strand_pos[c, :loc.shape[0], 2] *= 0.5
        edge_ids.append((c * edges.shape[0] + np.arange(int(counts[c]) * E_one)).astype(np.int32))
        cards = syn.make_cards(st, int(counts[c]), quads_along, quads_across)
        cp = (cards.verts - ctr) / half
        card_pos[c, :, :3] = cp.astype(np.float32)
        card_pos[c, :, 2] *= 0.5
        card_pos[c, :, 3] = 1.0
    ce, ce2t = build_edges_from_triangles(faces.astype(np.int32))
    return ClusterBatch(strand_pos, edges, np.concatenate(edge_ids), card_pos, faces.astype(np.int32), ce, ce2t,
                        np.concatenate([he, we], 0).astype(np.int32), H, W)


class BatchedClusterFit:
    """Device state of a batched fit; ``step()`` runs one iteration for every cluster."""

    def __init__(self, batch: ClusterBatch, device="cuda", lr: float = 0.25, lam: float = 0.5,
                 laplacian_steps: int = 10, kernel_radius: float = 7.0, rho: float = 1.0):
        dev = torch.device(device)
        self.batch = batch
        self.C = batch.card_pos.shape[0]
        self.H, self.W = batch.H, batch.W
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
        self.spos, self.sedges, self.edge_ids = t(batch.strand_pos), t(batch.strand_edges), t(batch.edge_ids)
        self.se2c = torch.zeros(batch.strand_edges.shape[0], dtype=torch.int32, device=dev)
        self.cpos = t(batch.card_pos)
        self.ctri, self.cedges, self.ce2t = t(batch.card_tri), t(batch.card_edges), t(batch.card_e2t)
        self.ct2c = torch.zeros(batch.card_tri.shape[0], dtype=torch.int32, device=dev)
        self.ce2c = torch.zeros(batch.card_edges.shape[0], dtype=torch.int32, device=dev)
        C, H, W = self.C, self.H, self.W
        L = _lib.lib()
        self.target = torch.empty((C, H, W, 1), dtype=torch.int32, device=dev)
        self.bits = torch.empty((C, H, W, 1), dtype=torch.int32, device=dev)
        self.rast = None
        self.d_pos = torch.zeros_like(self.cpos)
        self.xyz = torch.empty((C * self.cpos.shape[1], 3), dtype=torch.float32, device=dev)
        self.ws_dda = torch.empty(L.s2c_dda_cluster_bitset_workspace_size(self.edge_ids.shape[0], C, H, W, 1),
                                  dtype=torch.uint8, device=dev)
        self.ws_tri = torch.empty(L.s2c_rasterize_fused_workspace_size(C, H, W, self.ctri.shape[0]),
                                  dtype=torch.uint8, device=dev)
        aa_need = L.s2c_antialiased_cluster_bitset_grad_planes_workspace_size(C, self.cpos.shape[1],
                                                                                self.cedges.shape[0])
        self.ws_aa = torch.empty(aa_need, dtype=torch.uint8, device=dev)
        self.pplanes = torch.empty((C, 32, H, (W + 31) // 32), dtype=torch.int32, device=dev)
        self.tplanes = torch.empty_like(self.pplanes)
        self.lap = CardLaplacian(self.cpos.shape[1], batch.quad_edges, dev)
        self.lr, self.lam, self.nlap = float(lr), float(lam), int(laplacian_steps)
        self.kr, self.rho = float(kernel_radius), float(rho)
        self.side = torch.cuda.Stream(device=dev)
        self.graph = None
        self.mode = "eager"
        # the persistent launch: per-cluster segment ranges of edge_ids (grouped by cluster)
        E = batch.strand_edges.shape[0]
        owner = batch.edge_ids.astype(np.int64) // max(E, 1)
        if owner.size and np.any(np.diff(owner) < 0):
            raise ValueError("BatchedClusterFit: edge_ids must be grouped by cluster (b * E + e, b non-decreasing).")
        self.seg_counts = np.bincount(owner, minlength=C).astype(np.int64)[:C]
        self.coff = t(np.concatenate([[0], np.cumsum(self.seg_counts)]).astype(np.int32))
        self.ws_fit = torch.empty(L.s2c_fit_workspace_size(C, H, W), dtype=torch.uint8, device=dev)
        # the persistent launch reads strand vertices packed: cluster c's used vertices (up to
        # the largest index its segments reference) at rows voff[c] .. voff[c + 1]
        used = np.zeros(C, np.int64)
        if batch.edge_ids.size:
            mine = owner < C
            seg_max = batch.strand_edges[batch.edge_ids[mine] % max(E, 1)].max(1).astype(np.int64) + 1
            np.maximum.at(used, owner[mine], seg_max)
        used = np.minimum(used, batch.strand_pos.shape[1])
        self.voff_h = np.concatenate([[0], np.cumsum(used)]).astype(np.int64)
        if self.voff_h[-1] >= 2 ** 31:
            raise ValueError("BatchedClusterFit: more than 2^31 - 1 packed strand vertices.")
        self.voff = t(self.voff_h.astype(np.int32))
        self.spos_packed_h = np.concatenate([batch.strand_pos[c, :used[c]] for c in range(C)]) if C else \
            np.zeros((0, 4), np.float32)
        self.spos_packed = t(self.spos_packed_h)
        self.step_scale = float(np.float32(2.0 * self.lr / max(H, W)))
        self.params = dict(chunk=8192, threads=256, ctas_per_sm=2, aa_warp=0)
        self._items: Dict[int, tuple] = {}

    # -- the five parts of an iteration --
    def _coverage(self):
        dda_cluster_bitset((self.H, self.W), self.spos, self.sedges, self.se2c, 1, edge_ids=self.edge_ids,
                           out=self.target, workspace=self.ws_dda)

    def _raster(self):
        # the cards straight into cluster planes, the layout the gradient reads
        _core.rasterize_fused_planes(self.cpos, self.ctri, self.ct2c, 1, self.H, self.W, planes=self.pplanes,
                                     ws=self.ws_tri)

    def _update(self):
        self.d_pos.zero_()
        _core.bitset_to_planes(self.target, self.tplanes)
        _core.antialiased_cluster_bitset_grad_planes(self.pplanes, self.tplanes, (self.C, self.H, self.W, 1),
                                                     self.cpos, self.ctri, self.cedges, self.ce2t, self.ce2c, self.kr,
                                                     self.rho, d_pos=self.d_pos, ws=self.ws_aa)
        # gradient step on x, y (each cluster's largest move lr pixels), then Laplacian smoothing
        g = self.d_pos[..., :2]
        scale = (2.0 * self.lr / max(self.H, self.W)) / g.abs().amax(dim=(1, 2), keepdim=True).clamp_min(1e-30)
        self.cpos[..., :2].sub_(g * scale)
        self.xyz.copy_(self.cpos[..., :3].reshape(-1, 3))
        self.lap(self.xyz, self.lam, self.nlap, out=self.xyz)
        self.cpos[..., :3].copy_(self.xyz.view(self.C, -1, 3))

    # -- the persistent launch --
    def items(self, chunk: int):
        """(cluster, chunk) work items, largest clusters first, and chunks per cluster."""
        if chunk not in self._items:
            n = np.maximum(1, -(-self.seg_counts // chunk)).astype(np.int32)
            order = np.argsort(-self.seg_counts, kind="stable")
            it = np.array([(c, k) for c in order for k in range(int(n[c]))], np.int32).reshape(-1, 2)
            dev = self.cpos.device
            self._items[chunk] = (torch.from_numpy(it).to(dev), torch.from_numpy(n).to(dev), int(it.shape[0]))
        return self._items[chunk]

    def persistent_step(self, params: Optional[dict] = None):
        """One iteration for every cluster in one launch (``s2c_fit_iteration``)."""
        p = dict(self.params, **(params or {}))
        items, nch, n_items = self.items(int(p["chunk"]))
        lap = self.lap
        _lib.call("s2c_fit_iteration", self.C, self.H, self.W, 0, _lib.ptr(self.spos_packed), _lib.ptr(self.voff),
                  self.sedges.shape[0], _lib.ptr(self.sedges), _lib.ptr(self.edge_ids), _lib.ptr(self.coff),
                  self.cpos.shape[1], _lib.ptr(self.cpos), self.ctri.shape[0], _lib.ptr(self.ctri),
                  self.cedges.shape[0], _lib.ptr(self.cedges), _lib.ptr(self.ce2t), _lib.ptr(lap.offsets),
                  _lib.ptr(lap.adj), lap.num_adj, _lib.ptr(items), n_items, int(p["chunk"]), _lib.ptr(nch),
                  self.step_scale, self.lam, self.nlap, self.kr, self.rho, int(p["threads"]), int(p["ctas_per_sm"]),
                  int(p["aa_warp"]), _lib.ptr(self.ws_fit), self.ws_fit.numel(), _lib.stream_of(self.cpos))

    def shape_key(self) -> str:
        """Shape class of the problem for the tuning cache: frame, card, cluster count and the
        (log2-bucketed) total and largest cluster segment counts, and the GPU's SM count."""
        tot = int(self.seg_counts.sum())
        mx = int(self.seg_counts.max()) if self.seg_counts.size else 0
        sms = torch.cuda.get_device_properties(self.cpos.device).multi_processor_count
        return (f"C{self.C}_H{self.H}_W{self.W}_Vc{self.cpos.shape[1]}_Ec{self.cedges.shape[0]}_"
                f"seg2^{int(math.log2(max(tot, 1)))}_max2^{int(math.log2(max(mx, 1)))}_sm{sms}")

    def eager_step(self, two_streams: bool = False):
        if two_streams:
            cur = torch.cuda.current_stream()
            self.side.wait_stream(cur)
            with torch.cuda.stream(self.side):
                self._coverage()
            self._raster()
            cur.wait_stream(self.side)
        else:
            self._coverage()
            self._raster()
        self._update()

    def capture(self, two_streams: bool = False, persistent: bool = False):
        """Capture one iteration in a CUDA graph (after a warm-up on the side stream)."""
        body = self.persistent_step if persistent else (lambda: self.eager_step(two_streams))
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            body()
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            body()
        self.graph = g
        return g

    def step(self):
        if self.mode.startswith("graph") or self.mode == "persistent_graph":
            self.graph.replay()
        elif self.mode == "persistent":
            self.persistent_step()
        else:
            self.eager_step(self.mode == "eager2")

    def plain_iteration(self):
        """The same iteration as C independent per-cluster call sequences."""
        for c in range(self.C):
            sl = slice(c, c + 1)
            ids = self._plain_ids[c]
            dda_cluster_bitset((self.H, self.W), self.spos[sl], self.sedges, self.se2c, 1, edge_ids=ids,
                               out=self.target[sl])
            rasterize_fused((self.H, self.W), self.cpos[sl], self.ctri, self.ct2c, 1, want_rast=False,
                            bitset=self.bits[sl])
            d = _core.antialiased_cluster_bitset_grad(self.bits[sl], self.target[sl], self.cpos[sl].contiguous(),
                                                      self.ctri, self.cedges, self.ce2t, self.ce2c, self.kr, self.rho)
            p = self.cpos[c]
            g = d[0, :, :2]
            p[:, :2].sub_(g * ((2.0 * self.lr / max(self.H, self.W)) / g.abs().amax().clamp_min(1e-30)))
            xyz = p[:, :3].contiguous()
            self.lap(xyz, self.lam, self.nlap, out=xyz)
            p[:, :3].copy_(xyz)

    def prepare_plain(self):
        E = self.batch.strand_edges.shape[0]
        ids = self.batch.edge_ids
        b = ids // E
        self._plain_ids = [torch.from_numpy((ids[b == c] - c * E).astype(np.int32)).to(self.spos.device)
                           for c in range(self.C)]


def default_tuning_cache() -> str:
    return os.environ.get("S2C_TUNING_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "strns2cards_gb300", "fit_tuning.json"))


class FitSchedule:
    """Autotuner of ``BatchedClusterFit.step``.

    Candidates: the persistent launch over ``SPACE`` (segments per coverage chunk, threads
    per CTA, CTAs per SM, one thread or one warp per antialias fragment) and, with
    ``launch_sequences``, the launch sequence eager / eager on two streams / as a graph / as
    a two-stream graph.  Each is timed over ``trials`` iterations (CUDA events, one warm-up
    iteration first); the card positions are restored afterwards.  The fastest is applied
    (the persistent one then replayed from a CUDA graph) and stored in the JSON cache under
    ``fit.shape_key()``; a later schedule for the same shape class reads it instead of
    searching (``search=True`` searches regardless).  ``self.table`` lists every candidate
    with its time (ms per iteration)."""

    SPACE = dict(chunk=(2048, 4096, 8192, 16384, 32768), threads=(256, 512), ctas_per_sm=(1, 2, 4), aa_warp=(0, 1))

    def __init__(self, fit: BatchedClusterFit, trials: int = 3, cache: Optional[str] = None, search: bool = False,
                 launch_sequences: bool = True):
        self.fit = fit
        self.key = fit.shape_key()
        self.cache = default_tuning_cache() if cache is None else cache
        self.table: List[dict] = []
        self.from_cache = False
        stored = None if search else self._load().get(self.key)
        snap = fit.cpos.clone()
        if stored:
            self.table = stored["table"]
            best = stored["best"]
            self.from_cache = True
        else:
            best = self._search(trials, launch_sequences)
        self._apply(best)            # (a graph capture runs one warm-up iteration)
        fit.cpos.copy_(snap)
        self.best = best["mode"]
        self.best_params = best.get("params")
        self.results = {r["name"]: r["ms"] for r in self.table}
        if not stored:
            self._save(best)

    def _time(self, body, trials):
        body()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(trials):
            body()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / trials

    def _search(self, trials, launch_sequences):
        fit = self.fit
        best = None
        keys = list(self.SPACE)
        for combo in _product([self.SPACE[k] for k in keys]):
            params = dict(zip(keys, combo))
            ms = self._time(lambda: fit.persistent_step(params), trials)
            name = "persistent " + " ".join(f"{k}={v}" for k, v in params.items())
            self.table.append({"name": name, "mode": "persistent", "params": params, "ms": ms})
            if best is None or ms < best["ms"]:
                best = {"mode": "persistent", "params": params, "ms": ms}
        if launch_sequences:
            for mode in ("eager", "eager2", "graph", "graph2"):
                if mode.startswith("graph"):
                    fit.capture(two_streams=mode == "graph2")
                    body = fit.graph.replay
                else:
                    body = (lambda m=mode: fit.eager_step(m == "eager2"))
                ms = self._time(body, trials)
                self.table.append({"name": mode, "mode": mode, "ms": ms})
                if ms < best["ms"]:
                    best = {"mode": mode, "ms": ms}
        return best

    def _apply(self, best):
        fit = self.fit
        mode = best["mode"]
        if mode == "persistent":
            fit.params = dict(best["params"])
            fit.capture(persistent=True)
            fit.mode = "persistent_graph"
        elif mode.startswith("graph"):
            fit.capture(two_streams=mode == "graph2")
            fit.mode = mode
        else:
            fit.mode = mode

    def _load(self) -> dict:
        try:
            with open(self.cache) as f:
                return json.load(f)
        except (OSError, ValueError):
            return {}

    def _save(self, best):
        try:
            data = self._load()
            data[self.key] = {"best": best, "table": self.table}
            os.makedirs(os.path.dirname(self.cache) or ".", exist_ok=True)
            tmp = self.cache + ".tmp"
            with open(tmp, "w") as f:
                json.dump(data, f, indent=1)
            os.replace(tmp, self.cache)
        except OSError:
            pass   # an unwritable cache only costs a search next time


def _product(lists):
    if not lists:
        yield ()
        return
    for x in lists[0]:
        for rest in _product(lists[1:]):
            yield (x,) + rest
