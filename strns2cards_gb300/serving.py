"""Continuous-batching server for strands-to-cards fitting jobs.

A job is one model: its strands (clip space of the job's view), its card mesh and a
number of fitting iterations of the full-size single-model pipeline -- card raster
(cluster bitset), antialias forward (XOR loss) and backward, per-card IoU, a gradient
step on the card vertices.  The iteration runs in cluster-plane layout (the raster writes
planes, the loss, gradient and IoU read them).  The server keeps every admitted job's
state resident on the device (card positions, the target's planes, workspaces) and runs
each job on its own CUDA
stream; in every scheduling round it issues one iteration of every active job, so the
jobs' kernels overlap on the GPU.  Requests that arrive while others run wait in a queue
and are admitted, oldest first, as soon as the HBM budget has room for their footprint;
a finished job's memory is released before the next admission.

The scheduling thread never waits for the GPU or for host preparation: an admitted job's
preparation (pinned copies of its inputs, the card edge topology, the target's DDA and
cluster planes) runs on a worker thread, on the job's stream, and the job joins the
rounds when it is ready; per-iteration losses stay on the device; a finished job's
results are copied into pinned host memory asynchronously and collected when its event
has completed.

``serve(requests, budget_bytes)`` replays a timed request stream (arrival offsets in
seconds) and returns per-job latency (completion - arrival) and results;
``serve_serial`` runs the same jobs one after another with the plain per-call path.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import torch

from . import _core, _lib
from .dda import dda_cluster_bitset
from .mesh import build_edges_from_triangles
from .rasterize import rasterize_fused


@dataclass
class JobSpec:
    """Host payload of one request."""
    strand_pos: np.ndarray     # (1, N*V, 4) float32 clip positions
    strand_edges: np.ndarray   # (E, 2) int32
    strand_e2c: np.ndarray     # (E,) int32
    card_pos: np.ndarray       # (1, Vc, 4) float32
    card_tri: np.ndarray       # (T, 3) int32
    card_t2c: np.ndarray       # (T,) int32
    res: int
    clusters: int
    iterations: int = 50
    lr: float = 0.25          # largest vertex move per iteration, in pixels
    arrival: float = 0.0       # seconds after the start of the stream
    name: str = ""

    def footprint(self) -> int:
        """Device bytes the job holds while admitted (inputs, bitsets, planes, workspaces)."""
        S = (self.clusters + 31) // 32
        bits = self.res * self.res * S * 4
        Vc, T = self.card_pos.shape[1], self.card_tri.shape[0]
        E = self.strand_edges.shape[0]
        cards = Vc * 16 * 3 + T * 16 + 3 * T * 8 + 3 * T * 4
        return 3 * bits + 8 * self.res * self.res + 2 * cards + self.strand_pos.nbytes + E * 60 + (64 << 20)


def synthetic_job(n_strands: int, verts: int, res: int, clusters: int, seed: int, iterations: int = 50,
                  arrival: float = 0.0) -> JobSpec:
    """A job of the stream: strands of the generator, one 16 x 4-quad card per cluster."""
    from . import synthetic as syn
    strands = syn.make_strands(n_strands, verts, seed=seed)
    mvp = syn.ortho_cameras(strands, margin=0.3, num_views=1)
    pos = syn.project(strands.reshape(-1, 3), mvp)
    edges = syn.strand_edges(n_strands, verts)
    K = min(clusters, n_strands)
    e2c = (np.arange(edges.shape[0]) // (verts - 1) * K // n_strands).astype(np.int32)
    cards = syn.make_cards(strands, 0, 16, 4, num_cards=K)
    cpos = syn.project(cards.verts, mvp)
    return JobSpec(pos, edges, e2c, cpos, cards.tri, cards.tri2cluster.astype(np.int32), res, clusters,
                   iterations, arrival=arrival, name=f"{n_strands}x{verts}@{res}/K{clusters}")


def step_towards(pos: torch.Tensor, d_pos: torch.Tensor, lr: float, res: int):
    """Gradient step on the clip-space x, y of the vertices, normalised so that the largest
    move is ``lr`` pixels (2 / res NDC units per pixel); no host synchronisation."""
    g = d_pos[..., :2]
    scale = (2.0 * lr / res) / g.abs().amax().clamp_min(1e-30)
    pos[..., :2].sub_(g * scale)


@dataclass
class JobResult:
    name: str
    arrival: float
    admitted: float = 0.0
    finished: float = 0.0
    card_pos: Optional[np.ndarray] = None
    loss: List[int] = field(default_factory=list)
    iou_inter: Optional[np.ndarray] = None          # per-card counts after the last iteration
    iou_union: Optional[np.ndarray] = None
    iou_first_inter: Optional[np.ndarray] = None    # ... and of the first iteration
    iou_first_union: Optional[np.ndarray] = None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


class _Active:
    """Device state of an admitted job.  ``prepare()`` (any thread) uploads the inputs and
    builds the target's planes on the job's stream; ``iterate()`` enqueues one iteration;
    ``start_finish()`` enqueues the copies of the results into pinned host memory and
    ``collect()`` reads them once ``finished()``."""

    def __init__(self, spec: JobSpec, dev, stream):
        self.spec = spec
        self.dev = dev
        self.stream = stream
        self.done_iters = 0
        self.ready = None    # Future of prepare() when prepared on a worker thread

    def prepare(self):
        spec, dev, stream = self.spec, self.dev, self.stream
        H = W = spec.res
        S = (spec.clusters + 31) // 32
        L = _lib.lib()
        with torch.cuda.stream(stream):
            t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().to(dev, non_blocking=True)  # noqa
            spos, sedges, se2c = t(spec.strand_pos), t(spec.strand_edges), t(spec.strand_e2c)
            self.cpos = t(spec.card_pos)
            self.tri, self.t2c = t(spec.card_tri), t(spec.card_t2c)
            edges, e2t = build_edges_from_triangles(spec.card_tri)
            self.edges, self.e2t = t(edges), t(e2t)
            self.e2c = t(spec.card_t2c[e2t[:, 0]].astype(np.int32))
            target = dda_cluster_bitset((H, W), spos, sedges, se2c, spec.clusters)
            del spos, sedges, se2c
            # the target's cluster planes stay resident for the whole job, with the rectangle
            # of each plane's set bits; the prediction's planes start empty and each
            # iteration clears only the rectangles the previous one could have written
            self.shape = (1, H, W, S)
            self.tplanes = _core.bitset_to_planes(target)
            del target
            self.trects = _core.planes_bounds(self.tplanes, self.shape)
            self.pplanes = torch.zeros_like(self.tplanes)
            self.prects = torch.tensor([H, 0, (W + 31) // 32, 0], dtype=torch.int32, device=dev).repeat(1, 32 * S, 1)
            self.ws_tri = torch.empty(L.s2c_rasterize_fused_workspace_size(1, H, W, self.tri.shape[0]),
                                      dtype=torch.uint8, device=dev)
            self.ws_aa = torch.empty(L.s2c_antialiased_cluster_bitset_grad_planes_workspace_size(
                1, self.cpos.shape[1], self.edges.shape[0]), dtype=torch.uint8, device=dev)
            self.d_pos = torch.zeros_like(self.cpos)
            self.losses = torch.zeros(max(spec.iterations, 1), dtype=torch.int64, device=dev)
            self.iou_first = None
            self.iou = None
        return self

    def iterate(self):
        spec = self.spec
        with torch.cuda.stream(self.stream):
            # the iteration in cluster-plane layout (the target's planes were built at admission):
            # clear the last prediction's rectangles, raster onto the planes (new rectangles),
            # per-card counts and the XOR loss in one pass over the rectangles, the gradient
            _core.planes_clear_rects(self.pplanes, self.prects, self.shape)
            _core.rasterize_fused_planes_onto(self.cpos, self.tri, self.t2c, spec.clusters, spec.res, spec.res,
                                              self.pplanes, rects=self.prects, ws=self.ws_tri)
            inter, uni, xor = _core.cluster_iou_counts_planes_rects(self.pplanes, self.tplanes, self.prects,
                                                                    self.trects, self.shape, spec.clusters)
            self.losses[self.done_iters:self.done_iters + 1].copy_(xor)
            self.d_pos.zero_()
            _core.antialiased_cluster_bitset_grad_planes(self.pplanes, self.tplanes, self.shape, self.cpos, self.tri,
                                                         self.edges, self.e2t, self.e2c, 7.0, 0.5, d_pos=self.d_pos,
                                                         ws=self.ws_aa)
            self.iou = (inter, uni)
            if self.done_iters == 0:
                self.iou_first = self.iou
            step_towards(self.cpos, self.d_pos, spec.lr, spec.res)
        self.done_iters += 1

    def start_finish(self):
        """Asynchronous copies of the results into pinned host memory, then an event."""
        with torch.cuda.stream(self.stream):
            src = {"card_pos": self.cpos, "loss": self.losses[:self.done_iters]}
            if self.iou is not None:
                src.update(iou_inter=self.iou[0], iou_union=self.iou[1], iou_first_inter=self.iou_first[0],
                           iou_first_union=self.iou_first[1])
            self.host = {k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True) for k, v in src.items()}
            for k, v in src.items():
                self.host[k].copy_(v, non_blocking=True)
            self.event = torch.cuda.Event()
            self.event.record(self.stream)

    def finished(self) -> bool:
        return self.event.query()

    def collect(self, res: "JobResult"):
        h = self.host
        res.card_pos = h["card_pos"].numpy()
        res.loss = [int(x) for x in h["loss"].tolist()]
        if "iou_inter" in h:
            res.iou_inter, res.iou_union = h["iou_inter"].numpy(), h["iou_union"].numpy()
            res.iou_first_inter, res.iou_first_union = h["iou_first_inter"].numpy(), h["iou_first_union"].numpy()

    def finish(self, res: "JobResult"):
        self.start_finish()
        self.event.synchronize()
        self.collect(res)


def serve(requests: List[JobSpec], budget_bytes: int, device="cuda", max_active: int = 32,
          realtime: bool = True, prep_workers: int = 2) -> List[JobResult]:
    """Continuous batching over a timed request stream; returns results in request order."""
    from concurrent.futures import ThreadPoolExecutor
    dev = torch.device(device)
    order = sorted(range(len(requests)), key=lambda i: requests[i].arrival)
    results = [JobResult(r.name, r.arrival) for r in requests]
    pending: List[int] = []
    preparing = {}
    active = {}
    finishing = {}
    used = 0
    streams = [torch.cuda.Stream(device=dev) for _ in range(max_active)]
    free_streams = list(range(max_active))
    t0 = time.perf_counter()
    nxt = 0
    with ThreadPoolExecutor(max_workers=max(prep_workers, 1)) as pool:
        while nxt < len(order) or pending or preparing or active or finishing:
            now = time.perf_counter() - t0
            while nxt < len(order) and (requests[order[nxt]].arrival <= now or not realtime):
                pending.append(order[nxt])
                nxt += 1
            # admit, oldest first, while the budget and the stream pool allow; the job is
            # prepared on a worker thread and joins the rounds when ready
            while pending and free_streams:
                i = pending[0]
                need = requests[i].footprint()
                if used + need > budget_bytes and (active or preparing or finishing):
                    break
                pending.pop(0)
                used += need
                sid = free_streams.pop()
                results[i].admitted = time.perf_counter() - t0
                job = _Active(requests[i], dev, streams[sid])
                job.ready = pool.submit(job.prepare)
                preparing[i] = (job, sid, need)
            for i, (job, sid, need) in list(preparing.items()):
                if job.ready.done():
                    job.ready.result()          # re-raises a preparation error
                    active[i] = preparing.pop(i)
            # one iteration of every active job, each on its own stream
            for i, (job, sid, need) in list(active.items()):
                job.iterate()
                if job.done_iters >= job.spec.iterations:
                    job.start_finish()
                    finishing[i] = active.pop(i)
            # collect the finished jobs whose copies have landed; release their memory
            for i, (job, sid, need) in list(finishing.items()):
                if job.finished():
                    job.collect(results[i])
                    results[i].finished = time.perf_counter() - t0
                    del finishing[i]
                    used -= need
                    free_streams.append(sid)
                    del job
            if not active:
                # nothing to issue this round: wait a little for arrivals, preparations, copies
                wait = 0.0005
                if nxt < len(order) and not (pending or preparing or finishing):
                    wait = max(0.0, min(0.005, requests[order[nxt]].arrival - (time.perf_counter() - t0)))
                time.sleep(wait)
    torch.cuda.synchronize()
    return results


def serve_serial(requests: List[JobSpec], device="cuda", realtime: bool = True) -> List[JobResult]:
    """The same jobs one at a time (plain calls on the default stream), in arrival order."""
    dev = torch.device(device)
    order = sorted(range(len(requests)), key=lambda i: requests[i].arrival)
    results = [JobResult(r.name, r.arrival) for r in requests]
    t0 = time.perf_counter()
    stream = torch.cuda.current_stream(dev)
    for i in order:
        now = time.perf_counter() - t0
        if realtime and requests[i].arrival > now:
            time.sleep(requests[i].arrival - now)
        results[i].admitted = time.perf_counter() - t0
        job = _Active(requests[i], dev, stream).prepare()
        for _ in range(requests[i].iterations):
            job.iterate()
        job.finish(results[i])
        results[i].finished = time.perf_counter() - t0
        del job
    return results


def serve_serial_dropin(requests: List[JobSpec], device="cuda") -> List[JobResult]:
    """The same jobs one at a time, back to back, through the drop-in ops as the reference's
    fitting loop calls them (3_fitting.py:254-261, 381-406): the target by
    dda_compute_fragments + cluster_mask_from_fragments, then per iteration compute_fragments
    + cluster_mask_from_fragments, antialiased_cluster_bitset_loss (the XOR count) and its
    gradient, the per-card IoU counts and the step.  The plain per-call baseline of the
    served form."""
    from .antialias import antialiased_cluster_bitset_loss
    from .bitset_utils import cluster_iou
    from .dda import dda_compute_fragments
    from .rasterize import cluster_mask_from_fragments, compute_fragments
    dev = torch.device(device)
    results = [JobResult(r.name, r.arrival) for r in requests]
    t0 = time.perf_counter()
    for i, spec in enumerate(requests):
        results[i].admitted = time.perf_counter() - t0
        H = W = spec.res
        K = spec.clusters
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
        fp, fa = dda_compute_fragments((H, W), t(spec.strand_pos), t(spec.strand_edges))
        target = cluster_mask_from_fragments((H, W), fp, fa, t(spec.strand_e2c), K)
        del fp, fa
        cpos, tri, t2c = t(spec.card_pos), t(spec.card_tri), t(spec.card_t2c)
        edges_h, e2t_h = build_edges_from_triangles(spec.card_tri)
        edges, e2t = t(edges_h), t(e2t_h)
        e2c = t(spec.card_t2c[e2t_h[:, 0]].astype(np.int32))
        losses, iou = [], None
        for it in range(spec.iterations):
            fp, fa = compute_fragments((H, W), cpos, tri)
            bits = cluster_mask_from_fragments((H, W), fp, fa, t2c, K)
            p = cpos.detach().requires_grad_(True)
            loss = antialiased_cluster_bitset_loss(bits, target, p, tri, edges, e2t, e2c, 7.0, 0.5,
                                                   count_xor_error=True)
            loss.backward()
            iou = cluster_iou(bits, target, K)[1:]
            if it == 0:
                results[i].iou_first_inter, results[i].iou_first_union = (x.cpu().numpy() for x in iou)
            losses.append(loss.detach())
            with torch.no_grad():
                step_towards(cpos, p.grad, spec.lr, spec.res)
        res = results[i]
        res.card_pos = cpos.cpu().numpy()
        res.loss = [int(x) for x in torch.stack(losses).tolist()] if losses else []
        if iou is not None:
            res.iou_inter, res.iou_union = (x.cpu().numpy() for x in iou)
        res.finished = time.perf_counter() - t0
    return results


def poisson_stream(num_requests: int, rate: float = 20.0, seed: int = 1, scale: float = 1.0,
                   iterations: int = 50) -> List[JobSpec]:
    """Request stream: Poisson arrivals (rate per second, seed 1); strand count log-uniform in
    [5k, 200k] x ``scale``, vertices in {32, 64, 128}, resolution in {512, 1024, 2048},
    clusters in {256, 1024, 4096}."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=num_requests))
    out = []
    for k in range(num_requests):
        n = int(np.exp(rng.uniform(np.log(5_000), np.log(200_000))) * scale)
        v = int(rng.choice([32, 64, 128]))
        res = int(rng.choice([512, 1024, 2048]))
        K = int(rng.choice([256, 1024, 4096]))
        out.append(synthetic_job(max(n, 16), v, res, K, seed=1000 + k, iterations=iterations, arrival=float(t[k])))
    return out
