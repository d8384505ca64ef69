"""Benchmark: DDA line raster of strand segments into per-pixel cluster bitsets (Gseg/s).

Workload (one step): 50,000 synthetic strands x 100 vertices = 4.95M segments, one
orthographic 1024x1024 view, 2,048 clusters (k = strand_idx // 25) -> a 1024x1024x64-slot
int32 bitset (256 MiB), via the fused kernel path (s2c_dda_cluster_bitset).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

* value  = segments processed / device time of the steps (CUDA events on the launching
           stream; L2 flushed with a 256 MiB write between steps, outside the events).
* e2e    = the same metric through the public op with host buffers: each step copies the
           inputs from pinned host memory, runs the op and copies the bitset back.
* roofline: algorithmic bytes of the path (16 B/vertex + 12 B/segment read, 4 B/word
           bitset write) / device time, against the measured HBM copy bandwidth.
* --impl reference: the CPU oracle's fused DDA -> bitset (a restatement of the
           reference's dda.cu + cluster_mask kernels; the reference itself has no CPU
           path) on all host cores, same workload.
Under torchrun each rank rasterises its own view of the same model (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NUM_STRANDS, NUM_VERTS, PER_CLUSTER, RES, K = 50_000, 100, 25, 1024, 2048
# kernels one s2c_dda_cluster_bitset call launches: init, bin, scan (one CTA for <= 16,384
# tiles), scatter, tile raster, fixup
LAUNCHES_PER_STEP = 6
METRIC = "Gseg/s DDA+bitset"
WORKLOAD = (f"dda_cluster_bitset: {NUM_STRANDS}x{NUM_VERTS} synthetic strands "
            f"({NUM_STRANDS * (NUM_VERTS - 1)} segments) -> {RES}x{RES} view, {K} clusters "
            f"(int32 bitset {RES}x{RES}x{K // 32}, 256 MiB)")


def algorithmic_bytes(B, V, E, H, W, S):
    return 16 * B * V + 12 * B * E + 4 * B * H * W * S


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    p = os.path.join(ROOT, "profiles", "dda_cluster_bitset_50kx100_1024sq_k2048_traffic.json")
    if os.path.exists(p):
        try:
            return json.load(open(p)).get("bytes_per_step")
        except Exception:
            return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 20 ms during the timed region; the
    sampler has written its first sample before the region starts (it takes ~0.1 s to start)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < 3.0 and self.proc.poll() is None and os.path.getsize(self.path) == 0:
                time.sleep(0.01)
            # samples taken before the region are dropped in summary()
            self.skip = sum(1 for _ in open(self.path))
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        rows = []
        lines = open(self.path).readlines()
        # keep the pre-region sample(s) only when the region itself produced none
        if len(lines) > getattr(self, "skip", 0):
            lines = lines[getattr(self, "skip", 0):]
        for line in lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, fl in rows for i, f in enumerate(fl) if f.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def max_over_ranks(seconds: float, ws: int, device) -> float:
    """The slowest rank's time (all ranks get it); one rank: the value itself."""
    if ws <= 1:
        return seconds
    import torch
    import torch.distributed as dist
    t = torch.tensor([seconds], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, ws: int, seconds_max: float) -> float:
    """Units all ranks processed divided by the slowest rank's time (weak scaling)."""
    return units_per_rank * ws / seconds_max


def make_inputs(view):
    from strns2cards_gb300 import synthetic as syn
    sc = syn.strand_scene(NUM_STRANDS, NUM_VERTS, per_cluster=PER_CLUSTER, num_views=view + 1, seed=0)
    return np.ascontiguousarray(sc.pos[view:view + 1]), sc.edges, sc.edge2cluster


def cpu_oracle_rate(pos, edges, e2c, seconds=4.0):
    """Segments/s of the CPU oracle's fused DDA -> bitset on all host cores."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    O.dda_cluster_bitset(RES, RES, pos, edges, e2c, K)  # warm
    n, t0 = 0, time.perf_counter()
    while True:
        O.dda_cluster_bitset(RES, RES, pos, edges, e2c, K)
        n += 1
        dt = time.perf_counter() - t0
        if dt >= seconds:
            break
    return n * edges.shape[0] * pos.shape[0] / dt, threads, n


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    pos, edges, e2c = make_inputs(0)
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    for _ in range(args.warmup):
        O.dda_cluster_bitset(RES, RES, pos, edges, e2c, K)
    t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.dda_cluster_bitset(RES, RES, pos, edges, e2c, K)
        t.append(time.perf_counter() - t0)
    E = edges.shape[0]
    val = E * len(t) / sum(t) / 1e9
    line = {"metric": METRIC, "value": val, "unit": "Gseg/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(t) / len(t),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "host": "cpu", "sample": "full workload each step"},
            "cpu_baseline": {"value": val, "unit": "Gseg/s", "cores": threads, "kind": "port",
                             "sample": "the full 4.95M-segment workload per step"},
            "e2e": {"value": val, "unit": "Gseg/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.no_forms:
        line["reference_gpu"] = reference_gpu_numbers()
    print(json.dumps(line), flush=True)


def reference_gpu_numbers(reps=5):
    """The reference's own CUDA kernels (built unmodified from its sources into cubins by
    oracle/build_ref.sh) on this GPU, for the headline op and the fitting iteration's two
    main ops, called in the reference's op sequences; median ms of ``reps`` calls each.
    None when there is no GPU or the cubins were not built."""
    try:
        import torch
        if not torch.cuda.is_available():
            return None
        from oracle import refkern
        if not refkern.available():
            return None
    except Exception as e:  # pragma: no cover - reported, not fatal to the CPU arm
        return {"unavailable": str(e)}
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    rk = refkern.RefKernels()

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return float(np.median(ms))
    out = {}
    pos_h, edges_h, e2c_h = make_inputs(0)
    pos, edges, e2c = (torch.from_numpy(a).cuda() for a in (pos_h, edges_h, e2c_h))

    def dda_ref():
        (fp, fa), _ = rk.dda_compute_fragments(RES, RES, pos, edges)
        return rk.cluster_mask_from_fragments(RES, RES, fp, fa, e2c, K)
    ms = timed(dda_ref)
    out["dda_cluster_bitset"] = {"ms": ms, "Gseg_per_s": edges_h.shape[0] / ms / 1e6,
                                 "ops": "dda_compute_fragments + cluster_mask_from_fragments (reference kernels)"}
    strands = syn.make_strands(NUM_STRANDS, NUM_VERTS, seed=0)
    mvp = syn.ortho_cameras(strands, margin=0.3, num_views=1)
    cards = syn.make_cards(strands, 0, 16, 4, num_cards=2048)
    cpos = torch.from_numpy(syn.project(cards.verts, mvp)).cuda()
    tri, t2c = torch.from_numpy(cards.tri).cuda(), torch.from_numpy(cards.tri2cluster).cuda()

    def raster_ref():
        (fp, fa) = rk.compute_fragments(RES, RES, cpos, tri)[0]
        return rk.depth_test(1, RES, RES, fp, fa), rk.cluster_mask_from_fragments(RES, RES, fp, fa, t2c, K)
    ms = timed(raster_ref)
    out["card_raster"] = {"ms": ms, "Mtri_per_s": cards.tri.shape[0] / ms / 1e3,
                          "ops": "compute_fragments + depth_test + cluster_mask_from_fragments, 2,048 cards "
                                 "(262,144 triangles), 1024x1024, K=2048"}
    bits = raster_ref()[1]
    target = dda_ref()
    e_h, e2t_h = s2c.build_edges_from_triangles(cards.tri)
    ce2c = torch.from_numpy(cards.tri2cluster[e2t_h[:, 0]].astype(np.int32)).cuda()
    cedges, e2t = torch.from_numpy(e_h).cuda(), torch.from_numpy(e2t_h).cuda()
    ms = timed(lambda: rk.antialiased_loss_grad(bits, target, cpos, tri, cedges, e2t, ce2c, 7.0, 0.5))
    out["antialias_backward"] = {"ms": ms, "Medge_per_s": e_h.shape[0] / ms / 1e3,
                                 "ops": "mark_discontinuity_edges + compact + dda_compute_fragments + "
                                        "backward_antialiased_cluster_bitset, the cards against the strands' bitset"}
    out["gpu"] = torch.cuda.get_device_name(0)
    return out


def run_ours(args):
    import torch
    import torch.distributed as dist

    ws, rank, local = dist_env()
    if ws > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import _lib

    pos_h, edges_h, e2c_h = make_inputs(rank)
    B, V, _ = pos_h.shape
    E = edges_h.shape[0]
    S = K // 32
    pos = torch.from_numpy(pos_h).to(dev)
    edges = torch.from_numpy(edges_h).to(dev)
    e2c = torch.from_numpy(e2c_h).to(dev)
    out = torch.empty((B, RES, RES, S), dtype=torch.int32, device=dev)
    wsb = _lib.lib().s2c_dda_cluster_bitset_workspace_size(B * E, B, RES, RES, S)
    work = torch.empty(wsb, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        s2c.dda_cluster_bitset((RES, RES), pos, edges, e2c, K, out=out, workspace=work)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    n_ent, n_over = s2c._core.dda_cluster_bitset_stats(work)

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(i & 0xff)  # evict L2 (256 MiB write) outside the timed events
            evs[i][0].record(stream)
            step()
            evs[i][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    if ws > 1:
        dist.barrier()
    ms = [a.elapsed_time(b) for a, b in evs]
    dev_s = sum(ms) / 1e3
    t_max = max_over_ranks(dev_s, ws, dev)
    value = whole_job_rate(B * E * args.steps, ws, t_max) / 1e9

    # e2e through the public op with host buffers (pinned), copies inside the timed region.
    # Steps are pipelined on three streams: the inputs of step i+1 go up while step i runs
    # and the bitset of step i-1 comes back; every step copies its own inputs in and its
    # whole bitset out.  Device and host buffers are double-buffered, reuse ordered by events.
    pos_p = torch.from_numpy(pos_h).pin_memory()
    edges_p = torch.from_numpy(edges_h).pin_memory()
    e2c_p = torch.from_numpy(e2c_h).pin_memory()
    outs_p = [torch.empty(out.shape, dtype=torch.int32).pin_memory() for _ in range(2)]
    dins = [(torch.empty_like(pos), torch.empty_like(edges), torch.empty_like(e2c)) for _ in range(2)]
    douts = [out, torch.empty_like(out)]
    s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    e2e_steps = max(3, min(args.steps, 300))

    def e2e_run(k):
        ev_in = [torch.cuda.Event() for _ in range(k)]
        ev_op = [torch.cuda.Event() for _ in range(k)]
        ev_out = [torch.cuda.Event() for _ in range(k)]
        for i in range(k):
            pd, ed, cd = dins[i % 2]
            with torch.cuda.stream(s_in):
                if i >= 2:
                    s_in.wait_event(ev_op[i - 2])
                pd.copy_(pos_p, non_blocking=True)
                ed.copy_(edges_p, non_blocking=True)
                cd.copy_(e2c_p, non_blocking=True)
                ev_in[i].record(s_in)
            stream.wait_event(ev_in[i])
            if i >= 2:
                stream.wait_event(ev_out[i - 2])
            s2c.dda_cluster_bitset((RES, RES), pd, ed, cd, K, out=douts[i % 2], workspace=work)
            ev_op[i].record(stream)
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev_op[i])
                outs_p[i % 2].copy_(douts[i % 2], non_blocking=True)
                ev_out[i].record(s_out)
        stream.wait_stream(s_out)

    e2e_run(2)
    torch.cuda.synchronize()
    ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ea.record(stream)
    s_in.wait_stream(stream)
    e2e_run(e2e_steps)
    eb.record(stream)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(ea.elapsed_time(eb) / 1e3, ws, dev)
    e2e = whole_job_rate(B * E * e2e_steps, ws, e2e_s) / 1e9
    h2d = pos_h.nbytes + edges_h.nbytes + e2c_h.nbytes
    d2h = out.numel() * 4

    peak, peak_kind = load_peaks()
    alg = algorithmic_bytes(B, V, E, RES, RES, S)
    achieved = alg / (dev_s / args.steps) / 1e9
    traffic = load_traffic()
    line = None
    if rank == 0:
        cpu = None
        if ws == 1 and not args.no_cpu_baseline:
            rate, threads, n = cpu_oracle_rate(pos_h, edges_h, e2c_h)
            cpu = {"value": rate / 1e9, "unit": "Gseg/s", "cores": threads, "kind": "port",
                   "sample": f"the full workload, {n} repetitions (~4 s) of the CPU oracle's fused DDA->bitset"}
        clocks = clk.summary()
        line = {"metric": METRIC, "value": value, "unit": "Gseg/s", "n_gpus": ws, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "views_per_rank": B, "l2": "flushed between steps (256 MiB write)",
                           "parallelism": f"replicas x{ws} (one view per rank)", "bin_entries": n_ent,
                           "fallback_prims": n_over},
                "e2e": {"value": e2e, "unit": "Gseg/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "peak_kind": peak_kind,
                             "algorithmic_bytes_per_step": alg, "traffic": traffic,
                             "kernel": "s2c_dda_cluster_bitset (init, bin, tile scan, scatter, tile raster, fixup)"},
                "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": LAUNCHES_PER_STEP * args.steps,
                "wall_s": wall}
        if ws == 1 and not args.no_forms:
            # the chosen forms, after the headline's timed region: the batched fit of 256
            # uneven clusters against their per-cluster call sequence, and the continuous-
            # batching server on a short Poisson stream against serial plain calls
            del work, flush, dins, douts, outs_p
            torch.cuda.empty_cache()
            bt = batched_numbers(steps=20, plain_iters=2, trials=2)
            ms = bt.pop("schedule_ms")
            bt["candidates_timed"] = len(ms)
            bt["schedule_ms_fastest5"] = dict(sorted(ms.items(), key=lambda kv: kv[1])[:5])
            bt["schedule_ms_slowest"] = max(ms.values())
            line["batched"] = bt
            torch.cuda.empty_cache()
            line["serving"] = serving_numbers(args.serving_jobs)
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    return line


# ---------------------------------------------------------------------------------------
# Other rows of the path, each on its published configuration (``--workload NAME``).
# A workload gives host inputs, an untimed setup on the device copies, a step, the units
# one step processes and its algorithmic bytes; the harness below times it like the
# headline (CUDA events per step, 256 MiB L2 flush between steps, clocks sampled) and
# end to end (pinned host inputs copied in, result copied out, inside the timed region).
# ---------------------------------------------------------------------------------------
def _cards_scene(num_strands, num_verts, num_cards, quads_along, quads_across, res, seed=0):
    from strns2cards_gb300 import synthetic as syn
    strands = syn.make_strands(num_strands, num_verts, seed=seed)
    mvp = syn.ortho_cameras(strands, margin=0.3, num_views=1)
    cards = syn.make_cards(strands, 0, quads_along, quads_across, num_cards=num_cards)
    return strands, mvp, cards


def wl_tri_raster(list_path=False):
    """Card raster of the 50,000 x 100 strand model: 2,048 cards (16 x 4 quads; 174,080 V,
    262,144 T) -> rast (1, 1024, 1024, 4) and the cluster bitset (1, 1024, 1024, 64)."""
    import torch
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    _, mvp, cards = _cards_scene(50_000, 100, 2048, 16, 4, 1024)
    pos = syn.project(cards.verts, mvp)
    host = {"pos": pos, "tri": cards.tri, "t2c": cards.tri2cluster}
    V, T, H = pos.shape[1], cards.tri.shape[0], 1024

    def setup(d):
        from strns2cards_gb300 import _lib
        need = _lib.lib().s2c_rasterize_fused_workspace_size(1, H, H, T)
        return {"ws": torch.empty(need, dtype=torch.uint8, device=d["pos"].device),
                "rast": torch.empty((1, H, H, 4), dtype=torch.float32, device=d["pos"].device),
                "bits": torch.empty((1, H, H, 64), dtype=torch.int32, device=d["pos"].device)}

    def step(d, st):
        if list_path:
            fp, fa = s2c.compute_fragments((H, H), d["pos"], d["tri"])
            rast = s2c.depth_test(1, (H, H), fp, fa)
            bits = s2c.cluster_mask_from_fragments((H, H), fp, fa, d["t2c"], 2048)
            return rast, bits
        return s2c.rasterize_fused((H, H), d["pos"], d["tri"], d["t2c"], 2048, rast=st["rast"], bitset=st["bits"],
                                   workspace=st["ws"])
    how = ("compute_fragments + depth_test + cluster_mask_from_fragments (the reference's op sequence)"
           if list_path else "one fused pass (rasterize_fused)")
    return dict(name="tri_raster", host=host, setup=setup, step=step, units=T, unit="Mtri/s", scale=1e6,
                metric="card triangles rasterised per second (rast + cluster bitset)",
                alg_bytes=16 * V + 12 * T + 16 * H * H + 4 * H * H * 64, launches=None if list_path else 3,
                workload="2,048 cards (16x4 quads, 262,144 triangles) of the 50,000x100 strand model, 1024x1024, "
                         "K=2048: " + how)


def wl_antialias(list_path=False):
    """Antialias backward of the same cards against the strands' target bitset."""
    import torch
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    strands, mvp, cards = _cards_scene(50_000, 100, 2048, 16, 4, 1024)
    pos = syn.project(cards.verts, mvp)
    spos = syn.project(strands.reshape(-1, 3), mvp)
    sedges = syn.strand_edges(50_000, 100)
    se2c = (np.arange(sedges.shape[0]) * 2048 // sedges.shape[0]).astype(np.int32)
    edges, e2t = s2c.build_edges_from_triangles(cards.tri)
    e2c = cards.tri2cluster[e2t[:, 0]].astype(np.int32)
    host = {"pos": pos, "tri": cards.tri, "edges": edges, "e2t": e2t, "e2c": e2c}
    V, E, H = pos.shape[1], edges.shape[0], 1024

    def setup(d):
        dev = d["pos"].device
        tgt = s2c.dda_cluster_bitset((H, H), torch.from_numpy(spos).to(dev), torch.from_numpy(sedges).to(dev),
                                     torch.from_numpy(se2c).to(dev), 2048)
        fp, fa = s2c.compute_fragments((H, H), d["pos"], d["tri"])
        bits = s2c.cluster_mask_from_fragments((H, H), fp, fa, torch.from_numpy(cards.tri2cluster).to(dev), 2048)
        return {"tgt": tgt, "bits": bits}

    def step(d, st):
        return s2c.antialiased_cluster_bitset_grad(st["bits"], st["tgt"], d["pos"], d["tri"], d["edges"], d["e2t"],
                                                   d["e2c"], 7.0, 0.5, fused=not list_path)
    how = ("mark_discontinuity_edges + dda_compute_fragments + backward (the reference's op sequence)"
           if list_path else "one fused pass per (view, edge)")
    return dict(name="antialias", host=host, setup=setup, step=step, units=E, unit="Medge/s", scale=1e6,
                metric="card edges through the antialiased bitset-loss backward per second",
                alg_bytes=2 * 4 * H * H * 64 + 16 * V + 20 * E + 16 * V, launches=None if list_path else 2,
                workload="antialias backward (silhouette edges, edge DDA, 15x15 window, kernel_radius 7, rho 0.5) "
                         "of 2,048 cards (434k edges) against the 50,000x100 strands' bitset, 1024x1024, K=2048: "
                         + how)


def wl_antialias_2048():
    """The differentiation case at full size: antialias backward of 4,096 cards (16 x 4
    quads) of the 100,000 x 64 strand model against its strands' bitset, 2048x2048, K=4096
    (two 2 GiB bitsets); the gradient w.r.t. the card vertices (scalar upstream gradient:
    the loss has no image-gradient input)."""
    import torch
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    H, K = 2048, 4096
    strands, mvp, cards = _cards_scene(100_000, 64, 4096, 16, 4, H)
    pos = syn.project(cards.verts, mvp)
    spos = syn.project(strands.reshape(-1, 3), mvp)
    sedges = syn.strand_edges(100_000, 64)
    se2c = (np.arange(sedges.shape[0]) * K // sedges.shape[0]).astype(np.int32)
    edges, e2t = s2c.build_edges_from_triangles(cards.tri)
    e2c = cards.tri2cluster[e2t[:, 0]].astype(np.int32)
    host = {"pos": pos, "tri": cards.tri, "edges": edges, "e2t": e2t, "e2c": e2c}
    V, E = pos.shape[1], edges.shape[0]
    S = K // 32

    def setup(d):
        dev = d["pos"].device
        tgt = s2c.dda_cluster_bitset((H, H), torch.from_numpy(spos).to(dev), torch.from_numpy(sedges).to(dev),
                                     torch.from_numpy(se2c).to(dev), K)
        _, bits = s2c.rasterize_fused((H, H), d["pos"], d["tri"], torch.from_numpy(cards.tri2cluster).to(dev), K,
                                      want_rast=False)
        return {"tgt": tgt, "bits": bits}

    def step(d, st):
        return s2c.antialiased_cluster_bitset_grad(st["bits"], st["tgt"], d["pos"], d["tri"], d["edges"], d["e2t"],
                                                   d["e2c"], 7.0, 0.5)
    return dict(name="antialias_2048", host=host, setup=setup, step=step, units=E, unit="Medge/s", scale=1e6,
                metric="card edges through the antialiased bitset-loss backward per second",
                alg_bytes=2 * 4 * H * H * S + 16 * V + 20 * E + 16 * V, launches=None,
                workload="antialias backward of 4,096 cards (16x4 quads, %d edges) of the 100,000x64 strand "
                         "model against its strands' bitset, 2048x2048, K=4096: bitset planes + one fused pass "
                         "per (view, edge)" % E)


def _dda_scene_full():
    from strns2cards_gb300 import synthetic as syn
    sc = syn.strand_scene(NUM_STRANDS, NUM_VERTS, per_cluster=PER_CLUSTER, num_views=1, seed=0)
    return sc


def wl_dda_list():
    """The reference's op sequence for the strands' bitset (dda_compute_fragments, then
    cluster_mask_from_fragments), 50,000 x 100 strands, 1024x1024, K=2048."""
    import strns2cards_gb300 as s2c
    sc = _dda_scene_full()
    host = {"pos": sc.pos, "edges": sc.edges, "e2c": sc.edge2cluster}
    H = 1024

    def step(d, st):
        fp, fa = s2c.dda_compute_fragments((H, H), d["pos"], d["edges"])
        return s2c.cluster_mask_from_fragments((H, H), fp, fa, d["e2c"], 2048)
    E, V = sc.edges.shape[0], sc.pos.shape[1]
    return dict(name="dda_list", host=host, step=step, units=E, unit="Gseg/s", scale=1e9, dtype="i32",
                metric="Gseg/s DDA+bitset through the reference's op sequence (fragment list)",
                alg_bytes=16 * V + 12 * E + 4 * H * H * 64, launches=None,
                workload="dda_compute_fragments + cluster_mask_from_fragments of 50,000x100 strands (4.95M "
                         "segments), 1024x1024, K=2048: fragment list, order-preserving compaction, bit OR")


def _rast_scene_full():
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    _, mvp, cards = _cards_scene(50_000, 100, 2048, 16, 4, 1024)
    pos = syn.project(cards.verts, mvp)
    return pos, cards


def wl_interpolate():
    """Attribute interpolation forward + backward (upstream image gradient N(0,1), seed 0) over
    the rast of the 2,048 cards, 1024x1024, 3 channels."""
    import torch
    import strns2cards_gb300 as s2c
    pos, cards = _rast_scene_full()
    V, H, C = pos.shape[1], 1024, 3
    attr = np.random.default_rng(0).normal(size=(V, C)).astype(np.float32)
    grad = torch.randn((1, H, H, C), generator=torch.Generator().manual_seed(0)).numpy()
    host = {"pos": pos, "tri": cards.tri, "attr": attr, "grad": grad}

    def setup(d):
        return {"rast": s2c.rasterize((H, H), d["pos"], d["tri"])}

    def step(d, st):
        a = d["attr"].detach().requires_grad_(True)
        img = s2c.interpolate_triangle_attributes(st["rast"], a, d["tri"])
        img.backward(d["grad"])
        return img, a.grad
    return dict(name="interpolate", host=host, setup=setup, step=step, units=H * H, unit="Mpix/s", scale=1e6, graph=True,
                metric="pixels interpolated forward and backward per second (3 channels)",
                alg_bytes=2 * 16 * H * H + 4 * C * H * H * 2 + 12 * 2 * V * C, launches=None,
                workload="interpolate_triangle_attributes fwd + bwd (N(0,1) image gradient) of 3 channels over the "
                         "rast of 2,048 cards, 1024x1024")


def wl_dda_interpolate():
    """Line-attribute interpolation forward + backward over the strands' DDA rast (the
    fragment list's depth-resolved raster), 1024x1024, 3 channels."""
    import torch
    import strns2cards_gb300 as s2c
    sc = _dda_scene_full()
    V, H, C = sc.pos.shape[1], 1024, 3
    attr = np.random.default_rng(0).normal(size=(V, C)).astype(np.float32)
    grad = torch.randn((1, H, H, C), generator=torch.Generator().manual_seed(0)).numpy()
    host = {"pos": sc.pos, "edges": sc.edges, "attr": attr, "grad": grad}

    def setup(d):
        fp, fa = s2c.dda_compute_fragments((H, H), d["pos"], d["edges"])
        return {"rast": s2c.depth_test(1, (H, H), fp, fa)}

    def step(d, st):
        a = d["attr"].detach().requires_grad_(True)
        img = s2c.dda_interpolate_attributes(st["rast"], a, d["edges"])
        img.backward(d["grad"])
        return img, a.grad
    return dict(name="dda_interpolate", host=host, setup=setup, step=step, units=H * H, unit="Mpix/s", scale=1e6, graph=True,
                metric="pixels interpolated forward and backward per second (3 channels, line raster)",
                alg_bytes=2 * 16 * H * H + 4 * C * H * H * 2 + 12 * 2 * V * C, launches=None,
                workload="dda_interpolate_attributes fwd + bwd (N(0,1) image gradient) of 3 channels over the "
                         "depth-resolved DDA raster of 50,000x100 strands, 1024x1024")


def wl_bary_derivatives():
    """Barycentric derivatives d(b0, b1)/d(x, y) of the 2,048 cards' rast, 1024x1024."""
    import strns2cards_gb300 as s2c
    pos, cards = _rast_scene_full()
    H = 1024
    host = {"pos": pos, "tri": cards.tri}

    def setup(d):
        return {"rast": s2c.rasterize((H, H), d["pos"], d["tri"])}

    def step(d, st):
        return s2c.barycentric_derivatives(st["rast"], d["pos"], d["tri"])
    return dict(name="bary_derivatives", host=host, setup=setup, step=step, units=H * H, unit="Mpix/s", scale=1e6,
                metric="pixels of barycentric derivatives per second",
                alg_bytes=16 * H * H + 16 * H * H, launches=1,
                workload="barycentric_derivatives (rast + the triangles' clip corners -> d(b0,b1)/d(x,y)) of the "
                         "2,048 cards' rast, 1024x1024")


def wl_bitset_stats():
    """popcount_bitset and accumulate_bitset_rgb of the strands' cluster bitset (1024x1024, K=2048)."""
    import strns2cards_gb300 as s2c
    rng = np.random.default_rng(0)
    H, S = 1024, 64
    bits = rng.integers(0, 2 ** 31 - 1, size=(1, H, H, S), dtype=np.int64).astype(np.int32)
    bits &= (rng.random(bits.shape) < 0.05).astype(np.int32) * -1   # sparse, as hair bitsets are
    rgb = rng.random((32 * S, 3), dtype=np.float32)
    host = {"bits": bits, "rgb": rgb}

    def step(d, st):
        return s2c.popcount_bitset(d["bits"]), s2c.accumulate_bitset_rgb(d["bits"], d["rgb"])
    return dict(name="bitset_stats", host=host, step=step, units=2 * 4 * H * H * S, unit="GB/s", scale=1e9,
                metric="bitset bytes read per second (popcount + colour accumulation)",
                alg_bytes=2 * 4 * H * H * S + 4 * H * H + 12 * H * H, launches=2,
                workload="popcount_bitset + accumulate_bitset_rgb of an int32 bitset (1, 1024, 1024, 64), K=2048, "
                         "5 % of the words non-zero")


def wl_iteration():
    """One fit iteration of the 50,000 x 100 model in cluster-plane layout: the card raster
    onto the prediction's planes, per-card IoU counts and the XOR loss in one pass, the
    antialias backward.  Each plane is cleared and counted only inside its rectangle."""
    import torch
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import _core
    from strns2cards_gb300 import synthetic as syn
    strands, mvp, cards = _cards_scene(50_000, 100, 2048, 16, 4, 1024)
    pos = syn.project(cards.verts, mvp)
    spos = syn.project(strands.reshape(-1, 3), mvp)
    sedges = syn.strand_edges(50_000, 100)
    se2c = (np.arange(sedges.shape[0]) * 2048 // sedges.shape[0]).astype(np.int32)
    edges, e2t = s2c.build_edges_from_triangles(cards.tri)
    e2c = cards.tri2cluster[e2t[:, 0]].astype(np.int32)
    host = {"pos": pos, "tri": cards.tri, "t2c": cards.tri2cluster, "edges": edges, "e2t": e2t, "e2c": e2c}
    V, T, E, H = pos.shape[1], cards.tri.shape[0], edges.shape[0], 1024
    shape = (1, H, H, 64)

    def setup(d):
        dev = d["pos"].device
        tgt = s2c.dda_cluster_bitset((H, H), torch.from_numpy(spos).to(dev), torch.from_numpy(sedges).to(dev),
                                     torch.from_numpy(se2c).to(dev), 2048)
        from strns2cards_gb300 import _lib
        need = _lib.lib().s2c_rasterize_fused_workspace_size(1, H, H, T)
        tplanes = _core.bitset_to_planes(tgt)              # the target's planes and rectangles, once per fit
        trects = _core.planes_bounds(tplanes, shape)
        pplanes = torch.zeros_like(tplanes)
        ws = torch.empty(need, dtype=torch.uint8, device=dev)
        prects = _core.rasterize_fused_planes_onto(d["pos"], d["tri"], d["t2c"], 2048, H, H, pplanes, ws=ws)
        # algorithmic bytes: inputs, the rectangles' words (clear, raster, counts of both
        # planes), the antialias backward's
        def words(r):
            r = r.cpu().numpy().reshape(-1, 4).astype(np.int64)
            return int((np.maximum(r[:, 1] - r[:, 0], 0) * np.maximum(r[:, 3] - r[:, 2], 0)).sum())
        wp, wt = words(prects), words(trects)
        alg = (16 * V + 12 * T) + 4 * (2 * wp) + 4 * (wp + wt) + (2 * 4 * H * H * 64 + 16 * V + 20 * E + 16 * V)
        return {"tplanes": tplanes, "trects": trects, "pplanes": pplanes, "prects": prects, "ws": ws,
                "alg_bytes": alg,
                "config_extra": {"rectangle_words": {"prediction": wp, "target": wt, "all_planes": 2048 * H * H // 32}}}

    def step(d, st):
        _core.planes_clear_rects(st["pplanes"], st["prects"], shape)
        _core.rasterize_fused_planes_onto(d["pos"], d["tri"], d["t2c"], 2048, H, H, st["pplanes"], rects=st["prects"],
                                          ws=st["ws"])
        inter, uni, loss = _core.cluster_iou_counts_planes_rects(st["pplanes"], st["tplanes"], st["prects"],
                                                                 st["trects"], shape, 2048)
        d_pos = _core.antialiased_cluster_bitset_grad_planes(st["pplanes"], st["tplanes"], shape, d["pos"], d["tri"],
                                                             d["edges"], d["e2t"], d["e2c"], 7.0, 0.5)
        return (loss, d_pos, inter, uni)
    alg = (16 * V + 12 * T) + 4 * 2 * 4 * H * H * 64 + (2 * 4 * H * H * 64 + 16 * V + 20 * E + 16 * V)
    return dict(name="iteration", host=host, setup=setup, step=step, units=1, unit="iter/s", scale=1.0,
                metric="plain fit iterations per second", alg_bytes=alg, launches=None,
                workload="one fit iteration of 2,048 cards against the 50,000x100 strands' bitset, 1024x1024, "
                         "K=2048 in cluster-plane layout: fused raster onto the prediction's planes (each plane "
                         "cleared and counted inside its rectangle only), per-card IoU counts and XOR loss in one "
                         "pass, fused antialias backward (target planes and rectangles built once)")


def wl_cluster_iou():
    import torch
    import strns2cards_gb300 as s2c
    rng = np.random.default_rng(0)
    H, S = 1024, 64
    a = rng.integers(0, 2 ** 31 - 1, size=(1, H, H, S), dtype=np.int64).astype(np.int32)
    b = a ^ (rng.random(a.shape) < 0.05).astype(np.int32)
    host = {"a": a, "b": b}

    def step(d, st):
        return s2c.cluster_iou(d["a"], d["b"], 2048)[1:]
    return dict(name="cluster_iou", host=host, step=step, units=2 * 4 * H * H * S, unit="GB/s", scale=1e9,
                metric="per-card bitset IoU counts: bitset bytes read per second",
                alg_bytes=2 * 4 * H * H * S, launches=1,
                workload="per-card IoU counts of two int32 bitsets (1, 1024, 1024, 64), K=2048")


def _strand_batch(N, V, seed=0):
    from strns2cards_gb300 import synthetic as syn
    return syn.make_strands(N, V, seed=seed).astype(np.float32)


def wl_smooth_strands():
    import strns2cards_gb300 as s2c
    x = _strand_batch(100_000, 64)
    host = {"x": x}

    def step(d, st):
        return s2c.smooth_strands(d["x"], 0.05)
    n = x.shape[0] * x.shape[1]
    return dict(name="smooth_strands", host=host, step=step, units=n, unit="Mpts/s", scale=1e6,
                metric="strand points smoothed per second", alg_bytes=24 * n, launches=1,
                workload="smooth_strands of 100,000 x 64 strands, beta 0.05 (arclength computed in the kernel)")


def wl_skinning():
    import strns2cards_gb300 as s2c
    rng = np.random.default_rng(0)
    x = _strand_batch(100_000, 64)
    h = (x + rng.normal(scale=0.01, size=x.shape)).astype(np.float32)
    c = (x + rng.normal(scale=0.02, size=x.shape)).astype(np.float32)
    R = np.tile(np.eye(3, dtype=np.float32), (x.shape[0], x.shape[1], 1, 1))
    host = {"x": x, "h": h, "c": c, "R": R}

    def step(d, st):
        return s2c.skinning(d["x"], d["h"], d["c"], d["R"], 0.05)
    n = x.shape[0] * x.shape[1]
    return dict(name="skinning", host=host, step=step, units=n, unit="Mpts/s", scale=1e6,
                metric="strand points skinned per second", alg_bytes=(12 * 3 + 36 + 12) * n, launches=1,
                workload="skinning of 100,000 x 64 strands to per-point handle frames, beta 0.05")


def wl_lbs():
    """Linear blend skinning of 100,000 x 64 strand vertices to the 4 nearest of 69,632 guides
    (centre lines of 4,096 cards, 16 x 4 quads): forward + backward (dM and dx)."""
    import torch
    import strns2cards_gb300 as s2c
    strands, _, cards = _cards_scene(100_000, 64, 4096, 16, 4, 2048)
    x = strands.reshape(-1, 3).astype(np.float32)
    g = np.ascontiguousarray(cards.verts.reshape(-1, 5, 17, 3)[:, 2].reshape(-1, 3), dtype=np.float32)
    G = g.shape[0]
    rng = np.random.default_rng(0)
    M = (np.tile(np.eye(3, 4), (G, 1, 1)) + rng.normal(scale=0.05, size=(G, 3, 4))).astype(np.float32)
    gy = torch.randn((x.shape[0], 3), generator=torch.Generator().manual_seed(0)).numpy()
    host = {"x": x, "M": M, "gy": gy}

    def setup(d):
        return {"bind": s2c.LBSBinding(d["x"], torch.from_numpy(g).to(d["x"].device), 0.01)}

    def step(d, st):
        Mt = d["M"].requires_grad_(True)
        xt = d["x"].requires_grad_(True)
        y = s2c.lbs(xt, Mt, st["bind"])
        dx, dM = torch.autograd.grad(y, (xt, Mt), d["gy"])
        return y, dM, dx
    Nv = x.shape[0]
    fwd = 12 * Nv + 32 * Nv + 48 * G + 12 * Nv
    bwd = 12 * Nv + 32 * Nv + 12 * Nv + 48 * G + 16 * Nv + 12 * Nv + 16 * Nv   # dx pass + dM pass
    return dict(name="lbs", host=host, setup=setup, step=step, units=Nv, unit="Mverts/s", scale=1e6,
                metric="strand vertices through LBS forward + backward per second", alg_bytes=fwd + bwd, launches=3,
                workload="LBS of 100,000 x 64 strand vertices to 4 nearest of 69,632 guides (4,096 cards): "
                         "forward, backward dM (per-guide lists) and dx")


def wl_laplacian():
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    _, _, h, w = syn.grid_strip(5, 33)
    qe = np.concatenate([h, w], 0)
    nv, cards = 165, 4096
    p = np.random.default_rng(0).normal(size=(cards * nv, 3)).astype(np.float32)
    host = {"p": p}

    def setup(d):
        return {"lap": s2c.CardLaplacian(nv, qe, d["p"].device)}

    def step(d, st):
        return st["lap"](d["p"], 0.5, 10)
    return dict(name="laplacian", host=host, setup=setup, step=step, units=cards * nv * 10, unit="Mvert-steps/s",
                scale=1e6, metric="card vertex Jacobi steps per second", alg_bytes=24 * cards * nv, launches=1,
                workload="10 Jacobi Laplacian steps (lambda 0.5) on 4,096 cards of 32x4 quads (165 vertices each)")


def batched_numbers(steps, warmup=3, plain_iters=2, trials=3):
    """Batched cluster fit (256 clusters, log-uniform 20..2000 strands x 64 vertices, seed 0;
    local 128 x 512 frames, K = 1, one 32 x 4-quad card each): cluster-fit iterations per
    second of the autotuned schedule, the per-cluster call sequence timed beside it, and end
    to end with positions copied in from pinned host memory and cards copied out."""
    import torch
    from strns2cards_gb300.batched import BatchedClusterFit, FitSchedule, synthetic_clusters
    batch = synthetic_clusters()
    C = batch.card_pos.shape[0]
    fit = BatchedClusterFit(batch)
    sched = FitSchedule(fit, trials=trials, search=True)
    for _ in range(max(warmup, 3)):
        fit.step()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        a.record(stream)
        for _ in range(steps):
            fit.step()
        b.record(stream)
        torch.cuda.synchronize()
    t = a.elapsed_time(b) / 1e3
    value = C * steps / t
    # the per-cluster call sequence (the reference's way of fitting), a few iterations
    plain = BatchedClusterFit(batch)
    plain.prepare_plain()
    plain.plain_iteration()
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(plain_iters):
        plain.plain_iteration()
    b.record(stream)
    torch.cuda.synchronize()
    plain_rate = C * plain_iters / (a.elapsed_time(b) / 1e3)
    del plain
    # end to end: card and strand positions in from pinned host memory, cards out (the
    # strands as the applied schedule reads them: packed for the persistent launch)
    packed = fit.mode.startswith("persistent")
    sp = torch.from_numpy(fit.spos_packed_h if packed else batch.strand_pos).pin_memory()
    sp_dev = fit.spos_packed if packed else fit.spos
    cp = torch.from_numpy(batch.card_pos).pin_memory()
    out = torch.empty(cp.shape, dtype=torch.float32).pin_memory()
    # the schedule stays applied (its graph, or the eager sequence)

    def e2e_step():
        sp_dev.copy_(sp, non_blocking=True)
        fit.cpos.copy_(cp, non_blocking=True)
        fit.step()
        out.copy_(fit.cpos, non_blocking=True)
    e2e_step()
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(3):
        e2e_step()
    b.record(stream)
    torch.cuda.synchronize()
    e2e = C * 3 / (a.elapsed_time(b) / 1e3)
    return dict(clusters=C, value=value, unit="cluster-iter/s", ms_per_iteration=1e3 * t / steps, steps=steps,
                schedule=sched.best, schedule_params=sched.best_params, schedule_ms=sched.results,
                tuned_parameters=list(FitSchedule.SPACE),
                plain_per_cluster_calls=plain_rate, batched_over_plain=value / plain_rate, e2e=e2e,
                h2d_bytes_per_step=sp.nbytes + cp.nbytes, d2h_bytes_per_step=out.nbytes,
                strand_segments=int(batch.edge_ids.shape[0]), clocks=clk.summary())


def run_batched_fit(args):
    """Batched cluster fit on its own line (``--workload batched_fit``)."""
    r = batched_numbers(args.steps, args.warmup)
    C = r["clusters"]
    line = {"metric": "cluster-fit iterations per second (batched, autotuned schedule)", "value": r["value"],
            "unit": "cluster-iter/s", "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_step": r["ms_per_iteration"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{C} clusters (log-uniform 20..2000 strands x 64 verts, seed 0), 128x512 local "
                                   "frames, K=1, one 32x4-quad card each; iteration = fused DDA coverage + fused "
                                   "card raster + fused antialias backward + gradient step + 10 Laplacian steps",
                       "schedule": r["schedule"], "schedule_params": r["schedule_params"],
                       "schedule_ms": r["schedule_ms"], "tuned_parameters": r["tuned_parameters"],
                       "plain_per_cluster_calls": {"value": r["plain_per_cluster_calls"], "unit": "cluster-iter/s"},
                       "batched_over_plain": r["batched_over_plain"], "strand_segments": r["strand_segments"]},
            "e2e": {"value": r["e2e"], "unit": "cluster-iter/s", "h2d_bytes_per_step": r["h2d_bytes_per_step"],
                    "d2h_bytes_per_step": r["d2h_bytes_per_step"]},
            "roofline": None, "cpu_baseline": None, "clocks": r["clocks"], "gpu_launches": None}
    print(json.dumps(line), flush=True)


def serving_numbers(n_jobs):
    """Continuous-batching server on a Poisson request stream (20 req/s, seed 1) of fitting
    jobs (strands log-uniform 5k..200k, V in {32, 64, 128}, resolution in {512, 1024, 2048},
    K in {256, 1024, 4096}, 50 iterations each), HBM budget 150 GB; the same stream served
    one job at a time with plain calls is timed beside it."""
    import torch
    from strns2cards_gb300.serving import poisson_stream, serve, serve_serial, serve_serial_dropin
    n = max(n_jobs, 4)
    reqs = poisson_stream(n, rate=20.0, seed=1)
    warm = poisson_stream(2, rate=20.0, seed=2, scale=0.05, iterations=3)
    serve(warm, 150 << 30)
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        res = serve(reqs, 150 << 30)
        wall = time.perf_counter() - t0
    lat = np.array([r.latency for r in res])
    iters = sum(r.iterations for r in reqs)
    # capacity: the same jobs all waiting at the start (the GPU, not the stream, sets the rate)
    t0 = time.perf_counter()
    serve(reqs, 150 << 30, realtime=False)
    torch.cuda.synchronize()
    wall_c = time.perf_counter() - t0
    t0 = time.perf_counter()
    ser = serve_serial(reqs)
    wall_s = time.perf_counter() - t0
    lat_s = np.array([r.latency for r in ser])
    # the plain per-call path (the drop-in ops as the reference's fitting loop calls them),
    # one job at a time back to back, on the stream's first jobs
    m = min(n, 12)
    t0 = time.perf_counter()
    serve_serial_dropin(reqs[:m])
    torch.cuda.synchronize()
    wall_d = time.perf_counter() - t0
    iters_d = sum(r.iterations for r in reqs[:m])
    h2d = sum(r.strand_pos.nbytes + r.strand_edges.nbytes + r.strand_e2c.nbytes + r.card_pos.nbytes +
              r.card_tri.nbytes + r.card_t2c.nbytes for r in reqs)
    return dict(jobs=n, jobs_per_s=n / wall, iterations_per_s=iters / wall, wall_s=wall,
                latency_p50_s=float(np.percentile(lat, 50)), latency_p99_s=float(np.percentile(lat, 99)),
                serial_plain={"jobs_per_s": n / wall_s, "iterations_per_s": iters / wall_s,
                              "latency_p50_s": float(np.percentile(lat_s, 50)),
                              "latency_p99_s": float(np.percentile(lat_s, 99))},
                served_over_serial_iterations=(iters / wall) / (iters / wall_s),
                dropin_serial={"jobs": m, "iterations_per_s": iters_d / wall_d,
                               "ops": "compute_fragments + cluster_mask_from_fragments, "
                                      "antialiased_cluster_bitset_loss (XOR count) + backward, cluster_iou, step"},
                served_over_dropin_iterations=(iters / wall) / (iters_d / wall_d),
                capacity={"jobs_per_s": n / wall_c, "iterations_per_s": iters / wall_c,
                          "over_dropin_iterations": (iters / wall_c) / (iters_d / wall_d)},
                h2d_bytes_per_job=h2d // n, d2h_bytes_per_job=sum(r.card_pos.nbytes for r in reqs) // n,
                clocks=clk.summary())


def run_serving(args):
    """The served form on its own line (``--workload serving``)."""
    r = serving_numbers(args.steps)
    n = r["jobs"]
    line = {"metric": "served fitting jobs per second (continuous batching)", "value": r["jobs_per_s"],
            "unit": "jobs/s", "n_gpus": 1, "steps": n, "warmup": 2, "ms_per_step": 1e3 * r["wall_s"] / n,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{n} Poisson requests (20/s, seed 1): strands log-uniform 5k..200k, V in "
                                   "{32,64,128}, res in {512,1024,2048}, K in {256,1024,4096}, 50 iterations of the "
                                   "full-size pipeline each; HBM budget 150 GB",
                       "iterations_per_s": r["iterations_per_s"], "latency_p50_s": r["latency_p50_s"],
                       "latency_p99_s": r["latency_p99_s"], "serial_plain": r["serial_plain"],
                       "served_over_serial_iterations": r["served_over_serial_iterations"],
                       "dropin_serial": r["dropin_serial"],
                       "served_over_dropin_iterations": r["served_over_dropin_iterations"],
                       "capacity_all_jobs_waiting": r["capacity"]},
            "e2e": {"value": r["jobs_per_s"], "unit": "jobs/s", "h2d_bytes_per_step": r["h2d_bytes_per_job"],
                    "d2h_bytes_per_step": r["d2h_bytes_per_job"]},
            "roofline": None, "cpu_baseline": None, "clocks": r["clocks"], "gpu_launches": None}
    print(json.dumps(line), flush=True)


def wl_resample():
    """Arclength resampling of 100,000 ragged strands (50..200 points, seed 0) to 100 points."""
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import _core
    rng = np.random.default_rng(0)
    counts = rng.integers(50, 201, size=100_000).astype(np.int32)
    pts = np.cumsum(rng.normal(scale=0.02, size=(int(counts.sum()), 3)), 0).astype(np.float32)
    host = {"counts": counts, "points": pts}

    def setup(d):
        t0 = time.perf_counter()
        _core.resample_strands_by_arclength(counts, pts, 100)      # the host path, for the record
        return {"host_s": time.perf_counter() - t0}

    def step(d, st):
        return _core.resample_strands_by_arclength_device(d["counts"], d["points"], 100)
    n = counts.shape[0]
    return dict(name="resample", host=host, setup=setup, step=step, units=n, unit="Mstrands/s", scale=1e6,
                metric="strands resampled by arclength per second (device)",
                alg_bytes=4 * n + 12 * int(counts.sum()) + 12 * 100 * n, launches=4,
                workload="resample_strands_by_arclength of 100,000 strands with 50..200 points to 100 points")


def wl_msaa():
    """Software-MSAA render of one wisp (400 strands x 64 points as a tube of 8 sides:
    204,800 vertices, 403,200 triangles) into a 512 x 256 patch, 64 jittered samples."""
    import torch
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    verts, faces, attr = syn.wisp_patch(400, 64, n_circle=8, seed=0)
    offsets, weights = s2c.msaa_pattern(8)
    H, W = 512, 256
    host = {"pos": verts, "tri": faces, "attr": attr}

    def setup(d):
        # the reference's per-sample loop over the drop-in ops, timed for the record
        s2c.msaa_render_loop((H, W), d["pos"], d["tri"], d["attr"], offsets, weights)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        s2c.msaa_render_loop((H, W), d["pos"], d["tri"], d["attr"], offsets, weights)
        b.record()
        torch.cuda.synchronize()
        return {"config_extra": {"per_sample_loop_ms": a.elapsed_time(b)}}

    def step(d, st):
        return s2c.msaa_render((H, W), d["pos"], d["tri"], d["attr"], offsets, weights)
    T = faces.shape[0]
    return dict(name="msaa", host=host, setup=setup, step=step, units=64 * T, unit="Mtri-samples/s", scale=1e6,
                metric="triangle samples rasterised, interpolated and resolved per second (64-sample MSAA)",
                alg_bytes=64 * (16 * verts.shape[0] + 12 * T + 16 * H * W) + 20 * H * W, launches=None,
                workload="64-sample software MSAA of a 400x64-strand wisp tube (403,200 triangles) into 512x256: "
                         "all jitters in one fused raster + one resolve")


def _align_wisps_loop(strands, sizes, beta):
    """The reference's align_wisps structure (curve_utils.py:104-165, 481-607) over the
    drop-in ops, for the record: a Python loop over wisps with a host SVD of each wisp's
    roots, and the Bishop frame as a loop over the points (torch ops on all strands)."""
    import torch
    import strns2cards_gb300 as s2c
    dev = strands.device
    lengths = (strands[:, 1:] - strands[:, :-1]).norm(dim=2).sum(1)
    h_orig = s2c.smooth_strands(strands, beta)
    Td = torch.tensor([0.0, 1.0, 0.0], device=dev)
    Nd = torch.tensor([0.0, 0.0, -1.0], device=dev)
    Bd = torch.tensor([-1.0, 0.0, 0.0], device=dev)
    s_all, h_all, off = [], [], 0
    for n in sizes.tolist():
        sw, hw = strands[off:off + n].clone(), h_orig[off:off + n].clone()
        c = sw[:, 0].mean(0, keepdim=True)
        sw -= c
        hw -= c
        _, _, Vt = np.linalg.svd(sw[:, 0].cpu().numpy(), full_matrices=False)
        ax = torch.from_numpy(Vt[:3] if Vt.shape == (3, 3) else np.eye(3, dtype=np.float32)).float().to(dev)
        li = int(torch.argmax(lengths[off:off + n]).item())
        g = sw[li]
        view = (g[0] - g[1]) / (g[0] - g[1]).norm().clamp(min=1e-8)
        down = (g[-1] - g[0]) / (g[-1] - g[0]).norm().clamp(min=1e-8)
        sg = torch.sign(torch.dot(ax[2], view)).item()
        nsrc = ax[2] * (1.0 if sg == 0 else sg)
        tsrc = down - torch.dot(down, nsrc) * nsrc
        tsrc = tsrc / tsrc.norm()
        if not bool(torch.isfinite(tsrc).all()):
            tsrc = ax[1]
        Rg = torch.stack([Td, Nd, Bd], -1) @ torch.stack([tsrc, nsrc, torch.cross(tsrc, nsrc, dim=-1)], -1).T
        s_all.append(sw.reshape(-1, 3) @ Rg.T)
        h_all.append(hw.reshape(-1, 3) @ Rg.T)
        off += n
    S, V, _ = strands.shape
    sr = torch.cat(s_all).reshape(S, V, 3)
    hr = torch.cat(h_all).reshape(S, V, 3)
    # Bishop frame: loop over the points
    d = hr[:, 1:] - hr[:, :-1]
    T = torch.zeros_like(hr)
    T[:, :-1] += d
    T[:, 1:] += d
    T = T / T.norm(dim=-1, keepdim=True).clamp(min=1e-8)
    N, B = torch.zeros_like(hr), torch.zeros_like(hr)
    N[:, 0], B[:, 0] = s2c.tangent_frame(T[:, 0])
    for i in range(1, V):
        v1 = hr[:, i] - hr[:, i - 1]
        c1 = (v1 ** 2).sum(-1, keepdim=True).clamp(min=1e-8)
        nL = N[:, i - 1] - 2 * ((v1 * N[:, i - 1]).sum(-1, keepdim=True) / c1) * v1
        tL = T[:, i - 1] - 2 * ((v1 * T[:, i - 1]).sum(-1, keepdim=True) / c1) * v1
        v2 = T[:, i] - tL
        c2 = (v2 ** 2).sum(-1, keepdim=True).clamp(min=1e-8)
        n1 = nL - 2 * ((v2 * nL).sum(-1, keepdim=True) / c2) * v2
        N[:, i] = n1 / n1.norm(dim=-1, keepdim=True).clamp(min=1e-8)
        b1 = torch.cross(T[:, i], N[:, i], dim=-1)
        B[:, i] = b1 / b1.norm(dim=-1, keepdim=True).clamp(min=1e-8)
    Ra = s2c.minimal_rotation(T[:, 0], Td.expand(S, 3))
    nd = (Ra @ N[:, 0, :, None])[..., 0]
    bd = (Ra @ B[:, 0, :, None])[..., 0]
    Rdst = torch.stack([Td.expand(S, V, 3), nd[:, None].expand(S, V, 3), bd[:, None].expand(S, V, 3)], -1)
    R = Rdst @ torch.stack([T, N, B], -1).transpose(-1, -2)
    arc = torch.cat([torch.zeros((S, 1), device=dev), torch.cumsum(d.norm(dim=2), 1)], 1)
    canon = arc[..., None] * Td + sr[:, 0][:, None]
    return s2c.skinning(sr, hr, canon, R.contiguous(), beta), h_orig


def wl_align_wisps():
    """align_wisps of 100,000 x 64 strands in 2,048 wisps (sizes 1..~500)."""
    import torch
    import strns2cards_gb300 as s2c
    from strns2cards_gb300 import synthetic as syn
    x, sizes = syn.make_wisps(100_000, 64, 2048, seed=0)
    host = {"x": x}
    sz = torch.from_numpy(sizes)

    def setup(d):
        _align_wisps_loop(d["x"], sz, 0.05)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        _align_wisps_loop(d["x"], sz, 0.05)
        b.record()
        torch.cuda.synchronize()
        return {"config_extra": {"per_wisp_loop_ms": a.elapsed_time(b)}}

    def step(d, st):
        return s2c.align_wisps_packed(d["x"], sz, 0.05)
    n = x.shape[0] * x.shape[1]
    # wisp frames (read every point for the lengths: 12) + fused smoothing / rotation / frames /
    # skinning (read 12, write handles 12 and aligned strands 12) per point
    return dict(name="align_wisps", host=host, setup=setup, step=step, units=n, unit="Mpts/s", scale=1e6,
                metric="strand points aligned per second (align_wisps)",
                alg_bytes=(12 + 12 + 24) * n, launches=2,
                workload="align_wisps of 100,000 x 64 strands in 2,048 wisps, beta 0.05: per-wisp frames, then "
                         "smoothing, rotation, Bishop frames + canonical handles and skinning fused")


def wl_build_edges():
    """Edges of the card mesh of 2,048 cards (16 x 4 quads: 174,080 vertices, 262,144
    triangles) on the device; the host builder timed for the record."""
    import time
    import torch
    import strns2cards_gb300 as s2c
    _, _, cards = _cards_scene(50_000, 100, 2048, 16, 4, 1024)
    tri = np.ascontiguousarray(cards.tri, dtype=np.int32)
    nv = int(cards.verts.shape[0])
    host = {"tri": tri}

    def setup(d):
        s2c.build_edges_from_triangles(tri)
        t0 = time.perf_counter()
        s2c.build_edges_from_triangles(tri)
        return {"config_extra": {"host_builder_ms": 1e3 * (time.perf_counter() - t0)}}

    def step(d, st):
        return s2c.build_edges_from_triangles_device(d["tri"], nv)
    T = tri.shape[0]
    # triangles read (12 B per triangle, twice), per half-edge: bucket/sorted/flag/eid writes and
    # reads (4 B each, about 8 passes), edges + edge2tri written (16 B per edge, E ~ 1.5 T)
    return dict(name="build_edges", host=host, setup=setup, step=step, units=T, unit="Mtri/s", scale=1e6, dtype="i32",
                metric="card-mesh triangles turned into edges per second (device edge builder)",
                alg_bytes=24 * T + 3 * T * 32 + 16 * 3 * T // 2, launches=None,
                workload="unique edges + edge->triangle map of 2,048 cards (16x4 quads, 262,144 triangles) "
                         "on the device, in the host builder's order")


WORKLOADS = {"msaa": wl_msaa, "resample": wl_resample, "tri_raster": wl_tri_raster, "tri_raster_list": lambda: wl_tri_raster(True),
             "antialias": wl_antialias, "antialias_list": lambda: wl_antialias(True), "iteration": wl_iteration,
             "antialias_2048": wl_antialias_2048, "dda_list": wl_dda_list, "interpolate": wl_interpolate,
             "dda_interpolate": wl_dda_interpolate, "bary_derivatives": wl_bary_derivatives,
             "bitset_stats": wl_bitset_stats,
             "cluster_iou": wl_cluster_iou,
             "smooth_strands": wl_smooth_strands, "skinning": wl_skinning, "lbs": wl_lbs,
             "laplacian": wl_laplacian, "align_wisps": wl_align_wisps, "build_edges": wl_build_edges}


def run_workload(args):
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        print(json.dumps({"workload": args.workload, "skipped": "secondary workloads run on one GPU"}))
        return
    dev = torch.device("cuda", 0)
    wl = WORKLOADS[args.workload]()
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in wl["host"].items()}
    st = wl["setup"](d) if "setup" in wl else None
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(max(args.warmup, 3)):
        wl["step"](d, st)
    torch.cuda.synchronize()

    def timed(run):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for i in range(args.steps):
            flush.fill_(i & 0xff)
            evs[i][0].record(stream)
            run()
            evs[i][1].record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs]
    graph_note = {}
    with ClockSampler(local) as clk:
        ms = timed(lambda: wl["step"](d, st))
        if wl.get("graph"):
            # small ops whose eager step is bound by the host's launches and autograd: the
            # same step captured once as a CUDA graph (static inputs) and replayed
            g = torch.cuda.CUDAGraph()
            side = torch.cuda.Stream(device=dev)
            side.wait_stream(stream)
            with torch.cuda.stream(side):
                wl["step"](d, st)
            stream.wait_stream(side)
            with torch.cuda.graph(g):
                wl["step"](d, st)
            g.replay()
            torch.cuda.synchronize()
            eager = ms
            ms = timed(g.replay)
            graph_note = {"timed_as": "CUDA graph replay of the step", "eager_ms_per_step": sum(eager) / len(eager)}
    t = sum(ms) / 1e3
    value = wl["units"] * args.steps / t / wl["scale"]
    # end to end: pinned host inputs in, every output tensor back
    pinned = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in wl["host"].items()}
    h2d = sum(v.nbytes for v in wl["host"].values())

    def outs(r):
        return [x for x in (r if isinstance(r, (tuple, list)) else (r,)) if isinstance(x, torch.Tensor)]
    probe = outs(wl["step"](d, st))
    host_out = [torch.empty(x.shape, dtype=x.dtype).pin_memory() for x in probe]
    d2h = sum(x.numel() * x.element_size() for x in probe)

    def e2e_step():
        dd = {k: v.to(dev, non_blocking=True) for k, v in pinned.items()}
        for ho, x in zip(host_out, outs(wl["step"](dd, st))):
            ho.copy_(x, non_blocking=True)
    e2e_step()
    torch.cuda.synchronize()
    ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k = max(3, min(args.steps, 10))
    ea.record(stream)
    for _ in range(k):
        e2e_step()
    eb.record(stream)
    torch.cuda.synchronize()
    e2e = wl["units"] * k / (ea.elapsed_time(eb) / 1e3) / wl["scale"]
    peak, peak_kind = load_peaks()
    alg_bytes = st["alg_bytes"] if isinstance(st, dict) and "alg_bytes" in st else wl["alg_bytes"]
    achieved = alg_bytes / (t / args.steps) / 1e9
    line = {"metric": wl["metric"], "value": value, "unit": wl["unit"], "n_gpus": 1, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": wl.get("dtype", "f32"), "data": "synthetic",
            "config": dict({"workload": wl["workload"], "l2": "flushed between steps (256 MiB write)"},
                           **({"host_reference_algorithm_s": st["host_s"]} if isinstance(st, dict) and "host_s" in st
                              else {}),
                           **(st.get("config_extra", {}) if isinstance(st, dict) else {}), **graph_note),
            "e2e": {"value": e2e, "unit": wl["unit"], "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "algorithmic_bytes_per_step": alg_bytes, "traffic": None},
            "cpu_baseline": None, "clocks": clk.summary(), "gpu_launches": None, "step_ms": ms}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the batched / served forms (ours) and the reference-kernel timings (reference)")
    ap.add_argument("--serving-jobs", type=int, default=40, help="requests in the served form's stream")
    ap.add_argument("--workload", choices=["dda_bitset", "batched_fit", "serving"] + sorted(WORKLOADS),
                    default="dda_bitset",
                    help="dda_bitset (default) is the headline; the others time the remaining rows")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched_fit":
        run_batched_fit(args)
    elif args.workload == "serving":
        run_serving(args)
    elif args.workload != "dda_bitset":
        run_workload(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
