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
# kernels one s2c_dda_cluster_bitset call launches: init, bin, scan (3), scatter, tile raster, fixup
LAUNCHES_PER_STEP = 8
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
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

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
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
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
        for line in open(self.path):
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
    print(json.dumps(line), flush=True)


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
    t_max = dev_s
    if ws > 1:
        t = torch.tensor([dev_s], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max = float(t.item())
    segs_total = B * E * args.steps * ws
    value = segs_total / t_max / 1e9

    # e2e through the public op with host buffers (pinned), copies inside the timed region
    pos_p = torch.from_numpy(pos_h).pin_memory()
    edges_p = torch.from_numpy(edges_h).pin_memory()
    e2c_p = torch.from_numpy(e2c_h).pin_memory()
    out_p = torch.empty(out.shape, dtype=torch.int32).pin_memory()
    e2e_steps = max(3, min(args.steps, 10))

    def e2e_step():
        pd = pos_p.to(dev, non_blocking=True)
        ed = edges_p.to(dev, non_blocking=True)
        cd = e2c_p.to(dev, non_blocking=True)
        r = s2c.dda_cluster_bitset((RES, RES), pd, ed, cd, K, out=out, workspace=work)
        out_p.copy_(r, non_blocking=True)

    e2e_step()
    torch.cuda.synchronize()
    ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ea.record(stream)
    for _ in range(e2e_steps):
        e2e_step()
    eb.record(stream)
    torch.cuda.synchronize()
    e2e_s = ea.elapsed_time(eb) / 1e3
    if ws > 1:
        t = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = B * E * e2e_steps * ws / e2e_s / 1e9
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
                             "kernel": "s2c_dda_cluster_bitset (init, bin, 3-launch scan, scatter, tile raster, fixup)"},
                "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": LAUNCHES_PER_STEP * args.steps,
                "wall_s": wall}
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
