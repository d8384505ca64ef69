"""Rank logic of bench.py under torch.distributed on CPU (gloo, world size 2): each rank
draws its own view of the same model, the timing reduction gives every rank the slowest
rank's time, and the whole-job rate counts the units of all ranks."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, ws, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    w, r, lr = bench.dist_env()
    assert (w, r, lr) == (ws, rank, rank)
    t = bench.max_over_ranks(0.5 + rank, ws, "cpu")
    rate = bench.whole_job_rate(100.0, ws, t)
    from strns2cards_gb300 import synthetic as syn
    sc = syn.strand_scene(64, 8, per_cluster=4, num_views=ws, seed=0)
    out[rank] = (t, rate, float(np.abs(sc.pos[rank]).sum()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_gloo():
    ws = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(ws, _free_port(), out), nprocs=ws, start_method="spawn", join=True)
    assert out[0][0] == out[1][0] == 1.5              # the slower rank's time on both
    assert out[0][1] == out[1][1] == 100.0 * 2 / 1.5  # units of both ranks over the max time
    assert out[0][2] != out[1][2]                     # each rank rasterises its own view
