"""The host logic of bench.py's multi-GPU (replica) path on CPU with two gloo ranks: the reported
time is the slowest rank's, and the ranks' right-hand-side seeds are disjoint."""
import os
import socket
import sys

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    try:
        t = bench.max_over_ranks(10.0 * (rank + 1), dist, torch.device("cpu"))
        seeds = bench.rank_seeds(2, rank, 8)
        gathered = [None] * world
        dist.all_gather_object(gathered, seeds)
        out.put((rank, t, gathered))
    finally:
        dist.destroy_process_group()


def test_bench_replica_host_logic():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, gathered in res:
        assert t == 10.0 * world                      # max over ranks
        flat = [s for seeds in gathered for s in seeds]
        assert len(set(flat)) == len(flat) == 8 * world
