"""CPU, two ranks over gloo: the replica bookkeeping of bench.py.

A depth map does not shard, so N GPUs run N independent replicas; the only
exchange is the timing reduction (max over ranks) and barriers around the
timed region.  Here two CPU processes check that path: the rendezvous on
127.0.0.1, barrier_max returning the maximum on every rank, and the
barriers.
"""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")  # CPU ranks: gloo
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    w, r, _ = bench.dist_init()
    bench.barrier(w)
    v = bench.barrier_max(w, 10.0 * (rank + 1))
    total = bench.barrier_max(w, float(rank))
    bench.barrier(w)
    q.put((r, w, v, total))
    dist.destroy_process_group()


def test_two_rank_timing_reduction():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 2, 20.0, 1.0), (1, 2, 20.0, 1.0)]
