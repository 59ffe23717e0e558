"""Multi-process (replica) path of bench.py on the CPU: two ``gloo`` ranks run
the same setup, barrier and max-over-ranks timing that the GPU replicas use
under torchrun (no data-path collective)."""

import os
import socket

import pytest
import torch
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(world),
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    import bench
    w, r, local = bench.dist_setup("gloo")
    bench.barrier(w)
    # rank 1 is slower: the job time is the slowest rank's
    ms = 100.0 + 50.0 * r
    ms_max = bench.max_over_ranks(ms, w, torch.device("cpu"))
    rate = bench.aggregate_rate(w, 1024 * 5, ms_max)
    bench.barrier(w)
    q.put((r, w, ms_max, rate, bench.replica_seed(1000, r)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_replicas_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2, 2]
    assert all(o[2] == 150.0 for o in out)            # max over ranks
    assert all(abs(o[3] - 2 * 5120 / 0.15) < 1e-6 for o in out)
    assert out[0][4] != out[1][4]                       # each replica draws its own batch
