"""The multi-process path of bench.py (one replica per rank, barrier + max-over-ranks
timing) on CPU with the gloo backend, world size 2.  The step itself does not shard
(one scene per GPU), so the only cross-rank operations are the barrier and the max."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, local = bench.dist_env()
        assert (ws, r, local) == (world, rank, rank)
        bench.barrier(ws)
        t = bench.max_over_ranks(10.0 + rank, ws)          # per-rank elapsed times
        units = 131072 * 5 * ws                               # every rank processed its replica
        out[rank] = (t, units / t)
        bench.barrier(ws)
    finally:
        dist.destroy_process_group()


def test_bench_replicas_take_max_over_ranks():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 11.0   # slowest rank's time on every rank
    assert res[0][1] == pytest.approx(131072 * 5 * 2 / 11.0)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    bench.barrier(1)
