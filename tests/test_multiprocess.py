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
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 11.0   # slowest rank's time on every rank
    assert res[0][1] == pytest.approx(131072 * 5 * 2 / 11.0)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    bench.barrier(1)


def _batch_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    from realtimeparticles_gb300 import scenes
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = bench.WORKLOADS["pbf_batched_48"]
        sc = scenes.batched_dam_breaks(count=w["count"], seed=w["seed"] + rank)  # as make_model(w, rank)
        n = sc["pos"].shape[0]
        out[rank] = (n, bench.sum_over_ranks(n, world), [s[0] for s in sc["scenes"]])
    finally:
        dist.destroy_process_group()


def test_batch_shards_by_scene():
    """Each rank of a batch run holds its own seeded scene set; the throughput counts the
    particles of all ranks (no collective on the data path, one all-reduce of the count)."""
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_batch_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][2] != res[1][2]                          # different scenes
    assert res[0][1] == res[1][1] == res[0][0] + res[1][0]  # total particles on every rank
