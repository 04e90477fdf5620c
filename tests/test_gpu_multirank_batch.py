"""Batched scenes sharded over ranks (the multi-GPU plan for batches: scenes are independent, so
rank r steps its own scene set with no collective on the data path).

Two gloo ranks, each a separate process with its own library handle on the one GPU this run
has, step their shard (`batched_dam_breaks(seed = base + rank)`, as bench.py shards the batched
workload) for a few steps; a single-process batch of both shards' scenes steps the same scenes
in one handle.  Every scene must end where the single batch puts it (within the per-step
tolerance, times the steps), and the ranks exchange only host metadata (the gathered results).
The ranks' kernels never wait on one another: their handles are independent.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

pytestmark = pytest.mark.gpu

STEPS = 3
BASE_SEED = 11
KW = dict(count=3, n_range=(1500, 6000))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _step_set(sc, steps):
    from realtimeparticles_gb300 import abi, model
    with model.FluidsBatch(sc["scenes"], sc["h"]) as m:
        m.setFluidParams(sc["fluid_params"])
        m.setJacobiIterations(3)
        m.upload(abi.BUF_POS, sc["pos"])
        m.upload(abi.BUF_VEL, sc["vel"])
        m.update(steps)
        pos, ids = m.download(abi.BUF_POS), m.download(abi.BUF_ID)
        out = []
        for s in range(m.numScenes()):
            off, cnt = m.sceneRange(s)
            p = np.empty((cnt, 4), np.float32)
            p[ids[off:off + cnt] - off] = pos[off:off + cnt]  # by particle id within the scene
            out.append(p)
        return out


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from realtimeparticles_gb300 import scenes
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = _step_set(scenes.batched_dam_breaks(seed=BASE_SEED + rank, **KW), STEPS)
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)  # host metadata only: the final positions
        if rank == 0:
            out["shards"] = gathered
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_step_their_scene_shards_like_one_batch():
    from realtimeparticles_gb300 import scenes
    world = 2
    port = _free_port()
    # The manager's server process is started by spawn, not fork: this process may hold a CUDA
    # context already, and a child forked after that can hang.
    with mp.get_context("spawn").Manager() as man:
        out = man.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        shards = out["shards"]
    # The same scenes in one single-process batch, shard 0's scenes first.
    sets = [scenes.batched_dam_breaks(seed=BASE_SEED + r, **KW) for r in range(world)]
    union = {"scenes": sets[0]["scenes"] + sets[1]["scenes"], "h": sets[0]["h"],
             "fluid_params": sets[0]["fluid_params"],
             "pos": np.concatenate([s["pos"] for s in sets]), "vel": np.concatenate([s["vel"] for s in sets])}
    whole = _step_set(union, STEPS)
    k = 0
    for r in range(world):
        assert len(shards[r]) == KW["count"]
        for s, p in enumerate(shards[r]):
            box = max(sets[r]["scenes"][s][1])
            diff = np.abs(p[:, :3].astype(np.float64) - whole[k][:, :3])
            assert np.all(np.isfinite(p)), (r, s)
            assert diff.max() <= 1e-5 * box * STEPS, (r, s, diff.max())
            k += 1
