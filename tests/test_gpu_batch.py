"""Batched scenes against the oracle, scene by scene.

A batch steps many independent dam breaks of different sizes and box aspects in one set of
buffers.  Each scene must evolve exactly as the oracle evolves that scene alone on its own
grid (rtp_batch_scene_constants): the sorted order and cell keys inside the scene bit for bit,
positions within 1e-5 x the scene's box, velocities within 1e-5 x box / dt — for every
launch shape the autotuner can pick (lanes per particle, cell factor) and with the warm start.
"""
import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, model, scenes

from helpers import REL_BOX, assert_close_by_id, random_net

pytestmark = pytest.mark.gpu


def _batch(count=6, seed=3, n_range=(700, 3000), iters=2, **kw):
    sc = scenes.batched_dam_breaks(count=count, seed=seed, n_range=n_range, **kw)
    m = model.FluidsBatch(sc["scenes"], sc["h"])
    m.setFluidParams(sc["fluid_params"])
    m.setJacobiIterations(iters)
    m.upload(abi.BUF_POS, sc["pos"])
    m.upload(abi.BUF_VEL, sc["vel"])
    return sc, m


def _scene_states(m, sc):
    pos, vel, ids = m.download(abi.BUF_POS), m.download(abi.BUF_VEL), m.download(abi.BUF_ID)
    out = []
    for s in range(m.numScenes()):
        off, cnt = m.sceneRange(s)
        c = m.sceneConstants(s)
        st = oracle.new_state(cnt, c)
        st["pos"][:] = pos[off:off + cnt]
        st["vel"][:] = vel[off:off + cnt]
        st["id"][:] = ids[off:off + cnt] - off
        out.append((c, off, cnt, st))
    return out


def _compare(m, sc, before, fp):
    pos, vel, ids = m.download(abi.BUF_POS), m.download(abi.BUF_VEL), m.download(abi.BUF_ID)
    keys = m.download(abi.BUF_CELL_ID)
    for s, (c, off, cnt, st) in enumerate(before):
        box = max(sc["scenes"][s][1])
        gid = ids[off:off + cnt] - off
        assert np.array_equal(gid, st["id"]), "scene %d: sorted order" % s
        assert np.array_equal(keys[off:off + cnt] - m.sceneKeyBase(s), st["cellId"]), "scene %d: cell keys" % s
        assert_close_by_id(gid, pos[off:off + cnt], st["id"], st["pos"], REL_BOX * box, "scene %d pos" % s)
        assert_close_by_id(gid, vel[off:off + cnt], st["id"], st["vel"], REL_BOX * box / fp.timeStep, "scene %d vel" % s)


@pytest.mark.parametrize("lanes,factor", [(4, 1.0), (2, 1.0), (8, 1.0), (4, 1.25), (8, 1.5), (2, 2.0)])
def test_batch_steps_match_the_oracle_per_scene(lanes, factor):
    sc, m = _batch()
    with m:
        m.setTuning(lanes, factor)
        fp = sc["fluid_params"]
        for _ in range(3):
            before = _scene_states(m, sc)
            for c, off, cnt, st in before:
                oracle.fluids_step(c, fp, 2, st)
            m.update(1)
            _compare(m, sc, before, fp)


def test_large_batch_matches_the_oracle_per_scene():
    """A batch of more than 49,152 particles: its full sweeps run one lane per particle (the
    small batches above run lane groups)."""
    sc, m = _batch(count=4, seed=9, n_range=(14000, 20000))
    with m:
        assert m.nbParticles() > 49152
        fp = sc["fluid_params"]
        for _ in range(2):
            before = _scene_states(m, sc)
            for c, off, cnt, st in before:
                oracle.fluids_step(c, fp, 2, st)
            m.update(1)
            _compare(m, sc, before, fp)


def test_batch_over_1m_particles_matches_the_oracle_per_scene():
    """A batch of more than 2^20 particles: its full sweeps record hits through the bit-mask
    filter."""
    # Wide scenes (x extent 2): their lattices stay below 0.7 of the box height.
    sc, m = _batch(count=6, seed=13, n_range=(180000, 220000), aspect_range=(2.0, 2.0))
    with m:
        assert m.nbParticles() >= 1 << 20
        fp = sc["fluid_params"]
        before = _scene_states(m, sc)
        for c, off, cnt, st in before:
            oracle.fluids_step(c, fp, 2, st)
        m.update(1)
        _compare(m, sc, before, fp)


def test_batch_scene_equals_the_same_scene_alone():
    """One scene of a batch and the same scene on its own handle: same trajectory."""
    sc, m = _batch(count=4, seed=11)
    with m:
        s = 2
        off, cnt = m.sceneRange(s)
        n, box = sc["scenes"][s]
        c = m.sceneConstants(s)
        mp = abi.model_params(n, n, box, tuple(c.gridRes), 3)
        single = model.Fluids(mp)
        single.setFluidParams(sc["fluid_params"])
        single.setJacobiIterations(2)
        single.upload(abi.BUF_POS, sc["pos"][off:off + cnt])
        single.upload(abi.BUF_VEL, sc["vel"][off:off + cnt])
        with single:
            assert single.constants().cellSize == c.cellSize
            for _ in range(5):
                m.update(1)
                single.update(1)
            ids_b = m.download(abi.BUF_ID)[off:off + cnt] - off
            ids_s = single.download(abi.BUF_ID)
            assert np.array_equal(ids_b, ids_s)
            assert np.allclose(m.download(abi.BUF_POS)[off:off + cnt], single.download(abi.BUF_POS), atol=1e-6 * max(box))


def test_warm_started_batch_matches_the_oracle_per_scene():
    sc, m = _batch(count=4, seed=5)
    fp = sc["fluid_params"]
    net = random_net(np.random.default_rng(2), out_scale=np.array([2e-7, 2e-5, 2e-5, 2e-5], np.float32))
    with m:
        m.setWarmStart(net, extra_iterations=1, guard_tolerance=0.0)
        for _ in range(2):
            before = _scene_states(m, sc)
            for c, off, cnt, st in before:
                oracle.ws_step(c, fp, net, 1, 0.0, 2, st, np.zeros(cnt, np.float32))
            m.update(1)
            _compare(m, sc, before, fp)


def test_autotune_tries_every_candidate_and_keeps_the_fastest():
    sc, m = _batch(count=5, seed=7)
    with m:
        best, cands = m.autotune(steps=2)
        assert len(cands) == 12 and all(k[2] == 0 for k in cands)  # no tiled sweeps on a batch
        key = (best[0], round(best[1], 3), best[2])
        assert cands[key] == min(cands.values())
        assert m.tuning() == best
        m.update(2)  # still steps after the grid changed


def test_batch_refuses_per_scene_resizing():
    sc, m = _batch(count=2)
    with m:
        from realtimeparticles_gb300._lib import RtpError
        with pytest.raises(RtpError):
            m.setNbParticles(10)
        with pytest.raises(RtpError):
            m.reset()
