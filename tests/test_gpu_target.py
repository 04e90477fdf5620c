"""Boids target attractor on the GPU against the oracle (Boids.cpp:351-358, boids.cl:226-241,
Target.cpp:27-50).

The trajectory is host state: the library's positions must equal the oracle's bit for bit.
The device reads the target of each step from a track uploaded in chunks of 1024 steps, so
the checks cover a step count that crosses a chunk inside one update call.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, model, scenes
from realtimeparticles_gb300._lib import RtpError, call

from helpers import REL_BOX, assert_close_by_id, boids_model, box_size, gpu_state

pytestmark = pytest.mark.gpu


def _target(enabled=True, radius=2.0, sign=1, visible=True):
    tp = model.default_target_params()
    tp.enabled = int(enabled)
    tp.visible = int(visible)
    tp.radiusEffect = float(radius)
    tp.signEffect = int(sign)
    return tp


def _trajectory(sc, nsteps, dim=3):
    return oracle.target_trajectory(sc["model_params"].boxSize[0], dim, sc["boids_params"].velocityScale, nsteps)


@pytest.mark.parametrize("boundary,dt,radius", [(abi.CYCLIC_WALL, 0.01, 2.0), (abi.BOUNCING_WALL, 0.1, 0.7)])
def test_target_steps_match_the_oracle(boundary, dt, radius):
    sc = scenes.boids_cloud(n=20000, seed=5)
    c = oracle.derive_constants(abi.BOIDS, sc["model_params"])
    L = box_size(sc["model_params"])
    traj = _trajectory(sc, 4)
    with boids_model(sc, dt=dt, boundary=boundary) as m:
        assert m.targetPos() == (0.0, 0.0, 0.0) and not m.isTargetActivated()
        m.setTarget(_target(radius=radius))
        assert m.isTargetActivated() and m.isTargetVisible()
        for s in range(4):
            st = gpu_state(m, abi.BOIDS)
            ost = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
            oracle.boids_step(c, sc["boids_params"], dt, boundary, ost, target=traj[s], target_radius=radius)
            m.update(1)
            assert np.array_equal(np.array(m.targetPos(), np.float32), traj[s])
            g = gpu_state(m, abi.BOIDS)
            assert np.array_equal(g["id"], ost["id"])
            assert_close_by_id(g["id"], g["pos"], ost["id"], ost["pos"], REL_BOX * L, "pos")
            assert_close_by_id(g["id"], g["vel"], ost["id"], ost["vel"], REL_BOX * L / dt, "vel")
            assert np.allclose(m.download(abi.BUF_ACC), ost["acc"], rtol=1e-4, atol=1e-4)


def _acc_err(m, sc, c, T, radius):
    """Positions stand still at dt = 0, so the last step's accelerations are the rules plus
    the pull towards T at the downloaded positions."""
    st = gpu_state(m, abi.BOIDS)
    oracle.boids_step(c, sc["boids_params"], 0.0, abi.CYCLIC_WALL, st, target=T, target_radius=radius)
    return float(np.abs(m.download(abi.BUF_ACC) - st["acc"]).max())


def test_target_track_across_chunks_and_calls():
    sc = scenes.boids_cloud(n=6000, seed=6)
    c = oracle.derive_constants(abi.BOIDS, sc["model_params"])
    traj = _trajectory(sc, 1029)
    with boids_model(sc, dt=0.0) as m:
        m.setTarget(_target(radius=2.0))
        m.update(1025)  # steps 0..1023 from the first upload, step 1024 from the second
        assert np.array_equal(np.array(m.targetPos(), np.float32), traj[1024])
        right = _acc_err(m, sc, c, traj[1024], 2.0)
        wrong = min(_acc_err(m, sc, c, traj[k], 2.0) for k in (1023, 1022, 0))
        assert right < 2e-5 and wrong > 20 * right, (right, wrong)
        m.update(3)  # a new call restarts the track
        assert np.array_equal(np.array(m.targetPos(), np.float32), traj[1027])
        assert _acc_err(m, sc, c, traj[1027], 2.0) < 2e-5
        m.update(1)
        assert _acc_err(m, sc, c, traj[1028], 2.0) < 2e-5


def test_target_json_reset_and_disable():
    sc = scenes.boids_cloud(n=4000, seed=7, max_n=131072)  # room for the reset case
    sc["boids_params"] = model.default_boids_params()  # what every JSON update transfers
    c = oracle.derive_constants(abi.BOIDS, sc["model_params"])
    traj = _trajectory(sc, 12)
    with boids_model(sc, dt=0.0) as m:
        m.updateInputJson({"Boids": {"Target": {"Enable##Target": True, "Radius": [1.5, 1.0, 20.0]}}})
        assert m.isTargetActivated() and m.isTargetVisible()
        m.update(3)
        assert np.array_equal(np.array(m.targetPos(), np.float32), traj[2])
        assert _acc_err(m, sc, c, traj[2], 1.5) < 2e-5
        # Disabled: no pull and the trajectory waits.
        m.updateInputJson({"Boids": {"Target": {"Enable##Target": False}}})
        assert not m.isTargetActivated() and not m.isTargetVisible()
        m.update(2)
        assert np.array_equal(np.array(m.targetPos(), np.float32), traj[2])
        st = gpu_state(m, abi.BOIDS)
        oracle.boids_step(c, sc["boids_params"], 0.0, abi.CYCLIC_WALL, st)
        assert float(np.abs(m.download(abi.BUF_ACC) - st["acc"]).max()) < 2e-5
        # Attract = false casts to a sign of 0: enabled, moving, and without effect.
        m.updateInputJson({"Boids": {"Target": {"Enable##Target": True, "Attract": False, "Show": False}}})
        assert m.isTargetActivated() and not m.isTargetVisible()
        m.update(1)
        assert np.array_equal(np.array(m.targetPos(), np.float32), traj[3])
        st = gpu_state(m, abi.BOIDS)
        oracle.boids_step(c, sc["boids_params"], 0.0, abi.CYCLIC_WALL, st)
        assert float(np.abs(m.download(abi.BUF_ACC) - st["acc"]).max()) < 2e-5
        # reset() restores the JSON defaults (target off); the trajectory continues afterwards.
        m.reset()
        assert not m.isTargetActivated()
        m.setTarget(_target())
        m.update(1)
        assert np.array_equal(np.array(m.targetPos(), np.float32), traj[4])


def test_target_2d_and_other_models():
    sc = scenes.boids_plane(n=4096)
    with model.Boids(sc["model_params"]) as m:
        m.setBoidsParams(sc["boids_params"])
        m.upload(abi.BUF_POS, sc["pos"])
        m.upload(abi.BUF_VEL, sc["vel"])
        m.setTarget(_target(radius=1.0))
        m.update(5)
        want = oracle.target_trajectory(sc["model_params"].boxSize[0], 2, sc["boids_params"].velocityScale, 5)
        assert np.array_equal(np.array(m.targetPos(), np.float32), want[4])
        assert m.targetPos()[0] == 0.0
        assert np.all(m.download(abi.BUF_POS)[:, 0] == 0.0)  # the 2D plane is kept
    sf = scenes.dam_break(lattice=(8, 8, 8))
    with model.Fluids(sf["model_params"]) as f:
        assert f.targetPos() == (0.0, 0.0, 0.0) and not f.isTargetActivated() and not f.isTargetVisible()
        with pytest.raises(RtpError):  # rtp_set_target: boids only
            call("rtp_set_target", f._h, C.byref(_target()))
