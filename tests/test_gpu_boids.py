"""Boids step parity (Boids::update, physics/ocl/Boids.cpp:323-377)."""
import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, scenes

from helpers import REL_BOX, assert_close_by_id, boids_model, box_size, gpu_state

pytestmark = pytest.mark.gpu


def _compare(m, sc, dt, boundary, steps, acc_atol=1e-4):
    c = oracle.derive_constants(abi.BOIDS, sc["model_params"])
    L = box_size(sc["model_params"])
    for _ in range(steps):
        st = gpu_state(m, abi.BOIDS)
        ost = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
        oracle.boids_step(c, sc["boids_params"], dt, boundary, ost)
        m.update(1)
        g = gpu_state(m, abi.BOIDS)
        assert np.array_equal(m.download(abi.BUF_CELL_ID), ost["cellId"])
        assert np.array_equal(g["id"], ost["id"])
        assert np.array_equal(m.download(abi.BUF_CELL_TABLE), ost["table"])
        assert_close_by_id(g["id"], g["pos"], ost["id"], ost["pos"], REL_BOX * L, "pos")
        assert_close_by_id(g["id"], g["vel"], ost["id"], ost["vel"], REL_BOX * L / dt, "vel")
        acc = m.download(abi.BUF_ACC)
        assert np.allclose(acc, ost["acc"], rtol=1e-4, atol=acc_atol)
        speed = np.linalg.norm(g["vel"][:, :3], axis=1)
        v = sc["boids_params"].velocityScale
        if boundary == abi.CYCLIC_WALL:  # bd_updateVel clamps |v| to [0.2 v, v] (boids.cl:256)
            assert speed.min() >= 0.2 * v * (1 - 1e-5) and speed.max() <= v * (1 + 1e-5)


def test_boids_131k_periodic():
    sc = scenes.boids_cloud()
    with boids_model(sc) as m:
        _compare(m, sc, 0.01, abi.CYCLIC_WALL, steps=3)


def test_boids_wall_and_reference_dt():
    sc = scenes.boids_cloud(n=20000, seed=3)
    with boids_model(sc, dt=0.1, boundary=abi.BOUNCING_WALL) as m:
        _compare(m, sc, 0.1, abi.BOUNCING_WALL, steps=3)


def test_boids_dense_cell_cap():
    # All boids in a few cells: exercises the 3000 per-cell cap (Boids.cpp:78).
    sc = scenes.boids_cloud(n=9000, seed=4)
    sc["pos"][:, :3] = np.random.default_rng(1).uniform(-0.04, 0.04, (9000, 3)).astype(np.float32)
    with boids_model(sc) as m:
        # Each boid sums ~10^4 nearly cancelling unit vectors: float32 summation-order
        # differences reach ~1e-3 in the accelerations (positions still match to 1e-5 L).
        _compare(m, sc, 0.01, abi.CYCLIC_WALL, steps=2, acc_atol=5e-3)
