"""Edge sizes on the GPU: empty models and a handful of particles (sort tiles of one or two
keys, cells with a single member, the sorted index 0 that never starts a cell, grid.cl:103-112)
against the oracle, for the three models."""
import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, model, scenes

from helpers import REL_BOX, assert_close_by_id, box_size, boids_model, clouds_model, fluids_model, gpu_state

pytestmark = pytest.mark.gpu


def _take(sc, n):
    sc["pos"] = np.ascontiguousarray(sc["pos"][:n])
    sc["vel"] = np.ascontiguousarray(sc["vel"][:n])
    sc["model_params"].currNbParticles = n
    return sc


@pytest.mark.parametrize("n", [1, 2, 3, 33])
def test_fluids_few_particles(n):
    sc = _take(scenes.dam_break(lattice=(4, 8, 8), max_n=256), n)
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    fp = sc["fluid_params"]
    L = box_size(sc["model_params"])
    with fluids_model(sc, 3) as m:
        for _ in range(3):
            st = gpu_state(m, abi.FLUIDS)
            ost = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
            oracle.fluids_step(c, fp, 3, ost)
            m.update(1)
            g = gpu_state(m, abi.FLUIDS)
            assert np.array_equal(g["id"], ost["id"])
            assert np.array_equal(m.download(abi.BUF_CELL_TABLE), ost["table"])
            assert_close_by_id(g["id"], g["pos"], ost["id"], ost["pos"], REL_BOX * L, "pos")
            assert_close_by_id(g["id"], g["vel"], ost["id"], ost["vel"], REL_BOX * L / fp.timeStep, "vel")
        assert m.metrics().meanNeighbours >= 0.0


@pytest.mark.parametrize("n", [1, 2, 33])
def test_boids_few_particles(n):
    sc = scenes.boids_cloud(n=n, seed=9, max_n=256)
    c = oracle.derive_constants(abi.BOIDS, sc["model_params"])
    L = box_size(sc["model_params"])
    with boids_model(sc, dt=0.01) as m:
        for _ in range(3):
            st = gpu_state(m, abi.BOIDS)
            ost = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
            oracle.boids_step(c, sc["boids_params"], 0.01, abi.CYCLIC_WALL, ost)
            m.update(1)
            g = gpu_state(m, abi.BOIDS)
            assert np.array_equal(g["id"], ost["id"])
            assert_close_by_id(g["id"], g["pos"], ost["id"], ost["pos"], REL_BOX * L, "pos")


@pytest.mark.parametrize("n", [1, 3, 33])
def test_clouds_few_particles(n):
    sc = scenes.clouds_cumulus(n=n, noise=False, seed=4, max_n=256)
    c = oracle.derive_constants(abi.CLOUDS, sc["model_params"])
    fp, cp = sc["fluid_params"], sc["cloud_params"]
    L = box_size(sc["model_params"])
    with clouds_model(sc) as m:
        for _ in range(3):
            st = gpu_state(m, abi.CLOUDS)
            ost = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
            oracle.clouds_step(c, fp, cp, sc["env"], sc["ground"], 1, ost)
            m.update(1)
            g = gpu_state(m, abi.CLOUDS)
            assert np.array_equal(g["id"], ost["id"])
            assert_close_by_id(g["id"], g["pos"], ost["id"], ost["pos"], REL_BOX * L, "pos")
            assert_close_by_id(g["id"], g["temp"], ost["id"], ost["temp"], 1e-3, "temp")


@pytest.mark.parametrize("mtype", [abi.FLUIDS, abi.BOIDS, abi.CLOUDS])
def test_empty_model(mtype):
    """No particles: steps, downloads, side outputs and metrics all succeed and change nothing."""
    mp = abi.model_params(0, 1024, (1.0, 1.0, 1.0), (20, 20, 20), 3)
    with model.CreateModel(mtype, mp) as m:
        assert m.nbParticles() == 0
        m.update(3)
        assert m.download(abi.BUF_POS, 0).shape[0] == 0
        m.synchronize()
        if mtype != abi.BOIDS:
            mt = m.metrics()
            assert mt.meanDensityError == 0.0 and mt.kineticEnergy == 0.0
        m.fillGridDetector()
        assert not np.any(m.download(abi.BUF_GRID_DETECTOR, m.constants().numCells))
