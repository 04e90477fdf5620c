"""The CUDA path against golden outputs of the reference's own kernels (tests/golden):
three steps from the fixture's inputs, compared by particle id within 3 x 1e-5 x box
(positions) and 3 x 1e-5 x box / dt (velocities); the constants the library derives must
equal the fixture's."""
import ctypes as C
import os

import numpy as np
import pytest

from realtimeparticles_gb300 import abi, model, scenes

from helpers import REL_BOX, assert_close_by_id, boids_model, clouds_model, fluids_model

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _struct(cls, arr):
    s = cls()
    C.memmove(C.addressof(s), arr.tobytes(), C.sizeof(cls))
    return s


def test_fluids_matches_reference_fixture():
    g = np.load(os.path.join(GOLD, "fluids_3steps.npz"))
    sc = scenes.dam_break(lattice=(8, 16, 16), seed=5)
    c = _struct(abi.GridConstants, g["consts"])
    assert abi.struct_to_dict(model.get_constants(abi.FLUIDS, sc["model_params"])) == abi.struct_to_dict(c)
    fp = _struct(abi.FluidParams, g["params"])
    sc["pos"], sc["vel"] = g["pos0"], g["vel0"]
    with fluids_model(sc, int(g["iters"][0]), fp) as m:
        m.update(3)
        ids = m.download(abi.BUF_ID)
        assert_close_by_id(ids, m.download(abi.BUF_POS), g["id"], g["pos"], 3 * REL_BOX, "pos")
        assert_close_by_id(ids, m.download(abi.BUF_VEL), g["id"], g["vel"], 3 * REL_BOX / fp.timeStep, "vel")


def test_boids_matches_reference_fixture():
    g = np.load(os.path.join(GOLD, "boids_3steps.npz"))
    sb = scenes.boids_cloud(n=3000, seed=6)
    sb["pos"], sb["vel"] = g["pos0"], g["vel0"]
    dt = float(g["dt"][0])
    with boids_model(sb, dt=dt) as m:
        m.update(3)
        ids = m.download(abi.BUF_ID)
        assert_close_by_id(ids, m.download(abi.BUF_POS), g["id"], g["pos"], 3 * REL_BOX * 2.0, "pos")
        assert_close_by_id(ids, m.download(abi.BUF_VEL), g["id"], g["vel"], 3 * REL_BOX * 2.0 / dt, "vel")


def test_clouds_matches_reference_fixture():
    g = np.load(os.path.join(GOLD, "clouds_3steps.npz"))
    scc = scenes.clouds_cumulus(n=3000, noise=False, seed=7)
    scc["env"] = scenes.cloud_env_reference()
    scc["fluid_params"] = _struct(abi.FluidParams, g["fparams"])
    scc["cloud_params"] = _struct(abi.CloudParams, g["cparams"])
    scc["pos"], scc["vel"] = g["pos0"], g["vel0"]
    with clouds_model(scc, 1) as m:
        assert np.allclose(m.download(abi.BUF_TEMP), g["temp0"], atol=1e-3)
        m.update(3)
        ids = m.download(abi.BUF_ID)
        L = 2.0
        assert_close_by_id(ids, m.download(abi.BUF_POS), g["id"], g["pos"], 3 * REL_BOX * L, "pos")
        assert_close_by_id(ids, m.download(abi.BUF_TEMP), g["id"], g["temp"], 1e-2, "temp")
        assert_close_by_id(ids, m.download(abi.BUF_CLOUD), g["id"], g["cloud"], 1e-3, "cloud")
