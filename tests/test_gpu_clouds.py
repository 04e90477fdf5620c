"""Clouds step parity (Clouds::update, physics/ocl/Clouds.cpp:503-610)."""
import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, scenes

from helpers import REL_BOX, assert_close_by_id, box_size, clouds_model, gpu_state

pytestmark = pytest.mark.gpu


def _compare(m, sc, iters, steps):
    c = oracle.derive_constants(abi.CLOUDS, sc["model_params"])
    L = box_size(sc["model_params"])
    fp, cp = sc["fluid_params"], sc["cloud_params"]
    for _ in range(steps):
        st = gpu_state(m, abi.CLOUDS)
        ost = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
        oracle.clouds_step(c, fp, cp, sc["env"], sc["ground"], iters, ost)
        m.update(1)
        g = gpu_state(m, abi.CLOUDS)
        assert np.array_equal(g["id"], ost["id"])
        assert np.array_equal(m.download(abi.BUF_CELL_ID), ost["cellId"])
        assert_close_by_id(g["id"], g["pos"], ost["id"], ost["pos"], REL_BOX * L, "pos")
        assert_close_by_id(g["id"], g["vel"], ost["id"], ost["vel"], REL_BOX * L / fp.timeStep, "vel")
        assert_close_by_id(g["id"], g["temp"], ost["id"], ost["temp"], 1e-3, "temp")
        assert_close_by_id(g["id"], g["vapor"], ost["id"], ost["vapor"], 1e-4, "vapor")
        assert_close_by_id(g["id"], g["cloud"], ost["id"], ost["cloud"], 1e-4, "cloud")
        assert g["cloud"].min() >= 0 and g["vapor"].min() >= 0  # clouds.cl:236-237


def test_clouds_init_matches_oracle():
    sc = scenes.clouds_cumulus(n=8192)
    c = oracle.derive_constants(abi.CLOUDS, sc["model_params"])
    with clouds_model(sc) as m:
        g = gpu_state(m, abi.CLOUDS)
        ost = oracle.new_state(8192, c, abi.CLOUDS)
        ost["pos"][:] = sc["pos"]
        oracle.clouds_init(c, sc["cloud_params"], sc["env"], sc["ground"], ost)
        assert np.allclose(g["temp"], ost["temp"], rtol=0, atol=1e-3)
        assert np.allclose(g["vapor"], ost["vapor"], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("noise", [True, False])
def test_clouds_step_parity(noise):
    sc = scenes.clouds_cumulus(n=16384, noise=noise)
    with clouds_model(sc, iters=1) as m:
        _compare(m, sc, 1, steps=4)


def test_clouds_two_iterations_and_reference_env():
    sc = scenes.clouds_cumulus(n=8192, noise=False, seed=2)
    sc["env"] = scenes.cloud_env_reference()
    with clouds_model(sc, iters=2) as m:
        _compare(m, sc, 2, steps=3)
