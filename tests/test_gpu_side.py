"""Headless side outputs (render-only in the reference) against the oracle, bit for bit:
fluid colours from the density, float-quantity colours, camera distances and the draw
order, the grid occupancy detector."""
import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, scenes

from helpers import fluids_model

pytestmark = pytest.mark.gpu


def test_side_outputs_match_the_oracle():
    sc = scenes.dam_break(lattice=(16, 32, 32), max_n=20000)
    with fluids_model(sc, 3) as m:
        m.update(20)
        n = m.nbParticles()
        c = m.constants()
        fp = m.fluidParams()
        m.fillFluidColor()
        rho = m.download(abi.BUF_DENSITY)
        assert np.array_equal(m.download(abi.BUF_COLOR), oracle.fill_fluid_color(rho, fp.restDensity))
        lo, hi = float(rho.min()), float(np.median(rho))
        m.fillColorFloat(abi.BUF_DENSITY, lo, hi)
        assert np.array_equal(m.download(abi.BUF_COLOR), oracle.fill_color_float(rho, lo, hi))
        cam = np.array([0.2, 1.5, -3.0], np.float32)
        m.fillCameraOrder(cam)
        pos = m.download(abi.BUF_POS, m.maxNbParticles())
        dist = m.download(abi.BUF_CAMERA_DIST)
        assert dist.shape[0] == 20000
        assert np.array_equal(dist, oracle.fill_camera_dist(pos, n, cam))
        assert np.array_equal(m.download(abi.BUF_DRAW_ORDER), np.argsort(dist, kind="stable"))
        m.fillGridDetector()
        assert np.array_equal(m.download(abi.BUF_GRID_DETECTOR), oracle.fill_grid_detector(c, pos[:n]))
