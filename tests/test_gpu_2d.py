"""2D models (Model::setDimension, physics/Model.hpp:109-113) against the oracle.

A 2D model keeps its particles in the x = 0 plane.  Boids use the 9-cell 2D rules kernel
(boids.cl:137-221, picked at Boids.cpp:346-349); fluids and clouds run their 3D kernels with
dim = 2 in the parameters (the clouds wind drift in x is multiplied by dim - 2,
clouds.cl:951).  The reset cases are the reference's 2D ones (Fluids.cpp:287-333,
Boids.cpp:291-299, Clouds.cpp:417-446)."""
import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, model, scenes

from helpers import REL_BOX, assert_close_by_id, box_size, gpu_state

pytestmark = pytest.mark.gpu


def test_boids_2d_case_and_steps_match_the_oracle():
    import ctypes as C
    from realtimeparticles_gb300._lib import call
    mp = abi.model_params(4096, 4096, (2.0, 2.0, 2.0), (40, 40, 40), 2, abi.CASE_BOIDS_SMALL)
    with model.Boids(mp) as m:
        m.setCase(abi.CASE_BOIDS_SMALL)
        m.reset()
        assert m.nbParticles() == 512
        ref = scenes.boids_plane(n=512, box=2.0)
        pos = m.download(abi.BUF_POS)
        assert np.allclose(pos[:512], ref["pos"], atol=1e-6)
        assert np.all(pos[:512, 0] == 0.0)
        c = m.constants()
        bp = abi.BoidsParams()
        call("rtp_boids_params_default", C.byref(bp))
        dt, L = 0.1, box_size(mp)  # Boids.cpp:334 time step, the reset value
        # On the exact circular grid the neighbour sums cancel to rounding noise, whose
        # direction normalize() then amplifies: compare the steps from a jittered plane.
        rng = np.random.default_rng(4)
        jit = pos[:512].copy()
        jit[:, 1:3] += rng.uniform(-0.01, 0.01, (512, 2)).astype(np.float32)
        m.upload(abi.BUF_POS, jit)
        m.upload(abi.BUF_VEL, jit)
        for _ in range(4):
            st = gpu_state(m, abi.BOIDS)
            st["acc"] = np.zeros_like(st["pos"])
            ost = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
            oracle.boids_step(c, bp, dt, abi.BOUNCING_WALL, ost, dim=2)
            m.update(1)
            g = gpu_state(m, abi.BOIDS)
            assert np.array_equal(m.download(abi.BUF_CELL_ID), ost["cellId"])
            assert np.array_equal(g["id"], ost["id"])
            assert_close_by_id(g["id"], g["pos"], ost["id"], ost["pos"], REL_BOX * L, "pos")
            assert_close_by_id(g["id"], g["vel"], ost["id"], ost["vel"], REL_BOX * L / dt, "vel")
            assert np.allclose(m.download(abi.BUF_ACC), ost["acc"], rtol=1e-4, atol=1e-4)
        assert np.all(m.download(abi.BUF_POS)[:, 0] == 0.0)


def test_fluids_2d_dam_steps_match_the_oracle():
    mp = abi.model_params(8192, 8192, (1.0, 1.0, 1.0), (40, 40, 40), 3, abi.CASE_FLUIDS_DAM)
    with model.Fluids(mp) as m:
        m.setCase(abi.CASE_FLUIDS_DAM)
        m.setDimension(2)
        assert m.nbParticles() == 4096
        pos = m.download(abi.BUF_POS)
        assert np.all(pos[:, 0] == 0.0)
        # Rectangular grid (64 x 64) from (0, -0.5, -0.5) to (0, 0, 0), y-major.
        iy, iz = np.meshgrid(np.arange(64), np.arange(64), indexing="ij")
        assert np.allclose(pos[:, 1], -0.5 + iy.ravel() * np.float32(0.5 / 64), atol=1e-7)
        assert np.allclose(pos[:, 2], -0.5 + iz.ravel() * np.float32(0.5 / 64), atol=1e-7)
        assert m.fluidParams().dim == 2
        c = m.constants()
        # The reference's default rest density does not suit this lattice (spacing 1/128):
        # use the planar lattice's own poly6 sum, with the coefficients mapped as for 3D.
        d = 0.5 / 64
        k = np.arange(-4, 5)
        r2 = ((k[:, None] * d) ** 2 + (k[None, :] * d) ** 2).ravel()
        h2 = c.effectRadius ** 2
        rho0 = float(np.sum(c.poly6Coeff * np.clip(h2 - r2, 0, None) ** 3))
        fp = scenes.fluid_params(rho0)
        fp.dim = 2
        m.setFluidParams(fp)
        m.setJacobiIterations(2)
        rng = np.random.default_rng(8)
        jit = pos.copy()
        jit[:, 1:3] += rng.uniform(-0.01 * d, 0.01 * d, (pos.shape[0], 2)).astype(np.float32)
        m.upload(abi.BUF_POS, jit)
        for _ in range(4):
            st = gpu_state(m, abi.FLUIDS)
            ost = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
            oracle.fluids_step(c, fp, 2, ost)
            m.update(1)
            g = gpu_state(m, abi.FLUIDS)
            assert np.array_equal(g["id"], ost["id"])
            assert_close_by_id(g["id"], g["pos"], ost["id"], ost["pos"], REL_BOX, "pos")
            assert_close_by_id(g["id"], g["vel"], ost["id"], ost["vel"], REL_BOX / fp.timeStep, "vel")


def test_dimension_switch_resets_to_the_case():
    mp = abi.model_params(131072, 131072, (1.0, 1.0, 1.0), (40, 40, 40), 3, abi.CASE_FLUIDS_DAM)
    with model.Fluids(mp) as m:
        m.setCase(abi.CASE_FLUIDS_DAM)
        m.setDimension(2)
        assert m.nbParticles() == 4096 and m.dimension() == 2
        m.setDimension(3)
        assert m.nbParticles() == 131072 and m.dimension() == 3
        assert m.fluidParams().dim == 3
