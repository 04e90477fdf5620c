"""The reset cases' initial particles against the reference's own lattice code.

`rtp_reset` builds each case's positions on the host (Fluids::initFluidsParticles,
physics/ocl/Fluids.cpp:273-398; Boids::initBoidsParticles, physics/ocl/Boids.cpp:277-321) from
its own restatement of Geometry::Generate3DGrid / Generate2DGrid.  Here every deterministic case
is compared bit for bit with the reference's utils/Geometry.cpp itself, compiled for the CPU into
oracle/_ref (oracle/ref/build_ref.py), called with the case's arguments as the reference's
initialisation passes them (start/end corners, subdivisions of utils/Parameters.hpp:89-98).
The clouds cases are left out: the reference draws them with an unseeded rand().
"""
import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, model

pytestmark = pytest.mark.gpu

# utils/Parameters.hpp:89-98: particle count -> (subdiv2D, subdiv3D)
SUBDIV = {512: ((32, 16), (8, 8, 8)), 4096: ((64, 64), (16, 16, 16)), 16384: ((128, 128), (32, 32, 16)),
          65536: ((256, 256), (64, 32, 32)), 131072: ((256, 512), (64, 64, 32))}


@pytest.fixture(scope="module")
def geometry():
    if not oracle.ref_geometry_available():
        pytest.skip("the reference's Geometry.cpp is not compiled into oracle/_ref (no reference sources)")
    return oracle


def _reference_case(g, mtype, case, dim, box):
    """Positions the reference generates for the case, in its order."""
    bx, by, bz = (np.float32(b) for b in box)
    f = np.float32
    if mtype == abi.FLUIDS and dim == 3:
        if case == abi.CASE_FLUIDS_DAM:  # Fluids.cpp:341-346
            return g.ref_generate_3d_grid("box", SUBDIV[131072][1], (bx / f(-2), by / f(-2), bz / f(-2)),
                                          (bx / f(2), 0, 0))
        if case == abi.CASE_FLUIDS_BOMB:  # :347-352
            return g.ref_generate_3d_grid("sphere", SUBDIV[65536][1], (bx / f(-6), by / f(-6), bz / f(-6)),
                                          (bx / f(6), by / f(6), bz / f(6)))
        if case == abi.CASE_FLUIDS_DROP:  # :353-380
            a = g.ref_generate_3d_grid("box", SUBDIV[4096][1], (bx / f(-10), f(2) * by / f(10), bz / f(-10)),
                                       (bx / f(10), f(4) * by / f(10), bz / f(10)))
            b = g.ref_generate_3d_grid("box", (64, 16, 64), (bx / f(-2), by / f(-2), bz / f(-2)),
                                       (bx / f(2), by / f(-2.55), bz / f(2)))
            return np.concatenate([a, b])
    if mtype == abi.FLUIDS and dim == 2:
        if case == abi.CASE_FLUIDS_DAM:  # Fluids.cpp:293-298
            return g.ref_generate_2d_grid_yz("rect", SUBDIV[4096][0], (0, by / f(-2), bz / f(-2)), (0, 0, 0))
        if case == abi.CASE_FLUIDS_BOMB:  # :299-304
            return g.ref_generate_2d_grid_yz("rect", SUBDIV[4096][0], (0, by / f(-6), bz / f(-6)),
                                             (0, by / f(6), bz / f(6)))
        if case == abi.CASE_FLUIDS_DROP:  # :305-333
            a = g.ref_generate_2d_grid_yz("rect", SUBDIV[512][0], (0, f(2) * by / f(10), bz / f(-10)),
                                          (0, f(4) * by / f(10), bz / f(10)))
            b = g.ref_generate_2d_grid_yz("rect", (64, 128), (0, by / f(-2), bz / f(-2)), (0, 0, bz / f(2)))
            return np.concatenate([a, b])
    if mtype == abi.BOIDS:
        n = {abi.CASE_BOIDS_SMALL: 512, abi.CASE_BOIDS_MEDIUM: 16384, abi.CASE_BOIDS_LARGE: 65536,
             abi.CASE_BOIDS_XLARGE: 131072}[case]
        if dim == 3:  # Boids.cpp:300-308
            return g.ref_generate_3d_grid("sphere", SUBDIV[n][1], (bx / f(-6), by / f(-6), bz / f(-6)),
                                          (bx / f(6), by / f(6), bz / f(6)))
        # Boids.cpp:291-299
        return g.ref_generate_2d_grid_yz("circle", SUBDIV[n][0], (0, by / f(-6), bz / f(-6)),
                                         (0, by / f(6), bz / f(6)))
    raise AssertionError("no such case")


CASES = [(abi.FLUIDS, abi.CASE_FLUIDS_DAM, 3), (abi.FLUIDS, abi.CASE_FLUIDS_BOMB, 3),
         (abi.FLUIDS, abi.CASE_FLUIDS_DROP, 3), (abi.FLUIDS, abi.CASE_FLUIDS_DAM, 2),
         (abi.FLUIDS, abi.CASE_FLUIDS_BOMB, 2), (abi.FLUIDS, abi.CASE_FLUIDS_DROP, 2),
         (abi.BOIDS, abi.CASE_BOIDS_SMALL, 3), (abi.BOIDS, abi.CASE_BOIDS_MEDIUM, 3),
         (abi.BOIDS, abi.CASE_BOIDS_LARGE, 3), (abi.BOIDS, abi.CASE_BOIDS_XLARGE, 3),
         (abi.BOIDS, abi.CASE_BOIDS_SMALL, 2), (abi.BOIDS, abi.CASE_BOIDS_XLARGE, 2)]


@pytest.mark.parametrize("box", [(10.0, 10.0, 10.0), (7.0, 13.0, 9.0)])
@pytest.mark.parametrize("mtype,case,dim", CASES)
def test_reset_case_positions_equal_the_reference_geometry(geometry, mtype, case, dim, box):
    # ParticleSystemApp::initPhysicsEngine (app/ParticleSystemApp.cpp:275-318): maxNb 131,072
    # (the Drop case needs 69,632 in 3D), a 30^3 grid.
    p = abi.model_params(0, 131072, box, (30, 30, 30), dim, case)
    want = _reference_case(geometry, mtype, case, dim, box)
    with model.CreateModel(mtype, p) as m:
        m.reset()
        n = m.nbParticles()
        # The reference's particle count; the 2D Drop case counts 512 + 4096 particles
        # (Fluids.cpp:329) although its bottom grid has 64 x 128 vertices, all of which it
        # writes to the position buffer (Fluids.cpp:383-386).
        drop2d = mtype == abi.FLUIDS and case == abi.CASE_FLUIDS_DROP and dim == 2
        assert n == (512 + 4096 if drop2d else len(want))
        k = len(want)
        pos = m.download(abi.BUF_POS, m.maxNbParticles())
        assert np.array_equal(pos[:k, :3].view(np.uint32), want.view(np.uint32)), "positions differ in bits"
        assert np.all(pos[:k, 3] == 0)
        assert np.all(np.isinf(pos[k:, :3]))  # slots past the generated vertices at +inf (Fluids.cpp:383-384)
        if mtype == abi.BOIDS:  # the velocity buffer starts as a copy of the positions (Boids.cpp:317-318)
            vel = m.download(abi.BUF_VEL, n)
            assert np.array_equal(vel[:, :3].view(np.uint32), want.view(np.uint32))
