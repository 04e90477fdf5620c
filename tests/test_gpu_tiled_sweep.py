"""The lambda sweep tiled by bricks of cells (rtp_tuning.tiledSweeps) against the one-thread-
per-particle sweep and the oracle (fluids.cl:101-193 through Fluids.cpp:427-439).

The tiled sweep visits the same candidates in the same order and records the same pair list;
its sums can differ from the one-lane sweep's in the last bit because the compiler contracts
the SPH arithmetic into fused multiply-adds differently in the two kernels (on the first Jacobi
iteration of the 131k dam break every density is bit-identical and about 1 % of the lambdas
differ by an ulp).  So the two are compared step by step within the step tolerance of the
oracle tests (1e-5 x box).

Cases: the 131,072-particle dam break (the benchmark workload); a denser lattice whose bricks
overflow the shared-memory halo (those bricks' particles take the global path); particles
pressed onto the +x, +y and +z walls (cell keys aliased past the grid and particles whose
current cell left their brick); a grid that is not a multiple of the brick (partial bricks);
and, below the tiled sweep's size threshold, the untouched path."""
import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, scenes

from helpers import REL_BOX, assert_close_by_id, box_size, fluids_model, gpu_state

pytestmark = pytest.mark.gpu


def _compare_tiled(sc, steps, iters=3, lanes=4, warm=0):
    """Steps a tiled and an untiled model side by side from the same state: after every step the
    tiled one must agree with the untiled one within the step tolerance."""
    L = box_size(sc["model_params"])
    dt = sc["fluid_params"].timeStep
    with fluids_model(sc, iters) as a, fluids_model(sc, iters) as b:
        a.setTuning(lanes, 1.0, tiled=0)
        b.setTuning(lanes, 1.0, tiled=1)
        assert a.tuning()[2] == 0 and b.tuning()[2] == 1
        def copy_state():  # b takes a's particles (positions, velocities and ids, in a's order)
            for buf in (abi.BUF_POS, abi.BUF_VEL, abi.BUF_ID):
                b.upload(buf, a.download(buf))

        if warm:
            a.update(warm)
            copy_state()
        for step in range(steps):
            a.update(1)
            b.update(1)
            ga, gb = gpu_state(a, abi.FLUIDS), gpu_state(b, abi.FLUIDS)
            assert_close_by_id(ga["id"], ga["pos"], gb["id"], gb["pos"], REL_BOX * L, "pos step %d" % step)
            assert_close_by_id(ga["id"], ga["vel"], gb["id"], gb["vel"], REL_BOX * L / dt, "vel step %d" % step)
            copy_state()  # the next step restarts both from the untiled state


def test_tiled_sweep_matches_the_plain_sweep_at_131k():
    _compare_tiled(scenes.dam_break(lattice=(32, 64, 64)), 3, warm=30)


def test_tiled_sweep_matches_the_oracle():
    sc = scenes.dam_break(lattice=(32, 64, 64), seed=4)
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    fp = sc["fluid_params"]
    L = box_size(sc["model_params"])
    with fluids_model(sc, 3) as m:
        m.setTuning(4, 1.0, tiled=1)
        m.update(5)
        for _ in range(2):
            st = gpu_state(m, abi.FLUIDS)
            oracle.fluids_step(c, fp, 3, st)
            m.update(1)
            g = gpu_state(m, abi.FLUIDS)
            assert np.array_equal(g["id"], st["id"])
            assert_close_by_id(g["id"], g["pos"], st["id"], st["pos"], REL_BOX * L, "pos")
            assert_close_by_id(g["id"], g["vel"], st["id"], st["vel"], REL_BOX * L / fp.timeStep, "vel")


def test_tiled_sweep_with_overflowing_halos():
    """Spacing 0.7 d packs about 23 particles per cell: many bricks hold more halo particles
    than the shared-memory stage, and their particles take the global path."""
    sc = scenes.dam_break(lattice=(48, 48, 48), d=0.0125)
    sc["pos"][:, :3] = (sc["pos"][:, :3] + 0.49) * 0.7 - 0.49  # squeeze towards the -x -y -z corner
    _compare_tiled(sc, 3)


def test_tiled_sweep_with_particles_on_the_far_walls():
    """A quarter of the particles sit exactly on +W_x, +W_y or +W_z: their cell keys alias
    past the grid or into the next row, and their current cell is outside the brick that
    stores them."""
    sc = scenes.dam_break(lattice=(32, 64, 64), seed=2)
    W = 0.5
    pos = sc["pos"]
    rng = np.random.default_rng(0)
    for axis in range(3):
        sel = rng.choice(pos.shape[0], pos.shape[0] // 12, replace=False)
        pos[sel, axis] = W
    _compare_tiled(sc, 3)


def test_tiled_sweep_on_a_grid_that_is_not_a_multiple_of_the_brick():
    """Box 0.95 wide: 38 cells per axis, the last bricks two cells deep."""
    sc = scenes.dam_break(lattice=(32, 48, 48), box=0.95)
    assert sc["model_params"].gridRes[0] == 38
    _compare_tiled(sc, 3, lanes=2, warm=10)


def test_small_scenes_keep_the_group_sweep():
    sc = scenes.dam_break(lattice=(16, 32, 32))  # 16,384 particles: below the threshold
    _compare_tiled(sc, 3)
