"""PBF step parity (Fluids::update, physics/ocl/Fluids.cpp:400-457) of the CUDA library
against the oracle: every step starts from the same state on both; integer outputs
(cell keys, sorted order, table) must match bit for bit, floats within the tolerance
1e-5 x box (positions) and 1e-5 x box / dt (velocities)."""
import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, scenes

from helpers import REL_BOX, assert_close_by_id, box_size, fluids_model, gpu_state

pytestmark = pytest.mark.gpu


def _step_and_compare(m, c, fp, iters, steps=1, check_table=True):
    L = box_size(m._params)
    worst = 0.0
    for _ in range(steps):
        st = gpu_state(m, abi.FLUIDS)
        ost = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
        oracle.fluids_step(c, fp, iters, ost)
        m.update(1)
        g = gpu_state(m, abi.FLUIDS)
        # Bit-exact integer work: sorted keys and the permutation (ids in sorted order).
        assert np.array_equal(m.download(abi.BUF_CELL_ID), ost["cellId"])
        assert np.array_equal(g["id"], ost["id"])
        if check_table:
            assert np.array_equal(m.download(abi.BUF_CELL_TABLE), ost["table"])
        worst = max(worst, assert_close_by_id(g["id"], g["pos"], ost["id"], ost["pos"], REL_BOX * L, "pos"))
        assert_close_by_id(g["id"], g["vel"], ost["id"], ost["vel"], REL_BOX * L / fp.timeStep, "vel")
        if iters:
            rho = m.download(abi.BUF_DENSITY)
            assert np.allclose(rho, ost["density"], rtol=1e-4, atol=1e-3 * fp.restDensity)
    return worst


def test_dam_break_16k_step_parity():
    sc = scenes.dam_break()
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    with fluids_model(sc, 3) as m:
        _step_and_compare(m, c, sc["fluid_params"], 3, steps=8)


@pytest.mark.parametrize("iters", [0, 1, 2])
def test_iteration_counts(iters):
    sc = scenes.dam_break(lattice=(8, 16, 16))
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    with fluids_model(sc, iters) as m:
        _step_and_compare(m, c, sc["fluid_params"], iters, steps=3)


@pytest.mark.parametrize("vort,ap", [(0, 1), (1, 0), (0, 0)])
def test_switches(vort, ap):
    sc = scenes.dam_break(lattice=(8, 16, 16))
    fp = sc["fluid_params"]
    fp.isVorticityConfEnabled = vort
    fp.isArtPressureEnabled = ap
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    with fluids_model(sc, 2, fp) as m:
        _step_and_compare(m, c, fp, 2, steps=3)


@pytest.mark.parametrize("lattice,spare", [((8, 16, 16), 5000), ((16, 32, 64), 33000)])
def test_ragged_count_and_spare_capacity(lattice, spare):
    # N not a multiple of the sort tile nor of the particles per warp of the lane-group sweeps
    # (4 with 8 lanes at 2k, 8 with 4 lanes at 33k), maxNb > N: the tail stays untouched.
    sc = scenes.dam_break(lattice=lattice, max_n=spare)
    n = lattice[0] * lattice[1] * lattice[2] - 37
    sc["pos"] = sc["pos"][:n].copy()
    sc["vel"] = sc["vel"][:n].copy()
    sc["model_params"].currNbParticles = n
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    with fluids_model(sc, 2) as m:
        assert m.nbParticles() == n
        _step_and_compare(m, c, sc["fluid_params"], 2, steps=2)
        tail = m.download(abi.BUF_POS, spare)[n:]
        assert np.all(tail == 0)


def test_dam_break_131k_first_step_parity():
    sc = scenes.dam_break(lattice=(32, 64, 64))
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    with fluids_model(sc, 3) as m:
        _step_and_compare(m, c, sc["fluid_params"], 3, steps=2)


def test_dam_break_1m_first_step_parity():
    """2^20 particles: the full sweeps record their hits through the bit-mask filter (the path
    from 1M particles on)."""
    sc = scenes.dam_break(lattice=(64, 128, 128), box=2.0)
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    with fluids_model(sc, 3) as m:
        _step_and_compare(m, c, sc["fluid_params"], 3, steps=1)


def test_long_run_statistics_16k():
    """500 independent steps on each side (config 0): density error, kinetic energy
    and the neighbour-count histogram must agree (the trajectories themselves diverge)."""
    sc = scenes.dam_break()
    fp = sc["fluid_params"]
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    ost = oracle.new_state(sc["pos"].shape[0], c)
    ost["pos"][:] = sc["pos"]
    ost["vel"][:] = sc["vel"]
    steps = 500
    for _ in range(steps):
        oracle.fluids_step(c, fp, 3, ost)
    om = oracle.fluid_metrics(c, fp, ost["predPos"], ost["vel"], ost["table"])
    with fluids_model(sc, 3) as m:
        m.update(steps)
        gm = m.metrics()
    assert np.isfinite(gm.kineticEnergy) and gm.kineticEnergy > 0
    assert abs(gm.meanDensityError - om.meanDensityError) <= 0.25 * om.meanDensityError + 2e-3
    assert gm.kineticEnergy == pytest.approx(om.kineticEnergy, rel=0.15)
    hg = np.array(gm.neighbourHist, np.float64)
    ho = np.array(om.neighbourHist, np.float64)
    tv = 0.5 * np.abs(hg / hg.sum() - ho / ho.sum()).sum()
    assert tv < 0.08, tv
    assert gm.meanNeighbours == pytest.approx(om.meanNeighbours, rel=0.05)


def test_pair_lists_fit_in_the_dam_break():
    """The recorded pair lists (64 per particle, 32 per x-plane) never overflow in the
    131k dam break over 100 steps (an overflow falls back to a 27-cell search: correct
    but slow, so this guards the performance path)."""
    sc = scenes.dam_break(lattice=(32, 64, 64))
    with fluids_model(sc, 3) as m:
        for _ in range(5):
            m.update(20)
            mt = m.metrics()
            assert mt.pairListOverflows == 0, (mt.pairListOverflows, mt.pairListMax)
            assert 0 < mt.pairListMax <= 64


@pytest.mark.parametrize("iters,vort", [(1, 0), (0, 1), (2, 1)])
@pytest.mark.parametrize("lattice", [(8, 16, 16), (16, 32, 72), (24, 32, 72)])
def test_pair_list_overflow_parity(lattice, iters, vort):
    """A lattice compressed to 0.75 of its spacing and centred in the box puts about 79
    particles within h of an interior particle: the sweep that records the pair lists
    (density with one iteration, vorticity with none) finds more pairs than a list holds and
    those particles fall back to the 27-cell search.  Covers the sweeps with 8 lanes per
    particle (2k particles), 4 lanes (37k) and one lane (55k); random velocities make the
    vorticity non-zero.  The block starts well away from the walls: a compressed block
    pressed into a wall or corner is ill-conditioned, not a parity case, since clamped pairs
    at distance 0 (gradient 0) and 1e-7 (gradient of full size) lie one rounding apart."""
    sc = scenes.dam_break(lattice=lattice)
    xyz = sc["pos"][:, :3]
    mid = 0.5 * (xyz.min(axis=0) + xyz.max(axis=0))
    sc["pos"][:, :3] = (xyz - mid) * np.float32(0.75)
    rng = np.random.default_rng(5)
    sc["vel"][:, :3] = rng.normal(0.0, 0.05, size=(len(xyz), 3)).astype(np.float32)
    fp = sc["fluid_params"]
    fp.isVorticityConfEnabled = vort
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    with fluids_model(sc, iters, fp) as m:
        _step_and_compare(m, c, fp, iters, steps=1)
        if iters + vort == 1:  # the lists come from the compressed start
            mt = m.metrics()
            assert mt.pairListOverflows > 0, (mt.pairListOverflows, mt.pairListMax)
        _step_and_compare(m, c, fp, iters, steps=1)
