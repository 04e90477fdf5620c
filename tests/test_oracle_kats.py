"""Known-answer tests of the CPU oracle (the checker), from mathematics and from the
reference's own definitions.  The reference ships no tests or fixtures, so these pin
the oracle's grid, sort and SPH arithmetic independently of any GPU code."""
import numpy as np
import pytest

from realtimeparticles_gb300 import abi, scenes


def _fluid_consts(oracle_mod, box=1.0, res=40, n=1024):
    mp = abi.model_params(n, n, (box, box, box), (res, res, res))
    return oracle_mod.derive_constants(abi.FLUIDS, mp)


def test_constants_follow_reference_formulas(oracle_mod):
    # Fluids.cpp:104-119 with box 10, res 30 (the reference's default geometry).
    c = _fluid_consts(oracle_mod, box=10.0, res=30)
    h = np.float32(10.0) / np.float32(30.0)
    assert c.effectRadius == pytest.approx(float(h), rel=1e-7)
    assert c.absWall[0] == 5.0 and c.gridRes[1] == 30 and c.numCells == 27000
    assert c.maxPartsInCell == 100 and c.maxVel == 30.0
    pi_f = np.float32(3.1415927)
    poly6 = np.float32(315.0) / (np.float32(64.0) * pi_f * np.float32(h) ** np.float32(9))
    assert c.poly6Coeff == pytest.approx(float(poly6), rel=1e-6)
    spiky = np.float32(15.0) / (pi_f * np.float32(h) ** np.float32(6))
    assert c.spikyCoeff == pytest.approx(float(spiky), rel=1e-6)
    # Boids: cap 3000 (Boids.cpp:78), EFFECT_RADIUS_SQUARED = (box/res)^2 (Boids.cpp:104).
    mp = abi.model_params(8, 8, (2.0, 2.0, 2.0), (40, 40, 40))
    cb = oracle_mod.derive_constants(abi.BOIDS, mp)
    assert cb.maxPartsInCell == 3000
    assert cb.effectRadiusSquared == pytest.approx(0.0025, rel=1e-6)


def test_key_bound_covers_wall_alias(oracle_mod):
    c = _fluid_consts(oracle_mod)
    # Every axis exactly at +W gives index == GRID_RES (grid.cl:33-35).
    top = np.array([[0.5, 0.5, 0.5, 0.0]], np.float32)
    k = oracle_mod.fill_cell_ids(c, top)[0]
    assert k == 40 * 40 * 40 + 40 * 40 + 40
    assert c.keyBound == k + 1 and c.keyBits == 17


def test_cell_index_of_walls_and_clamp(oracle_mod):
    c = _fluid_consts(oracle_mod)
    pts = np.array([[-0.5, -0.5, -0.5, 0], [-7.0, -9.0, -100.0, 0], [0.5, 0.0, -0.5, 0], [np.inf, -np.inf, 0.0, 0],
                    [0.0, 0.0, 0.0, 0]], np.float32)
    k = oracle_mod.fill_cell_ids(c, pts)
    assert k[0] == 0 and k[1] == 0  # clamped to -W
    assert k[2] == 40 * 1600 + 20 * 40 + 0  # x at +W aliases to x index 40
    assert k[3] == 40 * 1600 + 0 + 20
    assert k[4] == 20 * 1600 + 20 * 40 + 20


def test_stable_sort_matches_numpy(oracle_mod):
    rng = np.random.default_rng(1)
    for n, hi in [(0, 5), (1, 5), (1000, 3), (5000, 70000), (4096, 1)]:
        keys = rng.integers(0, hi, n, dtype=np.uint32)
        sk, perm = oracle_mod.stable_sort(keys)
        ref = np.argsort(keys, kind="stable")
        assert np.array_equal(perm, ref) and np.array_equal(sk, keys[ref])


def _brute_table(sk, nc, cap):
    # grid.cl:91-152 restated with plain loops.
    t = np.zeros((nc, 2), np.int64)
    t[:, 0] = 1
    n = len(sk)
    for i in range(1, n):
        if sk[i] < nc and sk[i] != sk[i - 1]:
            t[sk[i], 0] = i
    for i in range(n):
        right = sk[i + 1] if i + 1 < n else -1
        if sk[i] < nc and sk[i] != right:
            t[sk[i], 1] = i
    for c in range(nc):
        s, e = t[c]
        if e > s:
            t[c, 1] = s + min(e - s, cap)
    return t


def test_cell_table_quirks(oracle_mod):
    c = _fluid_consts(oracle_mod, res=4)  # 64 cells, cap 100
    # Cell 0 holds sorted index 0 and 1: start stays 1 (ID 0 never starts a cell).
    sk = np.array([0, 0, 3, 3, 3, 5, 64, 70], np.uint32)
    t = oracle_mod.cell_table(c, sk)
    assert tuple(t[0]) == (1, 1) and tuple(t[3]) == (2, 4) and tuple(t[5]) == (5, 5)
    assert tuple(t[1]) == (1, 0)
    # A single particle in the first cell is invisible: (1, 0).
    t = oracle_mod.cell_table(c, np.array([2, 7, 7], np.uint32))
    assert tuple(t[2]) == (1, 0) and tuple(t[7]) == (1, 2)
    # Cap of NUM_MAX_PARTS_IN_CELL (+1 because end is inclusive).
    sk = np.array([1] + [9] * 300, np.uint32)
    t = oracle_mod.cell_table(c, sk)
    assert tuple(t[9]) == (1, 101)
    rng = np.random.default_rng(2)
    sk = np.sort(rng.integers(0, 80, 3000).astype(np.uint32))
    assert np.array_equal(oracle_mod.cell_table(c, sk), _brute_table(sk, 64, 100))


def test_poly6_lattice_sum_is_rest_density(oracle_mod):
    sc = scenes.dam_break(lattice=(12, 12, 12), jitter=0.0)
    c = oracle_mod.derive_constants(abi.FLUIDS, sc["model_params"])
    pos = sc["pos"]
    keys = oracle_mod.fill_cell_ids(c, pos)
    sk, perm = oracle_mod.stable_sort(keys)
    t = oracle_mod.cell_table(c, sk)
    sp = np.ascontiguousarray(pos[perm])
    rho = oracle_mod.fld_density(c, sc["fluid_params"], sp, t)
    # Interior particle (far from the lattice surface): density == lattice sum (double).
    centre = np.argmin(np.linalg.norm(sp[:, :3] - sp[:, :3].mean(0), axis=1))
    assert rho[centre] == pytest.approx(sc["fluid_params"].restDensity, rel=2e-5)
    # Continuum limit: sum of poly6 over a fine lattice -> 1/d^3.
    fine = scenes.lattice_rest_density(0.0025, 0.025)
    assert fine * 0.0025 ** 3 == pytest.approx(1.0, rel=2e-3)


def test_neighbour_search_complete_vs_brute_force(oracle_mod):
    rng = np.random.default_rng(3)
    n = 3000
    mp = abi.model_params(n, n, (1.0, 1.0, 1.0), (40, 40, 40))
    c = oracle_mod.derive_constants(abi.FLUIDS, mp)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(-0.3, 0.3, (n, 3))
    keys = oracle_mod.fill_cell_ids(c, pos)
    sk, perm = oracle_mod.stable_sort(keys)
    t = oracle_mod.cell_table(c, sk)
    sp = np.ascontiguousarray(pos[perm])
    fp = scenes.fluid_params(1000.0)
    rho = oracle_mod.fld_density(c, fp, sp, t)
    h = np.float64(c.effectRadius)
    d2 = ((sp[:, None, :3].astype(np.float64) - sp[None, :, :3]) ** 2).sum(-1)
    w = np.where(d2 < h * h, c.poly6Coeff * (h * h - d2) ** 3, 0.0)
    # Sorted index 0 is excluded by the fillStartCell quirk (unless alone, then invisible).
    w[:, 0] = 0.0
    w[0, 0] = 0.0
    brute = w.sum(1)
    assert np.allclose(rho[1:], brute[1:], rtol=2e-5, atol=1e-3)


def test_gradient_antisymmetry_through_corrections(oracle_mod):
    # Two isolated particles: Δp_i = -Δp_j (gradSpiky(-v) = -gradSpiky(v), grad(0) = 0).
    c = _fluid_consts(oracle_mod)
    fp = scenes.fluid_params(1000.0)
    fp.isArtPressureEnabled = 0
    pred = np.array([[0.1, 0.1, 0.1, 0], [0.112, 0.105, 0.1, 0], [0.3, 0.3, 0.3, 0], [0.3, 0.31, 0.3, 0]], np.float32)
    keys = oracle_mod.fill_cell_ids(c, pred)
    sk, perm = oracle_mod.stable_sort(keys)
    t = oracle_mod.cell_table(c, sk)
    sp = np.ascontiguousarray(pred[perm])
    lam = np.ones(4, np.float32)
    corr = oracle_mod.fld_correction(c, fp, sp, lam, t)
    # Sorted index 0 is invisible to others (quirk); check the pair that does not contain it.
    i, j = [k for k in range(4) if k != 0 and np.linalg.norm(sp[k, :3] - sp[0, :3]) > 0.05][:2]
    assert np.allclose(corr[i, :3], -corr[j, :3], rtol=1e-6, atol=1e-12)
    assert np.abs(corr[i, :3]).max() > 0
