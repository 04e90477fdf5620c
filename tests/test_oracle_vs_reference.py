"""The oracle against the reference's own step kernels (oracle/_ref/libref.so, built by
oracle/ref/build_ref.py from physics/ocl/kernels/*.cl) on fresh seeded scenes: every output
array must match bit for bit.  Skipped when the reference kernels are not built."""
import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, scenes

pytestmark = pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref/libref.so not built")


def _same(a, b):
    return np.array_equal(a.view(np.uint32) if a.dtype == np.float32 else a,
                          b.view(np.uint32) if b.dtype == np.float32 else b)


def _pair(n, c, model):
    return oracle.new_state(n, c, model), oracle.new_state(n, c, model)


@pytest.mark.parametrize("iters,vort,ap", [(3, 1, 1), (0, 1, 1), (1, 0, 1), (2, 1, 0)])
def test_fluids_matches_reference(iters, vort, ap):
    sc = scenes.dam_break(lattice=(8, 16, 12), seed=iters * 10 + vort)
    fp = sc["fluid_params"]
    fp.isVorticityConfEnabled = vort
    fp.isArtPressureEnabled = ap
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    a, b = _pair(sc["pos"].shape[0], c, abi.FLUIDS)
    for st in (a, b):
        st["pos"][:] = sc["pos"]
        st["vel"][:] = sc["vel"]
    for _ in range(4):
        oracle.fluids_step(c, fp, iters, a)
        oracle.ref_fluids_step(c, fp, iters, b)
        for k in ("pos", "vel", "predPos", "density", "lambda", "id", "cellId", "table"):
            assert _same(a[k], b[k]), k


def test_fluids_reference_geometry():
    # The reference's own defaults: box 10, grid 30^3, JSON defaults (Fluids.cpp:52-74).
    n = 4096
    mp = abi.model_params(n, n, (10.0,) * 3, (30,) * 3)
    c = oracle.derive_constants(abi.FLUIDS, mp)
    fp = abi.FluidParams(450.0, 600.0, 0.01, 3, 1, 0.006, 0.001, 4, 1, 0.0004, 0.0001)
    rng = np.random.default_rng(3)
    a, b = _pair(n, c, abi.FLUIDS)
    for st in (a, b):
        st["pos"][:, :3] = rng.uniform(-5.0, 0.0, (n, 3)).astype(np.float32) if st is a else a["pos"][:, :3]
    for _ in range(3):
        oracle.fluids_step(c, fp, 2, a)
        oracle.ref_fluids_step(c, fp, 2, b)
        for k in ("pos", "vel", "id", "table"):
            assert _same(a[k], b[k]), k


@pytest.mark.parametrize("boundary,dt", [(abi.CYCLIC_WALL, 0.01), (abi.BOUNCING_WALL, 0.1)])
def test_boids_matches_reference(boundary, dt):
    sb = scenes.boids_cloud(n=5000, seed=boundary + 2)
    c = oracle.derive_constants(abi.BOIDS, sb["model_params"])
    a, b = _pair(5000, c, abi.BOIDS)
    for st in (a, b):
        st["pos"][:] = sb["pos"]
        st["vel"][:] = sb["vel"]
    for _ in range(4):
        oracle.boids_step(c, sb["boids_params"], dt, boundary, a)
        oracle.ref_boids_step(c, sb["boids_params"], dt, boundary, b)
        for k in ("pos", "vel", "acc", "id", "table"):
            assert _same(a[k], b[k]), k


@pytest.mark.parametrize("boundary", [abi.CYCLIC_WALL, abi.BOUNCING_WALL])
def test_boids_2d_matches_reference(boundary):
    """The 2D rules kernel (boids.cl:137-221) on the reference's 2D start (x = 0 plane)."""
    sb = scenes.boids_plane(n=4096)
    c = oracle.derive_constants(abi.BOIDS, sb["model_params"])
    n = sb["pos"].shape[0]
    a, b = _pair(n, c, abi.BOIDS)
    for st in (a, b):
        st["pos"][:] = sb["pos"]
        st["vel"][:] = sb["vel"]
    for _ in range(4):
        oracle.boids_step(c, sb["boids_params"], 0.1, boundary, a, dim=2)
        oracle.ref_boids_step(c, sb["boids_params"], 0.1, boundary, b, dim=2)
        for k in ("pos", "vel", "acc", "id", "table"):
            assert _same(a[k], b[k]), k
    assert np.all(a["pos"][:, 0] == 0.0)  # the plane is kept


@pytest.mark.parametrize("smoothing,iters,dim", [(1, 1, 3), (0, 2, 3), (1, 1, 2)])
def test_clouds_matches_reference(smoothing, iters, dim):
    scc = scenes.clouds_cumulus(n=4000, noise=False, seed=smoothing + 3)
    cp = scc["cloud_params"]
    cp.isTempSmoothingEnabled = smoothing
    if dim == 2:  # a 2D model: particles in the x = 0 plane, no x wind (clouds.cl:951)
        cp.dim = 2
        scc["fluid_params"].dim = 2
        scc["pos"][:, 0] = 0.0
    c = oracle.derive_constants(abi.CLOUDS, scc["model_params"])
    env = scenes.cloud_env_reference()
    a, b = _pair(4000, c, abi.CLOUDS)
    for st in (a, b):
        st["pos"][:] = scc["pos"]
        st["vel"][:] = scc["vel"]
    oracle.clouds_init(c, cp, env, None, a)
    oracle.ref_clouds_init(c, cp, b)
    for _ in range(4):
        oracle.clouds_step(c, scc["fluid_params"], cp, env, None, iters, a)
        oracle.ref_clouds_step(c, scc["fluid_params"], cp, iters, b)
        for k in ("pos", "vel", "predPos", "totCorrPos", "temp", "vapor", "cloud", "buoyancy", "id", "cellId"):
            assert _same(a[k], b[k]), k


def test_side_outputs_match_reference():
    """Render-only side outputs: colours, camera distances, grid detector."""
    sc = scenes.dam_break(lattice=(8, 16, 16))
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    rng = np.random.default_rng(1)
    n = sc["pos"].shape[0]
    density = (sc["fluid_params"].restDensity * rng.uniform(0.5, 1.5, n)).astype(np.float32)
    density[:5] = sc["fluid_params"].restDensity
    q = rng.uniform(-1, 3, n).astype(np.float32)
    pos = np.concatenate([sc["pos"], np.full((100, 4), np.inf, np.float32)])
    pos[:, 3] = 0
    cam = np.array([0.3, 2.0, -4.0], np.float32)
    col_r, colf_r, dist_r, det_r = oracle.ref_side_outputs(c, sc["fluid_params"], density, q, 0.0, 2.0, pos, n, cam)
    assert _same(oracle.fill_fluid_color(density, sc["fluid_params"].restDensity), col_r)
    assert _same(oracle.fill_color_float(q, 0.0, 2.0), colf_r)
    assert _same(oracle.fill_camera_dist(pos, n, cam), dist_r)
    assert _same(oracle.fill_grid_detector(c, pos[:n]), det_r)
    assert det_r.sum() > 0 and np.all(dist_r[n:] == 1000000)
