"""Boids target attractor on the CPU: the oracle's Perlin noise and target rule against the
reference's own PerlinNoise.cpp and bd_addTargetRule kernel (oracle/_ref), and the
trajectory's invariants (Target.cpp:27-50)."""
import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, scenes


def _bits(a):
    return np.asarray(a, np.float32).view(np.uint32)


def _ref_or_skip():
    if not oracle.ref_available():
        pytest.skip("oracle/_ref not built")
    if oracle.ref_perlin_noise(1, 0.5, 0.5, 0.5) is None:
        pytest.skip("oracle/_ref built without PerlinNoise.cpp")


def test_perlin_noise_matches_reference():
    _ref_or_skip()
    rng = np.random.default_rng(21)
    pts = np.concatenate([rng.uniform(-300, 300, (1500, 3)), rng.uniform(0, 4, (1500, 3)),
                          np.array([[0, 0, 0], [1, 1, 1], [255, 256, 257], [-1e-6, 0.5, 1 - 1e-7]])])
    pts = pts.astype(np.float32)
    for seed in (1, 29, 246, 12345):
        got = np.array([oracle.perlin_noise(seed, *p) for p in pts], np.float32)
        want = np.array([oracle.ref_perlin_noise(seed, *p) for p in pts], np.float32)
        assert np.array_equal(_bits(got), _bits(want)), "seed %d" % seed
        assert got.min() >= 0.0 and got.max() <= 1.0


def test_trajectory_noise_is_the_reference_noise_along_the_walk():
    """The trajectory samples the three noises at (0.001 s, 0.002 s, 0.01 s) (float sums)."""
    _ref_or_skip()
    walk = np.zeros(3, np.float32)
    for _ in range(300):
        walk += np.array([0.001, 0.002, 0.01], np.float32)
        for seed in (1, 29, 246):
            assert _bits(oracle.perlin_noise(seed, *walk)) == _bits(oracle.ref_perlin_noise(seed, *walk))


@pytest.mark.parametrize("dim", [3, 2])
def test_trajectory_stays_inside_its_radius(dim):
    box, vel = 2.0, 1.0
    t = oracle.target_trajectory(box, dim, vel, 2000)
    r = np.linalg.norm(t.astype(np.float64), axis=1)
    assert r.max() <= 0.48 * box * (1 + 1e-6)
    if dim == 2:
        assert np.all(t[:, 0] == 0.0)
    # Prefix property: the first k positions do not depend on how many follow.
    assert np.array_equal(_bits(oracle.target_trajectory(box, dim, vel, 37)), _bits(t[:37]))
    # It moves, smoothly.
    step = np.linalg.norm(np.diff(t.astype(np.float64), axis=0), axis=1)
    assert step.max() < 0.05 and step.mean() > 1e-4


@pytest.mark.parametrize("boundary,dim,radius,sign", [(abi.CYCLIC_WALL, 3, 2.0, 1), (abi.BOUNCING_WALL, 3, 0.6, 1),
                                                      (abi.CYCLIC_WALL, 3, 2.0, 0), (abi.CYCLIC_WALL, 2, 1.0, 1)])
def test_target_step_matches_reference(boundary, dim, radius, sign):
    """bd_addTargetRule between the rules and bd_updateVel (Boids.cpp:351-358), bit for bit."""
    if not oracle.ref_available():
        pytest.skip("oracle/_ref not built")
    sb = scenes.boids_plane(n=4096) if dim == 2 else scenes.boids_cloud(n=5000, seed=8)
    c = oracle.derive_constants(abi.BOIDS, sb["model_params"])
    n = sb["pos"].shape[0]
    a, b = (oracle.new_state(n, c, abi.BOIDS) for _ in range(2))
    for st in (a, b):
        st["pos"][:] = sb["pos"]
        st["vel"][:] = sb["vel"]
    box = sb["model_params"].boxSize[0]
    traj = oracle.target_trajectory(box, dim, sb["boids_params"].velocityScale, 4)
    for s in range(4):
        oracle.boids_step(c, sb["boids_params"], 0.1, boundary, a, dim=dim, target=traj[s], target_radius=radius,
                          target_sign=sign)
        oracle.ref_boids_step(c, sb["boids_params"], 0.1, boundary, b, dim=dim, target=traj[s],
                              target_radius=radius, target_sign=sign)
        for k in ("pos", "vel", "acc", "id", "table"):
            assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k


def test_target_rule_changes_the_step_only_inside_its_radius():
    sb = scenes.boids_cloud(n=3000, seed=9)
    c = oracle.derive_constants(abi.BOIDS, sb["model_params"])
    base, tgt, off = (oracle.new_state(3000, c, abi.BOIDS) for _ in range(3))
    for st in (base, tgt, off):
        st["pos"][:] = sb["pos"]
        st["vel"][:] = sb["vel"]
    T = np.array([0.3, -0.2, 0.1], np.float32)
    oracle.boids_step(c, sb["boids_params"], 0.01, abi.CYCLIC_WALL, base)
    oracle.boids_step(c, sb["boids_params"], 0.01, abi.CYCLIC_WALL, tgt, target=T, target_radius=0.5)
    oracle.boids_step(c, sb["boids_params"], 0.01, abi.CYCLIC_WALL, off, target=T, target_radius=0.5, target_sign=0)
    assert np.array_equal(base["acc"], off["acc"])  # Attract = false: (int)false = 0, no pull
    x = sb["pos"][base["id"], :3]
    inside = np.linalg.norm(T[None, :] - x, axis=1) < 0.5
    changed = np.any(base["acc"] != tgt["acc"], axis=1)
    assert inside.sum() > 100
    assert np.array_equal(changed, inside)
    # The pull points at the target.
    d = (tgt["acc"] - base["acc"])[inside, :3]
    assert np.all(np.sum(d * (T[None, :] - x[inside]), axis=1) > 0)
