#!/usr/bin/env python3
"""Writes the golden fixtures in this directory from the reference's own step kernels
(physics/ocl/kernels/*.cl compiled for the CPU by oracle/ref/build_ref.py).

Each fixture holds the seeded inputs, the JIT constants and parameters, and the outputs of
the reference kernels driven in the reference's update() order.  Regenerate with
    python oracle/ref/build_ref.py && python tests/golden/make_golden.py
(needs the reference checkout); the tests only read the .npz files.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from realtimeparticles_gb300 import abi, scenes  # noqa: E402


def sbytes(s):
    return np.frombuffer(bytes(s), np.uint8).copy()


def save(name, **arrays):
    np.savez_compressed(os.path.join(HERE, name), **arrays)
    print("wrote", name, sum(a.nbytes for a in arrays.values()), "bytes uncompressed")


def main():
    assert oracle.ref_available(), "build oracle/_ref first (python oracle/ref/build_ref.py)"
    # fillCellIDs on walls, cell edges and their float neighbours, +-inf.
    mp = abi.model_params(16, 16, (1.0, 1.0, 1.0), (40, 40, 40))
    c = oracle.derive_constants(abi.FLUIDS, mp)
    edges = (np.arange(41, dtype=np.float32) * np.float32(c.cellSize) - np.float32(0.5)).astype(np.float32)
    vals = np.concatenate([edges, np.nextafter(edges, np.float32(-1)), np.nextafter(edges, np.float32(1)),
                           np.array([0.5, -0.5, np.inf, -np.inf, 0.0, 3.0], np.float32)])
    rng = np.random.default_rng(11)
    pos = np.zeros((600, 4), np.float32)
    pos[:, :3] = rng.choice(vals, size=(600, 3))
    save("cell_ids.npz", consts=sbytes(c), pos=pos, keys=oracle.ref_fill_cell_ids(c, pos))
    # Start/end table with the quirks (index 0, cap, aliased keys).
    c8 = oracle.derive_constants(abi.FLUIDS, abi.model_params(16, 16, (1.0,) * 3, (8,) * 3))
    sk = np.sort(np.concatenate([np.full(150, 17), np.full(101, 40), [3, 3, 600, 640], rng.integers(0, 700, 400)]))
    sk = sk.astype(np.uint32)
    save("cell_table.npz", consts=sbytes(c8), keys=sk, table=oracle.ref_cell_table(c8, sk))
    # PBF: 2048-particle dam break, 3 Jacobi iterations, 3 steps.
    sc = scenes.dam_break(lattice=(8, 16, 16), seed=5)
    cf = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    st = oracle.new_state(2048, cf)
    st["pos"][:] = sc["pos"]
    st["vel"][:] = sc["vel"]
    pos0, vel0 = st["pos"].copy(), st["vel"].copy()
    for _ in range(3):
        oracle.ref_fluids_step(cf, sc["fluid_params"], 3, st)
    save("fluids_3steps.npz", consts=sbytes(cf), params=sbytes(sc["fluid_params"]), iters=np.array([3]),
         steps=np.array([3]), pos0=pos0, vel0=vel0, **{k: st[k] for k in
                                                       ("pos", "vel", "predPos", "density", "lambda", "vort", "id",
                                                        "cellId", "table")})
    # Boids: 3000 boids, periodic, dt 0.01, 3 steps.
    sb = scenes.boids_cloud(n=3000, seed=6)
    cb = oracle.derive_constants(abi.BOIDS, sb["model_params"])
    st = oracle.new_state(3000, cb, abi.BOIDS)
    st["pos"][:] = sb["pos"]
    st["vel"][:] = sb["vel"]
    pos0, vel0 = st["pos"].copy(), st["vel"].copy()
    for _ in range(3):
        oracle.ref_boids_step(cb, sb["boids_params"], 0.01, abi.CYCLIC_WALL, st)
    save("boids_3steps.npz", consts=sbytes(cb), params=sbytes(sb["boids_params"]), dt=np.array([0.01], np.float32),
         pos0=pos0, vel0=vel0, **{k: st[k] for k in ("pos", "vel", "acc", "id", "cellId", "table")})
    # Boids target attractor: the reference's PerlinNoise at seeded points, then 3 boids steps
    # with bd_addTargetRule.  Target.cpp needs spdlog/nlohmann-json, so the positions come from
    # the oracle's Target::updatePos restatement and are stored as inputs.
    pts = np.random.default_rng(13).uniform(-50, 50, (256, 3)).astype(np.float32)
    seeds = np.array([1, 29, 246], np.int32)
    noise = np.array([[oracle.ref_perlin_noise(int(sd), *p) for p in pts] for sd in seeds], np.float32)
    sb = scenes.boids_cloud(n=3000, seed=12)
    cb = oracle.derive_constants(abi.BOIDS, sb["model_params"])
    st = oracle.new_state(3000, cb, abi.BOIDS)
    st["pos"][:] = sb["pos"]
    st["vel"][:] = sb["vel"]
    pos0, vel0 = st["pos"].copy(), st["vel"].copy()
    traj = oracle.target_trajectory(sb["model_params"].boxSize[0], 3, sb["boids_params"].velocityScale, 3)
    for s in range(3):
        oracle.ref_boids_step(cb, sb["boids_params"], 0.01, abi.CYCLIC_WALL, st, target=traj[s], target_radius=1.2,
                              target_sign=1)
    save("boids_target_3steps.npz", points=pts, seeds=seeds, noise=noise, consts=sbytes(cb),
         params=sbytes(sb["boids_params"]), dt=np.array([0.01], np.float32), radius=np.array([1.2], np.float32),
         target=traj, pos0=pos0, vel0=vel0, **{k: st[k] for k in ("pos", "vel", "acc", "id")})
    # Clouds: 3000 particles, the reference environment, 1 iteration, 3 steps.
    scc = scenes.clouds_cumulus(n=3000, noise=False, seed=7)
    cc = oracle.derive_constants(abi.CLOUDS, scc["model_params"])
    st = oracle.new_state(3000, cc, abi.CLOUDS)
    st["pos"][:] = scc["pos"]
    st["vel"][:] = scc["vel"]
    oracle.ref_clouds_init(cc, scc["cloud_params"], st)
    init = {k + "0": st[k].copy() for k in ("pos", "vel", "temp", "vapor", "cloud")}
    for _ in range(3):
        oracle.ref_clouds_step(cc, scc["fluid_params"], scc["cloud_params"], 1, st)
    save("clouds_3steps.npz", consts=sbytes(cc), fparams=sbytes(scc["fluid_params"]),
         cparams=sbytes(scc["cloud_params"]), **init,
         **{k: st[k] for k in ("pos", "vel", "predPos", "totCorrPos", "temp", "vapor", "cloud", "buoyancy",
                                "density", "lambda", "id", "cellId")})


if __name__ == "__main__":
    main()
