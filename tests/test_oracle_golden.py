"""The oracle reproduces, bit for bit, golden outputs of the reference's own step kernels
(tests/golden/*.npz, written by tests/golden/make_golden.py from physics/ocl/kernels/*.cl
compiled for the CPU)."""
import ctypes as C
import os

import numpy as np
import pytest

from realtimeparticles_gb300 import abi

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLD, name))


def _struct(cls, arr):
    s = cls()
    C.memmove(C.addressof(s), arr.tobytes(), C.sizeof(cls))
    return s


def _bits(a):
    return a.view(np.uint32) if a.dtype == np.float32 else a


def _assert_same(got, want, what):
    assert got.shape == want.shape, what
    diff = np.flatnonzero(_bits(got).ravel() != _bits(want).ravel())
    assert diff.size == 0, "%s: %d values differ (first flat index %d)" % (what, diff.size, diff[0])


def test_cell_ids_golden(oracle_mod):
    g = _load("cell_ids.npz")
    c = _struct(abi.GridConstants, g["consts"])
    _assert_same(oracle_mod.fill_cell_ids(c, g["pos"]), g["keys"], "keys")


def test_cell_table_golden(oracle_mod):
    g = _load("cell_table.npz")
    c = _struct(abi.GridConstants, g["consts"])
    _assert_same(oracle_mod.cell_table(c, g["keys"]), g["table"], "table")


def test_fluids_golden(oracle_mod):
    g = _load("fluids_3steps.npz")
    c = _struct(abi.GridConstants, g["consts"])
    fp = _struct(abi.FluidParams, g["params"])
    st = oracle_mod.new_state(g["pos0"].shape[0], c)
    st["pos"][:] = g["pos0"]
    st["vel"][:] = g["vel0"]
    for _ in range(int(g["steps"][0])):
        oracle_mod.fluids_step(c, fp, int(g["iters"][0]), st)
    for k in ("pos", "vel", "predPos", "density", "lambda", "vort", "id", "cellId", "table"):
        _assert_same(st[k], g[k], k)


def test_boids_golden(oracle_mod):
    g = _load("boids_3steps.npz")
    c = _struct(abi.GridConstants, g["consts"])
    bp = _struct(abi.BoidsParams, g["params"])
    st = oracle_mod.new_state(g["pos0"].shape[0], c, abi.BOIDS)
    st["pos"][:] = g["pos0"]
    st["vel"][:] = g["vel0"]
    for _ in range(3):
        oracle_mod.boids_step(c, bp, float(g["dt"][0]), abi.CYCLIC_WALL, st)
    for k in ("pos", "vel", "acc", "id", "cellId", "table"):
        _assert_same(st[k], g[k], k)


def test_boids_target_golden(oracle_mod):
    """The reference's PerlinNoise values and 3 boids steps with its bd_addTargetRule."""
    g = _load("boids_target_3steps.npz")
    for k, seed in enumerate(g["seeds"]):
        got = np.array([oracle_mod.perlin_noise(int(seed), *p) for p in g["points"]], np.float32)
        _assert_same(got, g["noise"][k], "noise seed %d" % seed)
    c = _struct(abi.GridConstants, g["consts"])
    bp = _struct(abi.BoidsParams, g["params"])
    st = oracle_mod.new_state(g["pos0"].shape[0], c, abi.BOIDS)
    st["pos"][:] = g["pos0"]
    st["vel"][:] = g["vel0"]
    assert np.array_equal(g["target"], oracle_mod.target_trajectory(c.absWall[0] * 2, 3, bp.velocityScale, 3))
    for s in range(3):
        oracle_mod.boids_step(c, bp, float(g["dt"][0]), abi.CYCLIC_WALL, st, target=g["target"][s],
                              target_radius=float(g["radius"][0]))
    for k in ("pos", "vel", "acc", "id"):
        _assert_same(st[k], g[k], k)


def test_clouds_golden(oracle_mod):
    from realtimeparticles_gb300 import scenes
    g = _load("clouds_3steps.npz")
    c = _struct(abi.GridConstants, g["consts"])
    fp = _struct(abi.FluidParams, g["fparams"])
    cp = _struct(abi.CloudParams, g["cparams"])
    env = scenes.cloud_env_reference()
    st = oracle_mod.new_state(g["pos0"].shape[0], c, abi.CLOUDS)
    st["pos"][:] = g["pos0"]
    st["vel"][:] = g["vel0"]
    oracle_mod.clouds_init(c, cp, env, None, st)
    for k in ("temp", "vapor", "cloud"):
        _assert_same(st[k], g[k + "0"], k + " (init)")
    for _ in range(3):
        oracle_mod.clouds_step(c, fp, cp, env, None, 1, st)
    for k in ("pos", "vel", "predPos", "totCorrPos", "temp", "vapor", "cloud", "buoyancy", "density", "lambda", "id",
              "cellId"):
        _assert_same(st[k], g[k], k)
