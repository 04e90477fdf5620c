"""Shared helpers of the GPU parity tests: build a model from a seeded scene, run the
same step on the CUDA library and on the oracle, and compare by particle id."""
import numpy as np

import oracle
from realtimeparticles_gb300 import abi, model

# Per-step tolerance: positions within 1e-5 x box size; velocities such that the
# displacement they produce over one step, |dv| * dt, is within the same bound.
REL_BOX = 1e-5


def box_size(mp):
    return max(mp.boxSize[0], mp.boxSize[1], mp.boxSize[2])


def fluids_model(sc, iters=3, fp=None):
    m = model.Fluids(sc["model_params"])
    m.setFluidParams(fp or sc["fluid_params"])
    m.setJacobiIterations(iters)
    m.upload(abi.BUF_POS, sc["pos"])
    m.upload(abi.BUF_VEL, sc["vel"])
    return m


def boids_model(sc, dt=0.01, boundary=abi.CYCLIC_WALL):
    m = model.Boids(sc["model_params"])
    m.setBoidsParams(sc["boids_params"])
    m.setTimeStep(dt)
    m.setBoundary(boundary)
    m.upload(abi.BUF_POS, sc["pos"])
    m.upload(abi.BUF_VEL, sc["vel"])
    return m


def clouds_model(sc, iters=1):
    m = model.Clouds(sc["model_params"])
    m.setFluidParams(sc["fluid_params"])
    m.setCloudParams(sc["cloud_params"])
    m.setEnvironment(sc["env"], sc["ground"])
    m.setJacobiIterations(iters)
    m.upload(abi.BUF_POS, sc["pos"])
    m.upload(abi.BUF_VEL, sc["vel"])
    m.initThermo()
    return m


def gpu_state(m, mtype):
    """Download the model's state into an oracle state dict."""
    n = m.nbParticles()
    c = m.constants()
    st = oracle.new_state(n, c, mtype)
    st["pos"][:] = m.download(abi.BUF_POS)
    st["vel"][:] = m.download(abi.BUF_VEL)
    st["id"][:] = m.download(abi.BUF_ID)
    if mtype == abi.CLOUDS:
        st["temp"][:] = m.download(abi.BUF_TEMP)
        st["vapor"][:] = m.download(abi.BUF_VAPOR)
        st["cloud"][:] = m.download(abi.BUF_CLOUD)
        st["buoyancy"][:] = m.download(abi.BUF_BUOYANCY)
    return st


def by_id(ids, arr):
    out = np.empty_like(arr)
    out[ids] = arr
    return out


def assert_close_by_id(ids_a, a, ids_b, b, atol, what):
    A = by_id(ids_a, a)
    B = by_id(ids_b, b)
    err = np.abs(A.astype(np.float64) - B.astype(np.float64))
    worst = float(np.nanmax(err)) if err.size else 0.0
    assert np.all(np.isfinite(A)) and np.all(np.isfinite(B)), what + ": non-finite values"
    assert worst <= atol, "%s: max |diff| %.3g > %.3g" % (what, worst, atol)
    return worst


def random_net(rng, scale=0.5, out_scale=None):
    """A random warm-start network (abi.Mlp) with weights of a trained network's magnitude."""
    net = abi.Mlp()
    a = abi.mlp_to_arrays(net)
    a["inMean"][:] = rng.normal(0, 0.3, 12)
    a["inScale"][:] = rng.uniform(0.5, 2.0, 12)
    a["w1"][:] = rng.normal(0, scale, (64, 12))
    a["b1"][:] = rng.normal(0, 0.1, 64)
    a["w2"][:] = rng.normal(0, scale / 4, (64, 64))
    a["b2"][:] = rng.normal(0, 0.1, 64)
    a["w3"][:] = rng.normal(0, scale / 4, (4, 64))
    a["b3"][:] = rng.normal(0, 0.1, 4)
    a["outScale"][:] = rng.uniform(0.5, 2.0, 4) if out_scale is None else out_scale
    return abi.mlp_from_arrays(a)
