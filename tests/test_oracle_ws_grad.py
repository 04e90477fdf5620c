"""The oracle's gradient of the warm start's training loss, pinned by finite differences.

The loss is the mean squared density constraint after the omega-relaxed first correction
(oracle.ws_loss_grad, restating warmstart.cu k_ws_loss_grad_x / k_ws_grad_y).  Its gradient
to the network's parameters is dL/dy through the network's backward (oracle.mlp_backward);
central differences of the loss in the output-layer parameters must agree with it.  Pure
double precision (no BF16 rounding).  CPU only."""
import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, scenes

from helpers import random_net


def _state(steps=3):
    sc = scenes.dam_break(lattice=(8, 16, 16))
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    fp = sc["fluid_params"]
    st = oracle.new_state(sc["pos"].shape[0], c)
    st["pos"][:] = sc["pos"]
    st["vel"][:] = sc["vel"]
    for _ in range(steps):
        oracle.fluids_step(c, fp, 2, st)
    return c, fp, st


def _copy(st):
    return {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}


def _net():
    rng = np.random.default_rng(3)
    net = random_net(rng, scale=0.4, out_scale=np.array([1.0, 1.0, 1.0, 1.0], np.float32))
    a = abi.mlp_to_arrays(net)
    a["inMean"][:] = 0.0
    a["inScale"][:] = 1.0
    a["inScale"][10] = 1e5  # lambda of order 1e-5
    a["inScale"][0] = 1.0 / 30.0
    a["inScale"][6] = 20.0
    return abi.mlp_from_arrays(a)


def _clamped(c, s):
    W = np.array(c.absWall[:3], np.float32)
    lo = np.append(-W + np.float32(0.01), 0).astype(np.float32)
    hi = np.append(W - np.float32(0.1), 0).astype(np.float32)
    return np.ascontiguousarray(np.clip(s["predPos"], lo, hi))


@pytest.mark.parametrize("steps,rtol", [(3, 1e-3), (30, 5e-3)])
def test_ws_loss_gradient_matches_finite_differences(steps, rtol):
    """The gradient treats the pairs within h as symmetric.  A particle whose correction moved
    it into another cell can see a neighbour that does not see it (the 27 cells come from the
    step's table), which the finite differences include: a small absolute difference, so the
    bound is relative to the largest of the checked entries."""
    c, fp, st = _state(steps)
    net = _net()
    loss, dy_id, om = oracle.ws_loss_grad(c, fp, net, _copy(st), emulate=False)
    assert loss > 0 and np.all(np.isfinite(dy_id))
    assert om.min() > 0.0 and om.max() < 3.0 and om.std() > 0.01  # a real relaxation, not omega = 1
    # Parameter gradient = backward of dy (rows in the presort's sorted order).
    s = _copy(st)
    n = s["pos"].shape[0]
    l2, _, _ = oracle.ws_loss_grad(c, fp, net, s, emulate=False)  # s now holds the sorted ids
    assert l2 == loss
    feats = oracle.ws_features(c, fp, _clamped(c, s), s["vel"], s["table"])
    dy = np.zeros((n, 4), np.float32)
    dy[:, 0] = dy_id[s["id"]]
    grad = oracle.mlp_backward(net, feats, dy, emulate=False)
    checks = []
    for name, idx in (("b3", (0,)), ("w3", (0, 5)), ("w3", (0, 17)), ("w3", (0, 40)), ("b2", (3,))):
        eps = 1e-4
        vals = []
        for sgn in (1, -1):
            a = abi.mlp_to_arrays(net)
            a[name][idx] += sgn * eps
            lv, _, _ = oracle.ws_loss_grad(c, fp, abi.mlp_from_arrays(a), _copy(st), emulate=False)
            vals.append(lv)
        checks.append((name, idx, (vals[0] - vals[1]) / (2 * eps), float(grad[name][idx])))
    scale = max(abs(fd) for _, _, fd, _ in checks)
    for name, idx, fd, an in checks:
        assert abs(fd - an) <= rtol * scale, (name, idx, fd, an)


def test_zero_output_layer_is_the_plain_solver():
    """A network with a zero output layer relaxes nothing (omega = 1): the warm-started step
    with no extra iteration is the plain one-iteration step, bit for bit."""
    c, fp, st = _state()
    a, b = _copy(st), _copy(st)
    n = a["pos"].shape[0]
    z = abi.mlp_to_arrays(_net())
    z["w3"][:] = 0.0
    z["b3"][:] = 0.0
    oracle.ws_step(c, fp, abi.mlp_from_arrays(z), 0, 0.0, 1, a, np.zeros(n, np.float32))
    oracle.fluids_step(c, fp, 1, b)
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])


def _clouds_state(n=4000, steps=2):
    sc = scenes.clouds_cumulus(n=n, noise=True, seed=5)
    c = oracle.derive_constants(abi.CLOUDS, sc["model_params"])
    st = oracle.new_state(n, c, abi.CLOUDS)
    st["pos"][:] = sc["pos"]
    st["vel"][:] = sc["vel"]
    oracle.clouds_init(c, sc["cloud_params"], sc["env"], sc["ground"], st)
    for _ in range(steps):
        oracle.clouds_step(c, sc["fluid_params"], sc["cloud_params"], sc["env"], sc["ground"], 1, st)
    return sc, c, st


@pytest.mark.parametrize("extra", [0, 1])
def test_clouds_zero_output_layer_is_the_plain_solver(extra):
    """The clouds warm start with a zero output layer and `extra` plain iterations after it is
    the plain clouds step with extra + 1 iterations, bit for bit; a network that does relax
    lambda changes the step."""
    sc, c, st = _clouds_state()
    fp, cp, env, gr = sc["fluid_params"], sc["cloud_params"], sc["env"], sc["ground"]
    a, b, r = _copy(st), _copy(st), _copy(st)
    z = abi.mlp_to_arrays(_net())
    z["w3"][:] = 0.0
    z["b3"][:] = 0.0
    feats, om = oracle.clouds_ws_step(c, fp, cp, env, gr, abi.mlp_from_arrays(z), extra, a)
    oracle.clouds_step(c, fp, cp, env, gr, extra + 1, b)
    for k in ("pos", "vel", "temp", "vapor", "cloud", "id"):
        assert np.array_equal(a[k], b[k]), k
    assert np.all(om == 1.0)
    # the features: integer neighbour counts, the plain lambda, the y-wall proximity in [-2, 2]
    assert np.all(feats[:, 0] == np.round(feats[:, 0])) and feats[:, 0].max() > 0
    assert np.all(np.abs(feats[:, 8]) <= 2.0) and np.any(feats[:, 8] > 0)  # particles start at the floor
    assert np.all(np.isfinite(feats))
    _, om_r = oracle.clouds_ws_step(c, fp, cp, env, gr, _net(), extra, r)
    assert om_r.std() > 0.01 and not np.array_equal(r["pos"], b["pos"])
