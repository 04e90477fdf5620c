"""Learned warm start of the clouds solve on the GPU against the oracle.

The clouds Jacobi loop (Clouds.cpp:570-587) starts every step from a zero correction as the
fluids one does; the network relaxes the first iteration's lambda by omega(y) in (0, 3), with
features that see the clouds' periodic images in x and z, their y walls, the step's buoyancy
and the temperature above the environment (clouds.cu k_cloud_ws_lambda).

- warm-started steps (network + 0 or 1 extra iteration) against the oracle's restatement
  (oracle.clouds_ws_step) within the clouds step tolerances;
- an untrained network (zero output layer) is the plain clouds solver bit for bit;
- the guard: a tolerance every step exceeds reruns each step as the plain solver, bit for bit,
  and one no step reaches leaves the warm start as it is;
- the loss through the solve and its gradient dL/dy against the oracle, with the state left
  where it was;
- a network trained through the clouds solve on one seeded column lowers the solver-output
  density error of the warm start with no extra iteration below the plain one-iteration
  solver's (the clouds configuration's own iteration count) on a held-out seed.
"""
import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, scenes, warmstart

from helpers import REL_BOX, assert_close_by_id, box_size, clouds_model, gpu_state, random_net

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _copy(st):
    return {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}


def _features(sc, st):
    """The oracle's warm-start features of state st (a copy advances one step to get them)."""
    c = oracle.derive_constants(abi.CLOUDS, sc["model_params"])
    z = abi.mlp_to_arrays(abi.Mlp())
    z["inScale"][:] = 1.0
    f, _ = oracle.clouds_ws_step(c, sc["fluid_params"], sc["cloud_params"], sc["env"], sc["ground"],
                                 abi.mlp_from_arrays(z), 0, _copy(st))
    return f


def _omega_net(rng, feats, out=0.3):
    """A random network normalised on the scene's own features whose omega spans about 0.6-1.8."""
    net = random_net(rng, out_scale=np.array([1.0, 1.0, 1.0, 1.0], np.float32))
    a = abi.mlp_to_arrays(net)
    mu, sd = feats.mean(axis=0), feats.std(axis=0)
    a["inMean"][:] = mu
    a["inScale"][:] = 1.0 / np.maximum(sd, 1e-6 * np.abs(mu) + 1e-30)
    a["w3"][:] *= out / max(1e-6, float(np.abs(a["w3"]).max()))
    a["b3"][:] = 0.0
    return abi.mlp_from_arrays(a)


def _zero_output(net):
    a = abi.mlp_to_arrays(net)
    a["w3"][:] = 0.0
    a["b3"][:] = 0.0
    return abi.mlp_from_arrays(a)


@pytest.mark.parametrize("extra", [0, 1])
def test_warm_started_clouds_steps_match_oracle(extra):
    sc = scenes.clouds_cumulus(n=32768, noise=True, seed=1)
    c = oracle.derive_constants(abi.CLOUDS, sc["model_params"])
    fp, cp = sc["fluid_params"], sc["cloud_params"]
    L = box_size(sc["model_params"])
    with clouds_model(sc, iters=1) as m:
        m.update(2)
        net = _omega_net(np.random.default_rng(9), _features(sc, gpu_state(m, abi.CLOUDS)))
        m.setWarmStart(net, extra_iterations=extra)
        for step in range(3):
            st = gpu_state(m, abi.CLOUDS)
            _, om = oracle.clouds_ws_step(c, fp, cp, sc["env"], sc["ground"], net, extra, st)
            if step == 0:
                assert om.std() > 0.05, om.std()  # the network does relax lambda
            m.update(1)
            g = gpu_state(m, abi.CLOUDS)
            assert np.array_equal(g["id"], st["id"])
            assert_close_by_id(g["id"], g["pos"], st["id"], st["pos"], REL_BOX * L, "pos step %d" % step)
            assert_close_by_id(g["id"], g["vel"], st["id"], st["vel"], REL_BOX * L / fp.timeStep, "vel")
            assert_close_by_id(g["id"], g["temp"], st["id"], st["temp"], 1e-3, "temp")
            assert_close_by_id(g["id"], g["vapor"], st["id"], st["vapor"], 1e-4, "vapor")


@pytest.mark.parametrize("extra", [0, 1])
def test_untrained_network_is_the_plain_clouds_solver(extra):
    sc = scenes.clouds_cumulus(n=131072, noise=True)
    with clouds_model(sc, iters=extra + 1) as plain, clouds_model(sc, iters=1) as warm:
        net = _zero_output(_omega_net(np.random.default_rng(4), _features(sc, gpu_state(warm, abi.CLOUDS))))
        warm.setWarmStart(net, extra_iterations=extra)
        for _ in range(3):
            plain.update(1)
            warm.update(1)
        a, b = gpu_state(plain, abi.CLOUDS), gpu_state(warm, abi.CLOUDS)
        for k in ("id", "pos", "vel", "temp", "vapor", "cloud"):
            assert np.array_equal(a[k], b[k]), k


def test_relax_all_is_refused_for_clouds():
    sc = scenes.clouds_cumulus(n=4096)
    with clouds_model(sc) as m:
        with pytest.raises(Exception):
            m.setWarmStart(abi.Mlp(), extra_iterations=0, relax_all=True)


@pytest.mark.parametrize("plain_iters", [1, 2])
def test_clouds_guard_reruns_as_the_plain_solver(plain_iters):
    """A guard tolerance every step exceeds reruns every step with the plain solver from the
    same predicted positions and the step's total correction restored: the guarded warm start
    equals the plain clouds solver bit for bit, and the statistics count a rerun per step."""
    sc = scenes.clouds_cumulus(n=32768, noise=True, seed=4)
    with clouds_model(sc, iters=plain_iters) as plain, clouds_model(sc, iters=plain_iters) as guarded:
        net = _omega_net(np.random.default_rng(1), _features(sc, gpu_state(guarded, abi.CLOUDS)))
        guarded.setWarmStart(net, extra_iterations=1, guard_tolerance=1e-12)
        for _ in range(3):
            plain.update(1)
            guarded.update(1)
        a, b = gpu_state(plain, abi.CLOUDS), gpu_state(guarded, abi.CLOUDS)
        for k in ("id", "pos", "vel", "temp", "vapor", "cloud"):
            assert np.array_equal(a[k], b[k]), k
        s = guarded.solverStats()
        assert s["steps"] == 3 and s["reruns"] == 3 and s["mean_first"] > 0.0


def test_clouds_guard_that_never_fires_is_the_unguarded_warm_start():
    sc = scenes.clouds_cumulus(n=32768, noise=True, seed=5)
    with clouds_model(sc, iters=1) as free, clouds_model(sc, iters=1) as guarded:
        net = _omega_net(np.random.default_rng(2), _features(sc, gpu_state(free, abi.CLOUDS)))
        free.setWarmStart(net, extra_iterations=0)
        guarded.setWarmStart(net, extra_iterations=0, guard_tolerance=1e6)
        for _ in range(3):
            free.update(1)
            guarded.update(1)
        a, b = gpu_state(free, abi.CLOUDS), gpu_state(guarded, abi.CLOUDS)
        for k in ("id", "pos", "vel", "temp", "vapor", "cloud"):
            assert np.array_equal(a[k], b[k]), k
        s = guarded.solverStats()
        assert s["steps"] == 3 and s["reruns"] == 0


def test_clouds_loss_and_gradient_through_the_solve():
    """The loss (mean squared density constraint after the relaxed first correction) against
    the oracle's (oracle.clouds_ws_loss, BF16 network emulated), and dL/dy projected on the
    output layer's parameters (the network's backward) against central differences of the
    oracle's loss in double precision.  The state does not advance, and a second call gives
    the same loss and gradient."""
    sc = scenes.clouds_cumulus(n=32768, noise=True, seed=2)
    c = oracle.derive_constants(abi.CLOUDS, sc["model_params"])
    fp, cp, env, ground = sc["fluid_params"], sc["cloud_params"], sc["env"], sc["ground"]
    with clouds_model(sc, iters=1) as m:
        m.update(3)
        st = gpu_state(m, abi.CLOUDS)
        net = _omega_net(np.random.default_rng(7), _features(sc, st))
        keep = {b: m.download(b) for b in (abi.BUF_POS, abi.BUF_VEL, abi.BUF_TEMP, abi.BUF_VAPOR, abi.BUF_CLOUD)}
        loss, dy = warmstart.loss_grad_solve(m, net)
        for b, v in keep.items():
            assert np.array_equal(m.download(b), v), "the state must not advance (buffer %d)" % b
        loss2, dy2 = warmstart.loss_grad_solve(m, net)
    dy = dy.cpu().numpy()
    assert loss2 == loss and np.array_equal(dy, dy2.cpu().numpy())
    s = _copy(st)
    l_emu, feats = oracle.clouds_ws_loss(c, fp, cp, env, ground, net, s, emulate=True)
    assert abs(loss - l_emu) <= 2e-3 * l_emu, (loss, l_emu)
    rows = np.zeros((dy.shape[0], 4), np.float32)
    rows[:, 0] = dy[s["id"]]  # dL/dy by sorted row
    grad = oracle.mlp_backward(net, feats, rows, emulate=False)
    checks = []
    for name, idx in (("b3", (0,)), ("w3", (0, 5)), ("w3", (0, 17)), ("w3", (0, 40))):
        eps = 1e-3
        vals = []
        for sgn in (1, -1):
            a = abi.mlp_to_arrays(net)
            a[name][idx] += sgn * eps
            lv, _ = oracle.clouds_ws_loss(c, fp, cp, env, ground, abi.mlp_from_arrays(a), _copy(st))
            vals.append(lv)
        checks.append((name, idx, (vals[0] - vals[1]) / (2 * eps), float(grad[name][idx])))
    scale = max(abs(fd) for _, _, fd, _ in checks)
    assert scale > 0
    for name, idx, fd, an in checks:
        assert abs(fd - an) <= 3e-2 * scale, (name, idx, fd, an, checks)


def _solver_error(sc, iters, net=None, extra=0, steps=200):
    with clouds_model(sc, iters=iters) as m:
        m.enableSolverStats(True)
        if net is not None:
            m.setWarmStart(net, extra_iterations=extra)
        m.update(steps)
        return m.solverStats()["mean"]


def test_network_trained_through_the_clouds_solve_beats_the_plain_iteration():
    n = 32768
    sc = scenes.clouds_cumulus(n=n, noise=True, seed=1)
    with clouds_model(sc, iters=1) as m:
        net, hist = warmstart.train_rollout(m, 300, extra_iterations=0, seed=1)
    assert np.all(np.isfinite(hist))
    test = scenes.clouds_cumulus(n=n, noise=True, seed=3)
    # At the same held-out states the trained network's loss is below the untrained one's.
    with clouds_model(test, iters=1) as m:
        for _ in range(3):
            m.update(40)
            l_trained, _ = warmstart.loss_grad_solve(m, net)
            l_plain, _ = warmstart.loss_grad_solve(m, _zero_output(net))
            assert l_trained < l_plain, (l_trained, l_plain)
    errs = {"plain1": _solver_error(test, 1), "plain2": _solver_error(test, 2),
            "learned+0": _solver_error(test, 1, net, 0), "learned+1": _solver_error(test, 1, net, 1)}
    print("clouds solver-output mean |rho/rho0 - 1| on a held-out column: %s"
          % {k: round(v, 5) for k, v in errs.items()})
    assert errs["learned+0"] < errs["plain1"], errs


def test_clouds_warm_start_stays_stable_over_3000_steps():
    """The 131k cumulus column: a network trained through the clouds solve on two seeded
    columns for 1,500 steps each keeps the one-solve warm start's error near 0.9 % for 3,000
    steps (blocks of 1,000), where the plain single iteration degrades (measured: 0.89, 0.92,
    0.90 % against 5.0, 7.0, 16.9 %).  Rollouts of 300 steps trained networks that drove the
    column unstable within 1,000 steps."""
    n = 131072
    net = None
    for seed in (1, 2):
        with clouds_model(scenes.clouds_cumulus(n=n, noise=True, seed=seed), iters=1) as m:
            net, _ = warmstart.train_rollout(m, 1500, extra_iterations=0, net=net, seed=0)
    sc = scenes.clouds_cumulus(n=n, noise=True)

    def blocks(use):
        out = []
        with clouds_model(sc, iters=1) as m:
            m.enableSolverStats(True)
            if use:
                m.setWarmStart(net, extra_iterations=0)
            for _ in range(3):
                m.resetSolverStats()
                m.update(1000)
                out.append(m.solverStats()["mean"])
        return out

    warm, plain = blocks(True), blocks(False)
    print("3,000 steps, block means: warm start + 0 %s, plain 1 %s" % (np.round(warm, 5), np.round(plain, 5)))
    assert max(warm) < 0.015, warm
    assert all(w < p for w, p in zip(warm, plain)), (warm, plain)
