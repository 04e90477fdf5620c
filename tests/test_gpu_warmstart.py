"""Learned warm start on the GPU against the oracle.

- inference kernel and the trainer's loss / gradient against the oracle's double-precision
  restatement, both with the GPU's BF16 operand rounding emulated (tight) and without it;
- the trainer lowers the loss and is deterministic;
- regression samples (features and targets) recorded by the library against the oracle's;
- the loss through the solve and its gradient dL/dy, and the network's backward with a given
  output gradient, against the oracle (whose gradient is pinned by finite differences);
- warm-started steps (network + 0, 1 or 2 extra iterations, relaxed or plain) against the
  oracle within the step tolerance 1e-5 x box; an untrained network (zero output layer) is the
  plain solver bit for bit;
- the guard: a step above tolerance reruns as the plain solver, bit for bit;
- what a network trained through the solve gains over the same solver without it, on a
  held-out scene.
"""
import numpy as np
import pytest

import oracle
from realtimeparticles_gb300 import abi, scenes, warmstart

from helpers import REL_BOX, assert_close_by_id, box_size, fluids_model, gpu_state, random_net

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def test_inference_kernel_matches_oracle():
    rng = np.random.default_rng(11)
    net = random_net(rng)
    feats = rng.normal(0, 1, (1000, 12)).astype(np.float32)  # 1000: a partial last warp
    gpu = warmstart.forward(net, _cuda(feats)).cpu().numpy()
    emu = oracle.mlp_forward(net, feats, emulate=True)
    exact = oracle.mlp_forward(net, feats, emulate=False)
    scale = np.abs(exact).max(axis=0)
    assert np.all(np.abs(gpu - emu).max(axis=0) <= 5e-3 * scale), np.abs(gpu - emu).max(axis=0) / scale
    assert np.all(np.abs(gpu - exact).max(axis=0) <= 3e-2 * scale)


@pytest.mark.parametrize("n", [4096, 4099])
def test_gradient_matches_oracle(n):
    rng = np.random.default_rng(5 + n)
    net = random_net(rng)
    feats = rng.normal(0, 1, (n, 12)).astype(np.float32)
    targets = rng.normal(0, 1, (n, 4)).astype(np.float32)
    lw = (1.0, 0.5, 0.5, 2.0)
    loss, grad = warmstart.loss_grad(net, _cuda(feats), _cuda(targets), lw)
    g = abi.mlp_to_arrays(grad)
    l_emu, g_emu = oracle.mlp_loss_grad(net, np.array(lw, np.float32), feats, targets, emulate=True)
    l_dbl, g_dbl = oracle.mlp_loss_grad(net, np.array(lw, np.float32), feats, targets, emulate=False)
    assert abs(loss - l_emu) <= 1e-3 * abs(l_emu)
    assert abs(loss - l_dbl) <= 2e-2 * abs(l_dbl)
    for name in abi.MLP_TRAINABLE:
        ref = g_emu[name]
        rel = np.linalg.norm(g[name] - ref) / np.linalg.norm(ref)
        assert rel <= 1e-2, (name, rel)
        rel_d = np.linalg.norm(g[name] - g_dbl[name]) / np.linalg.norm(g_dbl[name])
        assert rel_d <= 5e-2, (name, rel_d)
    # normalisation fields of a gradient are zero
    assert not np.any(g["inMean"]) and not np.any(g["outScale"])


def test_trainer_lowers_loss_and_is_deterministic():
    rng = np.random.default_rng(2)
    feats = rng.normal(0, 1, (20000, 12)).astype(np.float32)
    t = np.stack([np.tanh(feats[:, 0] + 0.5 * feats[:, 1]), feats[:, 2] * feats[:, 3],
                  np.sin(feats[:, 4]), 0.3 * feats[:, 5] ** 2], axis=1).astype(np.float32)
    f, y = _cuda(feats), _cuda(t)
    kw = dict(epochs=12, batch=2048, learning_rate=3e-3, seed=4, loss_weights=(1.0, 1.0, 1.0, 1.0))
    net1, hist1 = warmstart.train(f, y, **kw)
    net2, hist2 = warmstart.train(f, y, **kw)
    assert hist1[-1] < 0.15 * hist1[0], hist1
    a1, a2 = abi.mlp_to_arrays(net1), abi.mlp_to_arrays(net2)
    for k in abi.MLP_ARRAYS:
        assert np.array_equal(a1[k], a2[k]), k
    # the trained network reproduces the function on held-out inputs
    xt = rng.normal(0, 1, (4000, 12)).astype(np.float32)
    yt = np.stack([np.tanh(xt[:, 0] + 0.5 * xt[:, 1]), xt[:, 2] * xt[:, 3], np.sin(xt[:, 4]),
                   0.3 * xt[:, 5] ** 2], axis=1)
    pred = warmstart.forward(net1, _cuda(xt)).cpu().numpy()
    assert np.mean((pred - yt) ** 2) < 0.15 * np.mean(yt ** 2)


def _record_both(sc, iters, stride, phase, steps):
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    fp = sc["fluid_params"]
    n = sc["pos"].shape[0]
    cap = (n - phase + stride - 1) // stride
    out = []
    with fluids_model(sc, iters) as m:
        for _ in range(steps):
            st = gpu_state(m, abi.FLUIDS)
            f_o, t_o = oracle.ws_record_step(c, fp, iters, stride, phase, st, np.zeros(n, np.float32))
            f = torch.zeros((cap, 12), dtype=torch.float32, device="cuda")
            t = torch.zeros((cap, 4), dtype=torch.float32, device="cuda")
            w = m.recordWarmStartSamples(iters, stride, phase, f.data_ptr(), t.data_ptr(), cap)
            assert w == cap == f_o.shape[0]
            out.append((f.cpu().numpy(), t.cpu().numpy(), f_o, t_o))
            g = gpu_state(m, abi.FLUIDS)
            assert np.array_equal(g["id"], st["id"])  # same sorted order as the oracle
            assert_close_by_id(g["id"], g["pos"], st["id"], st["pos"], REL_BOX * box_size(m._params), "pos")
    return out


def test_recorded_samples_match_oracle():
    sc = scenes.dam_break(lattice=(8, 16, 16))
    for f, t, f_o, t_o in _record_both(sc, iters=4, stride=3, phase=1, steps=3):
        fs = np.maximum(np.abs(f_o).max(axis=0), 1e-30)
        assert np.all(np.abs(f - f_o).max(axis=0) <= 2e-4 * fs + 1e-6), np.abs(f - f_o).max(axis=0) / fs
        lam_scale = np.abs(t_o[:, 0]).max()
        assert np.abs(t[:, 0] - t_o[:, 0]).max() <= 1e-3 * lam_scale
        assert np.abs(t[:, 1:] - t_o[:, 1:]).max() <= REL_BOX * 1.0


# Typical magnitudes of the 12 features on the dam break (the inputs' normalisation).
FEATURE_SCALE = np.array([30.0, 0.05, 1.0, 1.0, 1.0, 5.0, 0.05, 1.0, 1.0, 1.0, 1e-5, 0.1], np.float32)


def _omega_net(rng, out=0.3):
    """A random network with normalised inputs whose relaxation omega spans about 0.6-1.8."""
    net = random_net(rng, out_scale=np.array([1.0, 1.0, 1.0, 1.0], np.float32))
    a = abi.mlp_to_arrays(net)
    a["inMean"][:] = 0.0
    a["inScale"][:] = 1.0 / FEATURE_SCALE
    a["w3"][:] *= out / max(1e-6, float(np.abs(a["w3"]).max()))
    a["b3"][:] = 0.0
    return abi.mlp_from_arrays(a)


def _zero_output(net):
    a = abi.mlp_to_arrays(net)
    a["w3"][:] = 0.0
    a["b3"][:] = 0.0
    return abi.mlp_from_arrays(a)


@pytest.mark.parametrize("extra,relax_all", [(0, False), (1, False), (2, True)])
def test_warm_started_steps_match_oracle(extra, relax_all):
    sc = scenes.dam_break(lattice=(8, 16, 16))
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    fp = sc["fluid_params"]
    L = box_size(sc["model_params"])
    rng = np.random.default_rng(9)
    net = _omega_net(rng)
    with fluids_model(sc, 3) as m:
        m.setWarmStart(net, extra_iterations=extra, guard_tolerance=0.0, relax_all=relax_all)
        for step in range(4):
            st = gpu_state(m, abi.FLUIDS)
            lam = np.zeros(st["pos"].shape[0], np.float32)
            err_o, rerun = oracle.ws_step(c, fp, net, extra, 0.0, 3, st, lam, relax_all=relax_all)
            assert not rerun
            m.update(1)
            g = gpu_state(m, abi.FLUIDS)
            assert np.array_equal(g["id"], st["id"])
            assert_close_by_id(g["id"], g["pos"], st["id"], st["pos"], REL_BOX * L, "pos step %d" % step)
            assert_close_by_id(g["id"], g["vel"], st["id"], st["vel"], REL_BOX * L / fp.timeStep, "vel")
            lam_g = m.download(abi.BUF_LAMBDA_TOTAL)
            # omega comes from the BF16 network (within 0.5 % of the oracle's BF16 emulation)
            assert np.abs(lam_g - lam).max() <= 1e-2 * np.abs(lam).max() + 1e-12
        stats = m.solverStats()
        assert stats["steps"] == 4 and stats["reruns"] == 0


@pytest.mark.parametrize("extra", [0, 2])
def test_untrained_network_is_the_plain_solver(extra):
    """A zero output layer sets omega = 1: the warm-started step with `extra` plain iterations
    after it equals the plain solver with extra + 1 iterations bit for bit (65,536 particles:
    the plain sweeps run one lane per particle, as the warm start's feature sweep does)."""
    sc = scenes.dam_break(lattice=(32, 64, 32))
    net = _zero_output(_omega_net(np.random.default_rng(4)))
    with fluids_model(sc, extra + 1) as plain, fluids_model(sc, 3) as warm:
        warm.setWarmStart(net, extra_iterations=extra, guard_tolerance=0.0)
        for _ in range(3):
            plain.update(1)
            warm.update(1)
        a, b = gpu_state(plain, abi.FLUIDS), gpu_state(warm, abi.FLUIDS)
        assert np.array_equal(a["id"], b["id"])
        assert np.array_equal(a["pos"], b["pos"])
        assert np.array_equal(a["vel"], b["vel"])


@pytest.mark.parametrize("lattice,steps", [((8, 16, 16), 3), ((16, 32, 32), 30)])
def test_loss_and_gradient_through_the_solve_match_oracle(lattice, steps):
    sc = scenes.dam_break(lattice=lattice)
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    fp = sc["fluid_params"]
    net = _omega_net(np.random.default_rng(7))
    with fluids_model(sc, 2) as m:
        m.update(steps)
        st = gpu_state(m, abi.FLUIDS)
        pos0 = m.download(abi.BUF_POS)
        loss, dy = warmstart.loss_grad_solve(m, net)
        assert np.array_equal(m.download(abi.BUF_POS), pos0), "the state must not advance"
    dy = dy.cpu().numpy().astype(np.float64)
    l_o, dy_o, om = oracle.ws_loss_grad(c, fp, net, st, emulate=True)
    assert om.std() > 0.05  # the network does relax lambda
    assert abs(loss - l_o) <= 2e-3 * l_o, (loss, l_o)
    rel = np.linalg.norm(dy - dy_o) / np.linalg.norm(dy_o)
    assert rel <= 2e-2, rel


def test_backward_with_given_output_gradient_matches_oracle():
    rng = np.random.default_rng(12)
    net = random_net(rng)
    n = 3001
    feats = rng.normal(0, 1, (n, 12)).astype(np.float32)
    dy = rng.normal(0, 1e-3, (n, 4)).astype(np.float32)
    grad = abi.mlp_to_arrays(warmstart.backward(net, _cuda(feats), _cuda(dy)))
    g_o = oracle.mlp_backward(net, feats, dy, emulate=True)
    for name in abi.MLP_TRAINABLE:
        rel = np.linalg.norm(grad[name] - g_o[name]) / np.linalg.norm(g_o[name])
        assert rel <= 1e-2, (name, rel)


def test_guard_reruns_as_the_plain_solver():
    sc = scenes.dam_break(lattice=(8, 16, 16))
    rng = np.random.default_rng(1)
    net = _omega_net(rng)
    with fluids_model(sc, 3) as plain, fluids_model(sc, 3) as guarded:
        guarded.setWarmStart(net, extra_iterations=0, guard_tolerance=1e-12)
        for _ in range(3):
            plain.update(1)
            guarded.update(1)
        a, b = gpu_state(plain, abi.FLUIDS), gpu_state(guarded, abi.FLUIDS)
        assert np.array_equal(a["id"], b["id"])
        assert np.array_equal(a["pos"], b["pos"])
        assert np.array_equal(a["vel"], b["vel"])
        s = guarded.solverStats()
        assert s["steps"] == 3 and s["reruns"] == 3
        assert s["mean"] > 0.0 and s["mean_first"] > 0.0


def _solver_error(sc, iters, net=None, extra=0, steps=160):
    with fluids_model(sc, iters) as m:
        m.enableSolverStats(True)
        if net is not None:
            m.setWarmStart(net, extra_iterations=extra, guard_tolerance=0.0)
        m.update(steps)
        return m.solverStats()["mean"]


def test_network_trained_through_the_solve_beats_the_plain_first_iteration():
    """Train on the rollout of one seeded dam break (16,384 particles) under the warm start with
    no extra iteration, evaluate on a held-out seed: the solver-output mean density error of the
    warm start with no extra iteration must be below the plain solver's with one iteration (the
    solve the warm start replaces), and on held-out states the trained network's training loss
    must be below the untrained one's.  The comparison with more iterations is printed."""
    lattice = (16, 32, 32)
    sc = scenes.dam_break(lattice=lattice, seed=1)
    with fluids_model(sc, 2) as m:
        net, hist = warmstart.train_rollout(m, 300, extra_iterations=0, seed=1)
    assert np.all(np.isfinite(hist))
    test = scenes.dam_break(lattice=lattice, seed=3)
    # The training loss falls: at the same held-out states, the trained network's loss is below
    # the untrained one's (a zero output layer: the plain first iteration).  (The rollout's own
    # loss history mixes learning with the flow's development, so it is not compared.)
    with fluids_model(test, 2) as m:
        for _ in range(3):
            m.update(40)
            l_trained, _ = warmstart.loss_grad_solve(m, net)
            l_plain, _ = warmstart.loss_grad_solve(m, _zero_output(net))
            assert l_trained < l_plain, (l_trained, l_plain)
    errs = {"plain1": _solver_error(test, 1), "plain2": _solver_error(test, 2), "plain3": _solver_error(test, 3),
            "learned+0": _solver_error(test, 3, net, 0), "learned+1": _solver_error(test, 3, net, 1)}
    print("solver-output mean |rho/rho0 - 1| on a held-out scene: %s" % {k: round(v, 5) for k, v in errs.items()})
    assert errs["learned+0"] < errs["plain1"], errs


def test_warm_start_stays_stable_over_a_long_run():
    """The 131k dam break over 2,000 steps (4 blocks of 500): the warm start + 5, trained as the
    bench trains it (four seeded rollouts of 300 steps under + 1), stays below the plain
    8-iteration solver in every block and does not drift (measured: 1.79, 1.73, 1.72, 1.71 %
    against 2.48-2.54 %)."""
    lattice = (32, 64, 64)
    net = None
    for seed in (1, 2, 3, 4):
        with fluids_model(scenes.dam_break(lattice=lattice, seed=seed), 2) as m:
            net, _ = warmstart.train_rollout(m, 300, extra_iterations=1, net=net, seed=0)
    test = scenes.dam_break(lattice=lattice)

    def blocks(iters, extra=None):
        out = []
        with fluids_model(test, iters) as m:
            m.enableSolverStats(True)
            if extra is not None:
                m.setWarmStart(net, extra_iterations=extra, guard_tolerance=0.0)
            for _ in range(4):
                m.resetSolverStats()
                m.update(500)
                out.append(m.solverStats()["mean"])
        return out

    warm, plain = blocks(3, 5), blocks(8)
    print("2,000 steps, block means: warm start + 5 %s, plain 8 %s" % (np.round(warm, 5), np.round(plain, 5)))
    assert all(w < p for w, p in zip(warm, plain)), (warm, plain)
    assert max(warm) < 1.2 * min(warm), warm  # no drift
