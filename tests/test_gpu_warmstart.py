"""Learned warm start on the GPU against the oracle.

- inference kernel and the trainer's loss / gradient against the oracle's double-precision
  restatement, both with the GPU's BF16 operand rounding emulated (tight) and without it;
- the trainer lowers the loss and is deterministic;
- training samples (features and targets) recorded by the library against the oracle's;
- warm-started steps (network + 0 or 1 extra iterations) against the oracle within the
  step tolerance 1e-5 x box;
- the guard: a step above tolerance reruns as the plain solver, bit for bit;
- what a trained network gains over the same solver without it.
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


def _small_net(rng, lam_scale, res_scale):
    return random_net(rng, out_scale=np.array([lam_scale, res_scale, res_scale, res_scale], np.float32))


@pytest.mark.parametrize("extra", [0, 1])
def test_warm_started_steps_match_oracle(extra):
    sc = scenes.dam_break(lattice=(8, 16, 16))
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    fp = sc["fluid_params"]
    L = box_size(sc["model_params"])
    rng = np.random.default_rng(9)
    # lambda of the plain first iteration is ~1e-6 here; residuals a fraction of a spacing
    net = _small_net(rng, 2e-7, 2e-5)
    with fluids_model(sc, 3) as m:
        m.setWarmStart(net, extra_iterations=extra, guard_tolerance=0.0)
        for step in range(4):
            st = gpu_state(m, abi.FLUIDS)
            lam = np.zeros(st["pos"].shape[0], np.float32)
            err_o, rerun = oracle.ws_step(c, fp, net, extra, 0.0, 3, st, lam)
            assert not rerun
            m.update(1)
            g = gpu_state(m, abi.FLUIDS)
            assert np.array_equal(g["id"], st["id"])
            assert_close_by_id(g["id"], g["pos"], st["id"], st["pos"], REL_BOX * L, "pos step %d" % step)
            assert_close_by_id(g["id"], g["vel"], st["id"], st["vel"], REL_BOX * L / fp.timeStep, "vel")
            lam_g = m.download(abi.BUF_LAMBDA_TOTAL)
            assert np.abs(lam_g - lam).max() <= 1e-3 * np.abs(lam).max() + 1e-12
        stats = m.solverStats()
        assert stats["steps"] == 4 and stats["reruns"] == 0


def test_guard_reruns_as_the_plain_solver():
    sc = scenes.dam_break(lattice=(8, 16, 16))
    rng = np.random.default_rng(1)
    net = _small_net(rng, 2e-7, 2e-5)
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


def test_trained_network_gain_over_the_plain_first_iteration():
    """Train on plain 8-iteration dam-break runs (2 seeded scenes), evaluate on a third.

    The network's multiplier replaces the plain solver's first-iteration lambda; its target
    is the converged one (lambda summed over the 8 reference iterations).  Gain: on held-out
    samples the network explains the target better (R^2) than the plain first-iteration
    lambda does under its best linear scaling.  The step-level outcome (solver-output mean
    density error of the warm start + 1 iteration against plain 2 and 8 iterations, same
    held-out scene) is printed, not asserted: on this workload a local network's multiplier
    errors, amplified by the correction's kernel gradients, cost about what it saves."""
    lattice = (16, 32, 32)
    feats, targets = warmstart.generate_samples(seeds=(1, 2), lattice=lattice, steps=160, record_every=10,
                                                stride=4, reference_iterations=8)
    assert feats.shape[0] == 2 * 16 * 4096
    net, hist = warmstart.train(feats, targets, epochs=16, batch=4096, learning_rate=2e-3, seed=1)
    assert hist[-1] < 0.7 * hist[0], hist
    fe, te = warmstart.generate_samples(seeds=(3,), lattice=lattice, steps=160, record_every=20, stride=4,
                                        reference_iterations=8)
    pred = warmstart.forward(net, fe).cpu().numpy()
    t = te.cpu().numpy()[:, 0]
    lam0 = fe.cpu().numpy()[:, 10].astype(np.float64)
    a = float(lam0 @ t / (lam0 @ lam0))
    r2_net = float(warmstart.r2(pred[:, 0], t))
    r2_plain = float(warmstart.r2(a * lam0, t))
    assert not np.any(pred[:, 1:]), "residual outputs are off by default"
    errs = {}
    sc = scenes.dam_break(lattice=lattice, seed=3)
    for name, iters, extra in (("plain2", 2, None), ("plain8", 8, None), ("learned+1", 8, 1)):
        with fluids_model(sc, iters) as m:
            m.enableSolverStats(True)
            if extra is not None:
                m.setWarmStart(net, extra_iterations=extra, guard_tolerance=0.0)
            m.update(160)
            errs[name] = round(m.solverStats()["mean"], 5)
    print("R2 of the converged multiplier: network %.3f, plain first iteration %.3f; "
          "solver-output density error %s" % (r2_net, r2_plain, errs))
    assert r2_net > r2_plain + 0.1, (r2_net, r2_plain)
