"""The oracle's restatement of the warm-start network: its analytic gradient (double
precision, no BF16 rounding) against central finite differences of its own loss, so the
gradient the GPU kernels are later compared with is itself checked."""
import numpy as np

import oracle
from helpers import random_net
from realtimeparticles_gb300 import abi


def test_mlp_gradient_matches_finite_differences():
    rng = np.random.default_rng(7)
    net = random_net(rng)
    feats = rng.normal(0, 1, (48, 12)).astype(np.float32)
    targets = rng.normal(0, 1, (48, 4)).astype(np.float32)
    lw = np.array([1.0, 0.5, 0.5, 2.0], np.float32)
    loss, grad = oracle.mlp_loss_grad(net, lw, feats, targets, emulate=False)
    base = abi.mlp_to_arrays(net)
    eps = 1e-3
    checked = 0
    for name in abi.MLP_TRAINABLE:
        flat = base[name].reshape(-1)
        for idx in rng.choice(flat.size, size=min(12, flat.size), replace=False):
            plus, minus = {k: v.copy() for k, v in base.items()}, {k: v.copy() for k, v in base.items()}
            plus[name].reshape(-1)[idx] += eps
            minus[name].reshape(-1)[idx] -= eps
            # the parameter as stored (float32) is what the oracle reads
            hp = float(plus[name].reshape(-1)[idx]) - float(flat[idx])
            hm = float(flat[idx]) - float(minus[name].reshape(-1)[idx])
            lp, _ = oracle.mlp_loss_grad(abi.mlp_from_arrays(plus), lw, feats, targets, emulate=False)
            lm, _ = oracle.mlp_loss_grad(abi.mlp_from_arrays(minus), lw, feats, targets, emulate=False)
            fd = (lp - lm) / (hp + hm)
            an = grad[name].reshape(-1)[idx]
            assert abs(fd - an) <= 2e-3 * max(1e-3, abs(an)) + 1e-6, (name, idx, fd, an)
            checked += 1
    assert checked >= 60
    assert np.isfinite(loss) and loss > 0


def test_mlp_forward_emulation_is_close_to_double():
    """BF16 operand rounding changes the outputs by well under a percent of their scale."""
    rng = np.random.default_rng(3)
    net = random_net(rng)
    feats = rng.normal(0, 1, (256, 12)).astype(np.float32)
    exact = oracle.mlp_forward(net, feats, emulate=False)
    emu = oracle.mlp_forward(net, feats, emulate=True)
    scale = np.abs(exact).max(axis=0)
    assert np.all(np.abs(emu - exact).max(axis=0) <= 0.03 * scale)
    assert not np.array_equal(emu, exact)


def test_oracle_guard_rerun_is_the_plain_step():
    """With a tolerance every step exceeds, the oracle's warm-started step is the plain step."""
    from realtimeparticles_gb300 import scenes
    sc = scenes.dam_break(lattice=(8, 8, 16))
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    fp = sc["fluid_params"]
    n = sc["pos"].shape[0]
    a = oracle.new_state(n, c)
    a["pos"][:] = sc["pos"]
    a["vel"][:] = sc["vel"]
    b = {k: v.copy() for k, v in a.items()}
    net = random_net(np.random.default_rng(0))
    lam = np.zeros(n, np.float32)
    for _ in range(2):
        oracle.fluids_step(c, fp, 3, a)
        err, rerun = oracle.ws_step(c, fp, net, 0, 1e-12, 3, b, lam)
        assert rerun and err > 0
    for k in ("pos", "vel", "id"):
        assert np.array_equal(a[k], b[k]), k
