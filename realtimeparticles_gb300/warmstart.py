"""Learned warm start of the PBF constraint solve: the network trained through the solve on the
model's own rollout by the library's GPU kernels, regression samples from plain runs, and the
network file format.

The network relaxes the plain first-iteration lambda per particle, lambda <- omega(y) lambda
with omega = 1 + tanh(y) (2 for y > 0, 1 otherwise); a zero output layer is the plain solver.
The C entry points are rtp_train_warm_start_rollout, rtp_warm_start_loss_grad,
rtp_set_warm_start, and for regression rtp_record_warm_start_samples / rtp_train_warm_start
(include/rtp.h).  PyTorch only provides device buffers; every computation is a library kernel.
"""
import ctypes as C

import numpy as np

from . import abi, scenes
from ._lib import call
from .model import Fluids

# The residual outputs are off by default (loss weight 0, output scale 0): on the dam break
# they are barely predictable from the features (R^2 ~ 0.1) and their errors only add
# position noise.  Pass loss_weights=(1, 1, 1, 1) to train them.
DEFAULT_TRAIN = dict(epochs=24, batch=8192, learning_rate=2e-3, final_lr_fraction=0.02, beta1=0.9, beta2=0.999,
                     eps=1e-8, weight_decay=1e-4, loss_weights=(1.0, 0.0, 0.0, 0.0), seed=0)


def _torch():
    import torch
    return torch


def record_run(model, steps, reference_iterations, stride, record_every, feats, targets, offset):
    """Advances `model` by `steps` plain steps with `reference_iterations` Jacobi
    iterations; every `record_every`-th step writes the samples of every `stride`-th
    particle (the phase rotates so that successive records cover different particles)
    into the float32 CUDA tensors feats[offset:], targets[offset:].  Returns the new offset."""
    model.setJacobiIterations(reference_iterations)
    cap = feats.shape[0]
    k = 0
    for s in range(steps):
        if s % record_every == 0 and offset < cap:
            phase = k % stride
            w = model.recordWarmStartSamples(reference_iterations, stride, phase,
                                             feats.data_ptr() + offset * feats.stride(0) * 4,
                                             targets.data_ptr() + offset * targets.stride(0) * 4, cap - offset)
            offset += w
            k += 1
        else:
            model.update(1)
    model.synchronize()
    return offset


def generate_samples(seeds=range(1, 9), lattice=(32, 64, 64), steps=400, record_every=25, stride=8,
                     reference_iterations=24):
    """Samples of `len(seeds)` seeded dam-break runs (scenes.dam_break) on cuda:0:
    returns (features [m, 12], targets [m, 4]) float32 CUDA tensors."""
    torch = _torch()
    n = int(np.prod(lattice))
    per_record = (n + stride - 1) // stride
    records = (steps + record_every - 1) // record_every
    cap = len(list(seeds)) * records * per_record
    feats = torch.empty((cap, abi.MLP_IN), dtype=torch.float32, device="cuda")
    targets = torch.empty((cap, abi.MLP_OUT), dtype=torch.float32, device="cuda")
    off = 0
    for seed in seeds:
        sc = scenes.dam_break(lattice=lattice, seed=int(seed))
        with Fluids(sc["model_params"]) as m:
            m.setFluidParams(sc["fluid_params"])
            m.upload(abi.BUF_POS, sc["pos"])
            m.upload(abi.BUF_VEL, sc["vel"])
            off = record_run(m, steps, reference_iterations, stride, record_every, feats, targets, off)
    return feats[:off], targets[:off]


def train_config(**kw):
    d = dict(DEFAULT_TRAIN)
    d.update(kw)
    cfg = abi.TrainConfig()
    cfg.epochs = int(d["epochs"])
    cfg.batch = int(d["batch"])
    cfg.learningRate = float(d["learning_rate"])
    cfg.finalLrFraction = float(d["final_lr_fraction"])
    cfg.beta1 = float(d["beta1"])
    cfg.beta2 = float(d["beta2"])
    cfg.eps = float(d["eps"])
    cfg.weightDecay = float(d["weight_decay"])
    for o in range(abi.MLP_OUT):
        cfg.lossWeights[o] = float(d["loss_weights"][o])
    cfg.seed = int(d["seed"])
    return cfg


def train(feats, targets, **kw):
    """Trains a network on CUDA float32 sample tensors with the library's kernels.
    Outputs trained with loss weight 0 are switched off (output scale 0).
    Returns (abi.Mlp, per-epoch mean losses)."""
    cfg = train_config(**kw)
    net = abi.Mlp()
    hist = (C.c_float * cfg.epochs)()
    n = int(feats.shape[0])
    assert feats.is_contiguous() and targets.is_contiguous() and int(targets.shape[0]) == n
    call("rtp_train_warm_start", C.c_void_p(feats.data_ptr()), C.c_void_p(targets.data_ptr()), n, C.byref(cfg),
         C.byref(net), hist, None)
    for o in range(abi.MLP_OUT):
        if cfg.lossWeights[o] == 0.0:
            net.outScale[o] = 0.0
    return net, [float(v) for v in hist]


ROLLOUT_TRAIN = dict(learning_rate=2e-3, final_lr_fraction=0.05, beta1=0.9, beta2=0.999, eps=1e-8,
                     weight_decay=0.0, seed=0)


def omega(y):
    """The relaxation the network's output y sets (numpy)."""
    y = np.asarray(y, np.float64)
    return 1.0 + np.tanh(y) * np.where(y > 0, 2.0, 1.0)


def train_rollout(model, steps, extra_iterations=0, net=None, **kw):
    """Trains the warm-start network through the solve on `model`'s own rollout (the model
    advances `steps` steps under the warm-started solver).  net=None starts a new network.
    Returns (abi.Mlp, per-step losses)."""
    d = dict(ROLLOUT_TRAIN)
    d.update(kw)
    cfg = train_config(epochs=1, batch=16, loss_weights=(1.0, 0.0, 0.0, 0.0), **d)
    init = net is None
    net = abi.Mlp() if init else net
    hist = (C.c_float * max(1, steps))()
    call("rtp_train_warm_start_rollout", model.handle, C.byref(cfg), int(steps), int(extra_iterations),
         1 if init else 0, C.byref(net), hist)
    return net, [float(v) for v in hist[:steps]]


def loss_grad_solve(model, net):
    """(loss, dL/dy by particle id as a CUDA tensor) of the warm start through the solve at the
    model's current state (the model is not advanced)."""
    torch = _torch()
    n = model.nbParticles()
    dy = torch.zeros(n, dtype=torch.float32, device="cuda")
    loss = C.c_double()
    call("rtp_warm_start_loss_grad", model.handle, C.byref(net), C.c_void_p(dy.data_ptr()), C.byref(loss))
    return loss.value, dy


def backward(net, feats, dy):
    """Parameter gradient (abi.Mlp) of sum dy * y for CUDA rows (the trainer's kernels)."""
    grad = abi.Mlp()
    call("rtp_mlp_backward", C.byref(net), C.c_void_p(feats.data_ptr()), C.c_void_p(dy.data_ptr()),
         int(feats.shape[0]), C.byref(grad), None)
    return grad


def r2(pred, target):
    """Coefficient of determination of pred against target (numpy, per column)."""
    pred = np.asarray(pred, np.float64)
    target = np.asarray(target, np.float64)
    return 1.0 - ((pred - target) ** 2).sum(0) / ((target - target.mean(0)) ** 2).sum(0)


def loss_grad(net, feats, targets, loss_weights=(1.0, 1.0, 1.0, 1.0)):
    """(loss, gradient as abi.Mlp) of `net` over CUDA sample tensors (the trainer's kernels)."""
    lw = (C.c_float * abi.MLP_OUT)(*loss_weights)
    loss = C.c_double()
    grad = abi.Mlp()
    call("rtp_mlp_loss_grad", C.byref(net), lw, C.c_void_p(feats.data_ptr()), C.c_void_p(targets.data_ptr()),
         int(feats.shape[0]), C.byref(loss), C.byref(grad), None)
    return loss.value, grad


def forward(net, feats):
    """Network outputs (target units) for CUDA feature rows, by the inference kernel."""
    torch = _torch()
    out = torch.empty((int(feats.shape[0]), abi.MLP_OUT), dtype=torch.float32, device=feats.device)
    call("rtp_mlp_forward", C.byref(net), C.c_void_p(feats.data_ptr()), int(feats.shape[0]),
         C.c_void_p(out.data_ptr()), None)
    return out


def save(net, path, **meta):
    """Writes the network (and string metadata) as .npz."""
    arrays = abi.mlp_to_arrays(net)
    np.savez(path, **arrays, **{"meta_" + k: np.array(str(v)) for k, v in meta.items()})


def load(path):
    with np.load(path) as z:
        return abi.mlp_from_arrays({k: z[k] for k in abi.MLP_ARRAYS})
