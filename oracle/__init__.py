"""Python front end of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: this package is the checker.  tests/, __graft_entry__.smoke()
and bench.py's CPU legs import it; the product package never does.  The C++ restatement
of the reference kernels lives in oracle.cpp; see oracle.h for what each function follows.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from realtimeparticles_gb300 import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build(quiet=True):
    """Compile liboracle.so with the Makefile next to this file."""
    out = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        src = os.path.join(_HERE, "oracle.cpp")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        L = C.CDLL(path)
        P = C.c_void_p
        L.or_derive_constants.argtypes = [C.c_int, C.POINTER(abi.ModelParams), C.POINTER(abi.GridConstants)]
        L.or_fill_cell_ids.argtypes = [C.POINTER(abi.GridConstants), P, C.c_uint32, P]
        L.or_stable_sort.argtypes = [P, C.c_uint32, P, P]
        L.or_cell_table.argtypes = [C.POINTER(abi.GridConstants), P, C.c_uint32, P]
        L.or_fluids_step.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.FluidParams), C.c_uint32,
                                     C.c_uint32, P]
        L.or_boids_step.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.BoidsParams), C.c_float,
                                    C.c_int, C.c_uint32, P]
        L.or_boids_step_dim.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.BoidsParams), C.c_float,
                                        C.c_int, C.c_int, C.c_uint32, P]
        L.or_boids_step_target.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.BoidsParams), C.c_float,
                                           C.c_int, C.c_int, P, C.c_float, C.c_int, C.c_uint32, P]
        L.or_perlin_noise.argtypes = [C.c_int, C.c_float, C.c_float, C.c_float]
        L.or_perlin_noise.restype = C.c_float
        L.or_target_trajectory.argtypes = [C.c_float, C.c_int, C.c_float, C.c_uint32, P]
        L.or_target_trajectory.restype = None
        L.or_clouds_step.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.FluidParams),
                                     C.POINTER(abi.CloudParams), C.POINTER(abi.CloudEnv), P, C.c_uint32,
                                     C.c_uint32, P]
        L.or_clouds_ws_step.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.FluidParams),
                                        C.POINTER(abi.CloudParams), C.POINTER(abi.CloudEnv), P,
                                        C.POINTER(abi.Mlp), C.c_uint32, C.c_uint32, P, P, P]
        L.or_clouds_ws_loss.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.FluidParams),
                                        C.POINTER(abi.CloudParams), C.POINTER(abi.CloudEnv), P,
                                        C.POINTER(abi.Mlp), C.c_int, C.c_uint32, P, C.POINTER(C.c_double), P]
        L.or_clouds_init.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.CloudParams),
                                     C.POINTER(abi.CloudEnv), P, C.c_uint32, P]
        L.or_fld_density.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.FluidParams), P, P,
                                     C.c_uint32, P]
        L.or_fld_lambda.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.FluidParams), P, P, P,
                                    C.c_uint32, P]
        L.or_fld_correction.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.FluidParams), P, P, P,
                                        C.c_uint32, P]
        L.or_fluid_metrics.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.FluidParams), P, P, P,
                                       C.c_uint32, C.POINTER(abi.Metrics)]
        L.or_ws_features.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.FluidParams), P, P, P,
                                     C.c_uint32, P]
        L.or_mlp_forward.argtypes = [C.POINTER(abi.Mlp), P, C.c_uint64, C.c_int, P]
        L.or_mlp_loss_grad.argtypes = [C.POINTER(abi.Mlp), P, P, P, C.c_uint64, C.c_int, C.POINTER(C.c_double), P]
        L.or_ws_step.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.FluidParams), C.POINTER(abi.Mlp),
                                 C.c_uint32, C.c_float, C.c_uint32, C.c_uint32, P, P, C.POINTER(C.c_double),
                                 C.POINTER(C.c_int), C.c_int]
        L.or_mlp_backward.argtypes = [C.POINTER(abi.Mlp), P, P, C.c_uint64, C.c_int, P]
        L.or_ws_loss_grad.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.FluidParams), C.POINTER(abi.Mlp),
                                      C.c_int, C.c_uint32, P, C.POINTER(C.c_double), P, P]
        L.or_ws_record_step.argtypes = [C.POINTER(abi.GridConstants), C.POINTER(abi.FluidParams), C.c_uint32,
                                        C.c_uint32, C.c_uint32, C.c_uint32, P, P, P, P, C.POINTER(C.c_uint32)]
        L.or_fill_fluid_color.argtypes = [P, C.c_uint32, C.c_float, P]
        L.or_fill_color_float.argtypes = [P, C.c_uint32, C.c_float, C.c_float, P]
        L.or_fill_camera_dist.argtypes = [P, C.c_uint32, C.c_uint32, P, P]
        L.or_fill_grid_detector.argtypes = [C.POINTER(abi.GridConstants), P, C.c_uint32, P]
        L.or_set_threads.argtypes = [C.c_int]
        L.or_get_threads.restype = C.c_int
        _LIB = L
    return _LIB


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class _State(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in (
        "pos", "vel", "predPos", "totCorrPos", "acc", "vort", "density", "lambda_", "temp", "vapor",
        "cloud", "buoyancy", "id", "cellId", "table")]


_STATE_KEYS = {"pos": "pos", "vel": "vel", "predPos": "predPos", "totCorrPos": "totCorrPos",
               "acc": "acc", "vort": "vort", "density": "density", "lambda": "lambda_", "temp": "temp",
               "vapor": "vapor", "cloud": "cloud", "buoyancy": "buoyancy", "id": "id",
               "cellId": "cellId", "table": "table"}


def _state(d):
    s = _State()
    for k, f in _STATE_KEYS.items():
        a = d.get(k)
        if a is not None:
            assert a.flags["C_CONTIGUOUS"], k
            setattr(s, f, a.ctypes.data)
    return s


def set_threads(n):
    lib().or_set_threads(int(n))


def get_threads():
    return lib().or_get_threads()


def derive_constants(model, mp):
    c = abi.GridConstants()
    rc = lib().or_derive_constants(int(model), C.byref(mp), C.byref(c))
    if rc != 0:
        raise ValueError("or_derive_constants failed: %d" % rc)
    return c


def fill_cell_ids(c, pos):
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    n = pos.shape[0]
    keys = np.empty(n, np.uint32)
    lib().or_fill_cell_ids(C.byref(c), _p(pos), n, _p(keys))
    return keys


def stable_sort(keys):
    keys = np.ascontiguousarray(keys, dtype=np.uint32)
    n = keys.shape[0]
    sk = np.empty(n, np.uint32)
    perm = np.empty(n, np.uint32)
    lib().or_stable_sort(_p(keys), n, _p(sk), _p(perm))
    return sk, perm


def cell_table(c, sorted_keys):
    sorted_keys = np.ascontiguousarray(sorted_keys, dtype=np.uint32)
    t = np.empty((c.numCells, 2), np.uint32)
    lib().or_cell_table(C.byref(c), _p(sorted_keys), sorted_keys.shape[0], _p(t))
    return t


def new_state(n, c=None, model=abi.FLUIDS):
    """Zeroed state arrays for n particles (float4 arrays are (n, 4))."""
    f4 = lambda: np.zeros((n, 4), np.float32)
    f1 = lambda: np.zeros(n, np.float32)
    d = {"pos": f4(), "vel": f4(), "predPos": f4(), "density": f1(), "lambda": f1(),
         "vort": f4(), "id": np.arange(n, dtype=np.uint32), "cellId": np.zeros(n, np.uint32)}
    if model == abi.BOIDS:
        d["acc"] = f4()
    if model == abi.CLOUDS:
        d.update(totCorrPos=f4(), temp=f1(), vapor=f1(), cloud=f1(), buoyancy=f1())
    if c is not None:
        d["table"] = np.zeros((c.numCells, 2), np.uint32)
    return d


def fluids_step(c, fp, iters, st):
    n = st["pos"].shape[0]
    s = _state(st)
    rc = lib().or_fluids_step(C.byref(c), C.byref(fp), int(iters), n, C.byref(s))
    if rc != 0:
        raise ValueError("or_fluids_step failed: %d" % rc)


def boids_step(c, bp, dt, boundary, st, dim=3, target=None, target_radius=2.0, target_sign=1):
    """One Boids::update; `target` (x, y, z) applies the target rule with that position."""
    n = st["pos"].shape[0]
    s = _state(st)
    t = None if target is None else np.ascontiguousarray(target, dtype=np.float32)
    rc = lib().or_boids_step_target(C.byref(c), C.byref(bp), float(dt), int(boundary), int(dim), _p(t),
                                    float(target_radius), int(target_sign), n, C.byref(s))
    if rc != 0:
        raise ValueError("or_boids_step failed: %d" % rc)


def perlin_noise(seed, x, y, z):
    return float(lib().or_perlin_noise(int(seed), float(x), float(y), float(z)))


def target_trajectory(box_width, dim, particles_vel, nsteps):
    """Target positions after each of nsteps Target::updatePos calls from a new Target: [nsteps, 3]."""
    out = np.empty((int(nsteps), 3), np.float32)
    lib().or_target_trajectory(float(box_width), int(dim), float(particles_vel), int(nsteps), _p(out))
    return out


def clouds_init(c, cp, env, ground, st):
    n = st["pos"].shape[0]
    s = _state(st)
    g = None if ground is None else np.ascontiguousarray(ground, dtype=np.float32)
    lib().or_clouds_init(C.byref(c), C.byref(cp), C.byref(env), _p(g), n, C.byref(s))


def clouds_step(c, fp, cp, env, ground, iters, st):
    n = st["pos"].shape[0]
    s = _state(st)
    g = None if ground is None else np.ascontiguousarray(ground, dtype=np.float32)
    rc = lib().or_clouds_step(C.byref(c), C.byref(fp), C.byref(cp), C.byref(env), _p(g), int(iters), n,
                              C.byref(s))
    if rc != 0:
        raise ValueError("or_clouds_step failed: %d" % rc)


def clouds_ws_step(c, fp, cp, env, ground, net, extra_iters, st):
    """One warm-started clouds step in place; returns (features [n, 12], omega [n]) by sorted
    index (the order of st after the step)."""
    n = st["pos"].shape[0]
    s = _state(st)
    g = None if ground is None else np.ascontiguousarray(ground, dtype=np.float32)
    feats = np.zeros((n, 12), np.float32)
    om = np.zeros(n, np.float32)
    rc = lib().or_clouds_ws_step(C.byref(c), C.byref(fp), C.byref(cp), C.byref(env), _p(g), C.byref(net),
                                 int(extra_iters), n, C.byref(s), _p(feats), _p(om))
    if rc != 0:
        raise ValueError("or_clouds_ws_step failed: %d" % rc)
    return feats, om


def clouds_ws_loss(c, fp, cp, env, ground, net, st, emulate=False):
    """(loss, features [n, 12]) of the clouds warm start at state st, which advances through
    the step's presort (sorted order and thermodynamics)."""
    n = st["pos"].shape[0]
    s = _state(st)
    g = None if ground is None else np.ascontiguousarray(ground, dtype=np.float32)
    feats = np.zeros((n, 12), np.float32)
    loss = C.c_double()
    rc = lib().or_clouds_ws_loss(C.byref(c), C.byref(fp), C.byref(cp), C.byref(env), _p(g), C.byref(net),
                                 1 if emulate else 0, n, C.byref(s), C.byref(loss), _p(feats))
    if rc != 0:
        raise ValueError("or_clouds_ws_loss failed: %d" % rc)
    return loss.value, feats


def fld_density(c, fp, pred, table):
    n = pred.shape[0]
    out = np.empty(n, np.float32)
    lib().or_fld_density(C.byref(c), C.byref(fp), _p(pred), _p(table), n, _p(out))
    return out


def fld_lambda(c, fp, pred, density, table):
    n = pred.shape[0]
    out = np.empty(n, np.float32)
    lib().or_fld_lambda(C.byref(c), C.byref(fp), _p(pred), _p(density), _p(table), n, _p(out))
    return out


def fld_correction(c, fp, pred, lam, table):
    n = pred.shape[0]
    out = np.empty((n, 4), np.float32)
    lib().or_fld_correction(C.byref(c), C.byref(fp), _p(pred), _p(lam), _p(table), n, _p(out))
    return out


def fluid_metrics(c, fp, pred, vel, table):
    m = abi.Metrics()
    lib().or_fluid_metrics(C.byref(c), C.byref(fp), _p(pred), _p(vel), _p(table), pred.shape[0], C.byref(m))
    return m


# ---- side outputs -----------------------------------------------------------------------
def fill_fluid_color(density, rest_density):
    d = np.ascontiguousarray(density, dtype=np.float32)
    out = np.empty((d.shape[0], 4), np.float32)
    lib().or_fill_fluid_color(_p(d), d.shape[0], float(rest_density), _p(out))
    return out


def fill_color_float(q, vmin, vmax):
    q = np.ascontiguousarray(q, dtype=np.float32)
    out = np.empty((q.shape[0], 4), np.float32)
    lib().or_fill_color_float(_p(q), q.shape[0], float(vmin), float(vmax), _p(out))
    return out


def fill_camera_dist(pos, n, cam):
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    cam = np.ascontiguousarray(cam, dtype=np.float32)
    out = np.empty(pos.shape[0], np.uint32)
    lib().or_fill_camera_dist(_p(pos), int(n), pos.shape[0], _p(cam), _p(out))
    return out


def fill_grid_detector(c, pos):
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    out = np.empty((c.numCells, 8), np.float32)
    lib().or_fill_grid_detector(C.byref(c), _p(pos), pos.shape[0], _p(out))
    return out


# ---- learned warm start (restates the GPU method) ---------------------------------------
MLP_GRAD_SHAPES = (("w1", (64, 12)), ("b1", (64,)), ("w2", (64, 64)), ("b2", (64,)), ("w3", (4, 64)), ("b3", (4,)))


def ws_features(c, fp, x0, vel, table):
    x0 = np.ascontiguousarray(x0, dtype=np.float32)
    vel = np.ascontiguousarray(vel, dtype=np.float32)
    table = np.ascontiguousarray(table, dtype=np.uint32)
    n = x0.shape[0]
    out = np.empty((n, 12), np.float32)
    lib().or_ws_features(C.byref(c), C.byref(fp), _p(x0), _p(vel), _p(table), n, _p(out))
    return out


def mlp_forward(net, feats, emulate=True):
    feats = np.ascontiguousarray(feats, dtype=np.float32)
    out = np.empty((feats.shape[0], 4), np.float32)
    lib().or_mlp_forward(C.byref(net), _p(feats), feats.shape[0], 1 if emulate else 0, _p(out))
    return out


def mlp_loss_grad(net, loss_weights, feats, targets, emulate=True):
    """(loss, {name: gradient array}) in double precision."""
    feats = np.ascontiguousarray(feats, dtype=np.float32)
    targets = np.ascontiguousarray(targets, dtype=np.float32)
    lw = np.ascontiguousarray(loss_weights, dtype=np.float32)
    g = np.empty(5252, np.float64)
    loss = C.c_double()
    lib().or_mlp_loss_grad(C.byref(net), _p(lw), _p(feats), _p(targets), feats.shape[0], 1 if emulate else 0,
                           C.byref(loss), _p(g))
    out, o = {}, 0
    for name, shape in MLP_GRAD_SHAPES:
        size = int(np.prod(shape))
        out[name] = g[o:o + size].reshape(shape)
        o += size
    return loss.value, out


def mlp_backward(net, feats, dy, emulate=True):
    """{name: gradient} of sum_s sum_o dy_so y_so (double precision)."""
    feats = np.ascontiguousarray(feats, dtype=np.float32)
    dy = np.ascontiguousarray(dy, dtype=np.float32)
    g = np.empty(5252, np.float64)
    lib().or_mlp_backward(C.byref(net), _p(feats), _p(dy), feats.shape[0], 1 if emulate else 0, _p(g))
    out, o = {}, 0
    for name, shape in MLP_GRAD_SHAPES:
        size = int(np.prod(shape))
        out[name] = g[o:o + size].reshape(shape)
        o += size
    return out


def ws_loss_grad(c, fp, net, st, emulate=True):
    """(loss, dL/dy by particle id, omega by particle id) of the warm start through the solve at
    the state st (advanced by the step's presort only)."""
    n = st["pos"].shape[0]
    s = _state(st)
    loss = C.c_double()
    dy = np.zeros(n, np.float64)
    om = np.zeros(n, np.float64)
    rc = lib().or_ws_loss_grad(C.byref(c), C.byref(fp), C.byref(net), 1 if emulate else 0, n, C.byref(s),
                               C.byref(loss), _p(dy), _p(om))
    if rc != 0:
        raise ValueError("or_ws_loss_grad failed: %d" % rc)
    return loss.value, dy, om


def ws_step(c, fp, net, extra_iters, guard_tol, plain_iters, st, lam_tot, relax_all=False):
    """One warm-started step in place; returns (solver-output mean error, rerun flag)."""
    n = st["pos"].shape[0]
    s = _state(st)
    err = C.c_double()
    rr = C.c_int()
    rc = lib().or_ws_step(C.byref(c), C.byref(fp), C.byref(net), int(extra_iters), float(guard_tol),
                          int(plain_iters), n, C.byref(s), _p(lam_tot), C.byref(err), C.byref(rr),
                          1 if relax_all else 0)
    if rc != 0:
        raise ValueError("or_ws_step failed: %d" % rc)
    return err.value, bool(rr.value)


def ws_record_step(c, fp, iters, stride, phase, st, lam_tot):
    """One plain step in place that also returns (features, targets) of the sampled particles."""
    n = st["pos"].shape[0]
    s = _state(st)
    cap = max(0, (n - phase + stride - 1) // stride)
    feats = np.zeros((max(cap, 1), 12), np.float32)
    tg = np.zeros((max(cap, 1), 4), np.float32)
    cnt = C.c_uint32()
    rc = lib().or_ws_record_step(C.byref(c), C.byref(fp), int(iters), int(stride), int(phase), n, C.byref(s),
                                 _p(lam_tot), _p(feats), _p(tg), C.byref(cnt))
    if rc != 0:
        raise ValueError("or_ws_record_step failed: %d" % rc)
    return feats[:cnt.value], tg[:cnt.value]


# ---- the reference's own kernels, compiled for the CPU (oracle/ref/build_ref.py) -------
_REF = None
REF_LIB_PATH = os.path.join(_HERE, "_ref", "libref.so")


def ref_available():
    return os.path.exists(REF_LIB_PATH)


def ref_lib():
    """libref.so: the reference's step kernels driven in the reference's update() order."""
    global _REF
    if _REF is None:
        if not ref_available():
            raise RuntimeError("oracle/_ref/libref.so not built (python oracle/ref/build_ref.py)")
        L = C.CDLL(REF_LIB_PATH)
        P = C.c_void_p
        G = C.POINTER(abi.GridConstants)
        L.ref_fill_cell_ids.argtypes = [G, P, C.c_uint32, P]
        L.ref_cell_table.argtypes = [G, P, C.c_uint32, P]
        L.ref_fluids_step.argtypes = [G, C.POINTER(abi.FluidParams), C.c_uint32, C.c_uint32, P]
        L.ref_boids_step.argtypes = [G, C.POINTER(abi.BoidsParams), C.c_float, C.c_int, C.c_int, C.c_uint32, P]
        L.ref_boids_step_target.argtypes = [G, C.POINTER(abi.BoidsParams), C.c_float, C.c_int, C.c_int, P,
                                            C.c_float, C.c_int, C.c_uint32, P]
        L.ref_perlin_noise.argtypes = [C.c_int, C.c_float, C.c_float, C.c_float]
        L.ref_perlin_noise.restype = C.c_float
        L.ref_clouds_step.argtypes = [G, C.POINTER(abi.FluidParams), C.POINTER(abi.CloudParams), C.c_uint32,
                                      C.c_uint32, P]
        L.ref_clouds_init.argtypes = [G, C.POINTER(abi.CloudParams), C.c_uint32, P]
        L.ref_fill_fluid_color.argtypes = [G, C.POINTER(abi.FluidParams), P, C.c_uint32, P]
        L.ref_fill_color_float.argtypes = [G, P, C.c_uint32, C.c_float, C.c_float, P]
        L.ref_fill_camera_dist.argtypes = [G, P, C.c_uint32, C.c_uint32, P, P]
        L.ref_fill_grid_detector.argtypes = [G, P, C.c_uint32, P]
        if hasattr(L, "ref_generate_3d_grid"):
            L.ref_generate_3d_grid.argtypes = [C.c_int, P, P, P, P]
            L.ref_generate_2d_grid_yz.argtypes = [C.c_int, P, P, P, P]
        _REF = L
    return _REF


def ref_fill_cell_ids(c, pos):
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    keys = np.empty(pos.shape[0], np.uint32)
    ref_lib().ref_fill_cell_ids(C.byref(c), _p(pos), pos.shape[0], _p(keys))
    return keys


def ref_cell_table(c, sorted_keys):
    sorted_keys = np.ascontiguousarray(sorted_keys, dtype=np.uint32)
    t = np.empty((c.numCells, 2), np.uint32)
    ref_lib().ref_cell_table(C.byref(c), _p(sorted_keys), sorted_keys.shape[0], _p(t))
    return t


def ref_fluids_step(c, fp, iters, st):
    s = _state(st)
    ref_lib().ref_fluids_step(C.byref(c), C.byref(fp), int(iters), st["pos"].shape[0], C.byref(s))


def ref_boids_step(c, bp, dt, boundary, st, dim=3, target=None, target_radius=2.0, target_sign=1):
    s = _state(st)
    t = None if target is None else np.ascontiguousarray(target, dtype=np.float32)
    ref_lib().ref_boids_step_target(C.byref(c), C.byref(bp), float(dt), int(boundary), int(dim), _p(t),
                                    float(target_radius), int(target_sign), st["pos"].shape[0], C.byref(s))


def ref_perlin_noise(seed, x, y, z):
    """The reference's PerlinNoise; None when its copy was not compiled in."""
    v = float(ref_lib().ref_perlin_noise(int(seed), float(x), float(y), float(z)))
    return None if v == -1.0 else v


def ref_clouds_step(c, fp, cp, iters, st):
    s = _state(st)
    ref_lib().ref_clouds_step(C.byref(c), C.byref(fp), C.byref(cp), int(iters), st["pos"].shape[0], C.byref(s))


def ref_clouds_init(c, cp, st):
    s = _state(st)
    ref_lib().ref_clouds_init(C.byref(c), C.byref(cp), st["pos"].shape[0], C.byref(s))


def ref_side_outputs(c, fp, density, q, vmin, vmax, pos, n, cam):
    """The reference's side-output kernels: (fluid colours, float colours, camera distances,
    grid detector)."""
    L = ref_lib()
    density = np.ascontiguousarray(density, dtype=np.float32)
    q = np.ascontiguousarray(q, dtype=np.float32)
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    cam = np.ascontiguousarray(cam, dtype=np.float32)
    col = np.empty((density.shape[0], 4), np.float32)
    L.ref_fill_fluid_color(C.byref(c), C.byref(fp), _p(density), density.shape[0], _p(col))
    colf = np.empty((q.shape[0], 4), np.float32)
    L.ref_fill_color_float(C.byref(c), _p(q), q.shape[0], float(vmin), float(vmax), _p(colf))
    dist = np.empty(pos.shape[0], np.uint32)
    L.ref_fill_camera_dist(C.byref(c), _p(pos), int(n), pos.shape[0], _p(cam), _p(dist))
    det = np.empty((c.numCells, 8), np.float32)
    L.ref_fill_grid_detector(C.byref(c), _p(pos), int(n), _p(det))
    return col, colf, dist, det


def ref_geometry_available():
    return ref_available() and hasattr(ref_lib(), "ref_generate_3d_grid")


def ref_generate_3d_grid(shape, res, start, end):
    """The reference's Geometry::Generate3DGrid (uniform); shape "box" or "sphere"."""
    res = np.ascontiguousarray(res, dtype=np.int32)
    s = np.ascontiguousarray(start, dtype=np.float32)
    e = np.ascontiguousarray(end, dtype=np.float32)
    out = np.zeros((int(np.prod(res)), 3), np.float32)
    k = ref_lib().ref_generate_3d_grid(1 if shape == "sphere" else 0, _p(res), _p(s), _p(e), _p(out))
    return out[:k]


def ref_generate_2d_grid_yz(shape, res, start, end):
    """The reference's Geometry::Generate2DGrid in the YZ plane (uniform); shape "rect" or "circle"."""
    res = np.ascontiguousarray(res, dtype=np.int32)
    s = np.ascontiguousarray(start, dtype=np.float32)
    e = np.ascontiguousarray(end, dtype=np.float32)
    out = np.zeros((int(np.prod(res)), 3), np.float32)
    k = ref_lib().ref_generate_2d_grid_yz(1 if shape == "circle" else 0, _p(res), _p(s), _p(e), _p(out))
    return out[:k]
