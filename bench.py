#!/usr/bin/env python3
"""Benchmark of the GB300 simulation step.

Workload (default): the 3D PBF dam break of 131,072 particles (32 x 64 x 64 jittered
lattice, d = 0.0125 in a unit box, h = 2d, substep dt = 1/240 s, 3 Jacobi iterations,
vorticity confinement + XSPH).  One step = one Model::update() (one substep).
Metric: particle-steps/s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

* autotune (fluids workloads): the launch shape (list-sweep lanes; for one scene whether the
  lambda sweep runs tiled by bricks of cells, for a batch the cell factor) is picked by the
  library's autotuner before warm-up; candidates (lanes/factor/tiled) and times reported.
* value: K device-timed steps (CUDA events around each graph replay on the model's
  stream), inputs resident in HBM, L2 flushed before every step by a 256 MiB write.
* e2e: K steps through the public API with host buffers: one rtp_update_host call per step
  (upload pos/vel from pinned host memory, one update, download pos/vel, one
  synchronisation), timed on the host clock.
* roofline: the dominant kernel's algorithmic bytes / its mean CUDA-event duration
  (captured event nodes inside the same graph replays), against MEASURED_PEAKS.json.
* sweep (fluids, when the dominant kernel is the density/lambda sweep): candidates tested and
  pairs within h evaluated per second by that kernel (it is bound by dependent loads, so its
  HBM fraction says little), with its L1 data-pipe fraction of peak from a committed ncu capture
  and the candidate-test rate that fraction extrapolates to at the L1 ceiling.
* cpu_baseline: the reference's own kernels (physics/ocl/kernels/*.cl compiled for the
  CPU by oracle/ref/build_ref.py, OpenMP over the host cores) on a bounded sample of the
  same workload; the oracle's restatement when those are not built.
* warm_start (default workload): the learned warm start measured against the plain solver
  at equal solver-output density error.  A network is trained through the solve on the GPU
  by the library's kernels (the rollouts of the same lattice with seeds 1-4, 300 steps each),
  then the plain solver (1-48 iterations) and the warm start (+0-11 plain iterations) each
  run 100 device-timed steps of the seed-0 scene after 100 warm-up steps with the solver
  statistics on; the speed-up at equal error compares each warm-started configuration with
  the plain solver's Pareto front interpolated (log-log) at its error, and at_error_le_1pct
  the fastest configurations of each whose mean error is at most 1 % of rho0.  `long_run`
  repeats the comparison over 2,000 steps from the start (plain 3-24 iterations, warm start
  +2, +5, +9), the error averaged over the whole run.
* warm_start (clouds_131k): the same comparison on the clouds solve over the clouds
  configuration's 4,000 steps: networks trained through the clouds solve on the rollouts of
  seeds 1-2 (1,500 steps each, under + 0 and under + 1), then the plain clouds solver (1-8
  iterations) and the warm start (+0-3) on the seed-0 column, 4 blocks of 1,000 steps each.
* --impl reference: that CPU implementation alone (rank 0), same metric and config.
Under torchrun (N > 1) each rank runs an independent replica of the workload on its
own GPU (one scene does not shard; a batch shards by scene: rank r steps its own seeded
scene set, seed + r): barrier + max-over-ranks timing, value = the particles of all ranks
over that time.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from realtimeparticles_gb300 import abi, scenes  # noqa: E402

L2_FLUSH_BYTES = 256 << 20
# The config's "l2" entry, identical on both arms so that their configs compare equal.
L2_NOTE = "GPU arm: L2 flushed before every timed step (256 MiB write); reference arm: host cores, no GPU L2"
REF_BUDGET_S = 150.0
WORKLOAD = "pbf_dam_break_131k"

# Workloads (seeded synthetic scenes, realtimeparticles_gb300/scenes.py).  The default is the
# configuration the headline metric is quoted on; the others are measured the same way.
WORKLOADS = {
    "pbf_dam_break_131k": dict(kind="fluids", lattice=(32, 64, 64), iters=3,
                               metric="PBF particle-steps/s @131k (plain, 3 Jacobi iterations)"),
    "pbf_dam_break_16k": dict(kind="fluids", lattice=(16, 32, 32), iters=3,
                              metric="PBF particle-steps/s @16k (plain, 3 Jacobi iterations)"),
    # 16.7M particles (256^3 lattice, box 6.4 = 256 cells of h per axis): the grid/sort path
    # at a size where its HBM traffic, not launch latency, sets the time.
    "pbf_dam_break_1m": dict(kind="fluids", lattice=(64, 128, 128), box=1.6, iters=3, max_steps=50,
                             metric="PBF particle-steps/s @1M (plain, 3 Jacobi iterations)"),
    "pbf_dam_break_4m": dict(kind="fluids", lattice=(128, 256, 128), box=3.2, iters=3, max_steps=20,
                             metric="PBF particle-steps/s @4.2M (plain, 3 Jacobi iterations)"),
    "pbf_dam_break_16m": dict(kind="fluids", lattice=(256, 256, 256), box=6.4, iters=3, max_steps=10,
                              metric="PBF particle-steps/s @16.7M (plain, 3 Jacobi iterations)"),
    "boids_131k": dict(kind="boids", n=131072, metric="boids particle-steps/s @131k"),
    # 48 independent dam breaks (4,096-65,536 particles, box aspect 0.5-2, seed 0) in one batch.
    "pbf_batched_48": dict(kind="batch", count=48, seed=0, iters=3, max_steps=300,
                           metric="batched PBF particle-steps/s (48 dam-break scenes, 3 Jacobi iterations)"),
    "clouds_131k": dict(kind="clouds", n=131072, iters=1, metric="clouds particle-steps/s @131k"),
}


def make_model(w, rank=0):
    """The model of workload w with its seeded inputs uploaded.  A batch shards by scene:
    rank r steps its own seeded scene set (seed + r)."""
    from realtimeparticles_gb300 import model
    if w["kind"] == "batch":
        sc = scenes.batched_dam_breaks(count=w["count"], seed=w["seed"] + rank)
        m = model.FluidsBatch(sc["scenes"], sc["h"])
        m.setFluidParams(sc["fluid_params"])
        m.setJacobiIterations(w["iters"])
        m.upload(abi.BUF_POS, sc["pos"])
        m.upload(abi.BUF_VEL, sc["vel"])
        m._scene_set = sc
        return m, sc["pos"].shape[0]
    if w["kind"] == "fluids":
        sc = scenes.dam_break(lattice=w["lattice"], box=w.get("box", 1.0))
        m = model.Fluids(sc["model_params"])
        m.setFluidParams(sc["fluid_params"])
        m.setJacobiIterations(w["iters"])
    elif w["kind"] == "boids":
        sc = scenes.boids_cloud(n=w["n"])
        m = model.Boids(sc["model_params"])
        m.setBoidsParams(sc["boids_params"])
        m.setTimeStep(0.01)
        m.setBoundary(abi.CYCLIC_WALL)
    else:
        return clouds_model(w["n"], 0, w["iters"]), w["n"]
    m.upload(abi.BUF_POS, sc["pos"])
    m.upload(abi.BUF_VEL, sc["vel"])
    return m, sc["pos"].shape[0]


def fluids_model(lattice, seed, iters):
    """A dam break (scenes.dam_break) of `lattice` with its inputs uploaded."""
    from realtimeparticles_gb300 import model
    sc = scenes.dam_break(lattice=lattice, seed=seed)
    m = model.Fluids(sc["model_params"])
    m.setFluidParams(sc["fluid_params"])
    m.setJacobiIterations(iters)
    m.upload(abi.BUF_POS, sc["pos"])
    m.upload(abi.BUF_VEL, sc["vel"])
    return m


def clouds_model(n, seed, iters):
    """A cumulus column (scenes.clouds_cumulus) of n particles with its inputs uploaded and
    its thermodynamic state initialised."""
    from realtimeparticles_gb300 import model
    sc = scenes.clouds_cumulus(n=n, seed=seed)
    m = model.Clouds(sc["model_params"])
    m.setFluidParams(sc["fluid_params"])
    m.setCloudParams(sc["cloud_params"])
    m.setEnvironment(sc["env"], sc["ground"])
    m.setJacobiIterations(iters)
    m.upload(abi.BUF_POS, sc["pos"])
    m.upload(abi.BUF_VEL, sc["vel"])
    m.initThermo()
    return m

# Algorithmic bytes per particle of each kernel of the PBF substep (minimal dataflow of
# the fused kernels: every array a kernel must read or write once).
# DRAM bytes (read + write) per launch of a workload's dominant kernel from one ncu capture
# (cold cache, serialised), with the summary that records the capture.
KERNEL_TRAFFIC = {
    ("pbf_dam_break_131k", "fld_lambda"): (6600021, "profiles/k_fluid_lambda_131k_traffic.md"),
    ("pbf_dam_break_16k", "fld_lambda"): (523520, "profiles/k_fluid_lambda_group_16k_traffic.md"),
}

# The dominant sweep's L1 data-pipe (LSU wavefront) fraction of peak from one ncu capture: the
# ceiling the sweep's candidate-test rate is measured against (it is bound by L1 and issue, not HBM).
SWEEP_L1 = {
    ("pbf_dam_break_131k", "fld_lambda"): (0.5654, "profiles/k_fluid_lambda_131k_l1.md"),
}

KERNEL_BYTES = {
    "fld_predict": 16 + 16 + 16 + 4,          # pos, vel in; predPos, key out
    "sort_pass": 4 + 4 + 4,                   # key in; key, index out
    "sort_pass_gather": 4 + 4 + 4 + 3 * 32 + 8,  # key, index in; key out; 3 float4 gathered; id
    "cellTable": 4 + 8,                       # sorted key in; table entries out (upper bound)
    "fld_lambda": 16 + 4 + 4,                 # predPos in; lambda, density out
    "fld_deltap": 16 + 4 + 16,                # predPos, lambda in; predPos out
    "fld_deltap_vel": 16 + 4 + 16 + 16 + 16,  # + pos in, vel out
    "fld_vorticity": 16 + 16 + 16,            # predPos, vel in; vorticity out
    "fld_confine": 16 + 16 + 16 + 16,         # predPos, vorticity, vel in; vel out
    "fld_xsph_final": 16 + 16 + 16 + 16 + 8,  # predPos, vel in; pos, vel out; ids
    "bd_keys": 16 + 4,                         # pos in; key out
    "bd_rules_update": 16 + 16 + 16 + 16 + 16 + 8,  # pos, vel in; pos, vel, acc out; ids
    "cld_thermo_predict": 16 + 16 + 4 * 4 + 4 * 4 + 16 + 16 + 4,
    "cld_temp_lambda": 16 + 4 + 4,
    "cld_temp_correct": 16 + 4 + 4 + 4,
    "cld_lambda": 16 + 4 + 4,
    "cld_deltap": 16 + 4 + 16 + 16 + 16,
    "cld_deltap_vel": 16 + 4 + 16 + 16 + 16 + 16,
    "cld_vorticity": 16 + 16 + 16,
    "cld_confine": 16 + 16 + 16 + 16,
    "cld_xsph_final": 16 + 16 + 16 + 16 + 4 * 4 * 2 + 8,
}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 20 ms while running.  start() returns
    once the first sample has arrived (nvidia-smi takes a while to start), and only the samples
    after that point count, so they cover the timed region rather than the idle start-up."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.idx = device_index
        self.proc = None
        self.lines = []
        self.t = None
        self.mark = 0

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        t0 = time.time()
        while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
            time.sleep(0.005)
        self.mark = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines[self.mark:] or self.lines[-1:]
        for line in lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(value, ws):
    """Max of a float over all ranks (identity for one rank)."""
    if ws <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, ws):
    """Sum of a count over all ranks (identity for one rank)."""
    if ws <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_baseline(steps_sample=None, budget_s=20.0, iters=3):
    """The CPU implementation (cpu_impl) on the host cores, on a bounded sample of the
    workload."""
    import oracle
    oracle.set_threads(0)
    cores = oracle.get_threads()
    step, kind = cpu_impl()
    sc = scenes.dam_break(lattice=(32, 64, 64))
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    st = oracle.new_state(sc["pos"].shape[0], c)
    st["pos"][:] = sc["pos"]
    st["vel"][:] = sc["vel"]
    step(c, sc["fluid_params"], iters, st)  # warm-up
    n = sc["pos"].shape[0]
    t0 = time.perf_counter()
    k = 0
    while True:
        step(c, sc["fluid_params"], iters, st)
        k += 1
        el = time.perf_counter() - t0
        if (steps_sample and k >= steps_sample) or (not steps_sample and el >= budget_s):
            break
    return {"value": n * k / el, "unit": "particle-steps/s", "cores": cores, "kind": kind,
            "sample": "%d steps of the %d-particle dam break (I=%d), %.1f s" % (k, n, iters, el)}


def cpu_impl():
    """The CPU implementation of the step: the reference's own kernels compiled for the CPU
    (oracle/_ref, kind "reference") when built, else the oracle's restatement (kind "port")."""
    import oracle
    if oracle.ref_available():
        return oracle.ref_fluids_step, "reference"
    return oracle.fluids_step, "port"


def run_reference(args):
    """The CPU implementation of the step on all host cores: W warm-up updates, then K timed
    updates of the same 131k workload (stopping early after REF_BUDGET_S, reported in the
    sample)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import oracle
    oracle.set_threads(0)
    cores = oracle.get_threads()
    step, kind = cpu_impl()
    iters = 3
    sc = scenes.dam_break(lattice=(32, 64, 64))
    n = sc["pos"].shape[0]
    c = oracle.derive_constants(abi.FLUIDS, sc["model_params"])
    st = oracle.new_state(n, c)
    st["pos"][:] = sc["pos"]
    st["vel"][:] = sc["vel"]
    for _ in range(args.warmup):
        step(c, sc["fluid_params"], iters, st)
    t0 = time.perf_counter()
    k = 0
    while k < args.steps:
        step(c, sc["fluid_params"], iters, st)
        k += 1
        if time.perf_counter() - t0 > REF_BUDGET_S:
            break
    el = time.perf_counter() - t0
    value = n * k / el
    what = "the reference's kernels (physics/ocl/kernels) compiled for the CPU" if kind == "reference" else \
        "the oracle's restatement of the reference's kernels"
    sample = "%d of %d requested updates of the %d-particle dam break (I=%d) in %.1f s; %s, OpenMP over %d threads" % (
        k, args.steps, n, iters, el, what, cores)
    line = {"metric": "PBF particle-steps/s @131k (plain, 3 Jacobi iterations)", "value": value,
            "unit": "particle-steps/s", "n_gpus": args.gpus, "steps": k, "warmup": args.warmup,
            "ms_per_step": 1000.0 * el / k, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattice)",
            "config": {"workload": WORKLOAD, "particles": n, "jacobi_iterations": iters, "substep_dt": 1 / 240.0,
                       "l2": L2_NOTE,
                       "parallelism": "single"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": kind,
                             "sample": sample},
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


PLAIN_ITERS = (1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48)
WARM_EXTRA = (0, 1, 2, 3, 5, 7, 8, 9, 11)


def _timed_config(open_model, iters, net, extra, tol, steps, warmup):
    """(ms per step, mean solver-output density error, reruns) of one configuration;
    open_model(iters) makes the seed-0 model."""
    with open_model(iters) as m:
        m.enableSolverStats(True)
        if net is not None:
            m.setWarmStart(net, extra_iterations=extra, guard_tolerance=tol)
        m.update(warmup)
        m.resetSolverStats()
        ms = m.timeSteps(steps, flush_bytes=L2_FLUSH_BYTES) / steps
        st = m.solverStats()
    return ms, st["mean"], st["reruns"]


def _pareto(curve):
    """The plain configurations no other one beats on both error and throughput (more Jacobi
    iterations stop helping past a point and then make the error grow again), error decreasing."""
    front = [(e, v) for e, v in curve if not any(e2 <= e and v2 >= v and (e2, v2) != (e, v) for e2, v2 in curve)]
    return sorted(front, key=lambda p: -p[0])


def _plain_at(curve, err):
    """Throughput of the plain solver at mean error `err`, log-log interpolated on the Pareto
    front of the measured (error, particle-steps/s) points; None outside it."""
    pts = _pareto(curve)
    for (e0, v0), (e1, v1) in zip(pts, pts[1:]):
        if e1 <= err <= e0 and e0 > 0 and e1 > 0:
            t = (np.log(err) - np.log(e0)) / (np.log(e1) - np.log(e0)) if e0 != e1 else 0.0
            return float(np.exp(np.log(v0) + t * (np.log(v1) - np.log(v0))))
    return None


def _at_threshold(plain, learned, tol):
    """The fastest plain and the fastest warm-started configuration whose mean error is <= tol,
    and their throughput ratio (None when either has none)."""
    p = [x for x in plain if x["mean_density_error"] <= tol]
    q = [x for x in learned if x["mean_density_error"] <= tol]
    if not p or not q:
        return {"error_bound": tol, "plain": None, "learned": None, "speedup": None}
    bp = max(p, key=lambda x: x["particle_steps_per_s"])
    bq = max(q, key=lambda x: x["particle_steps_per_s"])
    return {"error_bound": tol,
            "plain": {"iterations": bp["iterations"], "particle_steps_per_s": bp["particle_steps_per_s"],
                      "mean_density_error": bp["mean_density_error"]},
            "learned": {"extra_iterations": bq["extra_iterations"], "particle_steps_per_s": bq["particle_steps_per_s"],
                        "mean_density_error": bq["mean_density_error"]},
            "speedup": bq["particle_steps_per_s"] / bp["particle_steps_per_s"]}


WS_LONG_PLAIN_ITERS = (3, 8, 16, 24)
WS_LONG_EXTRA = (2, 5, 9)
WS_LONG_BLOCKS = 4
WS_LONG_BLOCK_STEPS = 500
WS_TRAIN_SEEDS = (1, 2, 3, 4)
WS_TRAIN_STEPS = 300
WS_EVAL_WARMUP = 100
WS_EVAL_STEPS = 100


def warm_start_study(w, steps, warmup):
    """The learned warm start against the plain solver at equal error.  The network is trained
    through the solve on the rollouts of other seeded scenes (WS_TRAIN_STEPS steps each, warm
    start + 1 extra iteration, one AdamW step per step); every configuration then runs the
    seed-0 scene for WS_EVAL_STEPS device-timed steps after WS_EVAL_WARMUP warm-up steps (the
    dam has collapsed by then: errors of the first steps say little), L2 flushed before every
    step.  The plain solver's throughput at a configuration's error is log-log interpolated on
    the Pareto front of the measured plain points; `at_error_le_1pct` compares the fastest
    configurations of each whose mean error is at most 1 % of rho0."""
    from realtimeparticles_gb300 import warmstart
    lattice = w["lattice"]

    def open_model(iters):
        return fluids_model(lattice, 0, iters)

    n = int(np.prod(lattice))
    t0 = time.perf_counter()
    net, losses = None, []
    for seed in WS_TRAIN_SEEDS:
        with fluids_model(lattice, seed, 2) as m:
            net, hist = warmstart.train_rollout(m, WS_TRAIN_STEPS, extra_iterations=1, net=net, seed=0)
            losses += hist
    t1 = time.perf_counter()
    out = {"training": {"method": "through the solve on the model's own rollout (one AdamW step per step)",
                        "scenes": len(WS_TRAIN_SEEDS), "steps": len(losses), "particles": n,
                        "extra_iterations": 1, "train_seconds": round(t1 - t0, 2)},
           "eval": {"warmup_steps": WS_EVAL_WARMUP, "timed_steps": WS_EVAL_STEPS}}
    plain, curve = [], []
    for it in PLAIN_ITERS:
        ms, err, _ = _timed_config(open_model, it, None, 0, 0.0, WS_EVAL_STEPS, WS_EVAL_WARMUP)
        v = n / (ms / 1000.0)
        plain.append({"iterations": it, "particle_steps_per_s": v, "ms_per_step": ms, "mean_density_error": err})
        curve.append((err, v))
    learned = []
    for e in WARM_EXTRA:
        ms, err, rr = _timed_config(open_model, 3, net, e, 0.0, WS_EVAL_STEPS, WS_EVAL_WARMUP)
        v = n / (ms / 1000.0)
        ref = _plain_at(curve, err)
        learned.append({"extra_iterations": e, "particle_steps_per_s": v, "ms_per_step": ms,
                        "mean_density_error": err, "plain_at_equal_error": ref,
                        "speedup_at_equal_error": (v / ref) if ref else None})
    # The guard on the warm start + 2 extra iterations (three in all): a step whose
    # solver-output error exceeds 1.25 x the plain 3-iteration mean reruns with the plain 3.
    e3 = next(p["mean_density_error"] for p in plain if p["iterations"] == 3)
    tol = 1.25 * e3
    ms, err, rr = _timed_config(open_model, 3, net, 2, tol, WS_EVAL_STEPS, WS_EVAL_WARMUP)
    guarded = {"extra_iterations": 2, "guard_tolerance": tol, "plain_iterations": 3,
               "particle_steps_per_s": n / (ms / 1000.0), "mean_density_error": err, "reruns": rr,
               "steps": WS_EVAL_STEPS}

    def best(cond):
        v = [x["speedup_at_equal_error"] for x in learned if x["speedup_at_equal_error"] and cond(x)]
        return max(v) if v else None

    out.update(plain=plain, learned=learned, guarded=guarded,
               best_speedup_at_equal_error=best(lambda x: True),
               best_speedup_at_or_below_plain3_error=best(lambda x: x["mean_density_error"] <= e3),
               at_error_le_1pct=_at_threshold(plain, learned, 0.01),
               at_error_le_plain3=_at_threshold(plain, learned, e3))
    # The same comparison over a long run: WS_LONG_BLOCKS x WS_LONG_BLOCK_STEPS steps from the
    # start (the collapse included), the error averaged over all of them.
    lplain, lcurve = [], []
    for it in WS_LONG_PLAIN_ITERS:
        ms, err, worst, blocks, _ = _timed_blocks(open_model, it, None, 0, WS_LONG_BLOCKS, WS_LONG_BLOCK_STEPS)
        v = n / (ms / 1000.0)
        lplain.append({"iterations": it, "particle_steps_per_s": v, "ms_per_step": ms, "mean_density_error": err,
                       "block_errors": blocks})
        lcurve.append((err, v))
    llearned = []
    for e in WS_LONG_EXTRA:
        ms, err, worst, blocks, _ = _timed_blocks(open_model, 3, net, e, WS_LONG_BLOCKS, WS_LONG_BLOCK_STEPS)
        v = n / (ms / 1000.0)
        ref = _plain_at(lcurve, err)
        llearned.append({"extra_iterations": e, "particle_steps_per_s": v, "ms_per_step": ms,
                         "mean_density_error": err, "block_errors": blocks, "plain_at_equal_error": ref,
                         "speedup_at_equal_error": (v / ref) if ref else None})
    out["long_run"] = {"steps": WS_LONG_BLOCKS * WS_LONG_BLOCK_STEPS, "blocks": WS_LONG_BLOCKS,
                       "plain": lplain, "learned": llearned,
                       "at_error_le_1pct": _at_threshold(lplain, llearned, 0.01)}
    return out


CLOUD_PLAIN_ITERS = (1, 2, 3, 4, 6, 8)
CLOUD_WARM_EXTRA = (0, 1, 2, 3)
CLOUD_WS_TRAIN_SEEDS = (1, 2)
CLOUD_WS_TRAIN_STEPS = 1500
CLOUD_EVAL_BLOCKS = 4
CLOUD_EVAL_BLOCK_STEPS = 1000


def _timed_blocks(open_model, iters, net, extra, blocks, block_steps, tol=0.0):
    """(ms per step, mean solver-output error, largest block mean, block means, guard reruns)
    of one configuration run for blocks x block_steps device-timed steps from the seed-0
    start, L2 flushed before every step, solver statistics reset per block."""
    with open_model(iters) as m:
        m.enableSolverStats(True)
        if net is not None:
            m.setWarmStart(net, extra_iterations=extra, guard_tolerance=tol)
        total_ms, errs, reruns = 0.0, [], 0
        for _ in range(blocks):
            m.resetSolverStats()
            total_ms += m.timeSteps(block_steps, flush_bytes=L2_FLUSH_BYTES)
            st = m.solverStats()
            errs.append(st["mean"])
            reruns += st["reruns"]
    return total_ms / (blocks * block_steps), float(np.mean(errs)), float(max(errs)), errs, reruns


def clouds_warm_start_study(w):
    """The learned warm start of the clouds solve against the plain clouds solver at equal
    error over the clouds configuration's own length (4,000 steps).  Two networks are trained
    through the clouds solve on the rollouts of other seeded columns (CLOUD_WS_TRAIN_SEEDS,
    CLOUD_WS_TRAIN_STEPS steps each): one under no extra iteration (used for + 0), one under one
    extra iteration (used for + 1 and more).  Rollouts of 300 steps trained networks that were
    good for a few hundred steps and then drove the column unstable; 1,500 steps reach the
    states of the developed convection.  Every configuration then runs CLOUD_EVAL_BLOCKS x
    CLOUD_EVAL_BLOCK_STEPS device-timed steps of the seed-0 column from its start, L2 flushed
    before every step; the error is the mean over all steps and the largest block mean is kept
    as a stability check."""
    from realtimeparticles_gb300 import warmstart
    n = w["n"]

    def open_model(iters):
        return clouds_model(n, 0, iters)

    t0 = time.perf_counter()
    nets, losses = {}, {}
    for e in (0, 1):
        net, hist = None, []
        for seed in CLOUD_WS_TRAIN_SEEDS:
            with clouds_model(n, seed, 1) as m:
                net, h = warmstart.train_rollout(m, CLOUD_WS_TRAIN_STEPS, extra_iterations=e, net=net, seed=0)
                hist += h
        nets[e], losses[e] = net, hist
    t1 = time.perf_counter()
    out = {"training": {"method": "through the solve on the model's own rollout (one AdamW step per step)",
                        "scenes": len(CLOUD_WS_TRAIN_SEEDS), "steps_per_scene": CLOUD_WS_TRAIN_STEPS,
                        "particles": n, "networks": {"+0": "trained under + 0", "+1 and more": "trained under + 1"},
                        "train_seconds": round(t1 - t0, 2)},
           "eval": {"blocks": CLOUD_EVAL_BLOCKS, "steps_per_block": CLOUD_EVAL_BLOCK_STEPS}}
    plain, curve = [], []
    for it in CLOUD_PLAIN_ITERS:
        ms, err, worst, blocks, _ = _timed_blocks(open_model, it, None, 0, CLOUD_EVAL_BLOCKS, CLOUD_EVAL_BLOCK_STEPS)
        v = n / (ms / 1000.0)
        plain.append({"iterations": it, "particle_steps_per_s": v, "ms_per_step": ms, "mean_density_error": err,
                      "largest_block_error": worst, "block_errors": blocks})
        curve.append((err, v))
    learned = []
    for e in CLOUD_WARM_EXTRA:
        net = nets[0] if e == 0 else nets[1]
        ms, err, worst, blocks, _ = _timed_blocks(open_model, 1, net, e, CLOUD_EVAL_BLOCKS, CLOUD_EVAL_BLOCK_STEPS)
        v = n / (ms / 1000.0)
        ref = _plain_at(curve, err)
        learned.append({"extra_iterations": e, "particle_steps_per_s": v, "ms_per_step": ms,
                        "mean_density_error": err, "largest_block_error": worst, "block_errors": blocks,
                        "plain_at_equal_error": ref, "speedup_at_equal_error": (v / ref) if ref else None})
    e2 = plain[1]["mean_density_error"]
    # The guarded warm start: one solve per step (+ 0), and a step whose error exceeds 1.25 x the
    # plain 2-iteration mean reruns with the plain 2 iterations.
    tol = 1.25 * e2
    ms, err, worst, blocks, rr = _timed_blocks(open_model, 2, nets[0], 0, CLOUD_EVAL_BLOCKS, CLOUD_EVAL_BLOCK_STEPS,
                                               tol)
    guarded = {"extra_iterations": 0, "guard_tolerance": tol, "plain_iterations": 2,
               "particle_steps_per_s": n / (ms / 1000.0), "ms_per_step": ms, "mean_density_error": err,
               "largest_block_error": worst, "block_errors": blocks, "reruns": rr,
               "steps": CLOUD_EVAL_BLOCKS * CLOUD_EVAL_BLOCK_STEPS}
    v = [x["speedup_at_equal_error"] for x in learned if x["speedup_at_equal_error"]]
    out.update(plain=plain, learned=learned, guarded=guarded, best_speedup_at_equal_error=max(v) if v else None,
               at_error_le_plain2=_at_threshold(plain, learned, e2),
               at_error_le_1pct=_at_threshold(plain, learned, 0.01))
    return out


GRID_SORT_KERNELS = ("fld_predict", "sort_clear", "sort_scan", "sort_pass", "sort_pass_gather", "cellTableClear",
                     "cellTable")


def mean_candidates(c, table, keys):
    """Mean number of particles in the 27 cells (wrapped modulo the grid, as the fluids sweeps
    visit them, fluids.cl:101-123) around each particle's cell: the candidates one full sweep
    tests per particle.  table: the reference-format cell table; keys: the sorted cell keys."""
    res = tuple(int(r) for r in c.gridRes)
    cnt = np.where(table[:, 1] >= table[:, 0], table[:, 1].astype(np.int64) - table[:, 0] + 1, 0)
    cnt = cnt[:int(np.prod(res))].reshape(res)
    cand = np.zeros_like(cnt)
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                cand += np.roll(cnt, (-dx, -dy, -dz), axis=(0, 1, 2))
    k = keys[keys < cand.size]
    return float(cand.reshape(-1)[k].mean()) if k.size else 0.0


def grid_sort_summary(kt, steps, n, c, nonempty, peak):
    """HBM roofline of the grid/sort path of the PBF step (predict + cell keys, stable radix
    sort with the payload gather, cell table): algorithmic bytes of its kernels per step
    over their summed device time."""
    passes = max(1, -(-int(c.keyBits) // 9))
    per_step = {
        "fld_predict": 52 * n,                                   # pos, vel in; predPos, key out
        "sort_clear": 0, "sort_scan": 0,                         # sort bookkeeping, not algorithmic
        "sort_pass": (12 + 16 * max(0, passes - 2)) * n if passes > 1 else 0,  # keys (+ index) in and out
        "sort_pass_gather": 112 * n,                             # key, index in; key out; 3 float4 + id moved
        "cellTableClear": 8 * int(c.numCells),                   # the table is written whole
        "cellTable": 4 * n + 8 * nonempty,                       # sorted keys in; begin/end of each cell
    }
    ms = sum(kt[k][1] for k in GRID_SORT_KERNELS if k in kt) / max(1, steps)
    b = sum(per_step.values())
    gbs = b / (ms / 1000.0) / 1e9 if ms > 0 else None
    return {"kernels": [k for k in GRID_SORT_KERNELS if k in kt], "algorithmic_bytes_per_step": b,
            "ms_per_step": ms, "achieved_gbs": gbs, "peak_gbs": peak, "frac": (gbs / peak) if gbs else None,
            "sort_passes": passes, "cells": int(c.numCells), "nonempty_cells": nonempty}


def batch_study(m, w, steps, warmup):
    """The batch against the same scenes on separate handles stepped one after another, and
    plain against warm-started solver error on the batch."""
    from realtimeparticles_gb300 import model, warmstart
    sc = m._scene_set
    lanes, factor, _ = m.tuning()
    n_total = sc["pos"].shape[0]
    ms_sum = 0.0
    for s, (n, box) in enumerate(sc["scenes"]):
        off = sc["offsets"][s]
        res = tuple(int(round(b / sc["h"])) for b in box)
        with model.Fluids(abi.model_params(n, n, box, res, 3)) as one:
            one.setFluidParams(sc["fluid_params"])
            one.setJacobiIterations(w["iters"])
            one.setTuning(lanes, 1.0)
            one.upload(abi.BUF_POS, sc["pos"][off:off + n])
            one.upload(abi.BUF_VEL, sc["vel"][off:off + n])
            one.update(warmup)
            ms_sum += one.timeSteps(steps, flush_bytes=L2_FLUSH_BYTES) / steps
    separate = n_total / (ms_sum / 1000.0)
    # Plain and warm-started solver error on the batch: the network trained through the solve
    # on the rollouts of two seeded 131k dam breaks (as the warm_start study trains it).
    net = None
    for seed in WS_TRAIN_SEEDS[:2]:
        with fluids_model((32, 64, 64), seed, 2) as mt:
            net, _ = warmstart.train_rollout(mt, WS_TRAIN_STEPS, extra_iterations=1, net=net, seed=0)
    errs = {}
    for name, extra in (("plain", None), ("learned_extra1", 1), ("learned_extra2", 2)):
        mb, _ = make_model(w)
        with mb:
            mb.setTuning(lanes, factor)
            mb.enableSolverStats(True)
            if extra is not None:
                mb.setWarmStart(net, extra_iterations=extra, guard_tolerance=0.0)
            mb.update(warmup)
            mb.resetSolverStats()
            ms = mb.timeSteps(steps, flush_bytes=L2_FLUSH_BYTES) / steps
            errs[name] = {"particle_steps_per_s": n_total / (ms / 1000.0), "ms_per_step": ms,
                          "mean_density_error": mb.solverStats()["mean"]}
    return {"scenes": len(sc["scenes"]), "particles": n_total,
            "scene_particles_min": min(n for n, _ in sc["scenes"]),
            "scene_particles_max": max(n for n, _ in sc["scenes"]),
            "separate_handles_particle_steps_per_s": separate,
            "separate_handles_ms_per_step": ms_sum, "solver": errs}


def run_ours(args):
    ws, rank, local = dist_env()
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from realtimeparticles_gb300._lib import lib
    if ws > 1:
        # The library uses the current device of the calling thread.
        import torch
        torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    if "max_steps" in w:
        args.steps = min(args.steps, w["max_steps"])
    m, n = make_model(w, rank)
    n_all = sum_over_ranks(n, ws)  # a batch's ranks hold different scene sets
    tune = None
    if w["kind"] in ("batch", "fluids") and not args.no_autotune:
        best, cands = m.autotune(steps=5)
        tune = {"best": {"lanes": best[0], "cell_factor": best[1], "tiled_sweeps": best[2]},
                "candidates_ms_per_step": {"%d/%.2f/%d" % k: v for k, v in sorted(cands.items())}}

    # Warm-up (graph capture happens here).
    m.update(max(3, args.warmup))
    m.synchronize()

    # Device-timed steps with an L2 flush before each.
    clocks = ClockSampler(local)
    clocks.start()
    barrier(ws)
    ms = m.timeSteps(args.steps, flush_bytes=L2_FLUSH_BYTES)
    barrier(ws)
    clk = clocks.stop()
    ms = max_over_ranks(ms, ws)
    value = n_all * args.steps / (ms / 1000.0)

    # Per-kernel times from captured events inside the same kind of graph replays.
    m.enableProfiling(True)
    m.resetKernelTimes()
    m.timeSteps(args.steps, flush_bytes=L2_FLUSH_BYTES)
    kt = m.kernelTimes()
    m.enableProfiling(False)
    launches_per_step = sum(v[0] for v in kt.values()) / max(1, args.steps)
    dom = max(kt.items(), key=lambda kv: kv[1][1])
    dom_name, (dom_launches, dom_ms) = dom
    dom_avg_ms = dom_ms / dom_launches
    peak, peak_kind = load_peaks()
    alg = KERNEL_BYTES.get(dom_name, 0) * n
    achieved = alg / (dom_avg_ms / 1000.0) / 1e9
    share = {k: round(v[1] / sum(x[1] for x in kt.values()), 4) for k, v in kt.items()}
    # Sum of the kernels' own durations per step (events around each kernel inside the same
    # graph replays): the step time minus this is the launch and drain gaps between kernels,
    # the most a single persistent launch over the step's stages could take back.
    kernels_ms = sum(v[1] for v in kt.values()) / max(1, args.steps)
    grid_sort = sweep = None
    if w["kind"] == "fluids":  # (a batch has one grid per scene)
        tab = m.download(abi.BUF_CELL_TABLE)
        nonempty = int(np.count_nonzero(tab[:, 1] >= tab[:, 0]))
        grid_sort = grid_sort_summary(kt, args.steps, n, m.constants(), nonempty, peak)
        if dom_name == "fld_lambda":
            # The dominant sweep is bound by dependent loads, not HBM: its work rates.
            cand = mean_candidates(m.constants(), tab, m.download(abi.BUF_CELL_ID))
            nbr = m.metrics().meanNeighbours
            sweep = {"kernel": dom_name, "candidates_per_particle": cand, "neighbours_per_particle": nbr,
                     "candidate_tests_per_s": n * cand / (dom_avg_ms / 1000.0),
                     "pair_evaluations_per_s": n * nbr / (dom_avg_ms / 1000.0)}
            l1 = SWEEP_L1.get((args.workload, dom_name))
            if l1:
                sweep.update(l1_wavefront_frac=l1[0], l1_source=l1[1],
                             candidate_tests_per_s_at_l1_ceiling=sweep["candidate_tests_per_s"] / l1[0])

    # End to end through the public API with pinned host buffers.
    try:
        import torch
        hpos = torch.empty((n, 4), dtype=torch.float32, pin_memory=True).numpy()
        hvel = torch.empty((n, 4), dtype=torch.float32, pin_memory=True).numpy()
        pinned = True
    except Exception:
        hpos = np.empty((n, 4), np.float32)
        hvel = np.empty((n, 4), np.float32)
        pinned = False
    hpos[:] = m.download(abi.BUF_POS)
    hvel[:] = m.download(abi.BUF_VEL)
    barrier(ws)
    t0 = time.perf_counter()
    hp, hv = hpos.ctypes.data_as(C.c_void_p), hvel.ctypes.data_as(C.c_void_p)
    for _ in range(args.steps):
        # rtp_update_host: upload pos + vel, one step, download pos + vel, one synchronisation.
        rc = lib().rtp_update_host(m.handle, hp, hv, n, 1, hp, hv)
        if rc != 0:
            raise RuntimeError("rtp_update_host failed: %d" % rc)
    t_e2e = time.perf_counter() - t0
    barrier(ws)
    t_e2e = max_over_ranks(t_e2e, ws)
    e2e = n_all * args.steps / t_e2e
    metrics = m.metrics() if w["kind"] != "boids" else None
    batch = batch_study(m, w, args.steps, max(3, args.warmup)) if w["kind"] == "batch" and rank == 0 else None
    m.close()

    out = None
    if rank == 0:
        cb = cpu_baseline(budget_s=args.cpu_seconds) if not args.no_cpu and args.workload == WORKLOAD else None
        out = {
            "metric": w["metric"],
            "value": value, "unit": "particle-steps/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded jittered lattice)",
            "config": {"workload": args.workload, "particles": n, "jacobi_iterations": w.get("iters"),
                       **({"substep_dt": 1 / 240.0} if w["kind"] in ("fluids", "batch") else {}),
                       "l2": L2_NOTE,
                       "parallelism": ("scenes by rank" if w["kind"] == "batch" else "replicas") if ws > 1
                       else "single"},
            "e2e": {"value": e2e, "unit": "particle-steps/s", "h2d_bytes_per_step": 2 * 16 * n,
                    "d2h_bytes_per_step": 2 * 16 * n, "pinned_host": pinned},
            "gpu_launches": int(round(launches_per_step * args.steps)),
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": KERNEL_TRAFFIC.get((args.workload, dom_name), (None, None))[0],
                         "traffic_source": KERNEL_TRAFFIC.get((args.workload, dom_name), (None, None))[1],
                         "algorithmic_bytes_per_launch": alg,
                         "mean_launch_ms": dom_avg_ms},
            "kernel_share": share,
            "kernels_ms_per_step": kernels_ms,
            "clocks": clk,
        }
        if grid_sort:
            out["grid_sort"] = grid_sort
        if sweep:
            out["sweep"] = sweep
        if tune:
            out["autotune"] = tune
        if batch:
            out["batch"] = batch
        if metrics is not None:
            out["state_check"] = {"mean_density_error": metrics.meanDensityError,
                                  "kinetic_energy": metrics.kineticEnergy,
                                  "pair_list_overflows": metrics.pairListOverflows}
        if cb:
            out["cpu_baseline"] = cb
        if w["kind"] == "fluids" and args.workload == WORKLOAD and not args.no_warm_start:
            out["warm_start"] = warm_start_study(w, args.steps, max(3, args.warmup))
        if w["kind"] == "clouds" and not args.no_warm_start:
            out["warm_start"] = clouds_warm_start_study(w)
        print(json.dumps(out))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-warm-start", action="store_true", help="skip the learned warm-start study")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default launch shape (for profiler runs, whose timings would mislead the autotuner)")
    ap.add_argument("--workload", default=WORKLOAD, choices=sorted(WORKLOADS))
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
