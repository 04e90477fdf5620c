"""Python mirror of the reference's Physics::Model interface over the C ABI.

physics/Model.hpp:81-216 (Model), physics/Model.cpp:10-24 (CreateModel) and
physics/ocl/OclModel.hpp:12-70 (JSON -> kernel inputs).  Method names follow the
reference (update, reset, setNbParticles, setDimension, setBoundary, pause,
updateInputJson, ...); buffers are exchanged as numpy arrays through rtp_upload /
rtp_download, or used in place through rtp_device_ptr.
"""
import copy
import ctypes as C

import numpy as np

from . import abi
from ._lib import RtpError, call, lib

# Default input JSON trees, [value, min, max] triplets (Fluids.cpp:52-74,
# Boids.cpp:41-73, Clouds.cpp:67-102).
_FLUIDS_JSON = {
    "Fluids": {
        "Rest Density": [450.0, 10.0, 1000.0],
        "Relax CFM": [600.0, 100.0, 1000.0],
        "Time Step": [0.010, 0.0001, 0.020],
        "Nb Jacobi Iterations": [2, 1, 6],
        "Artificial Pressure": {
            "Enable##Pressure": True,
            "Coefficient##Pressure": [0.001, 0.0, 0.001],
            "Radius": [0.006, 0.001, 0.015],
            "Exp": [4, 1, 6],
        },
        "Vorticity Confinement": {
            "Enable##Vorticity": True,
            "Coefficient##Vorticity": [0.0004, 0.0, 0.001],
            "xSPH Viscosity Coefficient": [0.0001, 0.0, 0.001],
        },
    }
}
_BOIDS_JSON = {
    "Boids": {
        "Velocity": [0.5, 0.01, 5.0],
        "Target": {"Enable##Target": False, "Show": True, "Radius": [2.0, 1.0, 20.0], "Attract": True},
        "Alignment": {"Enable##Alignment": True, "Scale##Alignment": [1.6, 0.0, 3.0]},
        "Cohesion": {"Enable##Cohesion": True, "Scale##Cohesion": [1.45, 0.0, 3.0]},
        "Separation": {"Enable##Separation": True, "Scale##Separation": [1.6, 0.0, 3.0]},
    }
}
_CLOUDS_JSON = {
    "Fluids": copy.deepcopy(_FLUIDS_JSON["Fluids"]),
    "Clouds": {
        "Enable Temperature Smoothing": True,
        "Ground Heat Coefficient": [10.0, 0.0, 1000.0],
        "Buoyancy Heat Coefficient": [0.10, 0.0, 5.0],
        "Gravity Coefficient": [0.0005, 0.0, 0.1],
        "Adiabatic Lapse Rate": [5.0, 0.0, 20.0],
        "Phase Transition Rate": [0.3485, 0.0, 20.0],
        "Latent Heat Coefficient": [0.07, 0.0, 0.100],
        "Wind Coefficient": [1.0, 0.0, 1.0],
    },
}
_CLOUDS_JSON["Fluids"]["Nb Jacobi Iterations"] = [2, 1, 6]

_F4 = {abi.BUF_POS, abi.BUF_VEL, abi.BUF_PRED_POS, abi.BUF_VORTICITY, abi.BUF_ACC, abi.BUF_COLOR}
_U32 = {abi.BUF_ID, abi.BUF_CELL_ID, abi.BUF_CAMERA_DIST, abi.BUF_DRAW_ORDER}


def _merge_patch(target, patch):
    """RFC 7386 merge patch (nlohmann::json::merge_patch, used by Model::updateInputJson)."""
    if not isinstance(patch, dict):
        return copy.deepcopy(patch)
    if not isinstance(target, dict):
        target = {}
    for k, v in patch.items():
        if v is None:
            target.pop(k, None)
        else:
            target[k] = _merge_patch(target.get(k), v)
    return target


class Model:
    """Physics::Model (physics/Model.hpp:81-216) backed by one rtp handle."""

    TYPE = None
    _DEFAULT_JSON = {}

    def __init__(self, params):
        self._h = C.c_void_p()
        call("rtp_create", int(self.TYPE), C.byref(params), C.byref(self._h))
        self._params = params
        self._input_json = copy.deepcopy(self._DEFAULT_JSON)
        self._boundary = abi.BOUNCING_WALL
        self._pause = False
        self._dimension = int(params.dimension)
        self._case = int(params.pCase)

    # lifecycle -------------------------------------------------------------------
    def close(self):
        if self._h:
            call("rtp_destroy", self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def update(self, nsteps=1):
        """Model::update(), called nsteps times (graph replays on the handle's stream)."""
        call("rtp_update", self._h, int(nsteps))

    def updateHost(self, pos, vel, nsteps=1):
        """rtp_update_host: uploads pos / vel ((n, 4) float32, C-contiguous; n = the particle
        count), runs nsteps updates and writes the result back into the same arrays."""
        for a in (pos, vel):
            if a.dtype != np.float32 or not a.flags["C_CONTIGUOUS"] or a.shape != (self.nbParticles(), 4):
                raise ValueError("updateHost: (n, 4) C-contiguous float32 arrays of the particle count")
        pp, vp = pos.ctypes.data_as(C.c_void_p), vel.ctypes.data_as(C.c_void_p)
        call("rtp_update_host", self._h, pp, vp, pos.shape[0], int(nsteps), pp, vp)

    def reset(self):
        """Model::reset(): default parameters and the case's initial particles."""
        self._input_json = copy.deepcopy(self._DEFAULT_JSON)
        call("rtp_reset", self._h)

    def synchronize(self):
        call("rtp_synchronize", self._h)

    # Model setters (physics/Model.hpp:104-128) ---------------------------------------
    def maxNbParticles(self):
        return int(self._params.maxNbParticles)

    def setNbParticles(self, n):
        call("rtp_set_nb_particles", self._h, int(n))

    def nbParticles(self):
        v = C.c_uint64()
        call("rtp_get_nb_particles", self._h, C.byref(v))
        return int(v.value)

    def setDimension(self, dim):
        call("rtp_set_dimension", self._h, int(dim))
        self._dimension = int(dim)

    def dimension(self):
        return self._dimension

    def setBoundary(self, boundary):
        call("rtp_set_boundary", self._h, int(boundary))
        self._boundary = int(boundary)

    def boundary(self):
        return self._boundary

    def pause(self, p):
        call("rtp_pause", self._h, 1 if p else 0)
        self._pause = bool(p)

    def onPause(self):
        return self._pause

    def setCase(self, case):
        call("rtp_set_case", self._h, int(case))
        self._case = int(case)

    def getCase(self):
        return self._case

    def isInit(self):
        return bool(self._h)

    # target (Model.hpp:130-132): the boids' attractor; other models report none --------
    def _target(self):
        pos = (C.c_float * 3)()
        act, vis = C.c_int(), C.c_int()
        call("rtp_get_target", self._h, pos, C.byref(act), C.byref(vis))
        return (float(pos[0]), float(pos[1]), float(pos[2])), bool(act.value), bool(vis.value)

    def targetPos(self):
        return self._target()[0]

    def isTargetActivated(self):
        return self._target()[1]

    def isTargetVisible(self):
        return self._target()[2]

    # profiling (OclModel.hpp:28-38) -------------------------------------------------
    def isProfilingEnabled(self):
        v = C.c_int()
        call("rtp_is_profiling_enabled", self._h, C.byref(v))
        return bool(v.value)

    def enableProfiling(self, enable):
        call("rtp_enable_profiling", self._h, 1 if enable else 0)

    def kernelTimes(self):
        """{kernel name: (launches, total ms)} accumulated while profiling was enabled."""
        n = C.c_uint32()
        call("rtp_get_kernel_times", self._h, None, 0, C.byref(n))
        arr = (abi.KernelTime * max(1, n.value))()
        call("rtp_get_kernel_times", self._h, arr, n.value, C.byref(n))
        return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].total_ms)) for i in range(n.value)}

    def resetKernelTimes(self):
        call("rtp_reset_kernel_times", self._h)

    def timeSteps(self, nsteps, flush_bytes=0):
        """Device time (ms) of nsteps updates, each bracketed by CUDA events; with
        flush_bytes > 0 a buffer that large is rewritten before every step."""
        t = C.c_double()
        call("rtp_time_steps", self._h, int(nsteps), int(flush_bytes), C.byref(t))
        return float(t.value)

    # JSON inputs (Model.hpp:154-174, OclModel.hpp:48-57) ---------------------------
    def getInputJson(self):
        return copy.deepcopy(self._input_json)

    def resetInputJson(self, js):
        self._input_json = copy.deepcopy(js)

    def updateInputJson(self, js):
        new = _merge_patch(copy.deepcopy(self._input_json), js)
        if new == self._input_json:
            return
        self._input_json = new
        self.updateModelWithInputJson(self._input_json)

    def updateModelWithInputJson(self, js):
        try:
            self.transferJsonInputsToModel(js)
        except (KeyError, TypeError, IndexError) as e:
            # Fluids.cpp:245-250: wrong JSON path -> std::runtime_error("Wrong Json parsing")
            raise RuntimeError("Wrong Json parsing") from e

    def transferJsonInputsToModel(self, js):
        raise NotImplementedError

    # buffers ------------------------------------------------------------------------
    def upload(self, buffer, array):
        a = np.ascontiguousarray(array)
        count = a.shape[0]
        call("rtp_upload", self._h, int(buffer), a.ctypes.data_as(C.c_void_p), int(count))

    def download(self, buffer, count=None):
        if count is None:
            if buffer in (abi.BUF_CELL_TABLE, abi.BUF_GRID_DETECTOR):
                count = self.constants().numCells
            elif buffer in (abi.BUF_CAMERA_DIST, abi.BUF_DRAW_ORDER):
                count = self.maxNbParticles()
            else:
                count = self.nbParticles()
        if buffer == abi.BUF_GRID_DETECTOR:
            out = np.empty((count, 8), np.float32)
        elif buffer in _F4:
            out = np.empty((count, 4), np.float32)
        elif buffer == abi.BUF_CELL_TABLE:
            out = np.empty((count, 2), np.uint32)
        elif buffer in _U32:
            out = np.empty(count, np.uint32)
        else:
            out = np.empty(count, np.float32)
        call("rtp_download", self._h, int(buffer), out.ctypes.data_as(C.c_void_p), int(count))
        return out

    def devicePtr(self, buffer):
        p = C.c_void_p()
        call("rtp_device_ptr", self._h, int(buffer), C.byref(p))
        return p.value

    def stream(self):
        p = C.c_void_p()
        call("rtp_stream", self._h, C.byref(p))
        return p.value

    def constants(self):
        c = abi.GridConstants()
        call("rtp_get_constants", int(self.TYPE), C.byref(self._params), C.byref(c))
        return c

    def metrics(self):
        m = abi.Metrics()
        call("rtp_get_metrics", self._h, C.byref(m))
        return m

    # headless side outputs (render-only in the reference) --------------------------------
    def fillFluidColor(self):
        call("rtp_fill_fluid_color", self._h)

    def fillColorFloat(self, buffer, min_val, max_val):
        call("rtp_fill_color_float", self._h, int(buffer), float(min_val), float(max_val))

    def fillCameraOrder(self, camera_pos):
        cam = (C.c_float * 3)(*[float(v) for v in camera_pos])
        call("rtp_fill_camera_order", self._h, cam)

    def fillGridDetector(self):
        call("rtp_fill_grid_detector", self._h)


class Fluids(Model):
    """Physics::CL::Fluids (physics/ocl/Fluids.hpp) on the GB300 path."""

    TYPE = abi.FLUIDS
    _DEFAULT_JSON = _FLUIDS_JSON

    def setFluidParams(self, fp):
        call("rtp_set_fluid_params", self._h, C.byref(fp))

    def fluidParams(self):
        fp = abi.FluidParams()
        call("rtp_get_fluid_params", self._h, C.byref(fp))
        return fp

    def setJacobiIterations(self, it):
        call("rtp_set_jacobi_iterations", self._h, int(it))

    # launch shape (new; rtp.h rtp_set_tuning) --------------------------------------------
    def setTuning(self, lanes=4, cell_factor=1.0, tiled=None):
        """Launch shape (rtp_set_tuning); tiled=None keeps the handle's tiled-sweep setting."""
        t = abi.Tuning()
        if tiled is None:
            call("rtp_get_tuning", self._h, C.byref(t))
        else:
            t.tiledSweeps = 1 if tiled else 0
        t.lanes = int(lanes)
        t.cellFactor = float(cell_factor)
        call("rtp_set_tuning", self._h, C.byref(t))

    def tuning(self):
        """(lanes, cell factor, tiled sweeps)."""
        t = abi.Tuning()
        call("rtp_get_tuning", self._h, C.byref(t))
        return int(t.lanes), float(t.cellFactor), int(t.tiledSweeps)

    def autotune(self, steps=5):
        """Times every launch-shape candidate over `steps` steps and keeps the fastest.
        Returns (best (lanes, cell factor, tiled), {(lanes, cell factor, tiled): ms per step})."""
        r = abi.TuneResult()
        call("rtp_autotune", self._h, int(steps), C.byref(r))
        key = lambda t: (int(t.lanes), round(float(t.cellFactor), 3), int(t.tiledSweeps))
        cands = {key(r.candidates[i]): float(r.msPerStep[i]) for i in range(r.tried)}
        return (int(r.best.lanes), float(r.best.cellFactor), int(r.best.tiledSweeps)), cands

    # learned warm start (new; rtp.h rtp_set_warm_start) --------------------------------
    def setWarmStart(self, net, extra_iterations=0, guard_tolerance=0.0, relax_all=False):
        """Warm-start the Jacobi solve with `net` (abi.Mlp); net=None switches it off.
        relax_all: the network's per-particle relaxation also applies to the extra iterations."""
        cfg = abi.WarmStartConfig()
        cfg.enabled = 0 if net is None else 1
        cfg.extraIterations = int(extra_iterations)
        cfg.guardTolerance = float(guard_tolerance)
        cfg.relaxAllIterations = 1 if relax_all else 0
        call("rtp_set_warm_start", self._h, None if net is None else C.byref(net), C.byref(cfg))

    def enableSolverStats(self, enable=True):
        call("rtp_enable_solver_stats", self._h, 1 if enable else 0)

    def solverStats(self):
        """dict: steps, reruns, mean (accepted solver-output mean |rho/rho0-1| per step),
        max, mean_first (before reruns)."""
        st = abi.SolverStats()
        call("rtp_get_solver_stats", self._h, C.byref(st))
        k = max(1, st.steps)
        return {"steps": int(st.steps), "reruns": int(st.reruns), "mean": st.sumDensityError / k,
                "max": st.maxDensityError, "mean_first": st.sumFirstError / k}

    def resetSolverStats(self):
        call("rtp_reset_solver_stats", self._h)

    def recordWarmStartSamples(self, reference_iterations, stride, phase, d_features, d_targets, capacity):
        """One plain step that writes training samples into device memory (pointers)."""
        w = C.c_uint64()
        call("rtp_record_warm_start_samples", self._h, int(reference_iterations), int(stride), int(phase),
             C.c_void_p(d_features), C.c_void_p(d_targets), int(capacity), C.byref(w))
        return int(w.value)

    # Fluids::transferJsonInputsToModel (Fluids.cpp:218-251).
    def transferJsonInputsToModel(self, js):
        f = js["Fluids"]
        fp = abi.FluidParams()
        fp.restDensity = float(f["Rest Density"][0])
        fp.relaxCFM = float(f["Relax CFM"][0])
        fp.timeStep = float(f["Time Step"][0])
        fp.dim = 2 if self._dimension == 2 else 3
        fp.isArtPressureEnabled = 1 if f["Artificial Pressure"]["Enable##Pressure"] is True else 0
        fp.artPressureCoeff = float(f["Artificial Pressure"]["Coefficient##Pressure"][0])
        fp.artPressureRadius = float(f["Artificial Pressure"]["Radius"][0])
        fp.artPressureExp = int(f["Artificial Pressure"]["Exp"][0])
        fp.isVorticityConfEnabled = 1 if f["Vorticity Confinement"]["Enable##Vorticity"] is True else 0
        fp.vorticityConfCoeff = float(f["Vorticity Confinement"]["Coefficient##Vorticity"][0])
        fp.xsphViscosityCoeff = float(f["Vorticity Confinement"]["xSPH Viscosity Coefficient"][0])
        iters = int(f["Nb Jacobi Iterations"][0])
        self.setFluidParams(fp)
        self.setJacobiIterations(iters)


class FluidsBatch(Fluids):
    """Many independent fluids scenes stepped together (rtp.h rtp_create_batch).  Buffers
    are the scenes' particles concatenated; sceneRange(s) gives scene s's slots."""

    def __init__(self, scenes, effect_radius, max_parts_in_cell=0):
        arr = (abi.BatchScene * len(scenes))()
        for i, (n, box) in enumerate(scenes):
            arr[i].nbParticles = int(n)
            for a in range(3):
                arr[i].boxSize[a] = float(box[a])
        self._h = C.c_void_p()
        call("rtp_create_batch", len(scenes), arr, float(effect_radius), int(max_parts_in_cell), C.byref(self._h))
        total = sum(int(n) for n, _ in scenes)
        self._params = abi.model_params(total, total, scenes[0][1], (1, 1, 1), 3)
        self._input_json = copy.deepcopy(self._DEFAULT_JSON)
        self._boundary = abi.BOUNCING_WALL
        self._pause = False
        self._dimension = 3
        self._case = abi.CASE_INVALID
        self._nscenes = len(scenes)

    def numScenes(self):
        return self._nscenes

    def sceneRange(self, s):
        off, cnt = C.c_uint64(), C.c_uint64()
        call("rtp_batch_scene_range", self._h, int(s), C.byref(off), C.byref(cnt))
        return int(off.value), int(cnt.value)

    def sceneConstants(self, s):
        c = abi.GridConstants()
        call("rtp_batch_scene_constants", self._h, int(s), C.byref(c))
        return c

    def sceneKeyBase(self, s):
        b = C.c_uint32()
        call("rtp_batch_scene_key_base", self._h, int(s), C.byref(b))
        return int(b.value)

    def constants(self):
        raise NotImplementedError("a batch has one grid per scene: sceneConstants(s)")


class Boids(Model):
    """Physics::CL::Boids (physics/ocl/Boids.hpp) on the GB300 path."""

    TYPE = abi.BOIDS
    _DEFAULT_JSON = _BOIDS_JSON

    def setBoidsParams(self, bp):
        call("rtp_set_boids_params", self._h, C.byref(bp))

    def setTimeStep(self, dt):
        call("rtp_set_boids_time_step", self._h, float(dt))

    def setTarget(self, tp):
        call("rtp_set_target", self._h, C.byref(tp))

    # Boids::transferJsonInputsToModel (Boids.cpp:177-210).
    def transferJsonInputsToModel(self, js):
        b = js["Boids"]
        bp = abi.BoidsParams()
        bp.velocityScale = float(b["Velocity"][0])
        bp.alignmentScale = float(b["Alignment"]["Scale##Alignment"][0]) if b["Alignment"]["Enable##Alignment"] else 0.0
        bp.separationScale = float(b["Separation"]["Scale##Separation"][0]) if b["Separation"]["Enable##Separation"] else 0.0
        bp.cohesionScale = float(b["Cohesion"]["Scale##Cohesion"][0]) if b["Cohesion"]["Enable##Cohesion"] else 0.0
        t = b["Target"]
        tp = abi.TargetParams()
        tp.enabled = 1 if t["Enable##Target"] else 0
        tp.visible = 1 if t["Show"] else 0
        tp.radiusEffect = float(t["Radius"][0])
        tp.signEffect = int(bool(t["Attract"]))  # (int)"Attract": 1 or 0
        self.setBoidsParams(bp)
        self.setTarget(tp)


class Clouds(Model):
    """Physics::CL::Clouds (physics/ocl/Clouds.hpp) on the GB300 path."""

    TYPE = abi.CLOUDS
    _DEFAULT_JSON = _CLOUDS_JSON

    def setFluidParams(self, fp):
        call("rtp_set_fluid_params", self._h, C.byref(fp))

    def setCloudParams(self, cp):
        call("rtp_set_cloud_params", self._h, C.byref(cp))

    def setJacobiIterations(self, it):
        call("rtp_set_jacobi_iterations", self._h, int(it))

    # learned warm start (new; rtp.h rtp_set_warm_start) --------------------------------
    def setWarmStart(self, net, extra_iterations=0, guard_tolerance=0.0, relax_all=False):
        """Warm-start the Jacobi solve with `net` (abi.Mlp); net=None switches it off.
        relax_all: the network's per-particle relaxation also applies to the extra iterations."""
        cfg = abi.WarmStartConfig()
        cfg.enabled = 0 if net is None else 1
        cfg.extraIterations = int(extra_iterations)
        cfg.guardTolerance = float(guard_tolerance)
        cfg.relaxAllIterations = 1 if relax_all else 0
        call("rtp_set_warm_start", self._h, None if net is None else C.byref(net), C.byref(cfg))

    def enableSolverStats(self, enable=True):
        call("rtp_enable_solver_stats", self._h, 1 if enable else 0)

    def solverStats(self):
        """dict: steps, reruns, mean (accepted solver-output mean |rho/rho0-1| per step),
        max, mean_first (before reruns)."""
        st = abi.SolverStats()
        call("rtp_get_solver_stats", self._h, C.byref(st))
        k = max(1, st.steps)
        return {"steps": int(st.steps), "reruns": int(st.reruns), "mean": st.sumDensityError / k,
                "max": st.maxDensityError, "mean_first": st.sumFirstError / k}

    def resetSolverStats(self):
        call("rtp_reset_solver_stats", self._h)

    def recordWarmStartSamples(self, reference_iterations, stride, phase, d_features, d_targets, capacity):
        """One plain step that writes training samples into device memory (pointers)."""
        w = C.c_uint64()
        call("rtp_record_warm_start_samples", self._h, int(reference_iterations), int(stride), int(phase),
             C.c_void_p(d_features), C.c_void_p(d_targets), int(capacity), C.byref(w))
        return int(w.value)

    def setEnvironment(self, env, ground=None):
        g = None
        if ground is not None:
            g = np.ascontiguousarray(ground, dtype=np.float32)
        call("rtp_set_cloud_environment", self._h, C.byref(env), None if g is None else g.ctypes.data_as(C.c_void_p))
        self._ground_keepalive = g

    def initThermo(self):
        call("rtp_clouds_init", self._h)

    # Clouds::transferJsonInputsToModel (Clouds.cpp:279-329).
    def transferJsonInputsToModel(self, js):
        f = js["Fluids"]
        c = js["Clouds"]
        fp = abi.FluidParams()
        fp.restDensity = float(f["Rest Density"][0])
        fp.relaxCFM = float(f["Relax CFM"][0])
        fp.timeStep = float(f["Time Step"][0])
        fp.dim = 2 if self._dimension == 2 else 3
        fp.isArtPressureEnabled = 1 if f["Artificial Pressure"]["Enable##Pressure"] is True else 0
        fp.artPressureCoeff = float(f["Artificial Pressure"]["Coefficient##Pressure"][0])
        fp.artPressureRadius = float(f["Artificial Pressure"]["Radius"][0])
        fp.artPressureExp = int(f["Artificial Pressure"]["Exp"][0])
        fp.isVorticityConfEnabled = 1 if f["Vorticity Confinement"]["Enable##Vorticity"] is True else 0
        fp.vorticityConfCoeff = float(f["Vorticity Confinement"]["Coefficient##Vorticity"][0])
        fp.xsphViscosityCoeff = float(f["Vorticity Confinement"]["xSPH Viscosity Coefficient"][0])
        cp = abi.CloudParams()
        cp.restDensity = fp.restDensity
        cp.timeStep = fp.timeStep
        cp.dim = fp.dim
        cp.relaxCFM = fp.relaxCFM
        cp.isTempSmoothingEnabled = 1 if c["Enable Temperature Smoothing"] else 0
        cp.groundHeatCoeff = float(c["Ground Heat Coefficient"][0])
        cp.buoyancyCoeff = float(c["Buoyancy Heat Coefficient"][0])
        cp.gravCoeff = float(c["Gravity Coefficient"][0])
        cp.adiabaticLapseRate = float(c["Adiabatic Lapse Rate"][0])
        cp.phaseTransitionRate = float(c["Phase Transition Rate"][0])
        cp.latentHeatCoeff = float(c["Latent Heat Coefficient"][0])
        cp.windCoeff = float(c["Wind Coefficient"][0])
        cp.initVaporDensityCoeff = 0.75
        iters = int(f["Nb Jacobi Iterations"][0])
        self.setFluidParams(fp)
        self.setCloudParams(cp)
        self.setJacobiIterations(iters)


def CreateModel(model_type, params):
    """Physics::CreateModel (physics/Model.cpp:10-24)."""
    if model_type == abi.BOIDS:
        return Boids(params)
    if model_type == abi.FLUIDS:
        return Fluids(params)
    if model_type == abi.CLOUDS:
        return Clouds(params)
    return None


def get_constants(model_type, params):
    """Host-only derivation of the JIT constants (no device needed)."""
    c = abi.GridConstants()
    call("rtp_get_constants", int(model_type), C.byref(params), C.byref(c))
    return c


def default_fluid_params():
    p = abi.FluidParams()
    call("rtp_fluid_params_default", C.byref(p))
    return p


def default_boids_params():
    p = abi.BoidsParams()
    call("rtp_boids_params_default", C.byref(p))
    return p


def default_target_params():
    p = abi.TargetParams()
    call("rtp_target_params_default", C.byref(p))
    return p


def default_cloud_params():
    p = abi.CloudParams()
    call("rtp_cloud_params_default", C.byref(p))
    return p


def reference_cloud_env():
    e = abi.CloudEnv()
    call("rtp_cloud_env_reference", C.byref(e))
    return e


__all__ = ["Model", "Fluids", "Boids", "Clouds", "CreateModel", "RtpError", "get_constants", "lib",
           "default_fluid_params", "default_boids_params", "default_cloud_params", "reference_cloud_env"]
