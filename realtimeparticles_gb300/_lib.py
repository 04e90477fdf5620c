"""ctypes binding of librtp_gb300.so (include/rtp.h).

The shared library is built in-tree by realtimeparticles_gb300/csrc/Makefile (see
realtimeparticles_gb300.build).  There is no fallback: if the library is missing or a
call fails, an RtpError is raised.
"""
import ctypes as C
import os
import threading

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "librtp_gb300.so")
_LIB = None
_LOCK = threading.Lock()


class RtpError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("rtp error %d: %s" % (code, msg))
        self.code = code


P = C.c_void_p
PP = C.POINTER(C.c_void_p)
U32 = C.c_uint32
U64 = C.c_uint64

# name -> argtypes; every function returns int (status) unless listed in _RESTYPES.
_SIGS = {
    "rtp_last_error": [],
    "rtp_abi_version": [],
    "rtp_get_constants": [C.c_int, C.POINTER(abi.ModelParams), C.POINTER(abi.GridConstants)],
    "rtp_fluid_params_default": [C.POINTER(abi.FluidParams)],
    "rtp_boids_params_default": [C.POINTER(abi.BoidsParams)],
    "rtp_cloud_params_default": [C.POINTER(abi.CloudParams)],
    "rtp_cloud_env_reference": [C.POINTER(abi.CloudEnv)],
    "rtp_create": [C.c_int, C.POINTER(abi.ModelParams), PP],
    "rtp_destroy": [P],
    "rtp_reset": [P],
    "rtp_update": [P, U32],
    "rtp_set_fluid_params": [P, C.POINTER(abi.FluidParams)],
    "rtp_get_fluid_params": [P, C.POINTER(abi.FluidParams)],
    "rtp_set_jacobi_iterations": [P, U32],
    "rtp_set_boids_params": [P, C.POINTER(abi.BoidsParams)],
    "rtp_set_boids_time_step": [P, C.c_float],
    "rtp_update_host": [P, P, P, C.c_uint64, U32, P, P],
    "rtp_target_params_default": [C.POINTER(abi.TargetParams)],
    "rtp_set_target": [P, C.POINTER(abi.TargetParams)],
    "rtp_get_target": [P, C.POINTER(C.c_float), C.POINTER(C.c_int), C.POINTER(C.c_int)],
    "rtp_set_cloud_params": [P, C.POINTER(abi.CloudParams)],
    "rtp_set_cloud_environment": [P, C.POINTER(abi.CloudEnv), P],
    "rtp_clouds_init": [P],
    "rtp_set_nb_particles": [P, U64],
    "rtp_get_nb_particles": [P, C.POINTER(U64)],
    "rtp_set_boundary": [P, C.c_int],
    "rtp_set_dimension": [P, U32],
    "rtp_set_case": [P, C.c_int],
    "rtp_pause": [P, C.c_int],
    "rtp_upload": [P, C.c_int, P, U64],
    "rtp_download": [P, C.c_int, P, U64],
    "rtp_device_ptr": [P, C.c_int, PP],
    "rtp_stream": [P, PP],
    "rtp_synchronize": [P],
    "rtp_enable_profiling": [P, C.c_int],
    "rtp_is_profiling_enabled": [P, C.POINTER(C.c_int)],
    "rtp_get_kernel_times": [P, C.POINTER(abi.KernelTime), U32, C.POINTER(U32)],
    "rtp_reset_kernel_times": [P],
    "rtp_time_steps": [P, U32, U64, C.POINTER(C.c_double)],
    "rtp_get_metrics": [P, C.POINTER(abi.Metrics)],
    "rtp_fill_cell_ids": [C.POINTER(abi.GridConstants), P, U32, P, P],
    "rtp_radix_sort_scratch_bytes": [U32, U32, C.POINTER(C.c_size_t)],
    "rtp_radix_sort": [P, U32, U32, P, P, P, C.c_size_t, P],
    "rtp_build_cell_table": [C.POINTER(abi.GridConstants), P, U32, P, P],
    "rtp_radix_sort_noalloc": [P, U32, U32, P, P, P],
    "rtp_radix_sort_pass": [P, U32, U32, U32, P, P, P, P, P, P],
    "rtp_set_warm_start": [P, C.POINTER(abi.Mlp), C.POINTER(abi.WarmStartConfig)],
    "rtp_enable_solver_stats": [P, C.c_int],
    "rtp_get_solver_stats": [P, C.POINTER(abi.SolverStats)],
    "rtp_reset_solver_stats": [P],
    "rtp_record_warm_start_samples": [P, U32, U32, U32, P, P, U64, C.POINTER(U64)],
    "rtp_train_warm_start": [P, P, U64, C.POINTER(abi.TrainConfig), C.POINTER(abi.Mlp), P, P],
    "rtp_mlp_loss_grad": [C.POINTER(abi.Mlp), P, P, P, U64, C.POINTER(C.c_double), C.POINTER(abi.Mlp), P],
    "rtp_mlp_forward": [C.POINTER(abi.Mlp), P, U64, P, P],
    "rtp_mlp_backward": [C.POINTER(abi.Mlp), P, P, U64, C.POINTER(abi.Mlp), P],
    "rtp_warm_start_loss_grad": [P, C.POINTER(abi.Mlp), P, C.POINTER(C.c_double)],
    "rtp_train_warm_start_rollout": [P, C.POINTER(abi.TrainConfig), U32, U32, C.c_int, C.POINTER(abi.Mlp), P],
    "rtp_fill_fluid_color": [P],
    "rtp_fill_color_float": [P, C.c_int, C.c_float, C.c_float],
    "rtp_fill_camera_order": [P, C.POINTER(C.c_float)],
    "rtp_fill_grid_detector": [P],
    "rtp_create_batch": [U32, C.POINTER(abi.BatchScene), C.c_float, U32, PP],
    "rtp_batch_scene_range": [P, U32, C.POINTER(U64), C.POINTER(U64)],
    "rtp_batch_scene_constants": [P, U32, C.POINTER(abi.GridConstants)],
    "rtp_batch_scene_key_base": [P, U32, C.POINTER(U32)],
    "rtp_set_tuning": [P, C.POINTER(abi.Tuning)],
    "rtp_get_tuning": [P, C.POINTER(abi.Tuning)],
    "rtp_autotune": [P, U32, C.POINTER(abi.TuneResult)],
}
_RESTYPES = {"rtp_last_error": C.c_char_p}


def header_symbols():
    """Function names declared in include/rtp.h (parsed from the header text)."""
    import re
    hdr = os.path.join(os.path.dirname(_HERE), "include", "rtp.h")
    txt = open(hdr).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(rtp_\w+)\s*\(", txt, re.M)))


def lib():
    """Load the CUDA library (once).  Raises RtpError if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    with _LOCK:
        if _LIB is None:
            if not os.path.exists(LIB_PATH):
                raise RtpError(-1, "librtp_gb300.so not built: run realtimeparticles_gb300.build() "
                                   "(make -C realtimeparticles_gb300/csrc)")
            L = C.CDLL(LIB_PATH)
            for name, args in _SIGS.items():
                f = getattr(L, name)
                f.argtypes = args
                f.restype = _RESTYPES.get(name, C.c_int)
            _LIB = L
    return _LIB


def last_error():
    return lib().rtp_last_error().decode(errors="replace")


def check(rc):
    if rc != 0:
        raise RtpError(rc, last_error())
    return rc


def call(name, *args):
    return check(getattr(lib(), name)(*args))
