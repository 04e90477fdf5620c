"""GB300-native RealTimeParticles simulation step.

The compute path is librtp_gb300.so (hand-written CUDA for sm_103a behind the C ABI in
include/rtp.h).  This package holds the Python mirror of the reference's
Physics::Model interface (model.py), the ctypes types (abi.py), seeded scene generators
(scenes.py) and the build recipe (build()).
"""
import os
import subprocess

from . import abi  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))


def build(jobs=8, quiet=True):
    """Compile librtp_gb300.so for sm_103a (make -C csrc)."""
    out = subprocess.run(["make", "-C", os.path.join(_HERE, "csrc"), "-j%d" % jobs], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("librtp_gb300 build failed:\n" + out.stdout[-4000:] + out.stderr[-8000:])
    if not quiet:
        print(out.stdout)
    return os.path.join(_HERE, "librtp_gb300.so")


def __getattr__(name):
    # Lazy: importing the package must not load the CUDA library (CPU-only tools and the
    # oracle import abi/scenes).
    if name in ("Model", "Fluids", "Boids", "Clouds", "CreateModel", "RtpError", "get_constants",
                "default_fluid_params", "default_boids_params", "default_cloud_params", "default_target_params",
                "reference_cloud_env"):
        from . import model
        return getattr(model, name)
    raise AttributeError(name)
