"""The C++ Physics::Model subclasses (realtimeparticles_gb300/cpp/CudaModels.hpp) compiled
against the reference's own physics/Model.hpp, utils/Parameters.hpp, Geometry.hpp and Math.hpp
(physics/Model.hpp:81-216), with a small nlohmann/json stand-in (tests/model_binding), and
linked with librtp_gb300.so.  A typo in the binding a maintainer would paste into the reference
tree fails here.

- `json`: the subclasses' JSON reads (Fluids.cpp:218-251, Boids.cpp:177-210,
  Clouds.cpp:279-329) on trees with the reference's paths;
- `create`: CreateModel for each model, a reset and two steps; without a CUDA device the
  library's error must come back as std::runtime_error carrying rtp_last_error().

Needs the reference checkout (REFERENCE_DIR, default: `reference` next to this repository) for
its headers; skipped without it.  No GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("REFERENCE_DIR", os.path.join(os.path.dirname(ROOT), "reference"))
LIB_DIR = os.path.join(ROOT, "realtimeparticles_gb300")

pytestmark = [
    pytest.mark.skipif(not os.path.exists(os.path.join(REF, "physics", "Model.hpp")),
                       reason="reference checkout with physics/Model.hpp not present"),
    pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not found"),
    pytest.mark.skipif(not os.path.exists(os.path.join(LIB_DIR, "librtp_gb300.so")),
                       reason="librtp_gb300.so not built"),
]


@pytest.fixture(scope="module")
def binary(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("binding") / "check_binding")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror",
           "-I", os.path.join(ROOT, "tests", "model_binding"),
           "-isystem", os.path.join(REF, "physics"), "-isystem", os.path.join(REF, "utils"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "realtimeparticles_gb300", "cpp"),
           os.path.join(ROOT, "tests", "model_binding", "check_binding.cpp"),
           "-L", LIB_DIR, "-lrtp_gb300", "-Wl,-rpath," + LIB_DIR, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return out


def test_json_paths_of_the_subclasses(binary):
    r = subprocess.run([binary, "json"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert lines[0] == "fluids 450.0000 600.0 0.0100 3 1 0.0060 0.0010 4 1 0.00040 0.00010 iters 2"
    assert lines[1] == "clouds smoothing 1 wind 0.30 rho0 450.0"
    assert lines[2] == "boids 2.00 1.50 0"


def test_create_reset_and_step(binary):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    r = subprocess.run([binary, "create"], capture_output=True, text=True, timeout=300)
    if has_gpu:
        assert r.returncode == 0, r.stdout + r.stderr
        assert r.stdout.splitlines() == ["created fluids 4096", "created boids 4096", "created clouds 4096"]
    else:
        assert r.returncode == 3, r.stdout + r.stderr
        assert r.stdout.startswith("error fluids: rtp_create: "), r.stdout
