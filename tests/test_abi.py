"""The C-ABI library loads, exports every symbol include/rtp.h declares, and its
host-only functions agree with the oracle.  No compute call is made here."""
import ctypes as C
import os
import subprocess

import pytest

from realtimeparticles_gb300 import _lib, abi, model

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_every_header_symbol_is_exported(rtp_lib):
    names = _lib.header_symbols()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(rtp_lib, n)]
    assert not missing, missing
    # Every declared symbol has a ctypes signature in the binding.
    assert set(names) <= set(_lib._SIGS), sorted(set(names) - set(_lib._SIGS))


def test_struct_layouts_match_reference_structs():
    assert C.sizeof(abi.FluidParams) == 44   # FluidKernelInputs, 11 x 4 bytes
    assert C.sizeof(abi.CloudParams) == 52   # CloudKernelInputs, 13 x 4 bytes
    assert C.sizeof(abi.BoidsParams) == 16   # BoidsRuleKernelInputs
    assert C.sizeof(abi.TargetParams) == 16  # JSON Target group; TargetKernelInputs is its last 8 bytes


def test_ctypes_layouts_match_the_c_header(tmp_path):
    """sizeof and field offsets of every struct, as compiled by the C compiler."""
    structs = {"rtp_model_params": abi.ModelParams, "rtp_fluid_params": abi.FluidParams,
               "rtp_boids_params": abi.BoidsParams, "rtp_cloud_params": abi.CloudParams,
               "rtp_cloud_env": abi.CloudEnv, "rtp_grid_constants": abi.GridConstants,
               "rtp_kernel_time": abi.KernelTime, "rtp_metrics": abi.Metrics, "rtp_mlp": abi.Mlp,
               "rtp_warm_start_config": abi.WarmStartConfig, "rtp_solver_stats": abi.SolverStats,
               "rtp_train_config": abi.TrainConfig, "rtp_batch_scene": abi.BatchScene, "rtp_tuning": abi.Tuning,
               "rtp_tune_result": abi.TuneResult, "rtp_target_params": abi.TargetParams}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "%s/include/rtp.h"' % ROOT, "int main(void) {"]
    for cname, py in structs.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-o", str(exe), str(src)], check=True)
    out = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(out[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(out["%s.%s" % (cname, f)]) == getattr(py, f).offset, (cname, f)


def test_abi_version(rtp_lib):
    assert rtp_lib.rtp_abi_version() == 2


@pytest.mark.parametrize("mtype,box,res", [(abi.FLUIDS, 1.0, 40), (abi.BOIDS, 2.0, 40), (abi.CLOUDS, (1.0, 2.0, 1.0),
                                                                                          (30, 60, 30)),
                                          (abi.FLUIDS, 10.0, 30)])
def test_constants_match_oracle(oracle_mod, mtype, box, res):
    box = box if isinstance(box, tuple) else (box,) * 3
    res = res if isinstance(res, tuple) else (res,) * 3
    mp = abi.model_params(100, 100, box, res)
    a = model.get_constants(mtype, mp)
    b = oracle_mod.derive_constants(mtype, mp)
    assert abi.struct_to_dict(a) == abi.struct_to_dict(b)


def test_reference_defaults():
    fp = model.default_fluid_params()
    assert (fp.restDensity, fp.relaxCFM, fp.artPressureExp) == (450.0, 600.0, 4)
    bp = model.default_boids_params()
    assert bp.velocityScale == pytest.approx(0.5)
    cp = model.default_cloud_params()
    assert cp.groundHeatCoeff == 10.0 and cp.isTempSmoothingEnabled == 1
    env = model.reference_cloud_env()
    assert (env.groundTemp0, env.lapseRate, env.heatDecay) == (293.0, 3.5, 3.0)


def test_invalid_arguments_are_rejected_without_device(rtp_lib):
    c = abi.GridConstants()
    rc = rtp_lib.rtp_get_constants(7, C.byref(abi.model_params(1, 1, (1, 1, 1), (2, 2, 2))), C.byref(c))
    assert rc == abi.ERR_INVALID_ARGUMENT
    assert "unknown model" in _lib.last_error()
    bad = abi.model_params(1, 1, (0.0, 1, 1), (2, 2, 2))
    assert rtp_lib.rtp_get_constants(abi.FLUIDS, C.byref(bad), C.byref(c)) == abi.ERR_INVALID_ARGUMENT
    sz = C.c_size_t()
    assert rtp_lib.rtp_radix_sort_scratch_bytes(1000, 33, C.byref(sz)) == abi.ERR_INVALID_ARGUMENT
    assert rtp_lib.rtp_radix_sort_scratch_bytes(131072, 17, C.byref(sz)) == 0 and sz.value > 4 * 131072 * 4


def test_merge_patch_semantics():
    a = {"Fluids": {"Rest Density": [450.0, 10.0, 1000.0], "Time Step": [0.01, 0, 1]}}
    b = model._merge_patch(a, {"Fluids": {"Rest Density": [500.0, 10.0, 1000.0], "Time Step": None}})
    assert b == {"Fluids": {"Rest Density": [500.0, 10.0, 1000.0]}}
