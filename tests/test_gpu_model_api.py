"""Model API behaviour on the GPU: reset cases, setters, JSON inputs, errors, buffers,
profiling (physics/Model.hpp:81-216, physics/ocl/OclModel.hpp)."""
import ctypes as C

import numpy as np
import pytest

from realtimeparticles_gb300 import RtpError, abi, model, scenes
from realtimeparticles_gb300._lib import call

pytestmark = pytest.mark.gpu


def _ref_params(mtype, case, box=(10.0, 10.0, 10.0), res=(30, 30, 30)):
    # ParticleSystemApp::initPhysicsEngine (app/ParticleSystemApp.cpp:275-318).
    return abi.model_params(0, 131072, box, res, 3, case)


@pytest.mark.parametrize("mtype,case,n", [(abi.FLUIDS, abi.CASE_FLUIDS_DAM, 131072),
                                          (abi.FLUIDS, abi.CASE_FLUIDS_BOMB, 65536),
                                          (abi.FLUIDS, abi.CASE_FLUIDS_DROP, 4096 + 65536),
                                          (abi.BOIDS, abi.CASE_BOIDS_SMALL, 512),
                                          (abi.BOIDS, abi.CASE_BOIDS_XLARGE, 131072)])
def test_reset_cases(mtype, case, n):
    with model.CreateModel(mtype, _ref_params(mtype, case)) as m:
        m.reset()
        assert m.nbParticles() == n
        pos = m.download(abi.BUF_POS, m.maxNbParticles())
        assert np.all(np.isfinite(pos[:n, :3]))
        if n < m.maxNbParticles():
            assert np.all(np.isinf(pos[n:, :3]))  # inactive slots at +inf (Fluids.cpp:383-384)
        m.update(2)
        assert np.all(np.isfinite(m.download(abi.BUF_POS)[:, :3]))


def test_clouds_reset_case():
    p = _ref_params(abi.CLOUDS, abi.CASE_CLOUDS_CUMULUS, box=(10.0, 20.0, 10.0), res=(30, 60, 30))
    with model.Clouds(p) as m:
        m.reset()
        assert m.nbParticles() == 65536
        t = m.download(abi.BUF_TEMP)
        assert t.min() >= 223.0 - 1e-3 and t.max() <= 293.0 + 1e-3
        m.update(3)
        t = m.download(abi.BUF_TEMP)
        assert np.all(np.isfinite(t))


def test_json_inputs_and_wrong_path():
    sc = scenes.dam_break(lattice=(8, 8, 8))
    with model.Fluids(sc["model_params"]) as m:
        m.updateInputJson({"Fluids": {"Rest Density": [500.0, 10.0, 1000.0], "Nb Jacobi Iterations": [3, 1, 6]}})
        assert m.fluidParams().restDensity == 500.0
        with pytest.raises(RuntimeError, match="Wrong Json parsing"):
            m.updateModelWithInputJson({"Fluid": {}})


def test_errors_and_capacity():
    sc = scenes.dam_break(lattice=(8, 8, 8))
    with model.Fluids(sc["model_params"]) as m:
        with pytest.raises(RtpError) as e:
            m.setNbParticles(10 ** 6)
        assert e.value.code == abi.ERR_CAPACITY
        with pytest.raises(RtpError):
            m.upload(abi.BUF_POS, np.zeros((10 ** 6, 4), np.float32))
        with pytest.raises(RtpError):
            m.setBoundary(7)
        with pytest.raises(RtpError) as e:
            m.setDimension(4)
        assert e.value.code == abi.ERR_INVALID_ARGUMENT
        with pytest.raises(RtpError) as e:  # the 2D dam case needs 4,096 particles: more than the 512 here
            m.setCase(abi.CASE_FLUIDS_DAM)
            m.setDimension(2)
        assert e.value.code == abi.ERR_CAPACITY
    with pytest.raises(RtpError):
        model.Fluids(abi.model_params(10, 5, (1, 1, 1), (4, 4, 4)))


def test_pause_profiling_and_device_pointers():
    sc = scenes.dam_break(lattice=(8, 16, 16))
    with model.Fluids(sc["model_params"]) as m:
        m.setFluidParams(sc["fluid_params"])
        m.upload(abi.BUF_POS, sc["pos"])
        before = m.download(abi.BUF_POS)
        m.pause(True)
        m.update(3)
        assert np.array_equal(m.download(abi.BUF_POS), before)
        m.pause(False)
        assert m.devicePtr(abi.BUF_POS) and m.stream()
        m.enableProfiling(True)
        assert m.isProfilingEnabled()
        m.update(2)
        kt = m.kernelTimes()
        assert kt["fld_lambda"][0] == 2 * 2 and kt["fld_lambda"][1] > 0
        assert kt["sort_pass_gather"][0] == 2
        ms = m.timeSteps(3, flush_bytes=1 << 24)
        assert ms > 0
        with pytest.raises(RtpError):
            m.download(abi.BUF_ACC)


def test_update_host_equals_upload_update_download():
    """rtp_update_host = rtp_upload(pos, vel) + rtp_update + rtp_download(pos, vel), bit for bit."""
    sc = scenes.dam_break(lattice=(8, 16, 16))
    n = sc["pos"].shape[0]
    outs = []
    for fused in (False, True):
        with model.Fluids(sc["model_params"]) as m:
            m.setFluidParams(sc["fluid_params"])
            m.setJacobiIterations(3)
            pos, vel = sc["pos"].copy(), sc["vel"].copy()
            for _ in range(3):
                if fused:
                    m.updateHost(pos, vel, nsteps=2)
                else:
                    m.upload(abi.BUF_POS, pos)
                    m.upload(abi.BUF_VEL, vel)
                    m.update(2)
                    pos, vel = m.download(abi.BUF_POS), m.download(abi.BUF_VEL)
            outs.append((pos, vel, m.download(abi.BUF_ID)))
            with pytest.raises(RtpError):  # count must be the particle count
                call("rtp_update_host", m.handle, None, None, n - 1, 1, None, None)
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)



def test_update_host_pinned_buffers():
    """Pinned host buffers take the path whose first and last kernels read and write host memory
    directly; results equal the copy path bit for bit, for shared and separate in/out buffers and
    after the buffers change."""
    torch = pytest.importorskip("torch")
    sc = scenes.dam_break(lattice=(8, 16, 16))
    n = sc["pos"].shape[0]

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True).numpy()
        t[:] = a
        return t

    ref, fast = model.Fluids(sc["model_params"]), model.Fluids(sc["model_params"])
    with ref, fast:
        for m in (ref, fast):
            m.setFluidParams(sc["fluid_params"])
            m.setJacobiIterations(3)
        rp, rv = sc["pos"].copy(), sc["vel"].copy()          # pageable: the copy path
        fp, fv = pinned(sc["pos"]), pinned(sc["vel"])        # pinned: the direct path
        for _ in range(3):
            ref.updateHost(rp, rv, 1)
            fast.updateHost(fp, fv, 1)
            assert np.array_equal(rp, fp) and np.array_equal(rv, fv)
        # Separate output buffers, then new input buffers (the step is captured again).
        op, ov = pinned(np.zeros_like(fp)), pinned(np.zeros_like(fv))
        P = lambda a: a.ctypes.data_as(C.c_void_p)
        call("rtp_update_host", fast.handle, P(fp), P(fv), n, 1, P(op), P(ov))
        ref.updateHost(rp, rv, 1)
        assert np.array_equal(op, rp) and np.array_equal(ov, rv)
        fp2, fv2 = pinned(op), pinned(ov)
        call("rtp_update_host", fast.handle, P(fp2), P(fv2), n, 2, P(fp2), P(fv2))   # two steps: copy path
        ref.updateHost(rp, rv, 2)
        assert np.array_equal(fp2, rp) and np.array_equal(fv2, rv)
        assert np.array_equal(fast.download(abi.BUF_POS), rp)  # the device state follows
        # Ping-pong between two pinned buffer pairs (kept captures are reused).
        qa = (pinned(fp2), pinned(fv2))
        qb = (pinned(np.zeros_like(fp2)), pinned(np.zeros_like(fv2)))
        for k in range(4):
            src, dst = (qa, qb) if k % 2 == 0 else (qb, qa)
            call("rtp_update_host", fast.handle, P(src[0]), P(src[1]), n, 1, P(dst[0]), P(dst[1]))
            ref.updateHost(rp, rv, 1)
            assert np.array_equal(dst[0], rp) and np.array_equal(dst[1], rv)


def test_update_host_pinned_boids_with_target():
    """The direct host path for boids (keys kernel reads, rules kernel writes host memory),
    target attractor on: equal to the copy path bit for bit."""
    torch = pytest.importorskip("torch")
    sc = scenes.boids_cloud(n=5000, seed=3)
    runs = []
    for use_pinned in (False, True):
        with model.Boids(sc["model_params"]) as m:
            m.setBoidsParams(sc["boids_params"])
            m.setTimeStep(0.01)
            m.setBoundary(abi.CYCLIC_WALL)
            tp = model.default_target_params()
            tp.enabled = 1
            tp.radiusEffect = 0.8
            m.setTarget(tp)
            if use_pinned:
                pos = torch.empty((5000, 4), dtype=torch.float32, pin_memory=True).numpy()
                vel = torch.empty((5000, 4), dtype=torch.float32, pin_memory=True).numpy()
                pos[:], vel[:] = sc["pos"], sc["vel"]
            else:
                pos, vel = sc["pos"].copy(), sc["vel"].copy()
            for _ in range(4):
                m.updateHost(pos, vel, 1)
            runs.append((pos.copy(), vel.copy(), m.download(abi.BUF_ACC), m.targetPos()))
    for a, b in zip(runs[0][:3], runs[1][:3]):
        assert np.array_equal(a, b)
    assert runs[0][3] == runs[1][3]


def test_inactive_slots_keep_sentinel_cell_ids():
    """resetCellIDs (grid.cl:65-71, run over maxNb at reset): the slots a step does not fill keep
    2 * numCells + slot and stay at the tail of the sorted keys."""
    sc = scenes.dam_break(lattice=(8, 16, 16), max_n=5000)
    n = sc["pos"].shape[0]
    with model.Fluids(sc["model_params"]) as m:
        m.setFluidParams(sc["fluid_params"])
        m.upload(abi.BUF_POS, sc["pos"])
        m.upload(abi.BUF_VEL, sc["vel"])
        m.update(2)
        keys = m.download(abi.BUF_CELL_ID, 5000)
        nc = m.constants().numCells
        assert np.all(keys[:n] < nc) and np.all(np.diff(keys[:n].astype(np.int64)) >= 0)
        assert np.array_equal(keys[n:], 2 * nc + np.arange(n, 5000, dtype=np.uint32))
