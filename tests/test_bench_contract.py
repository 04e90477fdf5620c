"""The reference arm of bench.py on the host cores (no GPU needed): one JSON line with the same
metric, unit, direction and workload configuration as the CUDA arm, the CPU implementation
described in cpu_baseline, and an end-to-end figure with no host<->device bytes."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    sys.path.insert(0, ROOT)
    import bench

    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    w = bench.WORKLOADS[bench.WORKLOAD]
    assert d["impl"] == "reference"
    assert d["metric"] == w["metric"]
    assert d["unit"] == "particle-steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] >= 1 and d["warmup"] == 3
    cfg = d["config"]
    assert cfg["workload"] == bench.WORKLOAD and cfg["particles"] == 131072 and cfg["jacobi_iterations"] == 3
    assert cfg["l2"] == bench.L2_NOTE  # the same "l2" entry as the GPU arm's config
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
