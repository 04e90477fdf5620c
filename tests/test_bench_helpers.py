"""bench.py helpers (CPU only): the equal-error comparison of the warm-start studies (the Pareto
front of the plain solver's (error, throughput) points, the log-log interpolation of the plain
throughput at a given error, the fastest-configuration pick under an error bound) and the byte
accounting of the grid/sort roofline."""
import math
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_pareto_front_drops_dominated_points():
    # (error, particle-steps/s): I = 4 is dominated by I = 3 (worse error and slower), and the
    # last point (error growing again at many iterations) by every point before it that is faster
    curve = [(0.28, 380.0), (0.045, 515.0), (0.033, 402.0), (0.0329, 343.0), (0.034, 300.0), (0.009, 78.0),
             (0.018, 65.0)]
    front = bench._pareto(curve)
    assert front == [(0.045, 515.0), (0.033, 402.0), (0.0329, 343.0), (0.009, 78.0)]
    assert all(e1 < e0 for (e0, _), (e1, _) in zip(front, front[1:]))  # error decreasing


def test_plain_throughput_interpolated_log_log_on_the_front():
    curve = [(0.04, 400.0), (0.01, 100.0), (0.02, 50.0)]  # the last point is off the front
    # halfway in log error between 0.04 and 0.01 -> halfway in log throughput
    v = bench._plain_at(curve, 0.02)
    assert v == pytest.approx(200.0, rel=1e-12)
    assert bench._plain_at(curve, 0.04) == pytest.approx(400.0)
    assert bench._plain_at(curve, 0.01) == pytest.approx(100.0)
    assert bench._plain_at(curve, 0.05) is None and bench._plain_at(curve, 0.005) is None
    # monotone between the endpoints
    xs = [0.039, 0.03, 0.02, 0.011]
    ys = [bench._plain_at(curve, x) for x in xs]
    assert all(a > b for a, b in zip(ys, ys[1:]))
    assert math.log(ys[1]) == pytest.approx(math.log(400.0) + (math.log(0.03) - math.log(0.04))
                                            / (math.log(0.01) - math.log(0.04)) * (math.log(100.0) - math.log(400.0)))


def test_threshold_pick_takes_the_fastest_under_the_bound():
    plain = [{"iterations": i, "particle_steps_per_s": v, "mean_density_error": e}
             for i, v, e in ((3, 400.0, 0.033), (16, 113.0, 0.0124), (24, 78.0, 0.009), (32, 65.0, 0.0183))]
    learned = [{"extra_iterations": k, "particle_steps_per_s": v, "mean_density_error": e}
               for k, v, e in ((2, 380.0, 0.028), (7, 199.0, 0.0102), (9, 166.0, 0.0084), (11, 142.0, 0.0073))]
    r = bench._at_threshold(plain, learned, 0.01)
    assert r["plain"]["iterations"] == 24 and r["learned"]["extra_iterations"] == 9
    assert r["speedup"] == pytest.approx(166.0 / 78.0)
    none = bench._at_threshold(plain, learned, 0.005)
    assert none["speedup"] is None and none["plain"] is None


def test_grid_sort_roofline_counts_the_algorithmic_bytes_of_each_kernel():
    class C:  # the grid constants grid_sort_summary reads
        keyBits = 18  # two 9-bit passes
        numCells = 64000
    n, nonempty, steps = 131072, 16000, 4
    # kernel -> (launches, total ms) over `steps` steps, as Model.kernelTimes() reports
    kt = {"fld_predict": (4, 0.04), "sort_scan": (8, 0.05), "sort_pass": (4, 0.04), "sort_pass_gather": (4, 0.056),
          "cellTable": (4, 0.024), "fld_lambda": (12, 0.7)}
    r = bench.grid_sort_summary(kt, steps, n, C, nonempty, 6800.0)
    expect = 52 * n + 12 * n + 112 * n + 8 * C.numCells + 4 * n + 8 * nonempty
    assert r["algorithmic_bytes_per_step"] == expect
    assert r["sort_passes"] == 2
    assert r["ms_per_step"] == pytest.approx((0.04 + 0.05 + 0.04 + 0.056 + 0.024) / steps)  # fld_lambda left out
    assert r["achieved_gbs"] == pytest.approx(expect / (r["ms_per_step"] / 1000.0) / 1e9)
    assert r["frac"] == pytest.approx(r["achieved_gbs"] / 6800.0)
    assert "fld_lambda" not in r["kernels"]
    C.keyBits = 26  # three passes: the middle one moves keys and indices in and out
    r3 = bench.grid_sort_summary(kt, steps, n, C, nonempty, 6800.0)
    assert r3["sort_passes"] == 3
    assert r3["algorithmic_bytes_per_step"] == expect + 16 * n
