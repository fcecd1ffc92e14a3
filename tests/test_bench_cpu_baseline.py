"""bench.py's CPU baseline leg on the host: the oracle on all host threads
and on one thread (the reference's C kernels are single-threaded), with the
oracle's thread count restored afterwards."""

import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
import oracle  # noqa: E402
from tupan_gb300 import ics  # noqa: E402


def test_cpu_baseline_reports_all_threads_and_one():
    ps = ics.plummer(2048, eps=1e-4, seed=4)
    before = oracle.max_threads()
    out = bench.cpu_baseline(2048, 256, ps)
    assert oracle.max_threads() == before
    assert out["kind"] == "port" and out["unit"] == "Gint/s"
    assert out["cores"] == before and out["value"] > 0
    one = out["single_core"]
    assert one["cores"] == 1 and one["value"] > 0
    assert "ni=16 x nj=2048" in one["sample"]


def test_nominal_fp32_peak_formula():
    # 152 SMs x 128 lanes x 2 flop x 2070 MHz
    assert abs(bench.nominal_fp32_tflops(152, 2070.0) - 80.54784) < 1e-9
    # 262144^2 interactions x 42 flop in 77.2 ms
    assert abs(bench.achieved_aj(262144, 0.0772) - 37.3862) < 1e-3
