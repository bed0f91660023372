"""Host-side pieces of bench.py and the roofline model (no GPU)."""
import sys
import os

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402
from gpumatfun_gb300 import roofline  # noqa: E402


def test_profiled_traffic_keys():
    # the committed summaries carry traffic for the benched launches
    assert bench.profiled_traffic("fe-disk-1M-fp64", "fp64", 1) > 1e10
    assert bench.profiled_traffic("fd3d-256-mixed", "mixed", 1) > 1e11
    assert bench.profiled_traffic("fd3d-256-mixed", "fp64", 1) > 1e11
    assert bench.profiled_traffic("fe-disk-1M-fp64", "fp64", 4) is None
    assert bench.profiled_traffic("no-such-workload", "fp64", 1) is None


@pytest.mark.parametrize("argv,want", [
    (["bench.py"], False),
    (["bench.py", "--workload", "fd2d-256"], True),
    (["bench.py", "--workload", "batch-64"], True),
    (["bench.py", "--workload", "batch-64", "--autotune", "off"], False),
    (["bench.py", "--workload", "fd3d-256", "--autotune", "on"], True),
])
def test_autotune_selection(monkeypatch, argv, want):
    monkeypatch.setattr(sys, "argv", argv)
    assert bench.use_autotune(bench.parse()) is want


def test_reorth_bytes_and_flops():
    s = roofline.Sizes(n=1000, nnz=7000, R=1, m=10, d=2, C=8, k=0)
    base_b, base_f = roofline.fused_solve_bytes(s), roofline.fused_solve_flops(s)
    s1 = roofline.Sizes(n=1000, nnz=7000, R=1, m=10, d=2, C=8, k=0, reorth=1)
    s2 = roofline.Sizes(n=1000, nnz=7000, R=1, m=10, d=2, C=8, k=0, reorth=2)
    extra1 = roofline.fused_solve_bytes(s1) - base_b
    extra2 = roofline.fused_solve_bytes(s2) - base_b
    # CGS reads V_0..V_j twice per step: 2 * 8 * n * sum_j (j + 1), plus the w traffic
    assert extra1 == pytest.approx(sum(roofline.reorth_step_bytes(s1, j) for j in range(10)))
    assert extra1 > 2 * 8 * 1000 * sum(j + 1 for j in range(10))
    assert extra2 > 1.9 * extra1
    assert roofline.fused_solve_flops(s1) - base_f == pytest.approx(4.0 * 1000 * sum(j + 1 for j in range(10)))
