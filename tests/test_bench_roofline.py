"""The bench's roofline record: the committed ncu traffic table covers every kernel the record names, and
the FP64 flop count of the benchmark stencil is the one the design states."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_traffic_table_covers_the_timed_kernels():
    t = bench.read_ncu_traffic()
    for pair in ("k_fx_split + k_predict_fx", "k_correct_fx", "k_predict", "k_correct"):
        for k in pair.split(" + "):
            assert k in t and 0 < t[k] < 400, (k, t.get(k))


def test_fp64_flops_of_the_benchmark_stencil():
    assert bench.fp64_flops_per_spin_step(26) == 1109
