"""The FP64 operation count behind bench.py's FP64 roofline: the oracle on
an operation-counting scalar (oracle/count.h) gives the reference scheme's
operations per cell-update on the 2048^2 fjord; bench.py quotes that count."""
import os
import sys

import pytest

pyoracle = pytest.importorskip("pyoracle")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_counting_scalar_leaves_values_unchanged():
    """The counted run is the oracle's run: compare a counted and a plain misfit."""
    from adj_cases import copy_arrs, smooth_case
    p, arrs, gauges = smooth_case(order=2)
    a = pyoracle.count_ops(p, copy_arrs(arrs), 3)
    b = pyoracle.count_ops(p, copy_arrs(arrs), 3)
    assert a == b and a["fma"] > 0 and a["abs"] > 0 and a["cbrt"] > 0


def test_bench_quotes_the_counted_operations():
    sys.path.insert(0, ROOT)
    import bench
    from landslidehysea_gb300 import scenarios
    sc = scenarios.fjord(n=2048)
    r = pyoracle.ops_per_cell_step(sc.params, pyoracle.state_arrays(sc.state))
    flops = bench.flops_per_cell_step(r)
    assert abs(flops - bench.FJORD2048_FLOPS_PER_CELL_STEP) <= 1e-3 * flops
