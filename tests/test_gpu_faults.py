"""Failures reported without faulting the GPU: a NaN in the input, the dt
stall guard, a grid too large for device memory, an empty checkpoint budget,
and the bounded waits between passes running out.  Each returns its status and
leaves the context usable."""
import copy

import numpy as np
import pytest

from landslidehysea_gb300 import scenarios
from landslidehysea_gb300._abi import (LSH_ERR_GPU_OOM, LSH_ERR_INVALID, LSH_ERR_NUMERIC, LSH_ERR_STALL,
                                       LSH_ERR_TIMEOUT, default_params)
from landslidehysea_gb300.solver import LshError

pytestmark = pytest.mark.gpu


def test_nan_in_the_input_is_reported(gpu_lib):
    from landslidehysea_gb300.solver import Solver
    sc = scenarios.shelf(n=24, dx=200.0)
    st = {k: v.copy() for k, v in sc.state.items()}
    st["q1x"][12, 12] = np.nan
    with Solver(sc.params) as s:
        s.set_state(st)
        s.step(5)
        with pytest.raises(LshError) as e:
            s.synchronize()
        assert e.value.status == LSH_ERR_NUMERIC
        # the context is still usable: a clean state steps again
        s.set_state(sc.state)
        s.step(3)
        s.synchronize()
        assert s.time()[2] == 3


def test_stall_guard(gpu_lib):
    from landslidehysea_gb300.solver import Solver
    sc = scenarios.shelf(n=24, dx=200.0)
    p = copy.copy(sc.params)
    p.dt_min = 1e6  # any dt is below it
    with Solver(p) as s:
        s.set_state(sc.state)
        s.step(4)
        with pytest.raises(LshError) as e:
            s.synchronize()
        assert e.value.status == LSH_ERR_STALL
        assert s.time()[2] == 1  # stopped after the step that produced the small dt


def test_grid_too_large_for_device_memory(gpu_lib):
    import ctypes
    p = default_params(46000, 46000, dx=10.0, dy=10.0)  # 2.1e9 cells, ~630 GB: valid, but too large
    ctx = ctypes.c_void_p()
    assert gpu_lib.lsh_create(ctypes.byref(p), 0, ctypes.byref(ctx)) == LSH_ERR_GPU_OOM
    assert not ctx


def test_adjoint_budget_without_room(gpu_lib):
    from landslidehysea_gb300.solver import Adjoint
    sc = scenarios.shelf(n=16, dx=300.0)
    with Adjoint(sc.params, [5]) as A:
        A.set_budget(0.0)
        with pytest.raises(LshError) as e:
            A.forward(sc.state, 3)
        assert e.value.status == LSH_ERR_INVALID
        A.set_budget(1e9)
        J, eta = A.forward(sc.state, 3)
        assert eta.shape == (3, 1)


def test_bounded_waits_give_up_and_report(gpu_lib):
    """The overlapped step's and the work queue's waits, on counters that
    nothing increments, give up after their ~2 s bounds and report
    LSH_ERR_TIMEOUT; the device keeps working."""
    from landslidehysea_gb300.solver import Solver, probe_wait_bound
    status, ms = probe_wait_bound(0)
    assert status == LSH_ERR_TIMEOUT
    assert 3000.0 < ms < 20000.0  # two waits of about 2 s each
    sc = scenarios.shelf(n=24, dx=200.0)
    with Solver(sc.params) as s:
        s.set_state(sc.state)
        s.step(3)
        s.synchronize()
        assert s.time()[2] == 3
