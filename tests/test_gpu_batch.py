"""Batched ensemble (lsh_batch_*): scenarios of different sizes and
parameters advanced together must each be bit-identical to their own
single-grid run, before and after the autotuner changes the work-item tiling."""
import numpy as np
import pytest

from landslidehysea_gb300 import scenarios
from landslidehysea_gb300._abi import VARS

pytestmark = pytest.mark.gpu


def make(order):
    out = []
    for k, (n, ang, r) in enumerate([(40, 9.0, 0.5), (64, 15.0, 0.46), (33, 19.0, 0.58), (96, 11.0, 0.52)]):
        sc = scenarios.shelf(n=n, dx=25.0 * 200 / n, seed=k, angle_deg=ang, r=r, order=order,
                             cfl=0.5 if order == 2 else 0.9)
        out.append(sc)
    if order == 2:
        sc = scenarios.fjord(n=48, dcell_deg=0.008, seed=3)
        out.append(sc)
    return out


@pytest.mark.parametrize("order", [1, 2])
def test_batch_matches_single_grid(gpu_lib, order):
    from landslidehysea_gb300.solver import Batch, Solver
    scs = make(order)
    steps1, steps2 = 11, 9
    with Batch([sc.params for sc in scs]) as b:
        dts = [b.set_state(k, sc.state) for k, sc in enumerate(scs)]
        b.step(steps1)
        b.synchronize()
        mid = [b.get_state(k) for k in range(len(scs))]
        b.set_tune(ctas_per_sm=4, items_per_fetch=2)
        b.step(steps2)
        b.synchronize()
        fin = [b.get_state(k) for k in range(len(scs))]
        times = [b.time(k) for k in range(len(scs))]
        assert b.launch_count() > 0
    for k, sc in enumerate(scs):
        with Solver(sc.params) as s:
            assert s.set_state(sc.state) == dts[k]
            s.step(steps1)
            ref_mid = s.get_state()
            s.step(steps2)
            ref = s.get_state()
            t, dt, n = s.time()
        for v in VARS[:6]:
            assert np.array_equal(mid[k][v], ref_mid[v]), (k, v, "mid")
            assert np.array_equal(fin[k][v], ref[v]), (k, v)
        assert times[k] == (t, dt, n)


def test_batch_autotune_keeps_results(gpu_lib):
    from landslidehysea_gb300.solver import Batch, Solver
    scs = make(2)
    with Batch([sc.params for sc in scs]) as b:
        for k, sc in enumerate(scs):
            b.set_state(k, sc.state)
        best = b.autotune(trial_steps=2)
        assert best["ms_per_step"] > 0
        b.synchronize()
        steps = [b.time(k)[2] for k in range(len(scs))]
        out = [b.get_state(k) for k in range(len(scs))]
    assert len(set(steps)) == 1 and steps[0] > 0
    for k, sc in enumerate(scs):
        with Solver(sc.params) as s:
            s.set_state(sc.state)
            s.step(steps[0])
            ref = s.get_state()
        for v in VARS[:6]:
            assert np.array_equal(out[k][v], ref[v]), (k, v)
