"""The batched paths against the FP64 oracle directly.

The batched ensemble (lsh_batch_*) and the batched adjoint
(lsh_adjoint_batch_*) share their per-edge and per-cell device code with the
single-grid path, so a test that compares them only with the single-grid GPU
path would pass on a bug common to both.  Here each member is compared with
the oracle:
  * ensemble members of uneven grids (Cartesian and spherical, both orders)
    after each of two runs of steps, with a work-item tiling change between
    them: every state field, t, dt and the step count bit-identical to
    pyoracle.run (each member reproduces the reference's single-grid loop,
    ShallowWater.cu:266-461);
  * batched-adjoint members (orders 1 and 2, Cartesian and spherical): the
    misfit and gauge series bit-identical to the oracle's misfit run, and
    <grad J, v> + <dJ/dtheta, w> equal to the oracle's tangent-linear dJ.v
    to 1e-10 for state and parameter directions.
"""
import numpy as np
import pytest

from adj_cases import copy_arrs, scenario_case, smooth_case, smooth_direction, wet_direction
from landslidehysea_gb300 import scenarios
from landslidehysea_gb300._abi import VARS

pytestmark = pytest.mark.gpu
pyoracle = pytest.importorskip("pyoracle")

TOL = 1e-10


def _ensemble(order):
    cfl = 0.5 if order == 2 else 0.9
    return [scenarios.shelf(n=40, dx=125.0, seed=0, angle_deg=9.0, r=0.5, order=order, cfl=cfl),
            scenarios.shelf(nx=57, ny=23, dx=110.0, seed=1, angle_deg=15.0, r=0.46, order=order, cfl=cfl),
            scenarios.shelf(nx=19, ny=70, dx=90.0, seed=2, angle_deg=19.0, r=0.58, order=order, cfl=cfl),
            scenarios.fjord(n=48, dcell_deg=0.008, seed=3, order=order)]


@pytest.mark.parametrize("order", [1, 2])
def test_ensemble_members_equal_the_oracle(gpu_lib, order):
    from landslidehysea_gb300.solver import Batch
    scs = _ensemble(order)
    assert len({(sc.nx, sc.ny) for sc in scs}) == len(scs)
    steps = (12, 7)
    with Batch([sc.params for sc in scs]) as b:
        dt0 = [b.set_state(k, sc.state) for k, sc in enumerate(scs)]
        got = []
        for i, n in enumerate(steps):
            if i == 1:
                b.set_tune(ctas_per_sm=3, items_per_fetch=4)
            b.step(n)
            b.synchronize()
            got.append(([b.get_state(k) for k in range(len(scs))], [b.time(k) for k in range(len(scs))]))
    for k, sc in enumerate(scs):
        p = sc.params
        arrs = pyoracle.state_arrays(sc.state)
        dt = pyoracle.initial_dt(p, arrs)
        assert dt0[k] == dt, (k, "initial dt")
        t, done = 0.0, 0
        for i, n in enumerate(steps):
            t, dt, nd = pyoracle.run(p, arrs, n, t=t, dt=dt)
            done += nd
            states, times = got[i]
            assert times[k] == (t, dt, done), (k, i, times[k], (t, dt, done))
            for j, v in enumerate(VARS[:6]):
                assert np.array_equal(states[k][v], arrs[j]), f"member {k} ({sc.nx}x{sc.ny}) {v} after run {i}"
        assert any(np.any(arrs[j] != sc.state[v]) for j, v in enumerate(VARS[:6])), k


def _state(p, arrs):
    return {v: arrs[i].reshape(p.ny, p.nx) for i, v in enumerate(VARS)}


def _slot_bytes(p):
    return 6 * 8 * ((p.nx * p.ny + 31) // 32 * 32)


def test_batched_adjoint_members_equal_the_tangent_linear(gpu_lib):
    from landslidehysea_gb300.solver import AdjointBatch
    mem = [("smooth", smooth_case(order=2, spherical=True)), ("fjord", scenario_case("fjord", 2)),
           ("shelf", scenario_case("shelf", 1)), ("smooth", smooth_case(nx=23, ny=9, order=1))]
    n = 6
    tg = []
    for i, (_, (p, a, g)) in enumerate(mem):
        _, _, eta = pyoracle.misfit_run(p, copy_arrs(a), n, gauges=g)
        tg.append(eta + 0.01 * np.random.default_rng(40 + i).standard_normal(eta.shape))
    with AdjointBatch([m[1][0] for m in mem], [m[1][2] for m in mem]) as B:
        B.set_budget(2 * sum(_slot_bytes(m[1][0]) for m in mem) + 1.0)
        J, series = B.forward([_state(p, a) for _, (p, a, _) in mem], n, tg)
        grads, gps = B.gradient()
    for i, (kind, (p, a, g)) in enumerate(mem):
        Jo, _, eta_o = pyoracle.misfit_run(p, copy_arrs(a), n, gauges=g, target=tg[i])
        assert J[i] == Jo and np.array_equal(series[i], eta_o), i
        grad = [grads[i][v].reshape(-1) for v in VARS[:6]]
        gpar = np.array([gps[i][k] for k in ("angle1", "mf0", "mfs", "r")])
        dirs = [(smooth_direction(p.nx, p.ny, 7, which=w) if kind == "smooth" else wet_direction(a, w, 7),
                 [0, 0, 0, 0]) for w in ((3,), (0, 1, 2), (4, 5))]
        dirs += [([None] * 6, [0.2, -0.1, 0.3, 0.4])]
        for d, dpar in dirs:
            dd = [None if x is None else x.copy() for x in d]
            _, dJ, _, _ = pyoracle.tl_run(p, copy_arrs(a), dd, dpar, n, gauges=g, target=tg[i])
            ad = sum(float(np.dot(grad[k], d[k])) for k in range(6) if d[k] is not None) + float(np.dot(gpar, dpar))
            assert dJ != 0.0, (i, dpar)
            assert abs(ad - dJ) <= TOL * abs(dJ), (i, kind, dpar, ad, dJ)
