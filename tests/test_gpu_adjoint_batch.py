"""The batched adjoint on the GPU (lsh_adjoint_batch_*): scenarios of
different sizes and schemes, run forward and reversed under one checkpoint
schedule with a joint budget, give each member's misfit, gauge series and
gradient bit for bit as an Adjoint of its own with the same slot count."""
import numpy as np
import pytest

from adj_cases import copy_arrs, scenario_case, smooth_case
from landslidehysea_gb300._abi import VARS

pytestmark = pytest.mark.gpu
pyoracle = pytest.importorskip("pyoracle")


def _members():
    return [smooth_case(order=2), scenario_case("fjord", 2), scenario_case("shelf", 1), smooth_case(nx=23, ny=9, order=1)]


def _target(p, arrs, gauges, n, seed):
    _, _, eta = pyoracle.misfit_run(p, copy_arrs(arrs), n, gauges=gauges)
    return eta + 0.01 * np.random.default_rng(seed).standard_normal(eta.shape)


def _state(p, arrs):
    return {v: arrs[i].reshape(p.ny, p.nx) for i, v in enumerate(VARS)}


def _slot_bytes(p):
    return 6 * 8 * ((p.nx * p.ny + 31) // 32 * 32)


def _single(p, arrs, gauges, n, tgt, slots, h_adj=0.0, weight=1.0):
    from landslidehysea_gb300.solver import Adjoint
    with Adjoint(p, gauges) as A:
        A.set_budget(slots * _slot_bytes(p) + 1.0)
        if h_adj:
            A.set_thin_layer(h_adj)
        J, eta = A.forward(_state(p, arrs), n, tgt)
        g, gp = A.gradient(weight)
        assert A.stats()["slots"] == slots
    return J, eta, g, gp


@pytest.mark.parametrize("slots,h_adj", [(3, 0.0), (1, 0.0), (4, 0.05)])
def test_batch_members_equal_their_own_adjoints(gpu_lib, slots, h_adj):
    from landslidehysea_gb300.solver import AdjointBatch, revolve_plan
    mem = _members()
    n = 13
    tg = [_target(p, a, g, n, seed=3 + i) for i, (p, a, g) in enumerate(mem)]
    weights = [1.0, 0.5, 2.0, 1.0]
    with AdjointBatch([m[0] for m in mem], [m[2] for m in mem]) as B:
        B.set_budget(slots * sum(_slot_bytes(m[0]) for m in mem) + 1.0)
        if h_adj:
            B.set_thin_layer(h_adj)
        J, series = B.forward([_state(p, a) for p, a, _ in mem], n, tg)
        grads, gps = B.gradient(weights)
        st = B.stats()
    assert st["slots"] == slots and st["nsteps"] == n and st["reversed_steps"] == n
    fw, _ = revolve_plan(n, slots)
    assert st["recompute_steps"] <= fw
    for i, (p, a, g) in enumerate(mem):
        J1, eta1, g1, gp1 = _single(p, a, g, n, tg[i], slots, h_adj, weights[i])
        assert J[i] == J1, i
        assert np.array_equal(series[i], eta1), i
        for v in VARS[:6]:
            assert np.array_equal(grads[i][v], g1[v]), (i, v)
        assert gps[i] == gp1, i
        assert any(np.any(grads[i][v] != 0.0) for v in VARS[:6]), i


def test_batch_second_gradient_and_member_runs(gpu_lib):
    from landslidehysea_gb300.solver import AdjointBatch, LshError
    mem = _members()[:2]
    n = 9
    tg = [_target(p, a, g, n, seed=11 + i) for i, (p, a, g) in enumerate(mem)]
    with AdjointBatch([m[0] for m in mem], [m[2] for m in mem]) as B:
        B.set_budget(2 * sum(_slot_bytes(m[0]) for m in mem) + 1.0)
        B.forward([_state(p, a) for p, a, _ in mem], n, tg)
        ga, pa = B.gradient()
        gb, pb = B.gradient()  # the same recorded run, slots reused
        for i in range(2):
            for v in VARS[:6]:
                assert np.array_equal(ga[i][v], gb[i][v])
        assert pa == pb
        # member 1 on its own keeps the batch's slot count and its results
        m1 = B.member(1)
        p, a, g = mem[1]
        m1.forward(_state(p, a), n, tg[1])
        assert m1.stats()["slots"] == 2
        # the members' records now stand at different points of the schedule
        with pytest.raises(LshError):
            B.gradient()
        g1, p1 = m1.gradient()
        for v in VARS[:6]:
            assert np.array_equal(g1[v], ga[1][v])
        assert p1 == pa[1]
