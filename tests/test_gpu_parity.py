"""CUDA path (liblsh.so through the C ABI) against the FP64 CPU oracle.

Bar: every state field within 1e-10 relative L-infinity of the oracle after
N steps, time and next dt within 1e-10, and the wet/dry and granular
stop/move masks bit-identical.  By construction the two are in fact
bit-identical (both evaluate the same IEEE operation sequence: no implicit FMA
contraction on either side, shared elementary functions), which the tests
check too: a lost bit shows where the two codes part.
"""
import numpy as np
import pytest

from landslidehysea_gb300._abi import VARS

from gpu_cases import PARITY_CASES, case, rel_linf

pytestmark = pytest.mark.gpu

TOL = 1e-10


def run_both(oracle, name):
    from landslidehysea_gb300.solver import Solver
    p, st, steps = case(name)
    p.track_eta_max = 1
    arrs = [np.ascontiguousarray(st[v], dtype=np.float64).copy() for v in VARS]
    dt0_o = oracle.initial_dt(p, arrs)
    em = arrs[0] + arrs[3] - arrs[6]
    et = np.zeros_like(em)
    t_o, dt_o, _ = oracle.run(p, arrs, steps, dt=dt0_o, eta=(em, et))
    with Solver(p) as s:
        dt0_g = s.set_state(st)
        s.step(steps)
        s.synchronize()
        out = s.get_state()
        t_g, dt_g, n_g = s.time()
        masks_g = s.masks()
        em_g, et_g = s.eta_max()
        launches = s.launch_count()
    return dict(p=p, arrs=arrs, out=out, dt0=(dt0_o, dt0_g), t=(t_o, t_g), dt=(dt_o, dt_g), n=n_g, steps=steps,
                masks=(oracle.masks(p, arrs), masks_g), eta=(em, em_g, et, et_g), launches=launches)


@pytest.mark.parametrize("name", PARITY_CASES)
def test_parity(gpu_lib, oracle, name):
    r = run_both(oracle, name)
    assert r["n"] == r["steps"]
    assert abs(r["dt0"][0] - r["dt0"][1]) <= TOL * r["dt0"][0]
    assert abs(r["t"][0] - r["t"][1]) <= TOL * abs(r["t"][0])
    assert abs(r["dt"][0] - r["dt"][1]) <= TOL * r["dt"][0]
    for i, v in enumerate(VARS[:6]):
        e = rel_linf(r["out"][v], r["arrs"][i])
        assert e <= TOL, f"{name}: {v} rel Linf {e:.3e}"
    assert np.array_equal(r["masks"][0], r["masks"][1]), f"{name}: masks differ in {(r['masks'][0] != r['masks'][1]).sum()} cells"
    for i, v in enumerate(VARS[:6]):
        assert np.array_equal(r["out"][v], r["arrs"][i]), f"{name}: {v} not bit-identical"
    assert r["t"][0] == r["t"][1] and r["dt"][0] == r["dt"][1]
    em, em_g, et, et_g = r["eta"]
    assert rel_linf(em_g, em) <= TOL
    assert r["launches"] >= r["steps"] * (6 if r["p"].order == 1 else 13)


def test_config0_full(gpu_lib, oracle):
    """The 200 x 200 first-order shelf for 1000 steps, GPU vs oracle."""
    oracle.set_threads(0)
    r = run_both(oracle, "shelf200_o1")
    for i, v in enumerate(VARS[:6]):
        e = rel_linf(r["out"][v], r["arrs"][i])
        assert e <= TOL, f"{v} rel Linf {e:.3e}"
    assert np.array_equal(r["masks"][0], r["masks"][1])
    assert abs(r["t"][0] - r["t"][1]) <= TOL * r["t"][0]


def test_run_until_matches_oracle(gpu_lib, oracle):
    from landslidehysea_gb300.solver import Solver
    p, st, _ = case("golden_dam1d")
    arrs = [np.ascontiguousarray(st[v], dtype=np.float64).copy() for v in VARS]
    t_end = 0.35
    t_o, dt_o, n_o = oracle.run(p, arrs, 0, t_end=t_end)
    with Solver(p) as s:
        s.set_state(st)
        n_g = s.run_until(t_end)
        t_g, dt_g, _ = s.time()
        out = s.get_state()
    assert n_g == n_o
    assert abs(t_g - t_o) <= TOL * t_o
    for i, v in enumerate(VARS[:6]):
        assert rel_linf(out[v], arrs[i]) <= TOL
