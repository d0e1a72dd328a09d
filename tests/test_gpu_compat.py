"""The reference-signature entry point shallowWater() (ShallowWater.cu:125)
on a data.dat problem: final state, NetCDF snapshots and gauge series
against the FP64 oracle driven through the reference's loop
(ShallowWater.cu:266-461: snapshot when t >= next save time, then step,
until t >= tiempo_tot)."""
import numpy as np
import pytest

from landslidehysea_gb300 import io
from landslidehysea_gb300._abi import VARS

from datafiles import write_case

pytestmark = pytest.mark.gpu


def f32(x):
    return float(np.float32(x))


def float_params(p):
    """shallowWater() takes its parameters as float (main.cxx:157-164 casts
    every one); the replay must use the same rounded values."""
    q = p.copy()
    for name, typ in q._fields_:
        if typ.__name__ == "c_double":
            setattr(q, name, f32(getattr(q, name)))
    return q


def oracle_replay(oracle, pr):
    """Replay the reference loop on the oracle; returns the snapshot states
    (with their times), the final state and the eta1 max (as float32 after
    the shim's float conversion of the input)."""
    p = float_params(pr.params)
    p.radius = pr.params.radius
    st = {v: pr.state[v].astype(np.float32).astype(np.float64) for v in VARS}
    arrs = oracle.state_arrays(st)
    em = arrs[0] + arrs[3] - arrs[6]
    et = np.zeros_like(em)
    t, dt = 0.0, oracle.initial_dt(p, arrs)
    nxt = 0.0
    snaps = []
    t_tot, t_save = f32(pr.tiempo_tot), f32(pr.tiempo_guardar)
    while t < t_tot:
        if t_save >= 0 and t >= nxt:
            snaps.append((t, [a.copy() for a in arrs]))
            nxt += t_save
        t, dt, _ = oracle.run(p, arrs, 1, t=t, dt=dt, eta=(em, et))
    return snaps, arrs, em, et


@pytest.mark.parametrize("gauges", [False, True])
def test_shallow_water_entry_point(gpu_lib, oracle, tmp_path, monkeypatch, gauges):
    monkeypatch.chdir(tmp_path)
    (tmp_path / "out").mkdir()
    if gauges:
        (tmp_path / "g.txt").write_text("2\n60 45\n270 139\n")
        write_case(tmp_path, normalizar=0, extra_gauge_file="g.txt")
    else:
        write_case(tmp_path, normalizar=1)
    pr = io.LoadedProblem(str(tmp_path / "data.dat"))
    status, wall, out, eta = io.shallow_water(pr)
    assert status == 0
    snaps, arrs, em, et = oracle_replay(oracle, pr)
    for k, v in enumerate(VARS[:6]):
        assert np.array_equal(out[v], arrs[k].astype(np.float32)), v
    assert np.array_equal(eta[..., 0], em.astype(np.float32))
    H, Q, T, hmin = f32(pr.params.H), f32(pr.Q), f32(pr.T), f32(pr.hmin)
    if not gauges:
        from scipy.io import netcdf_file
        with netcdf_file(str(tmp_path / "out" / "run1_eta1.nc"), "r", mmap=False) as d:
            times = d.variables["time"][:]
            assert len(times) == len(snaps)
            assert np.allclose(times, [s[0] * T for s in snaps], rtol=1e-6)
            for r, (t, a) in enumerate(snaps):
                want = ((a[0] + a[3] - a[6] - hmin) * H).astype(np.float32)
                assert np.array_equal(d.variables["eta1"][r], want)
            assert np.array_equal(d.variables["max_height"][:], ((em - hmin) * H).astype(np.float32))
            assert np.array_equal(d.variables["bathymetry"][:],
                                  ((pr.state["H"].astype(np.float32).astype(np.float64) + hmin) * H).astype(np.float32))
        with netcdf_file(str(tmp_path / "out" / "run1_q2y.nc"), "r", mmap=False) as d:
            assert np.array_equal(d.variables["q2y"][-1], (snaps[-1][1][5] * Q).astype(np.float32))
    else:
        lines = (tmp_path / "out" / "run1_eta_puntos.txt").read_text().splitlines()
        assert len(lines) == len(snaps)
        for line, (t, a) in zip(lines, snaps):
            vals = [float(v) for v in line.split()]
            assert vals[0] == pytest.approx(t * T, rel=1e-6)
            for gi, c in enumerate(pr.gauges):
                want = (a[0].ravel()[c] - a[6].ravel()[c] - hmin) * H
                assert vals[1 + gi] == pytest.approx(want, rel=1e-7, abs=1e-12)


def test_gauge_gather_equals_the_state(gpu_lib):
    """lsh_get_gauge_eta gathers h1 - H at the gauge cells on the device: the
    same bits as the downloaded state, NaN off the grid, and a changed cell
    list is taken up."""
    from landslidehysea_gb300 import scenarios
    from landslidehysea_gb300.solver import Solver
    sc = scenarios.fjord(n=48, dcell_deg=0.008, seed=2)
    n = sc.nx * sc.ny
    cells = np.array([0, 5, n // 2, n - 1, -3, n + 7], dtype=np.int32)
    with Solver(sc.params) as s:
        s.set_state(sc.state)
        for k, steps in enumerate((0, 7, 3)):
            s.step(steps)
            s.synchronize()
            if k == 2:
                cells = cells[::-1].copy()
            got = s.gauge_eta(cells)
            st = s.get_state()
            ref = (st["h1"] - st["H"]).reshape(-1)
            for c, g in zip(cells, got):
                if 0 <= c < n:
                    assert g == ref[c], (k, c)
                else:
                    assert np.isnan(g), (k, c)
        assert s.gauge_eta(np.zeros(0, dtype=np.int32)).size == 0
