"""Host-side input and output of the drop-in surface (no GPU):
the data.dat / .bat / .ini loader with the reference's istream semantics
(src/GPU/Problema.cxx:139-549) and the NetCDF-classic files of
src/GPU/netcdf.cu, read back with scipy's independent NetCDF reader."""
import math
import os

import numpy as np
import pytest

from landslidehysea_gb300 import io
from landslidehysea_gb300._abi import LSH_ERR_IO

from datafiles import write_case

scipy_io = pytest.importorskip("scipy.io")


def test_loader_istream_quirk_and_normalisation(tmp_path):
    depth, h1, h2, q = write_case(tmp_path)
    pr = io.LoadedProblem(str(tmp_path / "data.dat"))
    p = pr.params
    assert (p.nx, p.ny) == (6, 4)
    assert pr.leer_fichero_puntos == 0
    assert p.cfl == pytest.approx(0.85)       # ".85" left in the stream by the int read
    assert p.r == pytest.approx(0.45)
    assert p.angle1 == pytest.approx(math.radians(11.0))
    L, H = 1000.0, 100.0
    Q = math.sqrt(9.81 * H ** 3)
    T = L * H / Q
    assert pr.Q == pytest.approx(Q) and pr.T == pytest.approx(T)
    assert p.gravity == 1.0 and p.L == L and p.H == H
    assert p.eps_h == pytest.approx(5e-3 / H)
    assert pr.tiempo_tot == pytest.approx(12.5 / T) and pr.tiempo_guardar == pytest.approx(2.0 / T)
    assert p.mfc == pytest.approx(0.01 * L)
    fac = (Q / H) * math.sqrt(L) / H ** (7.0 / 6.0)
    assert p.mf0 == pytest.approx(0.02 * fac) and p.mfs == pytest.approx(0.03 * fac)
    assert p.vmax1 == pytest.approx(15 / (Q / H)) and p.vmax2 == pytest.approx(25 / (Q / H))
    assert p.dx == pytest.approx(50.0 / L) and p.dy == pytest.approx(40.0 / L)
    assert (p.borde_sup, p.borde_inf, p.borde_izq, p.borde_der) == (-1.0, 1.0, 0.0, 1.0)
    hmin = np.round(depth, 6).min() / H
    assert pr.hmin == pytest.approx(hmin)
    assert np.allclose(pr.state["H"], np.round(depth, 6) / H - hmin, rtol=0, atol=1e-12)
    assert np.allclose(pr.state["h1"], np.round(h1, 6) / H, atol=1e-12)
    assert np.allclose(pr.state["q2y"], np.round(q[3], 6) / Q, atol=1e-12)
    assert np.allclose(pr.eta1_max, pr.state["h1"] + pr.state["h2"] - pr.state["H"])
    assert pr.prefijo == "out/run1" and pr.nombre_bati == "my_bathymetry"


def test_loader_gauges_nearest_cell(tmp_path):
    # the third point lies past the last cell centre: outside, as in
    # obtenerIndicePunto (no centre >= the point)
    (tmp_path / "gauges.txt").write_text("3\n60 45\n270 139\n290 5\n")
    write_case(tmp_path, normalizar=0, extra_gauge_file="gauges.txt")
    pr = io.LoadedProblem(str(tmp_path / "data.dat"))
    assert pr.leer_fichero_puntos == 1
    assert pr.params.cfl == pytest.approx(0.8)
    # cell centres x = 25, 75, ..., 275; y = 20, 60, 100, 140
    assert list(pr.gauges) == [1 * 6 + 1, 3 * 6 + 5, -1]
    assert pr.params.gravity == pytest.approx(9.81)


def test_loader_errors(tmp_path):
    with pytest.raises(Exception) as e:
        io.LoadedProblem(str(tmp_path / "missing.dat"))
    assert getattr(e.value, "status", None) == LSH_ERR_IO
    write_case(tmp_path)
    (tmp_path / "state.ini").write_text("1 2 3\n")
    with pytest.raises(Exception) as e:
        io.LoadedProblem(str(tmp_path / "data.dat"))
    assert getattr(e.value, "status", None) == LSH_ERR_IO


def test_netcdf_layout_roundtrip(tmp_path):
    nx, ny = 5, 3
    x = np.arange(nx) * 10.0 + 5.0
    y = np.arange(ny) * 20.0 + 10.0
    bati = np.arange(nx * ny, dtype=np.float32).reshape(ny, nx) + 100
    nc = io.NcOutput(str(tmp_path / "res"), "bati_name", x, y, bati, tiempo_tot=60.0, cfl=0.9, r=0.5,
                     angles_deg=(12.0, 0, 0, 0), mf0=0.03)
    fields = []
    for rec in range(3):
        f = [np.full((ny, nx), 10 * rec + k, np.float32) + np.arange(nx)[None, :] for k in range(6)]
        nc.write(1.5 * rec, *f)
        fields.append(f)
    mh = np.random.default_rng(1).uniform(size=(ny, nx)).astype(np.float32)
    nc.close(mh)
    names = ["eta1", "q1x", "q1y", "eta2", "q2x", "q2y"]
    for k, nm in enumerate(names):
        path = tmp_path / f"res_{nm}.nc"
        assert path.exists()
        with scipy_io.netcdf_file(str(path), "r", mmap=False) as d:
            assert d.version_byte == 1
            assert d.dimensions["lon"] == nx and d.dimensions["lat"] == ny and d.dimensions["time"] is None
            assert np.allclose(d.variables["lon"][:], x) and np.allclose(d.variables["lat"][:], y)
            assert np.allclose(d.variables["time"][:], [0.0, 1.5, 3.0])
            v = d.variables[nm]
            assert v.dimensions == ("time", "lat", "lon")
            assert v.shape == (3, ny, nx)
            for rec in range(3):
                assert np.array_equal(v[rec], fields[rec][k])
            assert float(v._FillValue) == pytest.approx(-1e30)
            assert d.friction_law == b"Coulomb"
            assert float(d.CFL) == pytest.approx(0.9)
            if k == 0:
                assert np.array_equal(d.variables["bathymetry"][:], bati)
                assert d.variables["bathymetry"].dimensions == ("grid_y", "grid_x")
                assert np.array_equal(d.variables["max_height"][:], mh)
                assert np.allclose(d.variables["grid_x"][:], x)
