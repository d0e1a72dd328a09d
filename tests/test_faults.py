"""Host-side fault handling of the C ABI (no GPU): every entry point
validates its arguments before it touches a device and returns the
documented status, with a message in lsh_last_error."""
import copy
import ctypes

import numpy as np
import pytest

from landslidehysea_gb300._abi import (COORDS_SPHERICAL, FRICTION_POULIQUEN, LSH_ERR_INVALID, default_params)
from landslidehysea_gb300.solver import load


@pytest.fixture(scope="module")
def lib():
    from landslidehysea_gb300 import build as B
    B.build()
    return load()


def _bad_params():
    base = default_params(8, 6, dx=10.0, dy=10.0)
    cases = {}
    for name, kw in {
        "nx0": dict(nx=0), "ny_neg": dict(ny=-3), "order3": dict(order=3), "coords": dict(coords=7),
        "law": dict(friction_law=5), "eig_sort": dict(eig_sort=2), "r1": dict(r=1.0), "eps0": dict(eps_h=0.0),
        "cfl0": dict(cfl=0.0), "dx0": dict(dx=0.0), "H0": dict(H=0.0), "nan_g": dict(gravity=float("nan")),
        "huge": dict(nx=50000, ny=50000),
        "sph_lat": dict(coords=COORDS_SPHERICAL, dlon=0.01, dlat=0.01, lat0=89.99, radius=6.4e6),
        "sph_dlat0": dict(coords=COORDS_SPHERICAL, dlon=0.01, dlat=0.0, lat0=10.0, radius=6.4e6),
    }.items():
        p = copy.copy(base)
        for k, v in kw.items():
            setattr(p, k, v)
        cases[name] = p
    return cases


@pytest.mark.parametrize("name", list(_bad_params()))
def test_create_rejects_bad_parameters(lib, name):
    p = _bad_params()[name]
    ctx = ctypes.c_void_p()
    assert lib.lsh_create(ctypes.byref(p), 0, ctypes.byref(ctx)) == LSH_ERR_INVALID
    assert not ctx
    assert lib.lsh_last_error()


def test_batch_and_adjoint_reject_bad_input(lib):
    good = default_params(8, 6, dx=10.0, dy=10.0)
    bad = _bad_params()["r1"]
    arr = (type(good) * 2)(good, bad)
    b = ctypes.c_void_p()
    assert lib.lsh_batch_create(arr, 2, 0, ctypes.byref(b)) == LSH_ERR_INVALID
    assert b"scenario 1" in lib.lsh_last_error()
    o2 = copy.copy(good)
    o2.order = 2
    arr = (type(good) * 2)(good, o2)
    assert lib.lsh_batch_create(arr, 2, 0, ctypes.byref(b)) == LSH_ERR_INVALID  # mixed orders
    a = ctypes.c_void_p()
    pq = copy.copy(good)
    pq.friction_law = FRICTION_POULIQUEN
    assert lib.lsh_adjoint_create(ctypes.byref(pq), 0, 0, None, ctypes.byref(a)) == LSH_ERR_INVALID
    g = (ctypes.c_int * 1)(48)  # 8 x 6 grid: cell 48 does not exist
    assert lib.lsh_adjoint_create(ctypes.byref(good), 0, 1, g, ctypes.byref(a)) == LSH_ERR_INVALID
    assert lib.lsh_adjoint_create(ctypes.byref(good), 0, 1, None, ctypes.byref(a)) == LSH_ERR_INVALID


def test_adjoint_batch_rejects_bad_input(lib):
    good = default_params(8, 6, dx=10.0, dy=10.0)
    bad = _bad_params()["r1"]
    b = ctypes.c_void_p()
    arr = (type(good) * 2)(good, bad)
    assert lib.lsh_adjoint_batch_create(2, arr, None, None, 0, ctypes.byref(b)) == LSH_ERR_INVALID
    assert b"member 1" in lib.lsh_last_error()
    assert not b
    arr = (type(good) * 2)(good, good)
    ng = (ctypes.c_int * 2)(0, 1)
    assert lib.lsh_adjoint_batch_create(2, arr, ng, None, 0, ctypes.byref(b)) == LSH_ERR_INVALID
    assert lib.lsh_adjoint_batch_create(0, arr, None, None, 0, ctypes.byref(b)) == LSH_ERR_INVALID
    assert lib.lsh_adjoint_batch_forward(None, None, 3, None, None, None) == LSH_ERR_INVALID
    assert lib.lsh_adjoint_batch_gradient(None, None, None, None) == LSH_ERR_INVALID
    assert lib.lsh_adjoint_batch_set_budget(None, 1.0) == LSH_ERR_INVALID
    assert lib.lsh_adjoint_batch_destroy(None) == 0


def test_no_alloc_entry_rejects_oversize_and_second_order(lib):
    t, dt = ctypes.c_double(0.0), ctypes.c_double(0.1)
    fake = (ctypes.c_void_p * 7)(*([1] * 7))  # never dereferenced: rejected before any device work
    p = default_params(300, 300, dx=10.0, dy=10.0)  # 90,000 cells > 65,536
    assert lib.lsh_step_noalloc(ctypes.byref(p), fake, 1, ctypes.byref(t), ctypes.byref(dt), None) == LSH_ERR_INVALID
    p = default_params(1, 5000, dx=10.0, dy=10.0)  # 5000 rows > 4096
    assert lib.lsh_step_noalloc(ctypes.byref(p), fake, 1, ctypes.byref(t), ctypes.byref(dt), None) == LSH_ERR_INVALID
    p = default_params(16, 16, dx=10.0, dy=10.0, order=2)
    assert lib.lsh_step_noalloc(ctypes.byref(p), fake, 1, ctypes.byref(t), ctypes.byref(dt), None) == LSH_ERR_INVALID


def test_null_handles(lib):
    assert lib.lsh_step(None, 1) == LSH_ERR_INVALID
    assert lib.lsh_destroy(None) == 0
    assert lib.lsh_batch_step(None, 1) == LSH_ERR_INVALID
    assert lib.lsh_adjoint_gradient(None, 1.0, None, None, None) == LSH_ERR_INVALID
    assert lib.lsh_revolve_plan(0, 3, None, None) == LSH_ERR_INVALID
