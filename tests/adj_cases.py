"""Smooth two-layer cases for derivative checks: water and granular layers
everywhere (no dry cell, no empty granular layer), moving layers (no
Coulomb stop), so the forward map is differentiable around the state and
central finite differences converge.  Kinks (h = 0, stopped layers) are
points where only one-sided derivatives exist; the dry-front cases of the
real configurations are covered by the adjoint-vs-tangent-linear identity,
which needs no smoothness."""
import math

import numpy as np

from landslidehysea_gb300._abi import COORDS_SPHERICAL, VARS, default_params


def smooth_case(nx=18, ny=14, order=1, seed=0, walls=True, spherical=False, angle_deg=4.0):
    rng = np.random.default_rng(seed)
    dx = 40.0
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y)
    ph = rng.uniform(0, 2 * math.pi, 4)
    d = 40.0 + 8.0 * np.sin(2 * math.pi * X + ph[0]) * np.cos(math.pi * Y + ph[1])
    h2 = 1.5 + 2.5 * np.exp(-((X - 0.45) ** 2 + (Y - 0.5) ** 2) / 0.05)
    h1 = d - h2 + 0.3 * np.sin(3 * X + 2 * Y + ph[2])  # eta1 varies in x and y: no flat minmod
    q1x = h1 * (0.4 + 0.1 * np.cos(2 * Y + ph[3]))
    q1y = h1 * (-0.25 + 0.1 * np.sin(2 * X))
    q2x = h2 * (0.9 + 0.2 * np.sin(3 * Y))
    q2y = h2 * (0.5 + 0.2 * np.cos(2 * X))
    kw = dict(order=order, cfl=0.45, r=0.52, angle_deg=angle_deg, mf0=0.025, mfs=0.03, mfc=0.0, eps_h=1e-5,
              gravity=9.81)
    b = -1.0 if walls else 1.0
    kw.update(borde_sup=b, borde_inf=b, borde_izq=b, borde_der=b)
    if spherical:
        kw.update(coords=COORDS_SPHERICAL, dlon=0.0006, dlat=0.0003, lon0=10.0, lat0=60.0, radius=6378136.6)
    else:
        kw.update(dx=dx, dy=dx)
    p = default_params(nx, ny, **kw)
    state = {"h1": h1, "q1x": q1x, "q1y": q1y, "h2": h2, "q2x": q2x, "q2y": q2y, "H": d}
    arrs = [np.ascontiguousarray(state[v], dtype=np.float64).reshape(-1).copy() for v in VARS]
    gauges = np.array([(ny // 2) * nx + nx // 3, (ny // 3) * nx + (2 * nx) // 3, (2 * ny // 3) * nx + nx // 2],
                      dtype=np.int32)
    return p, arrs, gauges


def smooth_direction(nx, ny, seed, which=(3,)):
    """A smooth perturbation field for the state variables in `which`."""
    rng = np.random.default_rng(100 + seed)
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y)
    out = [None] * 6
    for k in which:
        a = rng.uniform(0.5, 1.5, 3)
        out[k] = (a[0] * np.sin(2 * math.pi * X * a[1]) * np.cos(math.pi * Y * a[2]) + 0.3).reshape(-1).copy()
    return out


def copy_arrs(arrs):
    return [a.copy() for a in arrs]


# ---------------------------------------------------------------- native test harnesses
import ctypes  # noqa: E402
import os  # noqa: E402
import subprocess  # noqa: E402

_HERE = os.path.dirname(os.path.abspath(__file__))
_NATIVE = os.path.join(_HERE, "native")
_CSRC = os.path.join(os.path.dirname(_HERE), "landslidehysea_gb300", "csrc")
_libs = {}


def native_lib(name):
    """Compile tests/native/<name>.cpp (host code including the product's
    scheme and adjoint headers) into tests/native/_build/ and load it."""
    if name in _libs:
        return _libs[name]
    src = os.path.join(_NATIVE, name + ".cpp")
    out = os.path.join(_NATIVE, "_build", name + ".so")
    deps = [src] + [os.path.join(_CSRC, f) for f in os.listdir(_CSRC) if f.endswith((".h", ".cuh"))]
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(f) for f in deps):
        os.makedirs(os.path.dirname(out), exist_ok=True)
        subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", out + ".tmp"],
                       check=True)
        os.replace(out + ".tmp", out)
    lib = ctypes.CDLL(out)
    P = ctypes.c_void_p
    D = ctypes.POINTER(ctypes.c_double)
    if name == "adj_local":
        for f in ("adjl_edge", "adjl_volume"):
            getattr(lib, f).restype = ctypes.c_double
            getattr(lib, f).argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int, D, D]
        lib.adjl_initial_wave.restype = ctypes.c_double
        lib.adjl_initial_wave.argtypes = [ctypes.c_uint64, ctypes.c_int, D, D]
        lib.adjl_set_component.argtypes = [ctypes.c_int]
        lib.adjl_set_bor.argtypes = [ctypes.c_double]
        lib.adjl_initial_wave_empty.restype = ctypes.c_int
    elif name == "cmp_check":
        lib.cmpc_check.restype = ctypes.c_longlong
        lib.cmpc_check.argtypes = [P, ctypes.c_longlong]
    elif name == "adj_host":
        lib.adjh_run.argtypes = [P, P, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_double, P, D, P, P, ctypes.c_double]
        lib.adjh_recon_check.restype = ctypes.c_longlong
        lib.adjh_recon_check.argtypes = [P, P]
    _libs[name] = lib
    return lib


def _ptrs(arrs):
    return (ctypes.c_void_p * len(arrs))(*[a.ctypes.data if a is not None else None for a in arrs])


def host_adjoint(p, arrs, nsteps, gauges, target, wj=1.0, wfin=None, h_adj=0.0):
    """Gradient of wj * J + <wfin, X_N> by the host emulation of the adjoint
    sweep (the product's per-edge / per-cell adjoint bodies in loops).
    Returns (J, grad[6], grad_params[4] = d/d(angle1, mf0, mfs, r))."""
    lib = native_lib("adj_host")
    N = arrs[0].size
    grad = [np.zeros(N) for _ in range(6)]
    gpar = np.zeros(4)
    J = ctypes.c_double()
    g = np.ascontiguousarray(gauges, dtype=np.int32)
    t = None if target is None else np.ascontiguousarray(target, dtype=np.float64)
    lib.adjh_run(ctypes.byref(p), _ptrs(arrs), int(nsteps), len(g), g.ctypes.data, t.ctypes.data if t is not None else None,
                 float(wj), _ptrs(wfin) if wfin is not None else None, ctypes.byref(J), _ptrs(grad), gpar.ctypes.data,
                 float(h_adj))
    return J.value, grad, gpar


def scenario_case(kind, order, seed=1):
    """A realistic small case (dry land, granular front, resting slide)."""
    from landslidehysea_gb300 import scenarios
    if kind == "shelf":
        sc = scenarios.shelf(n=32, dx=25 * 200 / 32, seed=seed, order=order, cfl=0.5 if order == 2 else 0.9)
    else:
        sc = scenarios.fjord(n=40, dcell_deg=0.008, seed=seed, order=order)
    arrs = [np.ascontiguousarray(sc.state[v], dtype=np.float64).reshape(-1).copy() for v in VARS]
    rng = np.random.default_rng(seed)
    wet = np.where(arrs[0] > 0)[0]
    gauges = np.sort(rng.choice(wet, 4, replace=False)).astype(np.int32)
    return sc.params, arrs, gauges


def wet_direction(arrs, which, seed):
    """Random direction on the wet cells of the variables in `which`."""
    rng = np.random.default_rng(500 + seed)
    wet = (arrs[0] > 0) | (arrs[3] > 0)
    out = [None] * 6
    for k in which:
        m = (arrs[3] > 0) if k in (3, 4, 5) else wet
        out[k] = rng.standard_normal(arrs[0].size) * m
    return out
