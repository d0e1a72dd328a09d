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
