"""Make the golden fixtures in tests/golden/ from the REFERENCE's own FP32
kernels (src/GPU/Arista_kernel.cu, Volumen_kernel.cu, unmodified, compiled
for the host by oracle/build_ref.sh and driven by oracle/ref_driver.cpp,
which replays shallowWater()'s launch order for one rank).

Run here, where the reference sources exist:
    python tests/golden/make_golden.py [case ...]      (all cases by default)
Each fixture (ref_<case>.npz) holds the float32 inputs, the parameters, the
initial dt, and the reference's state, dt trace and time after each listed
number of steps.  The reference has no tests or golden vectors of its own,
so these are the pins for the FP64 oracle (tests/test_oracle_golden.py).
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle  # noqa: E402
from landslidehysea_gb300 import scenarios  # noqa: E402
from landslidehysea_gb300._abi import VARS, default_params  # noqa: E402

PARAM_KEYS = ("borde_sup", "borde_inf", "borde_izq", "borde_der", "dx", "dy", "cfl", "r", "angle1",
              "mfc", "mf0", "mfs", "vmax1", "vmax2", "gravity", "eps_h", "peso", "beta", "L", "H")
# stored only for the Pouliquen cases (the Coulomb fixtures keep their keys)
POULIQUEN_KEYS = ("friction_law", "angle2", "angle3", "angle4")


def f32(a):
    return np.asarray(a, dtype=np.float32)


def case_shelf():
    sc = scenarios.shelf(n=40, dx=125.0, cap_radius=400.0)
    return sc.params, {v: f32(sc.state[v]) for v in VARS}, (1, 10)


def case_random():
    rng = np.random.default_rng(17)
    ny, nx = 9, 17
    H = f32(rng.uniform(2.0, 12.0, (ny, nx)))
    h2 = rng.uniform(0.0, 3.0, (ny, nx))
    h2[rng.uniform(size=(ny, nx)) < 0.3] = 0.0
    h1 = np.maximum(H - h2 + rng.uniform(-0.5, 0.5, (ny, nx)), 0.0)
    h1[rng.uniform(size=(ny, nx)) < 0.15] = 0.0
    st = {"h1": f32(h1), "q1x": f32(rng.uniform(-2, 2, (ny, nx)) * (h1 > 0)),
          "q1y": f32(rng.uniform(-2, 2, (ny, nx)) * (h1 > 0)), "h2": f32(h2),
          "q2x": f32(rng.uniform(-1, 1, (ny, nx)) * (h2 > 0)), "q2y": f32(rng.uniform(-1, 1, (ny, nx)) * (h2 > 0)),
          "H": H}
    p = default_params(nx, ny, dx=3.0, dy=2.0, borde_sup=1.0, borde_inf=1.0, borde_izq=1.0, borde_der=1.0,
                       cfl=0.8, r=0.3, angle_deg=20.0, mfc=0.02, mf0=0.03, mfs=0.05, vmax1=1.5, vmax2=0.8,
                       eps_h=1e-3, gravity=9.81)
    return p, st, (1, 3)


def case_dam1d():
    nx, ny = 32, 1
    x = np.arange(nx)
    H = np.full((ny, nx), 3.0)
    h1 = np.where(x < 16, 2.5, 0.0)[None, :]
    h2 = np.where(x < 10, 0.4, 0.0)[None, :]
    z = np.zeros((ny, nx))
    st = {"h1": f32(h1), "q1x": f32(z), "q1y": f32(z), "h2": f32(h2), "q2x": f32(z), "q2y": f32(z), "H": f32(H)}
    p = default_params(nx, ny, dx=0.5, dy=0.5, borde_sup=0.0, borde_inf=0.0, borde_izq=0.0, borde_der=0.0,
                       cfl=0.9, r=0.5, angle_deg=5.0, mf0=0.0, mfs=0.0, eps_h=1e-4, gravity=9.81)
    return p, st, (1, 5)


def case_column():
    nx, ny = 1, 24
    y = np.arange(ny)
    H = (4.0 + 0.1 * y)[:, None]
    h2 = np.where((y > 5) & (y < 12), 1.0, 0.0)[:, None]
    h1 = H - h2
    q1y = np.where(y < 8, 0.3, -0.2)[:, None] * np.ones((ny, nx))
    z = np.zeros((ny, nx))
    st = {"h1": f32(h1), "q1x": f32(z), "q1y": f32(q1y), "h2": f32(h2), "q2x": f32(z), "q2y": f32(z), "H": f32(H)}
    p = default_params(nx, ny, dx=1.0, dy=1.0, cfl=0.9, r=0.5, angle_deg=10.0, mf0=0.02, mfs=0.02,
                       eps_h=1e-3, gravity=9.81)
    return p, st, (1, 5)


def case_slope():
    nx, ny = 24, 20
    x = (np.arange(nx) + 0.5) * 10.0
    y = (np.arange(ny) + 0.5) * 10.0
    X, Y = np.meshgrid(x, y)
    H = 2.0 + 0.25 * X
    cap = 8.0 * np.maximum(0.0, 1.0 - ((X - 60.0) / 45.0) ** 2 - ((Y - 100.0) / 55.0) ** 2)
    h1 = np.maximum(H - 1.0 - cap, 0.0)   # free surface 1 m below the reference level: a dry strip inshore
    # a 1e-5 relative jitter keeps cells off exact branch ties (an at-rest,
    # symmetric state puts some limiter comparisons exactly on their threshold,
    # where FP32 and FP64 rounding pick different branches)
    cap = cap * (1.0 + 1e-5 * np.random.default_rng(5).uniform(size=cap.shape))
    z = np.zeros((ny, nx))
    st = {"h1": f32(h1), "q1x": f32(z), "q1y": f32(z), "h2": f32(cap), "q2x": f32(z), "q2y": f32(z), "H": f32(H)}
    p = default_params(nx, ny, dx=10.0, dy=10.0, borde_sup=1.0, borde_inf=-1.0, borde_izq=0.0, borde_der=1.0,
                       cfl=0.9, r=0.45, angle_deg=4.0, mfc=0.0, mf0=0.02, mfs=0.01, eps_h=1e-3, gravity=9.81)
    return p, st, (1, 10)


def case_film(vmax=0.0):
    """A 1 mm water film on a 0.1 m granular layer, moving at 100 m/s, in a
    cell walled in by higher dry ground.  With no interlayer friction (mfc =
    0) and no speed cap nothing damps it: the wet/dry fix zeroes its normal
    discharge at every face, and Manning friction acts on the water only where
    the granular layer is empty.  With vmax the filter caps it."""
    n = 5
    H = np.full((n, n), 5.0)
    H[2, 2] = 10.0
    z = np.zeros((n, n))
    h1, h2, q1x = z.copy(), z.copy(), z.copy()
    h1[2, 2], h2[2, 2], q1x[2, 2] = 1e-3, 0.1, 0.1
    st = {"h1": f32(h1), "q1x": f32(q1x), "q1y": f32(z), "h2": f32(h2), "q2x": f32(z), "q2y": f32(z), "H": f32(H)}
    p = default_params(n, n, dx=10.0, dy=10.0, cfl=0.5, r=0.5, angle_deg=10.0, mf0=0.025, mfs=0.025, eps_h=1e-5,
                       gravity=9.81, vmax1=vmax, vmax2=vmax)
    return p, st, (1, 50)


def pouliquen(case, angles_deg):
    """A case run with the Pouliquen friction law (Arista_kernel.cu:20-58):
    angles (delta1..delta4) in degrees, read like Problema.cxx:246-255."""
    p, st, steps = case()
    p.friction_law = 1
    p.angle1, p.angle2, p.angle3, p.angle4 = (math.radians(a) for a in angles_deg)
    return p, st, steps


CASES = {"shelf40": case_shelf, "random17x9": case_random, "dam1d": case_dam1d, "column": case_column,
         "slope": case_slope, "film": case_film, "film_vmax20": lambda: case_film(20.0),
         # the slide starts at rest (Froude number 0: the law's fr < EPSILON
         # branch), then creeps (0 < fr < beta: the power-law branch)
         "pouliquen_slope": lambda: pouliquen(case_slope, (4.0, 12.0, 6.0, 14.0)),
         # granular discharges up to 1 m^2/s on 0-3 m layers (fr > beta)
         "pouliquen_random": lambda: pouliquen(case_random, (18.0, 30.0, 21.0, 33.0))}


def main(names):
    if pyoracle.build_ref() is None:
        print("reference sources not available; fixtures unchanged")
        return 1
    for name in names or list(CASES):
        p, st, steps_list = CASES[name]()
        out = {"nx": p.nx, "ny": p.ny, "steps": np.array(steps_list)}
        for k in PARAM_KEYS + (POULIQUEN_KEYS if p.friction_law == 1 else ()):
            out["p_" + k] = getattr(p, k)
        for v in VARS:
            out["in_" + v] = st[v]
        for n in steps_list:
            arrs, trace, t = pyoracle.ref_run(p, st, n)
            for i, v in enumerate(VARS[:6]):
                out[f"out{n}_{v}"] = arrs[i]
            out[f"trace{n}"] = trace
            out[f"t{n}"] = np.float32(t)
        path = os.path.join(HERE, f"ref_{name}.npz")
        np.savez_compressed(path, **out)
        print("wrote", path, os.path.getsize(path), "bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
