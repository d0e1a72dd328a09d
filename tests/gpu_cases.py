"""Parity cases shared by the GPU tests and smoke(): small seeded inputs that
the CPU oracle finishes in seconds, covering both orders, both coordinate
systems, odd/1-wide grids, open / wall / zero-flux boundaries, dry cells,
speed caps, interlayer friction and the Pouliquen law."""
import glob
import os

import numpy as np

from landslidehysea_gb300 import scenarios
from landslidehysea_gb300._abi import VARS, default_params

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_case(name):
    d = np.load(os.path.join(GOLDEN_DIR, f"ref_{name}.npz"))
    p = default_params(int(d["nx"]), int(d["ny"]))
    for k in d.files:
        if k.startswith("p_"):
            setattr(p, k[2:], int(d[k]) if k == "p_friction_law" else float(d[k]))
    state = {v: d["in_" + v].astype(np.float64) for v in VARS}
    return p, state


def case(name):
    """-> (params, state dict, steps)"""
    if name == "shelf48_o1":
        sc = scenarios.shelf(n=48, dx=25.0 * 200 / 48)
        return sc.params, sc.state, 200
    if name == "shelf200_o1":   # the 200 x 200 first-order shelf, 1000 steps
        sc = scenarios.shelf(n=200)
        return sc.params, sc.state, 1000
    if name == "shelf40x24_o2":
        sc = scenarios.shelf(nx=40, ny=24, dx=120.0, order=2, cfl=0.5)
        return sc.params, sc.state, 60
    if name == "fjord64_o2":
        sc = scenarios.fjord(n=64, dcell_deg=0.0064)
        return sc.params, sc.state, 40
    if name == "fjord64_o1_sph":
        sc = scenarios.fjord(n=64, dcell_deg=0.0064, order=1, cfl=0.9)
        return sc.params, sc.state, 40
    if name.startswith("golden_"):
        p, st = golden_case(name[7:])
        return p, st, 25
    if name == "random_o2":
        p, st = golden_case("random17x9")
        p.order = 2
        p.cfl = 0.45
        return p, st, 20
    if name == "shelf48_o2_fullsort":
        sc = scenarios.shelf(n=48, dx=25.0 * 200 / 48, order=2, cfl=0.5)
        sc.params.eig_sort = 1
        return sc.params, sc.state, 60
    if name == "pouliquen":
        # the slope fixture with the angles of ref_pouliquen_slope.npz, run longer
        p, st = golden_case("pouliquen_slope")
        return p, st, 20
    if name == "pouliquen_random_o2":
        p, st = golden_case("pouliquen_random")
        p.order = 2
        p.cfl = 0.45
        return p, st, 20
    if name in ("dam1d_o2", "column_o2"):
        # one-row and one-column grids at second order: every slope stencil
        # meets a boundary across the degenerate direction
        p, st = golden_case(name[:-3])
        p.order = 2
        p.cfl = 0.45
        return p, st, 25
    if name in ("cell1x1_o1", "cell1x1_o2"):
        # a single cell between walls: only friction and the granular layer's
        # Coulomb stop act
        p = default_params(1, 1, dx=5.0, dy=5.0, cfl=0.5, r=0.5, angle_deg=8.0, mf0=0.03, mfs=0.03, eps_h=1e-4,
                           gravity=9.81)
        p.order = 2 if name.endswith("o2") else 1
        one = np.ones((1, 1))
        st = {"h1": 2.0 * one, "q1x": 0.3 * one, "q1y": -0.2 * one, "h2": 0.5 * one, "q2x": 0.1 * one,
              "q2y": 0.05 * one, "H": 3.0 * one}
        return p, st, 10
    raise KeyError(name)


PARITY_CASES = ["shelf48_o1", "golden_random17x9", "golden_dam1d", "golden_column", "golden_slope",
                "golden_shelf40", "shelf40x24_o2", "random_o2", "fjord64_o2", "fjord64_o1_sph", "pouliquen", "golden_pouliquen_random", "pouliquen_random_o2",
                "shelf48_o2_fullsort", "dam1d_o2", "column_o2", "cell1x1_o1", "cell1x1_o2"]


def rel_linf(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)
