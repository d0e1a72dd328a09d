"""Properties of the FP64 scheme that hold independently of any reference
output: per-layer mass conservation with walls, a lake at rest staying at
rest, mirror symmetry, and the convergence orders of the first- and
second-order schemes.  Run on the CPU oracle (the GPU path is bit-identical
to it, tests/test_gpu_parity.py)."""
import math
import os

import numpy as np
import pytest

from landslidehysea_gb300 import scenarios
from landslidehysea_gb300._abi import VARS, default_params


def masses(p, arrs):
    from landslidehysea_gb300.scenarios import EARTH_RADIUS  # noqa: F401
    if p.coords == 1:
        d2r = math.pi / 180
        lat_e = p.lat0 + np.arange(p.ny + 1) * p.dlat
        area = p.radius ** 2 * p.dlon * d2r * (np.sin(lat_e[1:] * d2r) - np.sin(lat_e[:-1] * d2r))
    else:
        area = np.full(p.ny, p.dx * p.dy)
    return [float((arrs[k] * area[:, None]).sum()) for k in (0, 3)]


@pytest.mark.parametrize("kind", ["shelf_o1", "shelf_o2", "fjord_o2_walls", "fjord_o1_walls"])
def test_mass_conserved_with_walls(oracle, kind):
    """With the eigenvalue bounds fully sorted (eig_sort 1) each layer's mass
    is conserved to rounding."""
    if kind.startswith("shelf"):
        sc = scenarios.shelf(n=40, dx=125.0, order=2 if kind.endswith("o2") else 1,
                             cfl=0.5 if kind.endswith("o2") else 0.9)
        steps = 60
    else:
        sc = scenarios.fjord(n=48, dcell_deg=0.008, order=2 if "o2" in kind else 1, borde=-1.0,
                             cfl=0.5 if "o2" in kind else 0.9)
        steps = 40
    sc.params.eig_sort = 1
    arrs = oracle.state_arrays(sc.state)
    m0 = masses(sc.params, arrs)
    oracle.run(sc.params, arrs, steps)
    m1 = masses(sc.params, arrs)
    for a, b in zip(m0, m1):
        assert abs(b - a) <= 1e-13 * abs(a), (a, b)


def test_reference_sort_network_leaks_at_walls(oracle):
    """The reference's compare-and-swap sequence (Arista_kernel.cu:193-234)
    is not a full sort; when a thin granular film's internal wave outruns the
    external one, the bounds of a wall edge and its mirror ghost come out
    asymmetric and the wall passes a little mass (here ~3.5e-11 of the
    granular volume in 60 steps).  Same input with eig_sort 1: exact."""
    out = []
    for full in (0, 1):
        sc = scenarios.shelf(n=40, dx=125.0, order=1)
        sc.params.eig_sort = full
        arrs = oracle.state_arrays(sc.state)
        m0 = masses(sc.params, arrs)
        oracle.run(sc.params, arrs, 60)
        out.append(abs(masses(sc.params, arrs)[1] - m0[1]) / m0[1])
    assert out[0] > 1e-12 and out[0] < 1e-9
    assert out[1] <= 1e-13


def test_reference_keeps_a_walled_in_film_on_the_granular_layer(oracle):
    """A water film on the granular layer, in a cell walled in by higher dry
    ground, keeps its discharge.  The wet/dry fix zeroes its normal
    discharge at every face (Arista_kernel.cu:301-321).  Manning friction
    acts on the water only where h2 < eps_h (Volumen_kernel.cu:75-82), and
    the interlayer term is proportional to mfc (:64-74).  The reference's
    own kernels do the same (tests/golden/ref_film.npz); its speed cap
    (:150-179) is the remedy (ref_film_vmax20.npz).  In the 2048^2 fjord,
    films left on the slide thin towards eps_h with their discharge, and
    u = q/h collapses dt."""
    from gpu_cases import golden_case
    here = os.path.join(os.path.dirname(__file__), "golden")
    for name, q_after in (("film", 0.1), ("film_vmax20", 0.02)):
        ref = np.load(os.path.join(here, f"ref_{name}.npz"))["out50_q1x"][2, 2]
        assert abs(ref - q_after) <= 1e-6 * q_after, (name, ref)
        p, st = golden_case(name)
        arrs = oracle.state_arrays(st)
        oracle.run(p, arrs, 50)
        assert abs(arrs[1][2, 2] - q_after) <= 1e-5 * q_after, (name, arrs[1][2, 2])
        assert arrs[0][2, 2] == st["h1"][2, 2]
    # interlayer friction damps it; without the granular layer Manning friction does
    for change in ("mfc", "no_layer2"):
        p, st = golden_case("film")
        if change == "mfc":
            p.mfc = 0.01
        else:
            st["h2"][2, 2] = 0.0
        arrs = oracle.state_arrays(st)
        oracle.run(p, arrs, 50)
        assert abs(arrs[1][2, 2]) < 1e-2 * 0.1, (change, arrs[1][2, 2])


@pytest.mark.parametrize("order", [1, 2])
def test_lake_at_rest(oracle, order):
    rng = np.random.default_rng(11)
    n = 32
    x = np.linspace(0, 1, n)
    H = 20.0 + 8.0 * np.sin(3 * x)[None, :] * np.cos(2 * x)[:, None] + rng.uniform(0, 0.5, (n, n))
    # a flat-topped granular layer under the water (interface at 12 m below the surface)
    h2 = np.maximum(H - 12.0, 0.0)
    h1 = H - h2                       # surface eta1 = 0
    z = np.zeros((n, n))
    st = {"h1": h1, "q1x": z, "q1y": z, "h2": h2, "q2x": z, "q2y": z, "H": H}
    p = default_params(n, n, order=order, dx=10.0, dy=10.0, cfl=0.5, r=0.5, angle_deg=10.0,
                       mf0=0.02, mfs=0.02, eps_h=1e-5)
    arrs = oracle.state_arrays(st)
    oracle.run(p, arrs, 50)
    eta = arrs[0] + arrs[3] - arrs[6]
    assert np.max(np.abs(eta)) <= 1e-11
    for k in (1, 2, 4, 5):
        assert np.max(np.abs(arrs[k])) <= 1e-10


@pytest.mark.parametrize("order", [1, 2])
def test_mirror_symmetry(oracle, order):
    """Reflecting x (nx even keeps the edge parities) reflects the solution."""
    sc = scenarios.shelf(nx=24, ny=18, dx=200.0, order=order, cfl=0.5)
    st = sc.state
    # put the cap in the middle so the flow is not trivially one-sided
    arrs = oracle.state_arrays(st)
    flip = {v: st[v][:, ::-1].copy() for v in VARS}
    flip["q1x"] = -flip["q1x"]
    flip["q2x"] = -flip["q2x"]
    arrs_f = oracle.state_arrays(flip)
    oracle.run(sc.params, arrs, 30)
    oracle.run(sc.params, arrs_f, 30)
    for k, v in enumerate(VARS[:6]):
        a = arrs[k]
        b = arrs_f[k][:, ::-1] * (-1.0 if v in ("q1x", "q2x") else 1.0)
        scale = max(np.abs(a).max(), 1e-300)
        assert np.max(np.abs(a - b)) <= 1e-12 * scale, v


def smooth_1d(oracle, nx, order, t_end=2.0, cfl=0.4):
    """Water-only smooth hump on a flat bed, walls, no friction: returns the
    depth at t_end sampled on the coarse grid's cells."""
    L = 100.0
    x = (np.arange(nx) + 0.5) * L / nx
    H = np.full((1, nx), 10.0)
    h1 = (10.0 + 0.5 * np.exp(-((x - 50.0) / 10.0) ** 2))[None, :]
    z = np.zeros((1, nx))
    st = {"h1": h1, "q1x": z, "q1y": z, "h2": z, "q2x": z, "q2y": z, "H": H}
    p = default_params(nx, 1, order=order, dx=L / nx, dy=L / nx, cfl=cfl, r=0.5, mf0=0.0, mfs=0.0,
                       eps_h=1e-6, borde_izq=-1.0, borde_der=-1.0, borde_sup=-1.0, borde_inf=-1.0)
    arrs = oracle.state_arrays(st)
    t = 0.0
    dt = oracle.initial_dt(p, arrs)
    # march to t_end, then take a final partial step exactly to t_end
    while True:
        if t + dt >= t_end:
            break
        t, dt, _ = oracle.run(p, arrs, 1, t=t, dt=dt)
    t, _, _ = oracle.run(p, arrs, 1, t=t, dt=t_end - t)
    return arrs[0][0]


def test_second_order_converges_faster(oracle):
    ref = smooth_1d(oracle, 2048, 2)

    def err(nx, order):
        h = smooth_1d(oracle, nx, order)
        r = ref.reshape(nx, -1).mean(axis=1)
        return float(np.abs(h - r).mean())

    e1 = [err(n, 1) for n in (64, 128)]
    e2 = [err(n, 2) for n in (64, 128)]
    rate1 = math.log2(e1[0] / e1[1])
    rate2 = math.log2(e2[0] / e2[1])
    assert e2[1] < e1[1]
    assert rate2 > 1.5, (e2, rate2)
    assert rate1 < rate2
