"""CPU checks of the derivative machinery (no GPU):
* the oracle's tangent-linear model (the oracle on dual numbers) has the
  oracle's values bit for bit and matches FP64 central finite differences of
  the oracle's misfit, including the state-dependent CFL step."""
import numpy as np
import pytest

from adj_cases import copy_arrs, smooth_case, smooth_direction

pyoracle = pytest.importorskip("pyoracle")


def _target(p, arrs, gauges, nsteps, seed=5):
    J, _, eta = pyoracle.misfit_run(p, copy_arrs(arrs), nsteps, gauges=gauges)
    rng = np.random.default_rng(seed)
    return eta + 0.01 * rng.standard_normal(eta.shape)


@pytest.mark.parametrize("order", [1, 2])
def test_tl_values_are_the_forward(order):
    p, arrs, gauges = smooth_case(order=order)
    n = 6
    tgt = _target(p, arrs, gauges, n)
    a1 = copy_arrs(arrs)
    J, dt, _ = pyoracle.misfit_run(p, a1, n, gauges=gauges, target=tgt)
    a2 = copy_arrs(arrs)
    d = smooth_direction(p.nx, p.ny, 0)
    J2, dJ, dt2, _ = pyoracle.tl_run(p, a2, d, [0.0, 0.0, 0.0, 0.0], n, gauges=gauges, target=tgt)
    assert J2 == J and dt2 == dt
    for u, v in zip(a1, a2):
        assert np.array_equal(u, v)


def _fd(p, arrs, gauges, tgt, n, dirs, dpar, eps):
    import copy
    vals = []
    for s in (+1.0, -1.0):
        q = copy.copy(p)
        q.angle1 = p.angle1 + s * eps * dpar[0]
        q.mf0 = p.mf0 + s * eps * dpar[1]
        q.mfs = p.mfs + s * eps * dpar[2]
        q.r = p.r + s * eps * dpar[3]
        a = copy_arrs(arrs)
        for k in range(6):
            if dirs[k] is not None:
                a[k] = a[k] + s * eps * dirs[k]
        J, _, _ = pyoracle.misfit_run(q, a, n, gauges=gauges, target=tgt)
        vals.append(J)
    return (vals[0] - vals[1]) / (2 * eps)


@pytest.mark.parametrize("order,spherical", [(1, False), (2, False), (2, True)])
@pytest.mark.parametrize("what", ["h2", "q1", "angle", "manning", "r"])
def test_tl_matches_central_fd(order, spherical, what):
    p, arrs, gauges = smooth_case(order=order, spherical=spherical)
    n = 8
    tgt = _target(p, arrs, gauges, n)
    dirs = [None] * 6
    dpar = [0.0, 0.0, 0.0, 0.0]
    if what == "h2":
        dirs = smooth_direction(p.nx, p.ny, 1, which=(3,))
    elif what == "q1":
        dirs = smooth_direction(p.nx, p.ny, 2, which=(1, 2))
    elif what == "angle":
        dpar[0] = 1.0
    elif what == "manning":
        dpar[1] = dpar[2] = 1.0
    else:
        dpar[3] = 1.0
    a = copy_arrs(arrs)
    d = [None if x is None else x.copy() for x in dirs]
    J, dJ, _, _ = pyoracle.tl_run(p, a, d, dpar, n, gauges=gauges, target=tgt)
    scale = {"h2": 1e-5, "q1": 1e-5, "angle": 1e-6, "manning": 1e-6, "r": 1e-6}[what]
    fd = _fd(p, arrs, gauges, tgt, n, dirs, dpar, scale)
    assert abs(dJ) > 0
    assert abs(fd - dJ) <= 2e-6 * abs(dJ), (fd, dJ)
