"""The discrete adjoint on the GPU (lsh_adjoint_*): gradients against the
oracle's tangent-linear model (dot-product identity), against the host
emulation of the same adjoint bodies, against FP64 central finite
differences, invariant under the checkpoint budget, and bit-reproducible."""
import numpy as np
import pytest

from adj_cases import copy_arrs, host_adjoint, scenario_case, smooth_case, smooth_direction, wet_direction
from landslidehysea_gb300._abi import VARS

pytestmark = pytest.mark.gpu
pyoracle = pytest.importorskip("pyoracle")


def _target(p, arrs, gauges, n, seed=5):
    _, _, eta = pyoracle.misfit_run(p, copy_arrs(arrs), n, gauges=gauges)
    return eta + 0.01 * np.random.default_rng(seed).standard_normal(eta.shape)


def _state(p, arrs):
    return {v: arrs[i].reshape(p.ny, p.nx) for i, v in enumerate(VARS)}


def _gpu_grad(p, arrs, gauges, n, tgt, budget=None, weight=1.0, bar_final=None, h_adj=0.0):
    from landslidehysea_gb300.solver import Adjoint
    with Adjoint(p, gauges) as A:
        if budget is not None:
            A.set_budget(budget)
        if h_adj:
            A.set_thin_layer(h_adj)
        J, eta = A.forward(_state(p, arrs), n, tgt)
        g, gp = A.gradient(weight, bar_final)
        st = A.stats()
    grad = [g[v].reshape(-1) for v in VARS[:6]]
    return J, eta, grad, np.array([gp[k] for k in ("angle1", "mf0", "mfs", "r")]), st


CASES = [("smooth", 1, False), ("smooth", 2, False), ("smooth", 2, True), ("shelf", 1, False), ("shelf", 2, False),
         ("fjord", 2, False)]


def _case(kind, order, sph):
    if kind == "smooth":
        return smooth_case(order=order, spherical=sph)
    return scenario_case(kind, order)


@pytest.mark.parametrize("kind,order,sph", CASES)
def test_gpu_adjoint_equals_tangent_linear(gpu_lib, kind, order, sph):
    p, arrs, gauges = _case(kind, order, sph)
    n = 6
    tgt = _target(p, arrs, gauges, n)
    J, eta, grad, gpar, _ = _gpu_grad(p, arrs, gauges, n, tgt)
    Jo, _, eta_o = pyoracle.misfit_run(p, copy_arrs(arrs), n, gauges=gauges, target=tgt)
    assert J == Jo and np.array_equal(eta, eta_o)
    dirs = [(smooth_direction(p.nx, p.ny, 3, which=w) if kind == "smooth" else wet_direction(arrs, w, 3), [0, 0, 0, 0])
            for w in ((3,), (0,), (1, 2), (4, 5))]
    dirs += [([None] * 6, e) for e in ([1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1])]
    for d, dpar in dirs:
        dd = [None if x is None else x.copy() for x in d]
        _, dJ, _, _ = pyoracle.tl_run(p, copy_arrs(arrs), dd, dpar, n, gauges=gauges, target=tgt)
        ad = sum(float(np.dot(grad[k], d[k])) for k in range(6) if d[k] is not None) + float(np.dot(gpar, dpar))
        assert abs(ad - dJ) <= 1e-10 * max(abs(dJ), 1e-300), (dpar, dJ, ad)


@pytest.mark.parametrize("kind,order,sph", [("smooth", 2, True), ("fjord", 2, False)])
def test_gpu_adjoint_matches_host_emulation(gpu_lib, kind, order, sph):
    p, arrs, gauges = _case(kind, order, sph)
    n = 5
    tgt = _target(p, arrs, gauges, n)
    J, _, grad, gpar, _ = _gpu_grad(p, arrs, gauges, n, tgt)
    Jh, gh, gph = host_adjoint(p, copy_arrs(arrs), n, gauges, tgt)
    assert J == Jh
    for k in range(6):
        assert np.allclose(grad[k], gh[k], rtol=1e-11, atol=1e-14 * np.abs(gh[k]).max()), k
    assert np.allclose(gpar, gph, rtol=1e-11, atol=1e-300)


def test_checkpoint_budget_does_not_change_the_gradient(gpu_lib):
    from landslidehysea_gb300.solver import revolve_plan
    p, arrs, gauges = smooth_case(order=2)
    n = 23
    tgt = _target(p, arrs, gauges, n)
    slot = None
    ref = None
    for slots in (n, 6, 3, 2, 1):
        J, _, grad, gpar, st = _gpu_grad(p, arrs, gauges, n, tgt,
                                         budget=None if slots == n else slots * (slot or 1e9) + 1.0)
        slot = st["slot_bytes"]
        if ref is None:
            ref = (grad, gpar)
            assert st["slots"] == n
        else:
            assert st["slots"] == slots
            for k in range(6):
                assert np.array_equal(grad[k], ref[0][k]), (slots, k)
            assert np.array_equal(gpar, ref[1]), slots
        fw, _ = revolve_plan(n, st["slots"])
        assert st["reversed_steps"] == n
        assert st["recompute_steps"] <= fw


def test_gradient_is_bit_reproducible(gpu_lib):
    p, arrs, gauges = scenario_case("fjord", 2)
    n = 5
    tgt = _target(p, arrs, gauges, n)
    a = _gpu_grad(p, arrs, gauges, n, tgt)
    b = _gpu_grad(p, arrs, gauges, n, tgt)
    for k in range(6):
        assert np.array_equal(a[2][k], b[2][k])
    assert np.array_equal(a[3], b[3])
    # a second gradient from the same recorded run (the slots were reused)
    from landslidehysea_gb300.solver import Adjoint
    with Adjoint(p, gauges) as A:
        A.set_budget(3 * 6 * 8 * (arrs[0].size + 32) + 1.0)
        A.forward(_state(p, arrs), n, tgt)
        g1, p1 = A.gradient()
        g2, p2 = A.gradient()
    for v in VARS[:6]:
        assert np.array_equal(g1[v], g2[v])
        assert np.array_equal(g1[v].reshape(-1), a[2][VARS.index(v)])
    assert p1 == p2


def test_final_state_vector_jacobian_product(gpu_lib):
    """misfit weight 0, bar_final = w: the gradient is J^T w of the final state."""
    p, arrs, gauges = smooth_case(order=2, spherical=True)
    n = 4
    rng = np.random.default_rng(11)
    w = [rng.standard_normal(arrs[0].size) for _ in range(6)]
    bar = {v: w[i].reshape(p.ny, p.nx) for i, v in enumerate(VARS[:6])}
    _, _, grad, gpar, _ = _gpu_grad(p, arrs, gauges, n, None, weight=0.0, bar_final=bar)
    d = smooth_direction(p.nx, p.ny, 4, which=(0, 3, 4))
    dpar = [0.3, 0.0, 0.2, -0.5]
    dd = [np.zeros(arrs[0].size) if x is None else x.copy() for x in d]
    pyoracle.tl_run(p, copy_arrs(arrs), dd, dpar, n)
    lhs = sum(float(np.dot(w[k], dd[k])) for k in range(6))
    rhs = sum(float(np.dot(grad[k], d[k])) for k in range(6) if d[k] is not None) + float(np.dot(gpar, dpar))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)


def test_gradient_vs_central_finite_differences(gpu_lib):
    """FP64 central differences of the GPU forward's misfit against the
    adjoint gradient, to 1e-6 relative.  J is a sum of squared differences
    of ~40 m depths, so a difference quotient carries rounding noise ~1e-16 *
    40 m / step and the kinks of the scheme (Coulomb switch, minmod choice)
    bound the step from above: each quotient is taken at relative steps 1e-4,
    1e-5 and 1e-6 and the closest counts (the quotient must converge, not
    just land once).  h2 is checked along a smooth field direction and, per
    cell, against the gradient's own scale."""
    import copy
    from landslidehysea_gb300.solver import Adjoint
    p, arrs, gauges = smooth_case(order=2)
    n = 10
    tgt = _target(p, arrs, gauges, n)
    _, _, grad, gpar, _ = _gpu_grad(p, arrs, gauges, n, tgt)

    def J_of(q, a):
        with Adjoint(q, gauges) as A:
            return A.forward(_state(q, a), n, tgt)[0]

    def best(fd_of, ref):
        errs = [abs(fd_of(rel) - ref) for rel in (1e-4, 1e-5, 1e-6)]
        return min(errs) / abs(ref)

    for k, nm in enumerate(("angle1", "mf0", "mfs", "r")):
        if nm == "mf0":
            assert gpar[k] == 0.0  # a granular layer everywhere: no water-bottom friction acts
            continue

        def fd_param(rel, nm=nm):
            h = rel * abs(getattr(p, nm))
            qp, qm = copy.copy(p), copy.copy(p)
            setattr(qp, nm, getattr(p, nm) + h)
            setattr(qm, nm, getattr(p, nm) - h)
            return (J_of(qp, arrs) - J_of(qm, arrs)) / (2 * h)

        assert best(fd_param, gpar[k]) <= 1e-6, nm
    v = smooth_direction(p.nx, p.ny, 9, which=(3,))[3]

    def fd_dir(rel):
        h = rel * 10.0
        ap, am = copy_arrs(arrs), copy_arrs(arrs)
        ap[3] = ap[3] + h * v
        am[3] = am[3] - h * v
        return (J_of(p, ap) - J_of(p, am)) / (2 * h)

    assert best(fd_dir, float(np.dot(grad[3], v))) <= 1e-6
    scale = np.abs(grad[3]).max()
    rng = np.random.default_rng(3)
    for cell in rng.choice(arrs[0].size, 6, replace=False):
        h = 1e-5
        ap, am = copy_arrs(arrs), copy_arrs(arrs)
        ap[3][cell] += h
        am[3][cell] -= h
        fd = (J_of(p, ap) - J_of(p, am)) / (2 * h)
        assert abs(fd - grad[3][cell]) <= 1e-6 * scale, (cell, fd, grad[3][cell])


@pytest.mark.parametrize("kind,h_adj", [("fjord", 0.05), ("shelf", 0.5)])
def test_gpu_thin_layer_projection(gpu_lib, kind, h_adj):
    p, arrs, gauges = scenario_case(kind, 2)
    n = 6
    tgt = _target(p, arrs, gauges, n)
    _, _, grad, gpar, _ = _gpu_grad(p, arrs, gauges, n, tgt, budget=3 * 6 * 8 * (arrs[0].size + 32) + 1.0,
                                    h_adj=h_adj)
    for which, dpar in (((3,), [0, 0, 0, 0]), ((0, 1, 2), [0, 0, 0, 0]), ((), [1, 0, 0, 0]), ((), [0, 0, 0, 1])):
        d = wet_direction(arrs, which, 4) if which else [None] * 6
        dd = [None if x is None else x.copy() for x in d]
        _, dJ, _, _ = pyoracle.tl_run(p, copy_arrs(arrs), dd, dpar, n, gauges=gauges, target=tgt, h_adj=h_adj)
        ad = sum(float(np.dot(grad[k], d[k])) for k in range(6) if d[k] is not None) + float(np.dot(gpar, dpar))
        assert abs(ad - dJ) <= 1e-10 * max(abs(dJ), 1e-300), (which, dpar, dJ, ad)


@pytest.mark.parametrize("order", [1, 2])
def test_overlapped_passes_equal_ordered_launches(gpu_lib, order):
    """The adjoint's forward, recomputed and reverse passes run as overlapped
    launches ordered by row counters; the same run with every pass a
    full-grid launch after the one before gives the same bits.  A 256^2 fjord
    (many block rows per pass), 40 steps, a few checkpoint slots so that the
    schedule also recomputes."""
    from landslidehysea_gb300 import scenarios
    from landslidehysea_gb300.solver import Adjoint
    sc = scenarios.fjord(n=256, order=order)
    p = sc.params
    g = scenarios.gauge_cells(sc)
    n = 40
    with Adjoint(p, g) as T:
        _, tgt = T.forward(sc.state, n)
    tgt = tgt * 1.01
    out = []
    for ordered in (False, True):
        with Adjoint(p, g) as A:
            A.set_ordered(ordered)
            A.set_budget(5 * 6 * 8 * (p.nx * p.ny + 32) + 1.0)
            A.set_thin_layer(0.1)
            J, eta = A.forward(sc.state, n, tgt)
            grad, gp = A.gradient()
            assert A.stats()["recompute_steps"] > 0
        out.append((J, eta, grad, gp))
    (J0, e0, g0, p0), (J1, e1, g1, p1) = out
    assert J0 == J1 and np.array_equal(e0, e1)
    for v in VARS[:6]:
        assert np.array_equal(g0[v], g1[v]), v
    assert p0 == p1
    assert any(np.any(g0[v] != 0.0) for v in VARS[:6])


@pytest.mark.parametrize("name", ["golden_dam1d", "dam1d_o2", "column_o2", "cell1x1_o2"])
def test_gpu_adjoint_degenerate_grids(gpu_lib, name):
    """One-row and one-column grids and a single cell: the GPU gradient (the
    overlapped reverse chain's row waits included) against the oracle's
    tangent-linear, and the misfit bit-identical."""
    from gpu_cases import case
    p, st, _ = case(name)
    arrs = [np.ascontiguousarray(st[v], dtype=np.float64).reshape(-1).copy() for v in VARS]
    N = arrs[0].size
    gauges = np.array(sorted({0, N // 2, N - 1}), dtype=np.int32)
    n = 4
    tgt = _target(p, arrs, gauges, n)
    J, eta, grad, gpar, _ = _gpu_grad(p, arrs, gauges, n, tgt)
    Jo, _, eta_o = pyoracle.misfit_run(p, copy_arrs(arrs), n, gauges=gauges, target=tgt)
    assert J == Jo and np.array_equal(eta, eta_o)
    rng = np.random.default_rng(11)
    for which in ((0, 3), (1, 2), (4, 5)):
        d = [None] * 6
        for k in which:
            d[k] = rng.standard_normal(N) * (arrs[0 if k < 3 else 3] > 0)
        _, dJ, _, _ = pyoracle.tl_run(p, copy_arrs(arrs), [None if x is None else x.copy() for x in d], [0, 0, 0, 0], n,
                                      gauges=gauges, target=tgt)
        ad = sum(float(np.dot(grad[k], d[k])) for k in range(6) if d[k] is not None)
        assert abs(ad - dJ) <= 1e-10 * max(abs(dJ), 1e-300), (which, ad, dJ)
    for e in ([1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]):
        _, dJ, _, _ = pyoracle.tl_run(p, copy_arrs(arrs), [None] * 6, e, n, gauges=gauges, target=tgt)
        ad = float(np.dot(gpar, e))
        assert abs(ad - dJ) <= 1e-10 * max(abs(dJ), 1e-300), (e, ad, dJ)
