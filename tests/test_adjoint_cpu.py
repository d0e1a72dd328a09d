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


# ---------------------------------------------------------------- local adjoints vs FD
from adj_cases import host_adjoint, native_lib, scenario_case, wet_direction  # noqa: E402


def _worst(fn, modes, seeds=30):
    import ctypes
    fd, ad = ctypes.c_double(), ctypes.c_double()
    out = {}
    for m in modes:
        errs = sorted(fn(s, m, 6, ctypes.byref(fd), ctypes.byref(ad)) for s in range(seeds))
        out[m] = (errs[len(errs) // 2], errs[-1])
    return out


def test_local_edge_adjoint_vs_fd():
    lib = native_lib("adj_local")
    lib.adjl_set_component(-1)
    # bit0 granular layer, bit1 limiter active, bit2 boundary edge, bit3 Coulomb regime
    for bor in (0.5, 1.0, -1.0):
        lib.adjl_set_bor(bor)
        for mode, (med, worst) in _worst(lib.adjl_edge, [0, 1, 2, 3, 4, 5, 7, 9, 11]).items():
            assert med < 1e-7 and worst < 5e-5, (bor, mode, med, worst)


def test_local_volume_adjoint_vs_fd():
    lib = native_lib("adj_local")
    lib.adjl_set_component(-1)
    # bit0 granular layer, bit1 spherical, bit2 thin layers, bit3 vmax caps
    for mode, (med, worst) in _worst(lib.adjl_volume, [0, 1, 2, 3, 4, 5, 8, 9]).items():
        assert med < 1e-7 and worst < 5e-5, (mode, med, worst)


def test_local_initial_wave_adjoint_vs_fd():
    import ctypes
    lib = native_lib("adj_local")
    fd, ad = ctypes.c_double(), ctypes.c_double()
    errs = sorted(lib.adjl_initial_wave(s, 6, ctypes.byref(fd), ctypes.byref(ad)) for s in range(30))
    assert errs[15] < 1e-6 and errs[-1] < 1e-4


# ---------------------------------------------------------------- the whole sweep vs the tangent-linear
def _dot_check(p, arrs, gauges, n, dirs_list, tol, h_adj=0.0):
    _, _, eta = pyoracle.misfit_run(p, copy_arrs(arrs), n, gauges=gauges)
    tgt = eta + 0.01 * np.random.default_rng(5).standard_normal(eta.shape)
    J, grad, gpar = host_adjoint(p, copy_arrs(arrs), n, gauges, tgt, h_adj=h_adj)
    Jo, _, _ = pyoracle.misfit_run(p, copy_arrs(arrs), n, gauges=gauges, target=tgt)
    assert J == Jo
    for dirs, dpar in dirs_list:
        dd = [None if x is None else x.copy() for x in dirs]
        _, dJ, _, _ = pyoracle.tl_run(p, copy_arrs(arrs), dd, dpar, n, gauges=gauges, target=tgt, h_adj=h_adj)
        ad = sum(float(np.dot(grad[k], dirs[k])) for k in range(6) if dirs[k] is not None) + float(np.dot(gpar, dpar))
        assert abs(ad - dJ) <= tol * max(abs(dJ), 1e-300), (dpar, dJ, ad)


@pytest.mark.parametrize("order,spherical", [(1, False), (2, False), (2, True)])
def test_host_adjoint_equals_tangent_linear_smooth(order, spherical):
    p, arrs, gauges = smooth_case(order=order, spherical=spherical)
    dl = [(smooth_direction(p.nx, p.ny, 3, which=w), [0, 0, 0, 0]) for w in ((3,), (0,), (1, 2), (4, 5))]
    dl += [([None] * 6, e) for e in ([1, 0, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1])]
    _dot_check(p, arrs, gauges, 4, dl, 1e-11)


@pytest.mark.parametrize("kind,order", [("shelf", 1), ("shelf", 2), ("fjord", 2)])
def test_host_adjoint_equals_tangent_linear_scenarios(kind, order):
    p, arrs, gauges = scenario_case(kind, order)
    dl = [(wet_direction(arrs, w, 7), [0, 0, 0, 0]) for w in ((3,), (0,), (1, 2), (4, 5))]
    dl += [([None] * 6, e) for e in ([1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1])]
    _dot_check(p, arrs, gauges, 5, dl, 1e-11)


@pytest.mark.parametrize("kind", ["shelf", "fjord", "smooth"])
def test_fused_reconstruction_slopes_are_the_forwards(kind):
    """The adjoint recomputation's reconstruction (slopes + branch tape in one
    pass) writes the forward's slopes bit for bit."""
    from adj_cases import _ptrs
    if kind == "smooth":
        p, arrs, _ = smooth_case(order=2)
    else:
        p, arrs, _ = scenario_case(kind, 2)
    lib = native_lib("adj_host")
    import ctypes
    assert lib.adjh_recon_check(ctypes.byref(p), _ptrs(arrs)) == 0


@pytest.mark.parametrize("kind,order,h_adj", [("shelf", 2, 0.5), ("fjord", 2, 0.05), ("fjord", 2, 5.0)])
def test_thin_layer_projection_adjoint_is_the_tangent_linears_transpose(kind, order, h_adj):
    """With the thin-layer projection on, the adjoint is still exactly the
    transpose of the (equally projected) tangent-linear model."""
    p, arrs, gauges = scenario_case(kind, order)
    dl = [(wet_direction(arrs, w, 8), [0, 0, 0, 0]) for w in ((3,), (0,), (1, 2), (4, 5))]
    dl += [([None] * 6, e) for e in ([1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1])]
    _dot_check(p, arrs, gauges, 6, dl, 1e-11, h_adj=h_adj)


def test_initial_wave_empty_edge_shortcut_is_exact():
    """The kernels skip the initial-dt bound's FP64 work on empty, still edge
    pairs: the general formula gives exactly len * eps_h there."""
    assert native_lib("adj_local").adjl_initial_wave_empty() == 0


# ---------------------------------------------------------------- the product's forward on the host
@pytest.mark.parametrize("kind,order", [("shelf", 1), ("shelf", 2), ("fjord", 2), ("smooth", 1), ("smooth", 2)])
def test_host_forward_equals_oracle(kind, order):
    """The product's per-edge / per-cell forward bodies (lsh_passes.cuh,
    compiled for the host in plain loops) against the oracle: every state
    field and every step's dt bit-identical.  The CUDA kernels run these
    bodies too, so this holds the shared device code to the oracle on a
    machine without a GPU."""
    import ctypes
    from adj_cases import _ptrs
    if kind == "smooth":
        p, arrs, _ = smooth_case(order=order, spherical=(order == 2))
    else:
        p, arrs, _ = scenario_case(kind, order)
    n = 6
    lib = native_lib("adj_host")
    a_host = copy_arrs(arrs)
    dts = np.zeros(n + 1)
    assert lib.adjh_forward(ctypes.byref(p), _ptrs(a_host), n, dts.ctypes.data) == 0
    a_o = copy_arrs(arrs)
    dt0 = pyoracle.initial_dt(p, a_o)
    assert dt0 == dts[0]
    t, dt, _ = pyoracle.run(p, a_o, n, dt=dt0)
    assert dt == dts[n]
    for k in range(6):
        assert np.array_equal(a_host[k], a_o[k]), k


@pytest.mark.parametrize("name", ["dam1d_o2", "column_o2", "cell1x1_o1", "cell1x1_o2", "golden_dam1d", "golden_column",
                                  "random_o2", "pouliquen_random_o2"])
def test_host_forward_equals_oracle_edge_cases(name):
    """The same on the GPU parity suite's degenerate and special cases: one-row
    and one-column grids, a single cell, random states, the Pouliquen law."""
    import ctypes
    from adj_cases import _ptrs
    from gpu_cases import case
    from landslidehysea_gb300._abi import VARS
    p, st, steps = case(name)
    n = min(steps, 10)
    arrs = [np.ascontiguousarray(st[v], dtype=np.float64).reshape(-1).copy() for v in VARS]
    lib = native_lib("adj_host")
    a_host = copy_arrs(arrs)
    dts = np.zeros(n + 1)
    assert lib.adjh_forward(ctypes.byref(p), _ptrs(a_host), n, dts.ctypes.data) == 0
    a_o = copy_arrs(arrs)
    dt0 = pyoracle.initial_dt(p, a_o)
    assert dt0 == dts[0]
    t, dt, _ = pyoracle.run(p, a_o, n, dt=dt0)
    assert dt == dts[n]
    for k in range(6):
        assert np.array_equal(a_host[k], a_o[k]), (name, k)


@pytest.mark.parametrize("name", ["golden_dam1d", "dam1d_o2", "golden_column", "column_o2", "cell1x1_o2"])
def test_host_adjoint_equals_tangent_linear_edge_cases(name):
    """The host emulation of the adjoint sweep on one-row and one-column grids
    and a single cell, against the oracle's tangent-linear."""
    from gpu_cases import case
    from landslidehysea_gb300._abi import VARS
    p, st, _ = case(name)
    arrs = [np.ascontiguousarray(st[v], dtype=np.float64).reshape(-1).copy() for v in VARS]
    N = arrs[0].size
    gauges = np.array(sorted({0, N // 2, N - 1}), dtype=np.int32)
    rng = np.random.default_rng(11)
    dl = []
    for which in ((0, 3), (1, 2), (4, 5)):
        d = [None] * 6
        for k in which:
            d[k] = rng.standard_normal(N) * (arrs[0 if k < 3 else 3] > 0)
        dl.append((d, [0, 0, 0, 0]))
    dl += [([None] * 6, e) for e in ([1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1])]
    _dot_check(p, arrs, gauges, 4, dl, 1e-10)
