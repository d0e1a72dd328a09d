"""The FP64 oracle against the reference's own FP32 kernels.

tests/golden/ref_*.npz were produced by tests/golden/make_golden.py from the
reference's unmodified kernel sources (src/GPU/Arista_kernel.cu,
Volumen_kernel.cu) compiled for the host.  The oracle is FP64 and the
reference FP32, so the bar is FP32 rounding: after one step every field
agrees to 2e-6 of its scale (plus a 2e-5 absolute floor for the momentum noise
an at-rest FP32 state produces), after a few steps to 1e-3.
"""
import glob
import os

import numpy as np
import pytest

from landslidehysea_gb300._abi import VARS, default_params

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "ref_*.npz")))


def load_case(path):
    d = np.load(path)
    p = default_params(int(d["nx"]), int(d["ny"]))
    for k in d.files:
        if k.startswith("p_"):
            setattr(p, k[2:], int(d[k]) if k == "p_friction_law" else float(d[k]))
    return d, p


def test_fixtures_present():
    assert len(GOLDEN) >= 5


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(g)[4:-4] for g in GOLDEN])
def test_oracle_matches_reference(oracle, path):
    d, p = load_case(path)
    for n in d["steps"]:
        n = int(n)
        arrs = [d["in_" + v].astype(np.float64) for v in VARS]
        dt0 = oracle.initial_dt(p, arrs)
        trace = d[f"trace{n}"]
        assert abs(dt0 - trace[0]) <= 2e-7 * trace[0], "initial dt"
        t, dtn, done = oracle.run(p, arrs, n, dt=dt0)
        assert done == n
        rtol, atol = (2e-6, 2e-5) if n == 1 else (1e-3, 1e-4)
        assert abs(t - float(d[f"t{n}"])) <= max(rtol, 2e-7) * abs(float(d[f"t{n}"])) + 1e-12
        assert abs(dtn - trace[-1]) <= max(rtol, 2e-7) * 10 * trace[-1]
        for i, v in enumerate(VARS[:6]):
            ref = d[f"out{n}_{v}"].astype(np.float64)
            scale = max(np.abs(ref).max(), np.abs(d["in_" + v]).max())
            err = np.abs(arrs[i] - ref).max()
            assert err <= rtol * scale + atol, f"{v} after {n} steps: err {err:.3e} scale {scale:.3e}"


POULIQUEN = [g for g in GOLDEN if "pouliquen" in os.path.basename(g)]


def test_pouliquen_fixtures_present():
    assert len(POULIQUEN) >= 2


@pytest.mark.parametrize("path", POULIQUEN, ids=[os.path.basename(g)[4:-4] for g in POULIQUEN])
def test_pouliquen_fixtures_tell_the_laws_apart(oracle, path):
    """The Pouliquen fixtures come from the reference built with COULOMB
    undefined (Arista_kernel.cu:20-58).  The oracle on the Coulomb law with
    the same angle1 misses them by far more than the one-step FP32 bar, so
    the match above pins the Pouliquen law itself."""
    d, p = load_case(path)
    assert p.friction_law == 1
    p.friction_law = 0
    arrs = [d["in_" + v].astype(np.float64) for v in VARS]
    oracle.run(p, arrs, 1, dt=oracle.initial_dt(p, arrs))
    worst = 0.0
    for i, v in enumerate(VARS[:6]):
        ref = d["out1_" + v].astype(np.float64)
        scale = max(np.abs(ref).max(), np.abs(d["in_" + v]).max())
        worst = max(worst, (np.abs(arrs[i] - ref).max() - 2e-5) / (scale * 2e-6))
    assert worst > 10.0, f"the Coulomb law is within {worst:.1f}x of the one-step bar"
