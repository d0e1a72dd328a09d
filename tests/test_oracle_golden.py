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
            setattr(p, k[2:], float(d[k]))
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
