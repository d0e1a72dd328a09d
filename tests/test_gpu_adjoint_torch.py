"""torch.autograd.Function over the C ABI's adjoint (test harness only: the
library's interface is the C ABI): torch.autograd.gradcheck of the gauge
misfit with respect to the initial granular thickness field and the
(angle1, mf0, mfs, r) parameters."""
import copy

import numpy as np
import pytest

from adj_cases import copy_arrs, smooth_case
from landslidehysea_gb300._abi import VARS

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
pyoracle = pytest.importorskip("pyoracle")


class GaugeMisfit(torch.autograd.Function):
    """J(h2_0, theta) of an n-step run; theta = (angle1, mf0, mfs, r)."""

    @staticmethod
    def forward(ctx, h2, theta, base_params, base_arrs, gauges, nsteps, target):
        from landslidehysea_gb300.solver import Adjoint
        p = copy.copy(base_params)
        p.angle1, p.mf0, p.mfs, p.r = [float(x) for x in theta.detach().cpu().numpy()]
        arrs = copy_arrs(base_arrs)
        arrs[3] = np.ascontiguousarray(h2.detach().cpu().numpy(), dtype=np.float64).reshape(-1).copy()
        A = Adjoint(p, gauges)
        J, _ = A.forward({v: arrs[i].reshape(p.ny, p.nx) for i, v in enumerate(VARS)}, nsteps, target)
        ctx.adj = A
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        g, gp = ctx.adj.gradient()  # callable again: gradcheck may run backward twice
        gh2 = torch.from_numpy(g["h2"].reshape(-1).copy()) * gJ
        gth = torch.tensor([gp["angle1"], gp["mf0"], gp["mfs"], gp["r"]], dtype=torch.float64) * gJ
        return gh2, gth, None, None, None, None, None


def test_gradcheck(gpu_lib):
    p, arrs, gauges = smooth_case(nx=10, ny=8, order=2)
    n = 6
    _, _, eta = pyoracle.misfit_run(p, copy_arrs(arrs), n, gauges=gauges[:2] % arrs[0].size)
    g = (gauges[:2] % arrs[0].size).astype(np.int32)
    tgt = eta + 0.01 * np.random.default_rng(1).standard_normal(eta.shape)
    h2 = torch.tensor(arrs[3].copy(), dtype=torch.float64, requires_grad=True)
    theta = torch.tensor([p.angle1, p.mf0, p.mfs, p.r], dtype=torch.float64, requires_grad=True)

    def f(h2_, th_):
        return GaugeMisfit.apply(h2_, th_, p, arrs, g, n, tgt)

    assert torch.autograd.gradcheck(f, (h2, theta), eps=1e-6, atol=1e-8, rtol=1e-5, nondet_tol=0.0)
