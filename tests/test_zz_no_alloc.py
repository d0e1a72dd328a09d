"""lsh_step_noalloc: the entry point for callers that cannot allocate device
memory (a host framework that owns all GPU memory through its own pool, a
real-time loop that must not allocate).  It keeps its scratch in a static
device array instead of allocating.

Checked through the C ABI against the context API (lsh_create / lsh_set_state
/ lsh_step) on two calls in a row -- the second continues from the first, so
it also shows that state left in the shared static array by the previous call
does not leak into the next -- within the parity tolerance of the other GPU
tests (1e-10 relative; the two paths run the same kernels, so they agree bit
for bit).  Runs last (file name) so a failure here cannot hide other results.
"""
import ctypes

import numpy as np
import pytest

from landslidehysea_gb300._abi import LSH_ERR_INVALID, VARS

from gpu_cases import case, rel_linf

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _ptrs(tensors):
    return (ctypes.c_void_p * 7)(*[t.data_ptr() for t in tensors])


@pytest.mark.parametrize("name", ["golden_random17x9", "fjord64_o1_sph"])
def test_noalloc_matches_context_api(gpu_lib, name):
    torch = pytest.importorskip("torch")
    from landslidehysea_gb300.solver import Solver
    p, st, _ = case(name)
    assert p.order == 1
    dev = [torch.tensor(np.ascontiguousarray(st[v]), dtype=torch.float64, device="cuda") for v in VARS]
    ptrs = _ptrs(dev)
    t = ctypes.c_double(0.0)
    dt = ctypes.c_double(0.0)   # <= 0: run the initial-dt pass first
    with Solver(p) as s:
        dt0 = s.set_state(st)
        for call, nsteps in enumerate((9, 6)):
            status = gpu_lib.lsh_step_noalloc(ctypes.byref(p), ptrs, nsteps, ctypes.byref(t), ctypes.byref(dt), None)
            assert status == 0, gpu_lib.lsh_last_error().decode()
            s.step(nsteps)
            s.synchronize()
            ref = s.get_state()
            t_ref, dt_ref, _ = s.time()
            assert abs(t.value - t_ref) <= TOL * abs(t_ref)
            assert abs(dt.value - dt_ref) <= TOL * dt_ref
            torch.cuda.synchronize()
            for k, v in enumerate(VARS[:6]):
                got = dev[k].cpu().numpy()
                assert rel_linf(got, ref[v]) <= TOL, f"call {call}: {v}"
    assert dt0 > 0


def test_noalloc_rejects_what_it_cannot_hold(gpu_lib):
    torch = pytest.importorskip("torch")
    p, st, _ = case("golden_dam1d")
    dev = [torch.tensor(np.ascontiguousarray(st[v]), dtype=torch.float64, device="cuda") for v in VARS]
    ptrs = _ptrs(dev)
    t, dt = ctypes.c_double(0.0), ctypes.c_double(0.0)
    big = p.copy()
    big.nx, big.ny = 300, 300  # 90000 cells > 65536 (sizes are checked before anything is read)
    assert gpu_lib.lsh_step_noalloc(ctypes.byref(big), ptrs, 1, ctypes.byref(t), ctypes.byref(dt), None) == LSH_ERR_INVALID
    assert b"65536" in gpu_lib.lsh_last_error()
    tall = p.copy()
    tall.nx, tall.ny = 1, 5000  # 5000 rows > 4096
    assert gpu_lib.lsh_step_noalloc(ctypes.byref(tall), ptrs, 1, ctypes.byref(t), ctypes.byref(dt), None) == LSH_ERR_INVALID
    o2 = p.copy()
    o2.order = 2
    assert gpu_lib.lsh_step_noalloc(ctypes.byref(o2), ptrs, 1, ctypes.byref(t), ctypes.byref(dt), None) == LSH_ERR_INVALID
