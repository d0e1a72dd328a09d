"""TEST INFRASTRUCTURE -- ctypes access to the FP64 CPU oracle
(oracle/_build/liblsh_oracle.so) and, where it was built, to the reference's
own FP32 kernels run on the host (oracle/_ref/liblsh_ref.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this
module.  The product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liblsh_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "liblsh_ref.so")
# the same kernels built with the Pouliquen friction law (COULOMB undefined)
REF_POULIQUEN_SO = os.path.join(HERE, "_ref", "liblsh_ref_pouliquen.so")

_lib = None
_ref = {}


def build(force=False):
    """Compile the oracle (a second or two)."""
    srcs = [os.path.join(HERE, "lsh_oracle.cpp"), os.path.join(HERE, "dual.h"), os.path.join(HERE, "count.h"),
            os.path.join(HERE, "..", "landslidehysea_gb300", "csrc", "lsh_fpmath.h")]
    if force or not os.path.exists(ORACLE_SO) or \
            os.path.getmtime(ORACLE_SO) < max(os.path.getmtime(f) for f in srcs):
        subprocess.run(["sh", os.path.join(HERE, "build_oracle.sh")], check=True)
    return ORACLE_SO


def build_ref(reference_root=None):
    """Compile the reference's kernels for the host when its sources exist
    (reference_root: default $LSH_REFERENCE_ROOT, else build_ref.sh's own)."""
    cmd = ["sh", os.path.join(HERE, "build_ref.sh")]
    if reference_root:
        cmd.append(reference_root)
    subprocess.run(cmd, check=True)
    return REF_SO if os.path.exists(REF_SO) else None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(ORACLE_SO)
        P = ctypes.c_void_p
        _lib.orc_initial_dt.argtypes = [P, P, ctypes.POINTER(ctypes.c_double)]
        _lib.orc_run.argtypes = [P, P, ctypes.c_longlong, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                 ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong), P, P]
        _lib.orc_masks.argtypes = [P, P, P]
        _lib.orc_set_threads.argtypes = [ctypes.c_int]
        _lib.orc_fpmath.argtypes = [ctypes.c_int, P, P, ctypes.c_longlong]
        D = ctypes.POINTER(ctypes.c_double)
        _lib.orc_misfit_run.argtypes = [P, P, ctypes.c_longlong, ctypes.c_int, D, ctypes.c_int, P, P, D, P]
        _lib.orc_count_ops.argtypes = [P, P, ctypes.c_longlong, P]
        _lib.orc_tl_run.argtypes = [P, P, P, P, ctypes.c_longlong, ctypes.c_int, D, D, ctypes.c_int, P, P, D, D, P,
                                    ctypes.c_double]
    return _lib


def ref_available():
    return os.path.exists(REF_SO)


def ref_lib(pouliquen=False):
    """The reference's kernels on the host: as shipped (Coulomb law), or
    with the Pouliquen law."""
    path = REF_POULIQUEN_SO if pouliquen else REF_SO
    if path not in _ref:
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib_ = ctypes.CDLL(path)
        f = ctypes.c_float
        P = ctypes.c_void_p
        lib_.lsh_ref_run.argtypes = [ctypes.c_int, ctypes.c_int, P] + [f] * 24 + [ctypes.c_int, P, P, P, P]
        _ref[path] = lib_
    return _ref[path]


def _ptrs(arrays):
    arr = (ctypes.c_void_p * len(arrays))(*[a.ctypes.data for a in arrays])
    return arr


def set_threads(n):
    return lib().orc_set_threads(int(n))


def state_arrays(state):
    from landslidehysea_gb300._abi import VARS
    return [np.ascontiguousarray(state[v], dtype=np.float64).copy() for v in VARS]


def initial_dt(params, arrays):
    dt = ctypes.c_double()
    st = lib().orc_initial_dt(ctypes.byref(params), _ptrs(arrays), ctypes.byref(dt))
    if st:
        raise RuntimeError(f"orc_initial_dt status {st}")
    return dt.value


def run(params, arrays, nsteps, t=0.0, dt=None, t_end=-1.0, eta=None):
    """Advance `arrays` (list of 7 float64 arrays, modified in place).  Returns
    (t, dt_next, steps_done).  `eta` = (eta_max, eta_time) arrays or None."""
    if dt is None:
        dt = initial_dt(params, arrays)
    tt = ctypes.c_double(t)
    dd = ctypes.c_double(dt)
    done = ctypes.c_longlong(0)
    em = eta[0].ctypes.data if eta is not None else None
    et = eta[1].ctypes.data if eta is not None else None
    st = lib().orc_run(ctypes.byref(params), _ptrs(arrays), int(nsteps), float(t_end), ctypes.byref(tt),
                       ctypes.byref(dd), ctypes.byref(done), em, et)
    if st:
        raise RuntimeError(f"orc_run status {st}")
    return tt.value, dd.value, done.value


def fpmath(which, x):
    """Shared elementary functions: 'exp_neg', 'cbrt', 'log', 'pow1e-3'."""
    code = {"exp_neg": 0, "cbrt": 1, "log": 2, "pow1e-3": 3}[which]
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    if lib().orc_fpmath(code, x.ctypes.data, y.ctypes.data, x.size):
        raise RuntimeError("orc_fpmath")
    return y


def masks(params, arrays):
    out = np.zeros(arrays[0].shape, dtype=np.uint8)
    lib().orc_masks(ctypes.byref(params), _ptrs(arrays), out.ctypes.data)
    return out


def ref_run(params, state, nsteps, eta=None):
    """Run the reference's FP32 kernels (host build; the Pouliquen build when
    params.friction_law is 1).  `state`: dict or list of 7 arrays.  Returns
    (float32 arrays list, dt_trace, t)."""
    from landslidehysea_gb300._abi import VARS
    if isinstance(state, dict):
        arrs = [np.ascontiguousarray(state[v], dtype=np.float32).copy() for v in VARS]
    else:
        arrs = [np.ascontiguousarray(a, dtype=np.float32).copy() for a in state]
    trace = np.zeros(nsteps + 1, dtype=np.float32)
    t = ctypes.c_float()
    p = params
    em = eta[0].ctypes.data if eta is not None else None
    et = eta[1].ctypes.data if eta is not None else None
    ref_lib(p.friction_law == 1).lsh_ref_run(
                          p.nx, p.ny, _ptrs(arrs), p.borde_sup, p.borde_inf, p.borde_izq, p.borde_der,
                          p.dx, p.dy, p.dx * p.dy, p.cfl, p.r, p.angle1, p.angle2, p.angle3, p.angle4,
                          p.peso, p.beta, p.mfc, p.mf0, p.mfs,
                          p.vmax1, p.vmax2, p.gravity, p.eps_h, p.L, p.H, int(nsteps), trace.ctypes.data,
                          ctypes.byref(t), em, et)
    return arrs, trace, t.value


def _gauge_args(gauges, target, nsteps):
    g = np.ascontiguousarray(gauges if gauges is not None else np.zeros(0), dtype=np.int32)
    t = None if target is None else np.ascontiguousarray(target, dtype=np.float64).reshape(nsteps, len(g))
    return g, t


def misfit_run(params, arrs, nsteps, dt=None, gauges=None, target=None):
    """Forward run of `nsteps` with the gauge misfit (oracle).  `arrs` (7
    arrays) is advanced in place.  dt None: the initial-dt pass.  Returns
    (J, dt_next, eta series [nsteps, n_gauges])."""
    g, t = _gauge_args(gauges, target, nsteps)
    eta = np.zeros((nsteps, len(g)))
    d = ctypes.c_double(0.0 if dt is None else dt)
    J = ctypes.c_double()
    st = lib().orc_misfit_run(ctypes.byref(params), _ptrs(arrs), int(nsteps), int(dt is None), ctypes.byref(d),
                              len(g), g.ctypes.data if len(g) else None, t.ctypes.data if t is not None else None,
                              ctypes.byref(J), eta.ctypes.data if len(g) else None)
    if st:
        raise RuntimeError(f"orc_misfit_run: status {st}")
    return J.value, d.value, eta


def tl_run(params, arrs, darrs, dpar, nsteps, dt=None, ddt=0.0, gauges=None, target=None, h_adj=0.0):
    """Tangent-linear run (oracle on dual numbers).  darrs: 6 tangent arrays
    (h1..q2y, None = 0), advanced in place with `arrs`; dpar: tangents of
    (angle1, mf0, mfs, r); h_adj > 0: tangents of layers thinner than h_adj
    are zeroed after every step.  Returns (J, dJ, dt_next, ddt_next)."""
    g, t = _gauge_args(gauges, target, nsteps)
    N = arrs[0].size
    dd = [np.zeros(N) if a is None else a for a in darrs]
    for a in dd:
        assert a.dtype == np.float64 and a.flags.c_contiguous
    dp = np.ascontiguousarray(dpar, dtype=np.float64)
    d = ctypes.c_double(0.0 if dt is None else dt)
    dd_t = ctypes.c_double(ddt)
    J = ctypes.c_double()
    dJ = ctypes.c_double()
    st = lib().orc_tl_run(ctypes.byref(params), _ptrs(arrs), _ptrs(dd), dp.ctypes.data, int(nsteps), int(dt is None),
                          ctypes.byref(d), ctypes.byref(dd_t), len(g), g.ctypes.data if len(g) else None,
                          t.ctypes.data if t is not None else None, ctypes.byref(J), ctypes.byref(dJ), None,
                          float(h_adj))
    if st:
        raise RuntimeError(f"orc_tl_run: status {st}")
    for a, b in zip(darrs, dd):
        if a is not None and a is not b:
            a[...] = b
    return J.value, dJ.value, d.value, dd_t.value


OP_KINDS = ("add", "mul", "fma", "div", "sqrt", "exp", "cbrt", "pow", "cmp", "abs")


def count_ops(params, arrs, nsteps):
    """FP64 operations of the initial-dt pass and `nsteps` steps from `arrs`
    as the oracle performs them, by kind (dict)."""
    counts = np.zeros(16, dtype=np.int64)
    held = [np.ascontiguousarray(a, dtype=np.float64).copy() for a in arrs]  # alive across the call
    st = lib().orc_count_ops(ctypes.byref(params), _ptrs(held), int(nsteps), counts.ctypes.data)
    if st:
        raise RuntimeError(f"orc_count_ops: status {st}")
    return dict(zip(OP_KINDS, counts[:len(OP_KINDS)].tolist()))


def ops_per_cell_step(params, arrs, steps=(1, 3)):
    """FP64 operations per cell-update of the step (the initial-dt pass
    removed by differencing two run lengths)."""
    a, b = steps
    ca, cb = count_ops(params, arrs, a), count_ops(params, arrs, b)
    n = params.nx * params.ny * (b - a)
    return {k: (cb[k] - ca[k]) / n for k in OP_KINDS}


REF_CUDA_SO = os.path.join(HERE, "_ref", "liblsh_ref_cuda.so")
REF_CUBIN = os.path.join(HERE, "_ref", "ref_kernels.cubin")


def ref_cuda_available():
    """The reference's own CUDA build: its kernels compiled for sm_103a from
    the reference sources (ref_kernels.cubin) and the driver that runs them
    (liblsh_ref_cuda.so)."""
    return os.path.exists(REF_CUDA_SO) and os.path.exists(REF_CUBIN)


def ref_cuda_run(params, state, warmup, nsteps, device=0):
    """Run the reference's CUDA kernels on the GPU (FP32, Coulomb law): one
    rank's shallowWater() step sequence, `warmup` untimed steps then
    `nsteps` timed ones.  Returns (float32 arrays list, dt trace of the timed
    steps, t, wall ms of the timed steps)."""
    from landslidehysea_gb300._abi import VARS
    lib_ = ctypes.CDLL(REF_CUDA_SO)
    f = ctypes.c_float
    P = ctypes.c_void_p
    lib_.lsh_ref_cuda_run.argtypes = ([ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, P] + [f] * 24 +
                                      [ctypes.c_int, ctypes.c_int, P, P, P])
    lib_.lsh_ref_cuda_error.restype = ctypes.c_char_p
    arrs = [np.ascontiguousarray(state[v], dtype=np.float32).copy() for v in VARS]
    trace = np.zeros(nsteps + 1, dtype=np.float32)
    t = ctypes.c_float()
    ms = ctypes.c_double()
    p = params
    st = lib_.lsh_ref_cuda_run(REF_CUBIN.encode(), int(device), p.nx, p.ny, _ptrs(arrs), p.borde_sup, p.borde_inf,
                               p.borde_izq, p.borde_der, p.dx, p.dy, p.dx * p.dy, p.cfl, p.r, p.angle1, p.angle2,
                               p.angle3, p.angle4, p.peso, p.beta, p.mfc, p.mf0, p.mfs, p.vmax1, p.vmax2, p.gravity,
                               p.eps_h, p.L, p.H, int(warmup), int(nsteps), trace.ctypes.data, ctypes.byref(t),
                               ctypes.byref(ms))
    if st:
        raise RuntimeError("reference CUDA build: " + lib_.lsh_ref_cuda_error().decode())
    return arrs, trace, t.value, ms.value
