"""Python host mirror of the C ABI (include/lsh.h) over ctypes.

The solver runs on the GPU through liblsh.so only: there is no CPU path.
Constructing a :class:`Solver` without the built library, or without a CUDA
device, raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _abi
from ._abi import LSH_NVARS, VARS, LshParams

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "liblsh.so")

_lib = None


class LshError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = f"{what}: status {status}"
        if _lib is not None:
            msg += f" ({_lib.lsh_status_string(status).decode()}; {_lib.lsh_last_error().decode()})"
        super().__init__(msg)


P = ctypes.c_void_p
DP = ctypes.POINTER(ctypes.c_double)

# name -> (restype, argtypes); the list of every entry point include/lsh.h declares
SIGNATURES = {
    "lsh_params_default": (ctypes.c_int, [P]),
    "lsh_check_device": (ctypes.c_int, []),
    "lsh_create": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(P)]),
    "lsh_destroy": (ctypes.c_int, [P]),
    "lsh_set_stream": (ctypes.c_int, [P, P]),
    "lsh_set_state": (ctypes.c_int, [P, P, DP]),
    "lsh_set_state_device": (ctypes.c_int, [P, P, DP]),
    "lsh_step": (ctypes.c_int, [P, ctypes.c_int]),
    "lsh_run_until": (ctypes.c_int, [P, ctypes.c_double, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)]),
    "lsh_synchronize": (ctypes.c_int, [P]),
    "lsh_get_state": (ctypes.c_int, [P, P]),
    "lsh_get_state_device": (ctypes.c_int, [P, P]),
    "lsh_get_time": (ctypes.c_int, [P, DP, DP, ctypes.POINTER(ctypes.c_longlong)]),
    "lsh_get_eta_max": (ctypes.c_int, [P, P, P]),
    "lsh_get_masks": (ctypes.c_int, [P, P]),
    "lsh_get_gauge_eta": (ctypes.c_int, [P, ctypes.c_int, P, P]),
    "lsh_get_launch_count": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_longlong)]),
    "lsh_profile_step": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "lsh_probe_fp64_peak": (ctypes.c_int, [ctypes.c_int, DP]),
    "lsh_probe_wait_bound": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int), DP]),
    "lsh_step_noalloc": (ctypes.c_int, [P, P, ctypes.c_int, DP, DP, P]),
    "lsh_batch_create": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(P)]),
    "lsh_batch_destroy": (ctypes.c_int, [P]),
    "lsh_batch_set_state": (ctypes.c_int, [P, ctypes.c_int, P, DP]),
    "lsh_batch_step": (ctypes.c_int, [P, ctypes.c_int]),
    "lsh_batch_synchronize": (ctypes.c_int, [P]),
    "lsh_batch_get_state": (ctypes.c_int, [P, ctypes.c_int, P]),
    "lsh_batch_get_time": (ctypes.c_int, [P, ctypes.c_int, DP, DP, ctypes.POINTER(ctypes.c_longlong)]),
    "lsh_batch_autotune": (ctypes.c_int, [P, ctypes.c_int, P]),
    "lsh_batch_set_tune": (ctypes.c_int, [P, P]),
    "lsh_batch_get_tune": (ctypes.c_int, [P, P]),
    "lsh_batch_get_launch_count": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_longlong)]),
    "lsh_adjoint_create": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P, ctypes.POINTER(P)]),
    "lsh_adjoint_destroy": (ctypes.c_int, [P]),
    "lsh_adjoint_set_budget": (ctypes.c_int, [P, ctypes.c_double]),
    "lsh_adjoint_set_thin_layer": (ctypes.c_int, [P, ctypes.c_double]),
    "lsh_adjoint_set_ordered": (ctypes.c_int, [P, ctypes.c_int]),
    "lsh_adjoint_forward": (ctypes.c_int, [P, P, ctypes.c_int, P, DP, P]),
    "lsh_adjoint_gradient": (ctypes.c_int, [P, ctypes.c_double, P, P, P]),
    "lsh_adjoint_get_stats": (ctypes.c_int, [P, P]),
    "lsh_adjoint_get_times": (ctypes.c_int, [P, DP]),
    "lsh_adjoint_get_state": (ctypes.c_int, [P, P]),
    "lsh_adjoint_batch_create": (ctypes.c_int, [ctypes.c_int, P, P, P, ctypes.c_int, ctypes.POINTER(P)]),
    "lsh_adjoint_batch_destroy": (ctypes.c_int, [P]),
    "lsh_adjoint_batch_set_thin_layer": (ctypes.c_int, [P, ctypes.c_double]),
    "lsh_adjoint_batch_set_budget": (ctypes.c_int, [P, ctypes.c_double]),
    "lsh_adjoint_batch_forward": (ctypes.c_int, [P, P, ctypes.c_int, P, DP, P]),
    "lsh_adjoint_batch_gradient": (ctypes.c_int, [P, P, P, P]),
    "lsh_adjoint_batch_get_stats": (ctypes.c_int, [P, P]),
    "lsh_adjoint_batch_member": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(P)]),
    "lsh_revolve_plan": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong),
                                        ctypes.POINTER(ctypes.c_longlong)]),
    "lsh_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "lsh_last_error": (ctypes.c_char_p, []),
}


def load(path=LIB_PATH):
    """Load liblsh.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with landslidehysea_gb300.build.build() "
                           "(there is no CPU fallback)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(status, what):
    if status != 0:
        raise LshError(status, what)


def _ptr_array(ptrs):
    return (ctypes.c_void_p * LSH_NVARS)(*ptrs)


def _ptrs(ptrs):
    """A C array of pointers of any length (0 entries are NULL)."""
    ptrs = list(ptrs)
    return (ctypes.c_void_p * max(1, len(ptrs)))(*[p or None for p in ptrs])


def device_available():
    return load().lsh_check_device() == 0


def probe_fp64_peak(device=0):
    """Measured FP64 FMA throughput of the device, GFLOP/s."""
    g = ctypes.c_double()
    _check(load().lsh_probe_fp64_peak(int(device), ctypes.byref(g)), "lsh_probe_fp64_peak")
    return g.value


def probe_wait_bound(device=0):
    """(status, ms): the status the bounded waits between passes report when
    their counters never complete (LSH_ERR_TIMEOUT expected), and the probe
    kernel's duration."""
    st = ctypes.c_int()
    ms = ctypes.c_double()
    _check(load().lsh_probe_wait_bound(int(device), ctypes.byref(st), ctypes.byref(ms)), "lsh_probe_wait_bound")
    return st.value, ms.value


class Solver:
    """One solver context on one GPU (wraps lsh_ctx)."""

    def __init__(self, params: LshParams, device: int = 0):
        self.lib = load()
        self.params = params.copy()
        self.nx, self.ny = params.nx, params.ny
        self._ctx = ctypes.c_void_p()
        _check(self.lib.lsh_create(ctypes.byref(self.params), int(device), ctypes.byref(self._ctx)), "lsh_create")

    def close(self):
        if self._ctx:
            self.lib.lsh_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---------------------------------------------------------------- state
    def set_state(self, state):
        """`state`: dict VARS -> array (ny, nx) or a list of 7 arrays.
        Returns the initial dt."""
        arrs = [np.ascontiguousarray(state[v] if isinstance(state, dict) else state[i], dtype=np.float64)
                for i, v in enumerate(VARS)]
        for a in arrs:
            if a.size != self.nx * self.ny:
                raise ValueError("state array size does not match nx*ny")
        dt = ctypes.c_double()
        _check(self.lib.lsh_set_state(self._ctx, _ptr_array([a.ctypes.data for a in arrs]), ctypes.byref(dt)),
               "lsh_set_state")
        return dt.value

    def set_state_device(self, ptrs):
        """`ptrs`: 7 device pointers (ints) of FP64 arrays on this device."""
        dt = ctypes.c_double()
        _check(self.lib.lsh_set_state_device(self._ctx, _ptr_array(list(ptrs)), ctypes.byref(dt)),
               "lsh_set_state_device")
        return dt.value

    def get_state(self, out=None):
        """The state as host arrays.  `out`: a dict of C-contiguous float64
        (ny, nx) arrays to fill (e.g. pinned buffers reused across calls)."""
        if out is None:
            out = {v: np.empty((self.ny, self.nx), dtype=np.float64) for v in VARS}
        for v in VARS:
            a = out[v]
            if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] or a.size != self.nx * self.ny:
                raise ValueError(f"get_state: out[{v!r}] must be a C-contiguous float64 array of ny*nx values")
        _check(self.lib.lsh_get_state(self._ctx, _ptr_array([out[v].ctypes.data for v in VARS])), "lsh_get_state")
        return out

    def get_state_device(self, ptrs):
        _check(self.lib.lsh_get_state_device(self._ctx, _ptr_array(list(ptrs))), "lsh_get_state_device")

    # ---------------------------------------------------------------- time
    def step(self, n=1):
        _check(self.lib.lsh_step(self._ctx, int(n)), "lsh_step")

    def synchronize(self):
        _check(self.lib.lsh_synchronize(self._ctx), "lsh_synchronize")

    def run_until(self, t_end, max_steps=0):
        done = ctypes.c_longlong()
        _check(self.lib.lsh_run_until(self._ctx, float(t_end), int(max_steps), ctypes.byref(done)), "lsh_run_until")
        return done.value

    def time(self):
        t, dt, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        _check(self.lib.lsh_get_time(self._ctx, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(n)), "lsh_get_time")
        return t.value, dt.value, n.value

    def eta_max(self):
        em = np.empty((self.ny, self.nx))
        et = np.empty((self.ny, self.nx))
        _check(self.lib.lsh_get_eta_max(self._ctx, em.ctypes.data, et.ctypes.data), "lsh_get_eta_max")
        return em, et

    def masks(self):
        m = np.empty((self.ny, self.nx), dtype=np.uint8)
        _check(self.lib.lsh_get_masks(self._ctx, m.ctypes.data), "lsh_get_masks")
        return m

    def gauge_eta(self, cells):
        """h1 - H at the given cell indices (row-major j*nx + i), gathered on
        the device; NaN for an index outside the grid."""
        c = np.ascontiguousarray(cells, dtype=np.int32).reshape(-1)
        out = np.empty(c.size)
        _check(self.lib.lsh_get_gauge_eta(self._ctx, int(c.size), c.ctypes.data if c.size else None,
                                          out.ctypes.data if c.size else None), "lsh_get_gauge_eta")
        return out

    def launch_count(self):
        n = ctypes.c_longlong()
        _check(self.lib.lsh_get_launch_count(self._ctx, ctypes.byref(n)), "lsh_get_launch_count")
        return n.value

    def profile_step(self):
        """Run one step with per-kernel CUDA events; returns a list of ms."""
        buf = (ctypes.c_float * 32)()
        n = ctypes.c_int()
        _check(self.lib.lsh_profile_step(self._ctx, buf, 32, ctypes.byref(n)), "lsh_profile_step")
        return [buf[i] for i in range(n.value)]

    def set_stream(self, stream_ptr):
        _check(self.lib.lsh_set_stream(self._ctx, ctypes.c_void_p(stream_ptr)), "lsh_set_stream")


class Tune(ctypes.Structure):
    """Mirror of lsh_tune."""
    _fields_ = [("ctas_per_sm", ctypes.c_int32), ("items_per_fetch", ctypes.c_int32),
                ("ms_per_step", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Batch:
    """A batched ensemble (wraps lsh_batch): scenarios with their own
    parameters and grid sizes, advanced together."""

    def __init__(self, params_list, device: int = 0):
        self.lib = load()
        self.params = [p.copy() for p in params_list]
        arr = (LshParams * len(self.params))(*self.params)
        self._b = ctypes.c_void_p()
        _check(self.lib.lsh_batch_create(arr, len(self.params), int(device), ctypes.byref(self._b)),
               "lsh_batch_create")

    def close(self):
        if self._b:
            self.lib.lsh_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_state(self, s, state):
        p = self.params[s]
        arrs = [np.ascontiguousarray(state[v] if isinstance(state, dict) else state[i], dtype=np.float64)
                for i, v in enumerate(VARS)]
        for a in arrs:
            if a.size != p.nx * p.ny:
                raise ValueError("state array size does not match nx*ny")
        dt = ctypes.c_double()
        _check(self.lib.lsh_batch_set_state(self._b, int(s), _ptr_array([a.ctypes.data for a in arrs]),
                                            ctypes.byref(dt)), "lsh_batch_set_state")
        return dt.value

    def step(self, n=1):
        _check(self.lib.lsh_batch_step(self._b, int(n)), "lsh_batch_step")

    def synchronize(self):
        _check(self.lib.lsh_batch_synchronize(self._b), "lsh_batch_synchronize")

    def get_state(self, s):
        p = self.params[s]
        out = {v: np.empty((p.ny, p.nx), dtype=np.float64) for v in VARS}
        _check(self.lib.lsh_batch_get_state(self._b, int(s), _ptr_array([out[v].ctypes.data for v in VARS])),
               "lsh_batch_get_state")
        return out

    def time(self, s):
        t, dt, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        _check(self.lib.lsh_batch_get_time(self._b, int(s), ctypes.byref(t), ctypes.byref(dt), ctypes.byref(n)),
               "lsh_batch_get_time")
        return t.value, dt.value, n.value

    def autotune(self, trial_steps=8):
        t = Tune()
        _check(self.lib.lsh_batch_autotune(self._b, int(trial_steps), ctypes.byref(t)), "lsh_batch_autotune")
        return t.as_dict()

    def set_tune(self, **kw):
        t = Tune()
        _check(self.lib.lsh_batch_get_tune(self._b, ctypes.byref(t)), "lsh_batch_get_tune")
        for k, v in kw.items():
            setattr(t, k, v)
        _check(self.lib.lsh_batch_set_tune(self._b, ctypes.byref(t)), "lsh_batch_set_tune")

    def launch_count(self):
        n = ctypes.c_longlong()
        _check(self.lib.lsh_batch_get_launch_count(self._b, ctypes.byref(n)), "lsh_batch_get_launch_count")
        return n.value


class AdjointStats(ctypes.Structure):
    """Mirror of lsh_adjoint_stats."""
    _fields_ = [("slots", ctypes.c_int32), ("nsteps", ctypes.c_int32), ("forward_steps", ctypes.c_int64),
                ("recompute_steps", ctypes.c_int64), ("reversed_steps", ctypes.c_int64), ("ms_forward", ctypes.c_double),
                ("ms_gradient", ctypes.c_double), ("slot_bytes", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


PARAM_NAMES = ("angle1", "mf0", "mfs", "r")


class Adjoint:
    """Discrete adjoint of the time loop (wraps lsh_adjoint): the gradient of
    w * sum_n sum_g (eta1_n[g] - target)^2 + <bar_final, X_N> with respect to
    the initial h1..q2y and to (angle1, mf0, mfs, r)."""

    def __init__(self, params, gauges=(), device: int = 0, _member=None):
        self.lib = load()
        self.params = params.copy()
        self.gauges = np.ascontiguousarray(np.asarray(gauges, dtype=np.int32).reshape(-1))
        self._a = ctypes.c_void_p()
        self._owner = None
        self.nsteps = 0
        if _member is not None:
            # a member of an AdjointBatch: owned (and destroyed) by it
            self._owner, handle = _member
            self._a = ctypes.c_void_p(handle)
            return
        g = self.gauges.ctypes.data if self.gauges.size else None
        _check(self.lib.lsh_adjoint_create(ctypes.byref(self.params), int(device), int(self.gauges.size), g,
                                           ctypes.byref(self._a)), "lsh_adjoint_create")

    def close(self):
        if self._a and self._owner is None:
            self.lib.lsh_adjoint_destroy(self._a)
        self._a = ctypes.c_void_p()
        self._owner = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_thin_layer(self, h_adj):
        """Thin-layer projection threshold (0: the exact adjoint)."""
        _check(self.lib.lsh_adjoint_set_thin_layer(self._a, float(h_adj)), "lsh_adjoint_set_thin_layer")

    def set_budget(self, nbytes):
        _check(self.lib.lsh_adjoint_set_budget(self._a, float(nbytes)), "lsh_adjoint_set_budget")

    def set_ordered(self, ordered=True):
        """Run every pass as a full-grid launch after the one before (no overlap)."""
        _check(self.lib.lsh_adjoint_set_ordered(self._a, int(bool(ordered))), "lsh_adjoint_set_ordered")

    def forward(self, state, nsteps, target=None):
        """Run `nsteps` from `state` (dict or 7 arrays); returns (J, eta series [nsteps, n_gauges])."""
        arrs = [np.ascontiguousarray(state[v] if isinstance(state, dict) else state[i], dtype=np.float64).reshape(-1)
                for i, v in enumerate(VARS)]
        ng = self.gauges.size
        t = None
        if target is not None:
            t = np.ascontiguousarray(target, dtype=np.float64).reshape(nsteps, ng)
        eta = np.zeros((nsteps, ng))
        J = ctypes.c_double()
        self._keep = (arrs, t)
        _check(self.lib.lsh_adjoint_forward(self._a, _ptr_array([a.ctypes.data for a in arrs]), int(nsteps),
                                            t.ctypes.data if t is not None else None, ctypes.byref(J),
                                            eta.ctypes.data if ng else None), "lsh_adjoint_forward")
        self.nsteps = nsteps
        return J.value, eta

    def gradient(self, misfit_weight=1.0, bar_final=None):
        """Returns (grad: dict h1..q2y -> (ny, nx), grad_params: dict angle1, mf0, mfs, r)."""
        p = self.params
        out = {v: np.zeros((p.ny, p.nx)) for v in VARS[:6]}
        bf = None
        if bar_final is not None:
            arrs = [None if bar_final[v] is None else np.ascontiguousarray(bar_final[v], dtype=np.float64).reshape(-1)
                    for v in VARS[:6]]
            bf = _ptr_array([0 if a is None else a.ctypes.data for a in arrs])
            self._keep_bf = arrs
        gp = np.zeros(4)
        _check(self.lib.lsh_adjoint_gradient(self._a, float(misfit_weight), bf,
                                             _ptr_array([out[v].ctypes.data for v in VARS[:6]]), gp.ctypes.data),
               "lsh_adjoint_gradient")
        return out, dict(zip(PARAM_NAMES, gp.tolist()))

    def times(self):
        """Simulated time after each step of the recorded run."""
        t = np.zeros(self.nsteps)
        _check(self.lib.lsh_adjoint_get_times(self._a, t.ctypes.data_as(DP)), "lsh_adjoint_get_times")
        return t

    def final_state(self):
        """X_N of the recorded run (after forward, before gradient)."""
        p = self.params
        out = {v: np.zeros((p.ny, p.nx)) for v in VARS[:6]}
        _check(self.lib.lsh_adjoint_get_state(self._a, _ptr_array([out[v].ctypes.data for v in VARS[:6]])),
               "lsh_adjoint_get_state")
        return out

    def stats(self):
        st = AdjointStats()
        _check(self.lib.lsh_adjoint_get_stats(self._a, ctypes.byref(st)), "lsh_adjoint_get_stats")
        return st.as_dict()


class AdjointBatch:
    """Batched adjoint (wraps lsh_adjoint_batch): scenarios on uneven grids run
    forward and reversed together under one checkpoint schedule and a joint
    memory budget; each member's results equal its own Adjoint's."""

    def __init__(self, params_list, gauges_list=None, device: int = 0):
        self.lib = load()
        n = len(params_list)
        self.params = [p.copy() for p in params_list]
        gl = gauges_list if gauges_list is not None else [()] * n
        if len(gl) != n:
            raise ValueError("one gauge list per scenario")
        self.gauges = [np.ascontiguousarray(np.asarray(g, dtype=np.int32).reshape(-1)) for g in gl]
        arr = (LshParams * n)(*self.params)
        ng = np.array([g.size for g in self.gauges], dtype=np.int32)
        gp = _ptrs([g.ctypes.data if g.size else 0 for g in self.gauges])
        self._b = ctypes.c_void_p()
        _check(self.lib.lsh_adjoint_batch_create(n, ctypes.cast(arr, P), ng.ctypes.data, gp, int(device),
                                                 ctypes.byref(self._b)), "lsh_adjoint_batch_create")
        self.n = n
        self.nsteps = 0
        self._members = {}

    def close(self):
        if self._b:
            for m in self._members.values():
                m._a = ctypes.c_void_p()
                m._owner = None
            self._members = {}
            self.lib.lsh_adjoint_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_thin_layer(self, h_adj):
        _check(self.lib.lsh_adjoint_batch_set_thin_layer(self._b, float(h_adj)), "lsh_adjoint_batch_set_thin_layer")

    def set_budget(self, nbytes):
        """Device bytes all members' checkpoint slots may take together."""
        _check(self.lib.lsh_adjoint_batch_set_budget(self._b, float(nbytes)), "lsh_adjoint_batch_set_budget")

    def forward(self, states, nsteps, targets=None):
        """Run `nsteps` from each member's state; returns (misfits [n], list of eta series [nsteps, n_gauges_i])."""
        if len(states) != self.n:
            raise ValueError("one state per scenario")
        arrs = []
        for st in states:
            arrs += [np.ascontiguousarray(st[v] if isinstance(st, dict) else st[i], dtype=np.float64).reshape(-1)
                     for i, v in enumerate(VARS)]
        tg = None
        tl = None
        if targets is not None:
            tl = [None if t is None else np.ascontiguousarray(t, dtype=np.float64).reshape(nsteps, g.size)
                  for t, g in zip(targets, self.gauges)]
            tg = _ptrs([0 if t is None else t.ctypes.data for t in tl])
        series = [np.zeros((nsteps, g.size)) for g in self.gauges]
        misfits = np.zeros(self.n)
        self._keep = (arrs, tl, series)
        _check(self.lib.lsh_adjoint_batch_forward(self._b, _ptrs([a.ctypes.data for a in arrs]), int(nsteps), tg,
                                                  misfits.ctypes.data_as(DP),
                                                  _ptrs([s.ctypes.data if s.size else 0 for s in series])),
               "lsh_adjoint_batch_forward")
        self.nsteps = nsteps
        return misfits, series

    def gradient(self, misfit_weights=None, want_state=True):
        """Returns (list of dicts h1..q2y -> (ny, nx) or None, list of dicts angle1, mf0, mfs, r)."""
        w = None
        if misfit_weights is not None:
            w = np.ascontiguousarray(misfit_weights, dtype=np.float64).reshape(self.n)
        outs = None
        gs = None
        if want_state:
            outs = [{v: np.zeros((p.ny, p.nx)) for v in VARS[:6]} for p in self.params]
            gs = _ptrs([o[v].ctypes.data for o in outs for v in VARS[:6]])
        gp = np.zeros((self.n, 4))
        _check(self.lib.lsh_adjoint_batch_gradient(self._b, w.ctypes.data if w is not None else None, gs,
                                                   gp.ctypes.data), "lsh_adjoint_batch_gradient")
        return (outs if outs is not None else [None] * self.n), [dict(zip(PARAM_NAMES, r.tolist())) for r in gp]

    def stats(self):
        st = AdjointStats()
        _check(self.lib.lsh_adjoint_batch_get_stats(self._b, ctypes.byref(st)), "lsh_adjoint_batch_get_stats")
        return st.as_dict()

    def member(self, i):
        """Member i as an Adjoint owned by this batch (run on its own with the batch's slot count)."""
        if i not in self._members:
            h = ctypes.c_void_p()
            _check(self.lib.lsh_adjoint_batch_member(self._b, int(i), ctypes.byref(h)), "lsh_adjoint_batch_member")
            m = Adjoint(self.params[i], self.gauges[i], _member=(self, h.value))
            m.nsteps = self.nsteps
            self._members[i] = m
        return self._members[i]


def revolve_plan(nsteps, slots):
    """(forward steps of the checkpoint schedule, optimal recomputation count),
    or raises if the schedule does not reverse every step once, in order."""
    fw, opt = ctypes.c_longlong(), ctypes.c_longlong()
    _check(load().lsh_revolve_plan(int(nsteps), int(slots), ctypes.byref(fw), ctypes.byref(opt)), "lsh_revolve_plan")
    return fw.value, opt.value


__all__ = ["Solver", "Batch", "Tune", "Adjoint", "AdjointBatch", "revolve_plan", "LshError", "load", "device_available", "SIGNATURES", "_abi"]
