"""ctypes mirror of include/lsh_compat.h: the data.dat loader, the NetCDF
output files and the reference-signature shallowWater() entry point.

The loader and the NetCDF writer are host code (no GPU needed);
shallow_water() runs the time loop on the GPU.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

from ._abi import LSH_NVARS, VARS, LshParams
from .solver import LshError, load

P = ctypes.c_void_p
F = ctypes.c_float
FP = ctypes.POINTER(ctypes.c_float)


class Float4(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float), ("w", ctypes.c_float)]


class Float2(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float)]


class DatoCluster(ctypes.Structure):
    """Layout of the reference's TDatoCluster (Constantes.hxx:23-43)."""
    _fields_ = [("num_volx", ctypes.c_int), ("num_voly", ctypes.c_int),
                ("datosVolumenes_1", P), ("datosVolumenes_2", P), ("eta1_maxima", P)] + \
               [(f"puntero_{i}", P) for i in range(8)]


class Problem(ctypes.Structure):
    _fields_ = [("params", LshParams),
                ("xmin", ctypes.c_double), ("xmax", ctypes.c_double), ("ymin", ctypes.c_double),
                ("ymax", ctypes.c_double), ("hmin", ctypes.c_double), ("Q", ctypes.c_double), ("T", ctypes.c_double),
                ("tiempo_tot", ctypes.c_double), ("tiempo_guardar", ctypes.c_double),
                ("leer_fichero_puntos", ctypes.c_int32), ("num_puntos_guardar", ctypes.c_int32),
                ("indice_puntos", ctypes.POINTER(ctypes.c_int32)),
                ("state", ctypes.POINTER(ctypes.c_double) * LSH_NVARS),
                ("eta1_max", ctypes.POINTER(ctypes.c_double)),
                ("nombre_bati", ctypes.c_char * 256), ("prefijo", ctypes.c_char * 512), ("error", ctypes.c_char * 512)]


SIGNATURES = {
    "lsh_load_datadat": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(Problem))]),
    "lsh_load_datadat_law": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.POINTER(Problem))]),
    "lsh_problem_free": (None, [ctypes.POINTER(Problem)]),
    "lsh_nc_create": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, FP, FP, FP, F, F, F,
                                     FP, ctypes.c_int, F, F, F, F, F, ctypes.POINTER(P)]),
    "lsh_nc_write": (ctypes.c_int, [P, F, FP, FP, FP, FP, FP, FP]),
    "lsh_nc_close": (ctypes.c_int, [P, FP]),
    "shallowWater": (ctypes.c_int, [ctypes.POINTER(DatoCluster), F, F, F, ctypes.c_char_p, ctypes.c_char_p,
                                    ctypes.c_int, ctypes.c_int] + [F] * 28 +
                     [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                      ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), ctypes.c_int]),
    "comprobarSoporteCUDA": (ctypes.c_int, []),
}

_bound = False


def lib():
    global _bound
    L = load()
    if not _bound:
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _bound = True
    return L


def _fptr(a):
    return a.ctypes.data_as(FP)


class LoadedProblem:
    """A data.dat problem (normalised units, Hmin shift applied)."""

    def __init__(self, path, friction_law=0):
        out = ctypes.POINTER(Problem)()
        st = lib().lsh_load_datadat_law(os.fsencode(path), int(friction_law), ctypes.byref(out))
        if st != 0:
            msg = out.contents.error.decode() if out else ""
            if out:
                lib().lsh_problem_free(out)
            raise LshError(st, f"lsh_load_datadat({path}): {msg}")
        pr = out.contents
        self.params = pr.params.copy()
        nx, ny = self.params.nx, self.params.ny
        self.state = {v: np.ctypeslib.as_array(pr.state[i], shape=(ny, nx)).copy() for i, v in enumerate(VARS)}
        self.eta1_max = np.ctypeslib.as_array(pr.eta1_max, shape=(ny, nx)).copy()
        self.xmin, self.xmax, self.ymin, self.ymax = pr.xmin, pr.xmax, pr.ymin, pr.ymax
        self.hmin, self.Q, self.T = pr.hmin, pr.Q, pr.T
        self.tiempo_tot, self.tiempo_guardar = pr.tiempo_tot, pr.tiempo_guardar
        self.leer_fichero_puntos = pr.leer_fichero_puntos
        n = pr.num_puntos_guardar
        self.gauges = np.ctypeslib.as_array(pr.indice_puntos, shape=(n,)).copy() if n > 0 else np.zeros(0, np.int32)
        self.nombre_bati = pr.nombre_bati.decode()
        self.prefijo = pr.prefijo.decode()
        lib().lsh_problem_free(out)


class NcOutput:
    """The six NetCDF-classic files <prefix>_{eta1,q1x,q1y,eta2,q2x,q2y}.nc."""

    def __init__(self, prefix, nombre_bati, x, y, bathymetry, tiempo_tot=0.0, cfl=0.9, r=0.5, angles_deg=(0, 0, 0, 0),
                 pouliquen=False, mfc=0.0, mf0=0.0, mfs=0.0, vmax1=0.0, vmax2=0.0):
        self.nx, self.ny = len(x), len(y)
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        b = np.ascontiguousarray(bathymetry, np.float32).reshape(self.ny, self.nx)
        ang = np.ascontiguousarray(angles_deg, np.float32)
        self._h = ctypes.c_void_p()
        st = lib().lsh_nc_create(os.fsencode(prefix), os.fsencode(nombre_bati), self.nx, self.ny, _fptr(x), _fptr(y),
                                 _fptr(b), tiempo_tot, cfl, r, _fptr(ang), int(bool(pouliquen)), mfc, mf0, mfs, vmax1,
                                 vmax2, ctypes.byref(self._h))
        if st:
            raise LshError(st, "lsh_nc_create")

    def write(self, time, eta1, q1x, q1y, eta2, q2x, q2y):
        arrs = [np.ascontiguousarray(a, np.float32) for a in (eta1, q1x, q1y, eta2, q2x, q2y)]
        st = lib().lsh_nc_write(self._h, float(time), *[_fptr(a) for a in arrs])
        if st:
            raise LshError(st, "lsh_nc_write")

    def close(self, max_height=None):
        if self._h:
            mh = None if max_height is None else np.ascontiguousarray(max_height, np.float32)
            lib().lsh_nc_close(self._h, _fptr(mh) if mh is not None else None)
            self._h = ctypes.c_void_p()


def shallow_water(problem: LoadedProblem):
    """Call the reference-signature entry point shallowWater()
    (ShallowWater.cu:125-131) on a loaded problem, as main.cxx:157-164 does.
    Returns (status, wall_seconds, final state dict (float32), eta1 max)."""
    p = problem.params
    nx, ny = p.nx, p.ny
    d1 = (Float4 * ((ny + 2) * nx))()
    d2 = (Float4 * ((ny + 2) * nx))()
    em = (Float2 * (nx * ny))()
    a1 = np.ctypeslib.as_array(d1).view(np.float32).reshape(ny + 2, nx, 4)
    a2 = np.ctypeslib.as_array(d2).view(np.float32).reshape(ny + 2, nx, 4)
    s = problem.state
    a1[1:ny + 1, :, 0] = s["h1"]; a1[1:ny + 1, :, 1] = s["q1x"]; a1[1:ny + 1, :, 2] = s["q1y"]; a1[1:ny + 1, :, 3] = s["H"]
    a2[1:ny + 1, :, 0] = s["h2"]; a2[1:ny + 1, :, 1] = s["q2x"]; a2[1:ny + 1, :, 2] = s["q2y"]; a2[1:ny + 1, :, 3] = s["H"]
    dc = DatoCluster()
    dc.num_volx, dc.num_voly = nx, ny
    dc.datosVolumenes_1 = ctypes.cast(d1, P)
    dc.datosVolumenes_2 = ctypes.cast(d2, P)
    dc.eta1_maxima = ctypes.cast(em, P)
    g = np.ascontiguousarray(problem.gauges, dtype=np.int32)
    gp = g.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if g.size else None
    wall = ctypes.c_double()
    st = lib().shallowWater(ctypes.byref(dc), problem.xmin, problem.ymin, problem.hmin, problem.nombre_bati.encode(),
                            problem.prefijo.encode(), ny, ny, p.borde_sup, p.borde_inf, p.borde_izq, p.borde_der,
                            p.dx, p.dy, p.dx * p.dy, problem.tiempo_tot, problem.tiempo_guardar, p.cfl, p.r,
                            p.angle1, p.angle2, p.angle3, p.angle4, 1.0, 1.0, p.mfc, p.mf0, p.mfs, p.vmax1, p.vmax2,
                            p.gravity, p.eps_h, p.L, p.H, problem.Q, problem.T, 1, 0, ctypes.byref(wall),
                            problem.leer_fichero_puntos, gp, None, int(g.size))
    out = {"h1": a1[1:ny + 1, :, 0].copy(), "q1x": a1[1:ny + 1, :, 1].copy(), "q1y": a1[1:ny + 1, :, 2].copy(),
           "h2": a2[1:ny + 1, :, 0].copy(), "q2x": a2[1:ny + 1, :, 1].copy(), "q2y": a2[1:ny + 1, :, 2].copy()}
    eta = np.ctypeslib.as_array(em).view(np.float32).reshape(ny, nx, 2).copy()
    return st, wall.value, out, eta


def reference_units_to_deg(rad):
    return rad * 180.0 / math.pi
