"""ctypes mirror of include/lsh.h (structs and constants only, no library loading)."""
import ctypes
import math

LSH_OK = 0
LSH_ERR_GPU_OOM = 1
LSH_ERR_HOST_OOM = 2
LSH_ERR_INVALID = 3
LSH_ERR_CUDA = 4
LSH_ERR_NUMERIC = 5
LSH_ERR_IO = 6
LSH_ERR_NO_DEVICE = 7
LSH_ERR_TIMEOUT = 8
LSH_ERR_STALL = 9

LSH_NVARS = 7
VARS = ("h1", "q1x", "q1y", "h2", "q2x", "q2y", "H")

COORDS_CARTESIAN = 0
COORDS_SPHERICAL = 1
FRICTION_COULOMB = 0
FRICTION_POULIQUEN = 1


class LshParams(ctypes.Structure):
    """Field-for-field mirror of `lsh_params` (include/lsh.h)."""

    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
        ("order", ctypes.c_int32), ("coords", ctypes.c_int32),
        ("friction_law", ctypes.c_int32), ("track_eta_max", ctypes.c_int32),
        ("eig_sort", ctypes.c_int32),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double),
        ("lon0", ctypes.c_double), ("lat0", ctypes.c_double),
        ("dlon", ctypes.c_double), ("dlat", ctypes.c_double),
        ("radius", ctypes.c_double),
        ("borde_sup", ctypes.c_double), ("borde_inf", ctypes.c_double),
        ("borde_izq", ctypes.c_double), ("borde_der", ctypes.c_double),
        ("cfl", ctypes.c_double), ("r", ctypes.c_double),
        ("angle1", ctypes.c_double), ("angle2", ctypes.c_double),
        ("angle3", ctypes.c_double), ("angle4", ctypes.c_double),
        ("mfc", ctypes.c_double), ("mf0", ctypes.c_double), ("mfs", ctypes.c_double),
        ("vmax1", ctypes.c_double), ("vmax2", ctypes.c_double),
        ("gravity", ctypes.c_double), ("eps_h", ctypes.c_double),
        ("L", ctypes.c_double), ("H", ctypes.c_double),
        ("peso", ctypes.c_double), ("beta", ctypes.c_double),
        ("dt_min", ctypes.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}

    def copy(self):
        out = LshParams()
        ctypes.pointer(out)[0] = self
        return out


def default_params(nx=1, ny=1, **kw):
    """The reference defaults (Coulomb law, first order, Cartesian, walls,
    peso = beta = 1, eps_h = 5e-3 with H = 1), overridden by `kw`."""
    p = LshParams()
    p.nx, p.ny = nx, ny
    p.order = 1
    p.coords = COORDS_CARTESIAN
    p.friction_law = FRICTION_COULOMB
    p.track_eta_max = 0
    p.eig_sort = 0
    p.dx = p.dy = 1.0
    p.lon0 = p.lat0 = 0.0
    p.dlon = p.dlat = 0.0
    p.radius = 6378136.6
    p.borde_sup = p.borde_inf = p.borde_izq = p.borde_der = -1.0
    p.cfl = 0.9
    p.r = 0.5
    p.angle1 = p.angle2 = p.angle3 = p.angle4 = 0.0
    p.mfc = p.mf0 = p.mfs = 0.0
    p.vmax1 = p.vmax2 = 0.0
    p.gravity = 9.81
    p.eps_h = 5e-3
    p.L = p.H = 1.0
    p.peso = p.beta = 1.0
    p.dt_min = 0.0
    for k, v in kw.items():
        if k == "angle_deg":
            p.angle1 = math.radians(v)
            continue
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p
