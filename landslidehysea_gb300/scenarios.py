"""Seeded synthetic scenarios (the reference ships no usable input data: its one
example, PValdez/, lacks its .bat/.ini files).

Every generator returns a :class:`Scenario`: solver parameters plus the FP64
initial state (h1, q1x, q1y, h2, q2x, q2y, H), rows j = 0..ny-1, columns
i = 0..nx-1.  Depth H is positive downward; the water starts at rest
(eta1 = h1 + h2 - H = 0 where wet).  As the reference loader does for files
(Problema.cxx:463-481), depths are shifted by H -= Hmin when land (H < 0)
exists; `hmin` records the shift so outputs can add it back.

* :func:`shelf`   -- planar shelf d = 5 + 0.1 x m plus seeded Gaussian random
                     bumps, granular cap at the 100 m isobath (first-order,
                     Cartesian; the 200 x 200 case is the reference-runnable one).
* :func:`fjord`   -- spherical fjord: 2 km channel, 100-300 m deep, seeded
                     sinusoidal walls at 20 degrees inside land at +50 m, an
                     elliptic granular cap of given volume on a wall, 16 gauges
                     along the channel axis (second order).
* :func:`ensemble` -- uneven-size shelf scenarios with per-scenario seeds and
                     random friction angle, density ratio and slide volume.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from ._abi import COORDS_CARTESIAN, COORDS_SPHERICAL, VARS, default_params

EARTH_RADIUS = 6378136.6


@dataclasses.dataclass
class Scenario:
    name: str
    params: object              # _abi.LshParams
    state: dict                 # VARS -> float64 (ny, nx)
    hmin: float = 0.0
    gauges: np.ndarray | None = None   # (G, 2) int cell indices (i, j), -1 off-grid
    meta: dict = dataclasses.field(default_factory=dict)

    @property
    def nx(self):
        return self.params.nx

    @property
    def ny(self):
        return self.params.ny

    def arrays(self):
        return [np.ascontiguousarray(self.state[v], dtype=np.float64) for v in VARS]


def _smooth_noise(rng, ny, nx, corr_cells):
    """White noise convolved (periodically, by FFT) with exp(-(r/l)^2)."""
    noise = rng.standard_normal((ny, nx))
    ky = np.fft.fftfreq(ny)[:, None]
    kx = np.fft.fftfreq(nx)[None, :]
    # Fourier transform of exp(-(r/l)^2) is proportional to exp(-(pi l k)^2)
    filt = np.exp(-((math.pi * corr_cells) ** 2) * (kx * kx + ky * ky))
    field = np.real(np.fft.ifft2(np.fft.fft2(noise) * filt))
    m = np.max(np.abs(field))
    return field / m if m > 0 else field


def _shift_land(H):
    hmin = float(H.min())
    if hmin >= 0.0:
        return H, 0.0
    return H - hmin, hmin


def shelf(n=200, nx=None, ny=None, seed=0, dx=25.0, r=0.5, angle_deg=12.0, manning=0.03,
          cap_volume=None, cap_radius=400.0, cap_height=30.0, bump_amp=20.0, corr_len=500.0,
          cfl=0.9, eps_h=1e-5, order=1, borde=-1.0):
    """Planar shelf d = 5 + 0.1 x (x from the west edge, metres) plus seeded
    Gaussian random bumps (max |bump| = bump_amp, correlation length corr_len),
    water at rest, granular cap h2 = cap_height*max(0, 1-(r/R)^2) centred on
    the mid-row cell whose depth is closest to 100 m.  `cap_volume` (m^3), if
    given, sets R = sqrt(2 V / (pi cap_height))."""
    nx = nx or n
    ny = ny or n
    rng = np.random.default_rng(seed)
    x = (np.arange(nx) + 0.5) * dx
    y = (np.arange(ny) + 0.5) * dx
    d = np.broadcast_to(5.0 + 0.1 * x[None, :], (ny, nx)).copy()
    d += bump_amp * _smooth_noise(rng, ny, nx, corr_len / dx)
    jc = ny // 2
    ic = int(np.argmin(np.abs(d[jc] - 100.0)))
    if cap_volume is not None:
        cap_radius = math.sqrt(2.0 * cap_volume / (math.pi * cap_height))
    rr = np.hypot(x[None, :] - x[ic], y[:, None] - y[jc])
    h2 = cap_height * np.maximum(0.0, 1.0 - (rr / cap_radius) ** 2)
    h2 = np.where(d > 0.0, h2, 0.0)
    h1 = np.maximum(d - h2, 0.0)
    H, hmin = _shift_land(d)
    z = np.zeros((ny, nx))
    p = default_params(nx, ny, order=order, dx=dx, dy=dx, cfl=cfl, r=r, angle_deg=angle_deg,
                       mf0=manning, mfs=manning, mfc=0.0, eps_h=eps_h, gravity=9.81,
                       borde_sup=borde, borde_inf=borde, borde_izq=borde, borde_der=borde)
    state = {"h1": h1, "q1x": z.copy(), "q1y": z.copy(), "h2": h2, "q2x": z.copy(), "q2y": z.copy(), "H": H}
    return Scenario(f"shelf{nx}x{ny}_s{seed}", p, state, hmin,
                    meta={"cap_cell": (ic, jc), "cap_radius": cap_radius,
                          "slide_volume": float((h2 * dx * dx).sum())})


def fjord(n=2048, seed=0, dcell_deg=0.0002, lat_c=60.0, lon_c=10.0, r=0.48, angle_deg=10.0,
          manning=0.025, volume=2.0e7, width=2000.0, depth_s=100.0, depth_n=300.0, wall_deg=20.0,
          land=50.0, cfl=0.5, eps_h=1e-5, order=2, n_gauges=16, borde=1.0):
    """Spherical fjord (0.0002 degree cells at lat_c): a `width` channel along
    the meridian whose axis depth runs depth_s -> depth_n from the south to
    the north edge, centreline x_c(y) = A sin(2 pi y / lam + phi) with seeded
    A, lam, phi, walls sloping at wall_deg up to land at +land metres.  The
    slide is a seeded elliptic cap of `volume` m^3 on one wall at half the
    axis depth (footprint 1 - 1.2 km by 0.5 - 0.7 km, shrunk to 1/20 of a
    small domain; thickness at most 0.9 of the depth at its centre, so the
    centre starts submerged while the upslope rim can stand above the water
    on the steep wall -- 715 of the 2685 slide cells at 2048^2; meta["volume"]
    is what it holds); 16 gauges sit on the
    channel axis."""
    rng = np.random.default_rng(seed)
    nx = ny = n
    d2r = math.pi / 180.0
    lat0 = lat_c - 0.5 * n * dcell_deg
    lon0 = lon_c - 0.5 * n * dcell_deg
    latc = lat0 + (np.arange(ny) + 0.5) * dcell_deg
    lonc = lon0 + (np.arange(nx) + 0.5) * dcell_deg
    # local metric coordinates of the cell centres (metres from the domain centre)
    xm = EARTH_RADIUS * math.cos(lat_c * d2r) * (lonc - lon_c) * d2r
    ym = EARTH_RADIUS * (latc - lat_c) * d2r
    amp = rng.uniform(300.0, 800.0)
    lam = rng.uniform(8000.0, 16000.0)
    phase = rng.uniform(0.0, 2.0 * math.pi)
    xc = amp * np.sin(2.0 * math.pi * ym / lam + phase)                  # (ny,)
    yspan = ym[-1] - ym[0] if ny > 1 else 1.0
    daxis = depth_s + (depth_n - depth_s) * (ym - ym[0]) / yspan          # (ny,)
    s = np.abs(xm[None, :] - xc[:, None])
    half = 0.5 * width
    slope = math.tan(wall_deg * d2r)
    depth = np.where(s <= half, daxis[:, None], daxis[:, None] - slope * (s - half))
    depth = np.maximum(depth, -land)
    # slide: elliptic cap on one wall at half the local axis depth
    js = int(rng.integers(ny // 3, max(ny // 3 + 1, 2 * ny // 3)))
    side = 1.0 if rng.uniform() < 0.5 else -1.0
    sw = half + 0.5 * daxis[js] / slope
    xs, ys = xc[js] + side * sw, ym[js]
    a_len = rng.uniform(500.0, 700.0)
    b_wid = rng.uniform(250.0, 350.0)
    # a footprint within 1/20 of a small domain, but at least 3 cells
    a_len = max(min(a_len, (ym[-1] - ym[0]) / 20.0), 3.0 * EARTH_RADIUS * dcell_deg * d2r)
    b_wid = max(min(b_wid, (xm[-1] - xm[0]) / 20.0), 3.0 * EARTH_RADIUS * math.cos(lat_c * d2r) * dcell_deg * d2r)
    shape = np.maximum(0.0, 1.0 - ((xm[None, :] - xs) / b_wid) ** 2 - ((ym[:, None] - ys) / a_len) ** 2)
    # exact spherical cell areas
    lat_e = lat0 + np.arange(ny + 1) * dcell_deg
    area_row = EARTH_RADIUS ** 2 * (dcell_deg * d2r) * (np.sin(lat_e[1:] * d2r) - np.sin(lat_e[:-1] * d2r))
    vol_unit = float((shape * area_row[:, None]).sum())
    thick = volume / vol_unit if vol_unit > 0 else 0.0
    # at most 0.9 of the water depth where it is centred (its centre submerged)
    # (half the axis depth); a thinner cap carries less than `volume`
    thick = min(thick, 0.9 * 0.5 * daxis[js])
    volume = thick * vol_unit
    h2 = thick * shape
    h1 = np.maximum(depth - h2, 0.0)
    h2 = np.where(depth > -land, h2, 0.0)
    H, hmin = _shift_land(depth)
    z = np.zeros((ny, nx))
    gy = np.linspace(0.5 * yspan / n_gauges, yspan - 0.5 * yspan / n_gauges, n_gauges) + ym[0]
    gj = np.clip(np.searchsorted(ym, gy), 0, ny - 1)
    gi = np.clip(np.searchsorted(xm, xc[gj]), 0, nx - 1)
    p = default_params(nx, ny, order=order, coords=COORDS_SPHERICAL, lon0=lon0, lat0=lat0,
                       dlon=dcell_deg, dlat=dcell_deg, radius=EARTH_RADIUS, cfl=cfl, r=r,
                       angle_deg=angle_deg, mf0=manning, mfs=manning, mfc=0.0, eps_h=eps_h,
                       gravity=9.81, borde_sup=borde, borde_inf=borde, borde_izq=borde, borde_der=borde)
    state = {"h1": h1, "q1x": z.copy(), "q1y": z.copy(), "h2": h2, "q2x": z.copy(), "q2y": z.copy(), "H": H}
    return Scenario(f"fjord{n}_s{seed}", p, state, hmin, gauges=np.stack([gi, gj], axis=1),
                    meta={"amp": amp, "lambda": lam, "phase": phase, "slide_thickness": thick,
                          "slide_cell": (int(np.argmin(np.abs(xm - xs))), js), "volume": volume,
                          "wet_fraction": float((h1 + h2 > 0).mean())})


ENSEMBLE_SIZES = (128, 256, 512, 768)


def ensemble_member(k, seed0=0, sizes=ENSEMBLE_SIZES, order=2, cfl=0.5):
    """Scenario k of :func:`ensemble`, on its own (ensembles split over GPUs
    build only their share)."""
    rng = np.random.default_rng(1_000_003 + seed0 + k)
    n = int(sizes[int(rng.integers(0, len(sizes)))])
    ang = float(rng.uniform(8.0, 20.0))
    rr = float(rng.uniform(0.45, 0.6))
    vol = float(math.exp(rng.uniform(math.log(1e6), math.log(1e8))))
    return shelf(n=n, seed=seed0 + k, r=rr, angle_deg=ang, cap_volume=vol, order=order, cfl=cfl)


def ensemble(count=256, seed0=0, sizes=ENSEMBLE_SIZES, order=2, cfl=0.5, ids=None):
    """`count` shelf scenarios, scenario k seeded with seed0 + k: size drawn
    uniformly from `sizes`, Coulomb angle ~ U[8, 20] deg, r ~ U[0.45, 0.6],
    slide volume ~ log-U[1e6, 1e8] m^3 (cap radius scaled to match).  `ids`:
    only those members."""
    ks = range(count) if ids is None else ids
    return [ensemble_member(k, seed0, sizes, order, cfl) for k in ks]


CALIBRATION_SIZES = (256, 512, 768, 1024)


def calibration_member(k, seed0=0, sizes=CALIBRATION_SIZES, order=2):
    """Scenario k of a batched calibration: the fjord generator with seed
    seed0 + k on a grid drawn uniformly from `sizes`, plus its twin's
    parameters (Coulomb angle, Manning coefficients and density ratio
    scaled by seeded +-5%), whose gauge series is the calibration target.
    Returns (scenario, twin parameters)."""
    import copy
    rng = np.random.default_rng(2_000_003 + seed0 + k)
    n = int(sizes[int(rng.integers(0, len(sizes)))])
    sc = fjord(n=n, seed=seed0 + k, order=order)
    f = 1.0 + 0.05 * rng.choice([-1.0, 1.0], 4)
    twin = copy.copy(sc.params)
    p = sc.params
    twin.angle1, twin.mf0, twin.mfs, twin.r = p.angle1 * f[0], p.mf0 * f[1], p.mfs * f[2], p.r * f[3]
    return sc, twin


def gauge_cells(sc):
    """Flat cell indices of a scenario's gauges that lie on the grid."""
    p = sc.params
    return np.array([int(j) * p.nx + int(i) for i, j in sc.gauges if i >= 0 and j >= 0], dtype=np.int32)

