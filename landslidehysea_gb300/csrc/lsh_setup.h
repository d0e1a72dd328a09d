// lsh_setup.h -- host-side setup shared by the single-grid context, the
// allocation-free entry point and the batched ensemble: parameter checks,
// the device constant block and the per-row geometry.  One definition, so
// every path feeds the kernels bit-identical constants.
#pragma once

#include <cmath>
#include <cstddef>
#include <string>

#include "../../include/lsh.h"
#include "lsh_scheme.cuh"

namespace lsh {

// The thread's message behind lsh_last_error (defined with the C ABI).
void set_last_error(const std::string& msg);

// nullptr when `p` describes a grid the kernels accept, else the reason.
inline const char* params_problem(const lsh_params* p) {
    if (!p) return "null parameters";
    if (p->nx < 1 || p->ny < 1) return "nx and ny must be >= 1";
    if ((long long)p->nx * p->ny >= (1LL << 31) - 1024) return "grid too large for 32-bit indexing";
    if (p->order != 1 && p->order != 2) return "order must be 1 or 2";
    if (p->coords != LSH_COORDS_CARTESIAN && p->coords != LSH_COORDS_SPHERICAL) return "bad coords";
    if (p->friction_law != LSH_FRICTION_COULOMB && p->friction_law != LSH_FRICTION_POULIQUEN) return "bad friction law";
    if (p->eig_sort != 0 && p->eig_sort != 1) return "eig_sort must be 0 or 1";
    if (!(p->eps_h > 0) || !(p->gravity > 0) || !(p->r >= 0 && p->r < 1) || !(p->peso > 0) || !(p->cfl > 0) ||
        !(p->H > 0) || !(p->L > 0))
        return "eps_h, gravity, peso, cfl, L, H must be > 0 and 0 <= r < 1";
    if (p->coords == LSH_COORDS_CARTESIAN && !(p->dx > 0 && p->dy > 0)) return "dx, dy must be > 0";
    if (p->coords == LSH_COORDS_SPHERICAL &&
        !(p->dlon > 0 && p->dlat > 0 && p->radius > 0 && std::fabs(p->lat0) < 90 &&
          std::fabs(p->lat0 + p->ny * p->dlat) < 90))
        return "spherical grid needs dlon, dlat, radius > 0 and latitudes inside (-90, 90)";
    return nullptr;
}

inline Consts make_consts(const lsh_params& p) {
    Consts c{};
    c.g = p.gravity; c.r = p.r; c.gp = p.gravity * (1.0 - p.r);
    c.eps_h = p.eps_h; c.peso = p.peso; c.beta = p.beta; c.cfl = p.cfl;
    c.mu = std::fabs(std::tan(p.angle1)) * (p.L / p.H);  // defTerminoFriccion, Coulomb
    c.mfc = p.mfc; c.mf0 = p.mf0; c.mfs = p.mfs; c.vmax1 = p.vmax1; c.vmax2 = p.vmax2;
    c.L = p.L; c.H = p.H;
    c.tan1 = std::tan(p.angle1); c.tan2 = std::tan(p.angle2); c.tan3 = std::tan(p.angle3); c.tan4 = std::tan(p.angle4);
    c.borde_sup = p.borde_sup; c.borde_inf = p.borde_inf; c.borde_izq = p.borde_izq; c.borde_der = p.borde_der;
    c.omr = 1.0 - p.r;
    c.inv_gp = 1.0 / c.gp;
    c.inv_eps = 1.0 / p.eps_h;
    c.inv_peso = 1.0 / p.peso;
    c.eps_1r = p.eps_h * (1.0 + p.r);
    c.g_mf02 = (p.gravity * p.mf0) * p.mf0;
    c.g_mfs2 = (p.gravity * p.mfs) * p.mfs;
    c.sqrt_g = std::sqrt(p.gravity);
    c.law = p.friction_law; c.order = p.order; c.nx = p.nx; c.ny = p.ny; c.track_eta = p.track_eta_max;
    c.eig_sort = p.eig_sort;
    return c;
}

// Per-row geometry (the CPU oracle uses the same formulas) into one array of
// 7 rows of `stride` >= ny + 1 doubles: area, len_v, len_h (ny + 1 entries),
// tanR, wx, wy, inv_area.  Cartesian cells are dx * dy (Problema.cxx:296);
// spherical cells use the exact band area R^2 dlon (sin phi_n - sin phi_s).
inline void fill_geo(const lsh_params& p, double* g, size_t stride) {
    constexpr double kPiG = 3.14159265358979323846;
    double* area = g;
    double* len_v = g + stride;
    double* len_h = g + 2 * stride;
    double* tanR = g + 3 * stride;
    double* wx = g + 4 * stride;
    double* wy = g + 5 * stride;
    double* inv_area = g + 6 * stride;
    const int ny = p.ny;
    if (p.coords == LSH_COORDS_SPHERICAL) {
        const double d2r = kPiG / 180.0;
        const double R = p.radius, dl = p.dlon * d2r, dp = p.dlat * d2r;
        for (int y = 0; y <= ny; ++y) len_h[y] = R * std::cos((p.lat0 + y * p.dlat) * d2r) * dl;
        for (int j = 0; j < ny; ++j) {
            const double ps = (p.lat0 + j * p.dlat) * d2r, pn = (p.lat0 + (j + 1) * p.dlat) * d2r;
            const double pc = (p.lat0 + (j + 0.5) * p.dlat) * d2r;
            area[j] = R * R * dl * (std::sin(pn) - std::sin(ps));
            len_v[j] = R * dp;
            tanR[j] = std::tan(pc) / R;
            wx[j] = area[j] / (R * std::cos(pc) * dl);
            wy[j] = area[j] / (R * dp);
        }
    } else {
        for (int y = 0; y <= ny; ++y) len_h[y] = p.dx;
        for (int j = 0; j < ny; ++j) {
            area[j] = p.dx * p.dy;
            len_v[j] = p.dy;
            tanR[j] = 0.0;
            wx[j] = p.dy;
            wy[j] = p.dx;
        }
    }
    for (int j = 0; j < ny; ++j) inv_area[j] = 1.0 / area[j];
}

}  // namespace lsh
