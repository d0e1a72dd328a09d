// lsh_oracle.cpp -- TEST INFRASTRUCTURE: the FP64 CPU oracle.
//
// Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
// leg load this library, and only as the checker or as the timed CPU
// baseline.  The product (landslidehysea_gb300) never links, loads or calls it.
//
// It restates in double precision the two-layer scheme of LandSlide-HySEA's
// GPU solver (water layer: shallow-water equations; granular layer:
// Savage-Hutter), a path-conservative PVM/IFCP Roe-type finite-volume method:
//   edge flux           src/GPU/Arista_kernel.cu:324-645  (procesarArista)
//     flux / pressure   src/GPU/Arista_kernel.cu:62-150   (getFlujo_1dC, terminosPresion1D[Mod])
//     eigenvalues       src/GPU/Arista_kernel.cu:152-237  (aproximarAutovalores1D)
//     identity mod.     src/GPU/Arista_kernel.cu:239-276  (identityModification)
//     wet/dry fix       src/GPU/Arista_kernel.cu:301-321  (tratamientoSecoMojado)
//     friction law      src/GPU/Arista_kernel.cu:11-58    (defTerminoFriccion)
//   edge index maps     src/GPU/Arista_kernel.cu:651-838  (procesarAristasGPU)
//   initial dt pass     src/GPU/Arista_kernel.cu:1040-1127 (procesarAristaDeltaTInicial)
//   state update        src/GPU/Volumen_kernel.cu:7-180, 215-284
//   step ordering       src/GPU/ShallowWater.cu:236-263, 266-461
// and adds the numerics the reference lacks, defined by this project:
// second order (minmod MUSCL on eta1, q, eta2, q2, H + Heun TVD-RK2 with a
// cell-midpoint volume integral of the non-conservative pressure product) and
// spherical cells (exact cell areas, latitude-dependent edge lengths,
// tan(phi)/R metric source).
//
// Floating-point conventions shared with the CUDA kernels (so that both are
// the same FP64 scheme up to rounding):
//   * the reference's EPSILON (FLT_EPSILON, Constantes.hxx:13) keeps its value;
//   * the desingularised velocity u = sqrt(2) h q / sqrt(h^4 + max(h,eps_h)^4)
//     is evaluated as vfac(h) * q with vfac(h) = sqrt(2) h / sqrt(h^4 + m^4),
//     and h^4 as (h*h)*(h*h);
//   * exp, cbrt and log come from landslidehysea_gb300/csrc/lsh_fpmath.h, which
//     uses IEEE basic operations only (no vendor libm), so host and device agree
//     bit for bit; h^(4/3) is h*cbrt(h).
// Built with -ffp-contract=off (the CUDA side with --fmad=false), so x86, Arm
// and the GPU evaluate the same operation sequence and give identical bits.

#include "../include/lsh.h"
#include "../landslidehysea_gb300/csrc/lsh_fpmath.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

constexpr double kEps = 1.1920928955078125e-07;  // FLT_EPSILON, Constantes.hxx:13
constexpr double kSqrt2 = 1.41421356237309504880;
constexpr double kBig = 1e30;                       // "no limit" dt, Volumen_kernel.cu:226,256
constexpr double kPi = 3.14159265358979323846;

using std::fabs;
using std::sqrt;
using std::tan;

struct Consts {
    double g, r, gp, eps_h, peso, beta, cfl, mu, mfc, mf0, mfs, vmax1, vmax2, L, H;
    double tan1, tan2, tan3, tan4;
    int law;
    int eig_sort;
};

struct Geo {
    int nx, ny;
    std::vector<double> area;    // [ny]   cell area of row j
    std::vector<double> len_v;   // [ny]   length of the vertical edges of row j
    std::vector<double> len_h;   // [ny+1] length of horizontal edge row y
    std::vector<double> tanR;    // [ny]   tan(lat_j)/R, 0 for Cartesian
    std::vector<double> wx, wy;  // [ny]   second-order volume-integral weights
};

static Consts make_consts(const lsh_params& p) {
    Consts c;
    c.g = p.gravity; c.r = p.r; c.gp = p.gravity * (1.0 - p.r);
    c.eps_h = p.eps_h; c.peso = p.peso; c.beta = p.beta; c.cfl = p.cfl;
    // defTerminoFriccion, Coulomb law (Arista_kernel.cu:11-16): |tan(angle1)| * L/H
    c.mu = fabs(tan(p.angle1)) * (p.L / p.H);
    c.mfc = p.mfc; c.mf0 = p.mf0; c.mfs = p.mfs; c.vmax1 = p.vmax1; c.vmax2 = p.vmax2;
    c.L = p.L; c.H = p.H;
    c.tan1 = tan(p.angle1); c.tan2 = tan(p.angle2); c.tan3 = tan(p.angle3); c.tan4 = tan(p.angle4);
    c.law = p.friction_law;
    c.eig_sort = p.eig_sort;
    return c;
}

static Geo make_geo(const lsh_params& p) {
    Geo g;
    g.nx = p.nx; g.ny = p.ny;
    g.area.resize(p.ny); g.len_v.resize(p.ny); g.len_h.resize(p.ny + 1);
    g.tanR.resize(p.ny); g.wx.resize(p.ny); g.wy.resize(p.ny);
    if (p.coords == LSH_COORDS_SPHERICAL) {
        const double d2r = kPi / 180.0;
        const double R = p.radius, dl = p.dlon * d2r, dp = p.dlat * d2r;
        for (int y = 0; y <= p.ny; ++y) g.len_h[y] = R * std::cos((p.lat0 + y * p.dlat) * d2r) * dl;
        for (int j = 0; j < p.ny; ++j) {
            const double ps = (p.lat0 + j * p.dlat) * d2r, pn = (p.lat0 + (j + 1) * p.dlat) * d2r;
            const double pc = (p.lat0 + (j + 0.5) * p.dlat) * d2r;
            g.area[j] = R * R * dl * (std::sin(pn) - std::sin(ps));
            g.len_v[j] = R * dp;
            g.tanR[j] = std::tan(pc) / R;
            g.wx[j] = g.area[j] / (R * std::cos(pc) * dl);
            g.wy[j] = g.area[j] / (R * dp);
        }
    } else {
        for (int y = 0; y <= p.ny; ++y) g.len_h[y] = p.dx;
        for (int j = 0; j < p.ny; ++j) {
            g.area[j] = p.dx * p.dy;  // Problema.cxx:296
            g.len_v[j] = p.dy;
            g.tanR[j] = 0.0;
            g.wx[j] = p.dy;
            g.wy[j] = p.dx;
        }
    }
    return g;
}

// ---------------------------------------------------------------- helpers
template <class T> inline T tmin(const T& a, const T& b) { return (b < a) ? b : a; }
template <class T> inline T tmax(const T& a, const T& b) { return (b > a) ? b : a; }
template <class T> inline T max0(const T& a) { return (a > 0.0) ? a : T(0.0); }

inline double exp_neg(double x) { return lshm::exp_neg(x); }

// sqrt(2) h / sqrt(h^4 + max(h, eps_h)^4): the desingularised 1/h factor
// (Arista_kernel.cu:74,380; Volumen_kernel.cu:13,44,48)
template <class T> inline T vfac(const T& h, double eps_h) {
    const T m = (h > eps_h) ? h : T(eps_h);
    const T h2 = h * h, m2 = m * m;
    return (kSqrt2 * h) / sqrt(h2 * h2 + m2 * m2);
}

template <class T> inline T pow43(const T& h) { return h * lshm::cbrt_pos(h); }

inline int sgn(double x) { return (fabs(x) < kEps) ? 0 : ((x > 0) ? 1 : -1); }  // Constantes.hxx:14

template <class T> struct V4 { T x, y, z, w; };

// The fixed compare-and-swap sequence of Arista_kernel.cu:193-234, including
// its (i=2, j=1) compare, which leaves the larger of y/z in y (eig_sort 0);
// with eig_sort 1 that compare is (1,2) and the sequence is a true sort.
template <class T> inline void sort_eig(V4<T>& D, int full) {
    auto cs = [](T& a, T& b) { if (a > b) { T t = b; b = a; a = t; } };
    cs(D.x, D.y); cs(D.x, D.z); cs(D.x, D.w); cs(D.y, D.z); cs(D.y, D.w);
    if (full) cs(D.y, D.z);
    else if (D.z > D.y) { T t = D.y; D.y = D.z; D.z = t; }
    cs(D.z, D.w);
}

// aproximarAutovalores1D (Arista_kernel.cu:152-237).  conserved == false:
// (a1, a2) are the edge-averaged normal velocities (flag 0); conserved == true:
// (a1, a2) are the rotated normal discharges of one cell (flag 1).
template <class T>
inline V4<T> eig(const T& h1, const T& a1, const T& h2, const T& a2, bool conserved, const Consts& c) {
    const T h = h1 + h2;
    const T F = vfac(h, c.eps_h);
    T u1, u2, q;
    if (conserved) { q = a1 + a2; u1 = vfac(h1, c.eps_h) * a1; u2 = vfac(h2, c.eps_h) * a2; }
    else           { q = h1 * a1 + h2 * a2; u1 = a1; u2 = a2; }
    const T u = q * F;
    const T cg = sqrt(c.g * h);
    const T uu = (u1 * h2 + u2 * h1) * F;
    const T d = u1 - u2;
    const T aux = 1.0 - d * d * F / c.gp;
    const T ci = sqrt(c.gp * h1 * h2 * F * fabs(aux));
    V4<T> D{u - cg, uu - ci, uu + ci, u + cg};
    sort_eig(D, c.eig_sort);
    return D;
}

// defTerminoFriccion (Arista_kernel.cu:11-58): friction coefficient mu.
template <class T>
inline T friction_mu(const T& h1, const T& u1, const T& h2, const T& u2, const Consts& c) {
    if (c.law == LSH_FRICTION_COULOMB) return T(c.mu);
    // Pouliquen law (the reference's #ifndef COULOMB branch)
    const T a = 10.0 * h1 / c.eps_h;
    const T rr = 1.0 - c.r * (1.0 - exp_neg(a * a));
    const T gp = c.g * rr;
    const T fr1 = u1 * u1 * vfac(h1, c.eps_h) / gp;
    const T fr2 = u2 * u2 * vfac(h2, c.eps_h) / gp;
    const T fr = sqrt(fr1 + fr2 + (1.0 - rr) * fr1 * fr2);
    const double beta = 0.136, L2 = 8.0e-4, chi = 1.0e-3;
    const T mustop = c.tan1 + (c.tan2 - c.tan1) / (1.0 + h2 / L2);
    const T mustart = c.tan3 + (c.tan4 - c.tan3) / (1.0 + h2 / L2);
    T muf;
    if (fr > beta) muf = c.tan1 + (c.tan2 - c.tan1) / (1.0 + beta * h2 / (fr * L2));
    else if (fabs(fr) < kEps) muf = c.tan3 + (c.tan4 - c.tan3) / (1.0 + h2 / L2);
    else muf = mustart + lshm::pow_pos(fr / beta, chi) * (mustop - mustart);
    return muf * c.L / c.H;
}

// 1 - r (1 - exp(-(10 h1 / eps_h)^2)) (Arista_kernel.cu:136, Volumen_kernel.cu:15)
template <class T> inline T fsc_of(const T& h1, const Consts& c) {
    const T a = 10.0 * h1 / c.eps_h;
    return 1.0 - c.r * (1.0 - exp_neg(a * a));
}

// ---------------------------------------------------------------- edge flux
// Inputs of one edge.  W0 / W1 are the two states facing the edge (cell
// values at first order, reconstructed face values at second order; W1 is the
// ghost at a boundary); hc* are the cell-average depths and acc*h the partial
// accumulators (h1, h2) the positivity limiter reads.
template <class T> struct EdgeIn {
    T W0[6], W1[6];
    T H0, H1;
    double nx, ny, len, area0, area1;
    bool interior;
    T hc0[2], hc1[2];
    T acc0h[2], acc1h[2];
};

// procesarArista (Arista_kernel.cu:324-645).  Returns false for a dry edge
// (no contribution at all, :397).  d0 / d1 are subtracted from the
// accumulators of cell 0 / cell 1 (already multiplied by peso), `wave` is
// added to their dt accumulator.
template <class T>
bool edge_flux(const EdgeIn<T>& e, const T& dt, const Consts& c, T d0[6], T d1[6], T& wave) {
    const double nx = e.nx, ny = e.ny, eps = c.eps_h;
    V4<T> A{e.W0[0], e.W0[1] * nx + e.W0[2] * ny, e.W0[3], e.W0[4] * nx + e.W0[5] * ny};
    V4<T> B{e.W1[0], e.W1[1] * nx + e.W1[2] * ny, e.W1[3], e.W1[4] * nx + e.W1[5] * ny};
    const T H0 = e.H0, H1 = e.H1;

    // tratamientoSecoMojado (Arista_kernel.cu:301-321)
    if ((A.z < eps) && (H1 - B.z > H0)) B.w = 0.0;
    if ((B.z < eps) && (H0 - A.z > H1)) A.w = 0.0;
    if ((A.x < eps) && (H1 - B.x - B.z > H0 - A.z)) B.y = 0.0;
    if ((B.x < eps) && (H0 - A.x - A.z > H1 - B.z)) A.y = 0.0;
    if ((A.z + A.x < eps) && (H1 - B.x - B.z > H0)) { B.y = 0.0; B.w = 0.0; }
    if ((B.z + B.x < eps) && (H0 - A.x - A.z > H1)) { A.y = 0.0; A.w = 0.0; }

    // Roe-type averages (Arista_kernel.cu:375-395)
    const T fA1 = vfac(A.x, eps), fB1 = vfac(B.x, eps);
    const T fA2 = vfac(A.z, eps), fB2 = vfac(B.z, eps);
    const T h1ij = 0.5 * (A.x + B.x);
    T sa = sqrt(A.x), sb = sqrt(B.x);
    const T u1ij = (sa * (fA1 * A.y) + sb * (fB1 * B.y)) / (sa + sb + kEps);
    const T h2ij = 0.5 * (A.z + B.z);
    sa = sqrt(A.z); sb = sqrt(B.z);
    const T u2ij = (sa * (fA2 * A.w) + sb * (fB2 * B.w)) / (sa + sb + kEps);

    if (!((h1ij >= kEps) || (h2ij >= kEps))) return false;  // :397

    // hydrostatic reconstruction (terminosPresion1D, :94-115)
    const T Hm = tmin(H0, H1);
    const T deta1 = max0(B.x + B.z - H1 + Hm) - max0(A.x + A.z - H0 + Hm);
    const T deta2 = max0(B.z - H1 + Hm) - max0(A.z - H0 + Hm);
    V4<T> tp{T(0.0), c.g * h1ij * deta1, T(0.0), c.g * h2ij * ((1.0 - c.r) * deta2 + c.r * deta1)};

    // edge Coulomb switch (terminosPresion1DMod :134-147, identityModification :259-264)
    const T mu = friction_mu(h1ij, u1ij, h2ij, u2ij, c);
    const T sc = fsc_of(h1ij, c) * mu * c.g * h2ij;
    const bool coul = fabs(h2ij * u2ij) < c.peso * sc * dt;
    V4<T> tp2 = tp;
    if (coul) tp2.w = c.g * h2ij * c.r * deta1;

    // eigenvalue bounds (:427-444)
    const V4<T> D = eig(h1ij, u1ij, h2ij, u2ij, false, c);
    const V4<T> E0 = eig(A.x, A.y, A.z, A.w, true, c);
    const V4<T> E1 = eig(B.x, B.y, B.z, B.w, true, c);
    const T aut1 = tmin(D.x, tmin(E0.x, E1.x));
    const T aut3 = tmax(D.w, tmax(E0.w, E1.w));
    T lmax = tmax(fabs(aut3), fabs(aut1));
    const T umax = tmax(fabs(u1ij), fabs(u2ij));
    if (umax > lmax) lmax = umax;
    T aut2 = tmax(fabs(D.y), fabs(D.z));
    if (sgn(double(aut1 + aut3)) < 0) aut2 = -aut2;

    // PVM / IFCP coefficients (:446-465)
    T a0, a1, a2;
    if ((fabs(aut1 - aut3) >= kEps) && (fabs(aut1 - aut2) >= kEps) && (fabs(aut2 - aut3) >= kEps)) {
        if ((h1ij >= eps) && (h2ij >= eps)) {
            const T a = fabs(aut1) / ((aut1 - aut3) * (aut1 - aut2));
            const T b = fabs(aut2) / ((aut2 - aut1) * (aut2 - aut3));
            const T cc = fabs(aut3) / ((aut3 - aut1) * (aut3 - aut2));
            a0 = a * aut2 * aut3 + b * aut1 * aut3 + cc * aut1 * aut2;
            a1 = -a * (aut2 + aut3) - b * (aut1 + aut3) - cc * (aut1 + aut2);
            a2 = a + b + cc;
        } else {
            a0 = (aut3 * fabs(aut1) - aut1 * fabs(aut3)) / (aut3 - aut1);
            a1 = (fabs(aut3) - fabs(aut1)) / (aut3 - aut1);
            a2 = 0.0;
        }
    } else {
        a0 = lmax; a1 = 0.0; a2 = 0.0;
    }

    // physical fluxes (getFlujo_1dC :62-92)
    const V4<T> FA{A.y, (A.x < kEps) ? T(0.0) : (fA1 * A.y) * A.y, A.w, (A.z < kEps) ? T(0.0) : (fA2 * A.w) * A.w};
    const V4<T> FB{B.y, (B.x < kEps) ? T(0.0) : (fB1 * B.y) * B.y, B.w, (B.z < kEps) ? T(0.0) : (fB2 * B.w) * B.w};
    const V4<T> dF{FB.x - FA.x, FB.y - FA.y, FB.z - FA.z, FB.w - FA.w};
    tp2 = V4<T>{tp2.x + dF.x, tp2.y + dF.y, tp2.z + dF.z, tp2.w + dF.w};
    const V4<T> half{0.5 * (dF.x + tp.x), 0.5 * (dF.y + tp.y), 0.5 * (dF.z + tp.z), 0.5 * (dF.w + tp.w)};

    // A * tp2 (:476-482)
    const T ga = c.g * h1ij, gb = c.g * h2ij;
    const V4<T> At{tp2.y,
                   (ga - u1ij * u1ij) * tp2.x + 2.0 * u1ij * tp2.y + ga * tp2.z,
                   tp2.w,
                   c.r * gb * tp2.x + (gb - u2ij * u2ij) * tp2.z + 2.0 * u2ij * tp2.w};

    // identityModification (:239-276)
    V4<T> I{deta1, B.y - A.y, T(0.0), B.w - A.w};
    if (!coul) {
        if ((A.x > eps) && (B.x > eps)) I.x = I.x - deta2;
        I.z = deta2;
    }

    // viscosity and the two one-sided fluxes (:488-504)
    const V4<T> Q{0.5 * (a0 * I.x + a1 * tp2.x + a2 * At.x), 0.5 * (a0 * I.y + a1 * tp2.y + a2 * At.y),
                  0.5 * (a0 * I.z + a1 * tp2.z + a2 * At.z), 0.5 * (a0 * I.w + a1 * tp2.w + a2 * At.w)};
    const V4<T> Fm{half.x + (FA.x - Q.x), half.y + (FA.y - Q.y), half.z + (FA.z - Q.z), half.w + (FA.w - Q.w)};
    const V4<T> Fp{half.x + (Q.x - FB.x), half.y + (Q.y - FB.y), half.z + (Q.z - FB.z), half.w + (Q.w - FB.w)};

    // upwinded tangential velocity (:506-532)
    const T ut0 = fA1 * (e.W0[2] * nx - e.W0[1] * ny), ut1 = fB1 * (e.W1[2] * nx - e.W1[1] * ny);
    const T u1t = (fabs(Fm.x) < kEps) ? T(0.0) : ((Fm.x > 0.0) ? ut0 : ut1);
    const T vt0 = fA2 * (e.W0[5] * nx - e.W0[4] * ny), vt1 = fB2 * (e.W1[5] * nx - e.W1[4] * ny);
    const T u2t = (fabs(Fm.z) < kEps) ? T(0.0) : ((Fm.z > 0.0) ? vt0 : vt1);

    // rotate back and scale by the edge length (:534-552)
    const T s1 = Fm.x * u1t, s2 = Fm.z * u2t;
    T P[6] = {Fp.x, Fp.y * nx + s1 * ny, Fp.y * ny - s1 * nx, Fp.z, Fp.w * nx + s2 * ny, Fp.w * ny - s2 * nx};
    T M[6] = {Fm.x, Fm.y * nx - s1 * ny, Fm.y * ny + s1 * nx, Fm.z, Fm.w * nx - s2 * ny, Fm.w * ny + s2 * nx};
    for (int k = 0; k < 6; ++k) { P[k] = e.len * P[k]; M[k] = e.len * M[k]; }

    // positivity limiter on the partially accumulated depths (:554-609)
    const T b0 = dt / e.area0;
    const T hp00 = e.hc0[0] + b0 * e.acc0h[0], hp01 = e.hc0[1] + b0 * e.acc0h[1];
    T hp10 = 0.0, hp11 = 0.0;
    if (e.interior) {
        const T b1 = dt / e.area1;
        hp10 = e.hc1[0] + b1 * e.acc1h[0]; hp11 = e.hc1[1] + b1 * e.acc1h[1];
    }
    const double factor = 1.0 * c.beta;
    for (int layer = 0; layer < 2; ++layer) {
        const int k = 3 * layer;
        T dta = kBig, dtb = kBig;
        if (M[k] > 0.0) dta = (layer ? hp01 : hp00) * e.area0 / (factor * M[k] + kEps);
        if (e.interior && P[k] > 0.0) dtb = (layer ? hp11 : hp10) * e.area1 / (factor * P[k] + kEps);
        const T dtl = tmin(dta, dtb);
        if (!(dt <= dtl)) {
            const T alpha = dtl / (dt + kEps);
            for (int q = k; q < k + 3; ++q) { M[q] = alpha * M[q]; P[q] = alpha * P[q]; }
        }
    }

    if (lmax < eps) lmax = lmax + eps;  // :611-612
    wave = e.len * lmax / c.peso;
    for (int k = 0; k < 6; ++k) { d0[k] = c.peso * M[k]; d1[k] = c.peso * P[k]; }
    return true;
}

// procesarAristaDeltaTInicial (Arista_kernel.cu:1040-1127): wave-speed bound
// for the initial dt.  No wet/dry fix, no dry-edge skip, and the max of the
// signed sorted external eigenvalues (:1107).
template <class T>
T edge_initial_wave(const T W0[6], const T W1[6], double nx, double ny, double len, const Consts& c) {
    const double eps = c.eps_h;
    const V4<T> A{W0[0], W0[1] * nx + W0[2] * ny, W0[3], W0[4] * nx + W0[5] * ny};
    const V4<T> B{W1[0], W1[1] * nx + W1[2] * ny, W1[3], W1[4] * nx + W1[5] * ny};
    const T h1ij = 0.5 * (A.x + B.x);
    T sa = sqrt(A.x), sb = sqrt(B.x);
    const T u1ij = (sa * (vfac(A.x, eps) * A.y) + sb * (vfac(B.x, eps) * B.y)) / (sa + sb + kEps);
    const T h2ij = 0.5 * (A.z + B.z);
    sa = sqrt(A.z); sb = sqrt(B.z);
    const T u2ij = (sa * (vfac(A.z, eps) * A.w) + sb * (vfac(B.z, eps) * B.w)) / (sa + sb + kEps);
    const V4<T> D = eig(h1ij, u1ij, h2ij, u2ij, false, c);
    T lmax = tmax(D.x, D.w);
    const T b = tmax(fabs(u1ij), fabs(u2ij));
    if (b > lmax) lmax = b;
    if (lmax < eps) lmax = lmax + eps;
    return len * lmax;
}

// ---------------------------------------------------------------- state update
// filtroEstado (Volumen_kernel.cu:92-180); its "complex" block is dead (cf = 0).
template <class T> inline void filtro(T w[6], const T& dt, const Consts& c) {
    if (w[0] < 0.0) w[0] = 0.0;
    if (w[3] < 0.0) w[3] = 0.0;
    for (int layer = 0; layer < 2; ++layer) {
        const int k = 3 * layer;
        const T x = w[k] / c.eps_h;
        const T x2 = x * x;
        const T aux0 = 1.0 / (x2 * x2 + kEps);
        const T aux = exp_neg(dt * aux0);
        w[k + 1] = w[k + 1] * aux;
        w[k + 2] = w[k + 2] * aux;
    }
    for (int layer = 0; layer < 2; ++layer) {
        const double vmax = layer ? c.vmax2 : c.vmax1;
        if (vmax > 0.0) {
            const int k = 3 * layer;
            const T h = w[k];
            const T f = vfac(h, c.eps_h);
            T ux = f * w[k + 1], uy = f * w[k + 2];
            const T u = sqrt(ux * ux + uy * uy);
            if (u > vmax) {
                ux = ux * (vmax / u); uy = uy * (vmax / u);
                w[k + 1] = ux * h; w[k + 2] = uy * h;
            }
        }
    }
}

// disImplicita (Volumen_kernel.cu:31-90): semi-implicit interlayer and bottom
// friction.  Speeds of the previous state `wo` enter the coefficients.
template <class T> inline void dis_implicita(const T wo[6], T w[6], const T& dt, const Consts& c) {
    if (w[0] < 0.0) w[0] = 0.0;
    if (w[3] < 0.0) w[3] = 0.0;
    const double eps = c.eps_h;
    const T h1 = w[0], h2 = w[3];
    const T f1 = vfac(h1, eps), f2 = vfac(h2, eps);
    T u1x = f1 * w[1], u1y = f1 * w[2], u2x = f2 * w[4], u2y = f2 * w[5];
    const T fo1 = vfac(wo[0], eps), fo2 = vfac(wo[3], eps);
    const T uo1x = fo1 * wo[1], uo1y = fo1 * wo[2], uo2x = fo2 * wo[4], uo2y = fo2 * wo[5];
    const T dx = uo1x - uo2x, dy = uo1y - uo2y;
    const T du = sqrt(dx * dx + dy * dy);
    const T u1 = sqrt(uo1x * uo1x + uo1y * uo1y);
    const T u2 = sqrt(uo2x * uo2x + uo2y * uo2y);
    const T hmod = h2 + c.r * h1;
    const T m = (hmod > eps * (1.0 + c.r)) ? hmod : T(eps * (1.0 + c.r));
    const T hm2 = hmod * hmod, m2 = m * m;
    const T hmodm = sqrt(hm2 * hm2 + m2 * m2);
    if ((h1 > 0.0) && (h2 > 0.0)) {
        const T c1 = dt * kSqrt2 * h2 * hmod / hmodm * c.mfc * du;
        const T c2 = dt * c.r * kSqrt2 * h1 * hmod / hmodm * c.mfc * du;
        const T c3 = dt * c.g * c.mfs * c.mfs * u2 / (pow43(h2) + kEps);
        const T det = 1.0 / ((1.0 + c1) * (1.0 + c2 + c3) - c1 * c2);
        w[1] = h1 * (u1x * (1.0 + c2 + c3) + c1 * u2x) * det;
        w[4] = h2 * (u2x * (1.0 + c1) + c2 * u1x) * det;
        w[2] = h1 * (u1y * (1.0 + c2 + c3) + c1 * u2y) * det;
        w[5] = h2 * (u2y * (1.0 + c1) + c2 * u1y) * det;
    }
    if ((h1 > 0.0) && (h2 < eps)) {
        u1x = f1 * w[1]; u1y = f1 * w[2];
        const T c1 = dt * c.g * c.mf0 * c.mf0 * u1 / (pow43(h1) + kEps);
        w[1] = h1 * u1x / (1.0 + c1);
        w[2] = h1 * u1y / (1.0 + c1);
    }
    if ((h2 > 0.0) && (h1 < eps)) {
        u2x = f2 * w[4]; u2y = f2 * w[5];
        const T c1 = dt * c.g * c.mfs * c.mfs * u2 / (pow43(h2) + kEps);
        w[4] = h2 * u2x / (1.0 + c1);
        w[5] = h2 * u2y / (1.0 + c1);
    }
}

// coulomb (Volumen_kernel.cu:7-26): granular stop / slow-down.
template <class T> inline void coulomb(T w[6], const T& dt, const Consts& c) {
    T mu = c.mu;
    if (c.law != LSH_FRICTION_COULOMB) {
        const T u1 = sqrt(w[1] * w[1] + w[2] * w[2]) * vfac(w[0], c.eps_h);
        const T u2 = sqrt(w[4] * w[4] + w[5] * w[5]) * vfac(w[3], c.eps_h);
        mu = friction_mu(w[0], u1, w[3], u2, c);
    }
    const T sc = fsc_of(w[0], c) * mu * c.g * w[3] * dt * 1.0;
    const T normq = sqrt(w[4] * w[4] + w[5] * w[5]);
    T aux = 0.0;
    if ((normq + sc >= kEps) && (w[3] > 0.0)) aux = (normq >= sc) ? normq / (normq + sc) : T(0.0);
    w[4] = w[4] * aux;
    w[5] = w[5] * aux;
}

// obtenerEstadoYDeltaTVolumenesGPU (Volumen_kernel.cu:231-284) for one cell:
// per-cell dt from the wave accumulator, forward Euler stage, the spherical
// metric source (new), then filtroEstado -> disImplicita -> coulomb.
template <class T>
inline void volume_update(const T wo[6], const T acc[7], T w[6], T& dti, double area, double tanR,
                          const T& dt, const Consts& c) {
    dti = (acc[6] < kEps) ? T(kBig) : (2.0 * c.cfl * area) / acc[6];
    const T b = dt / area;
    for (int k = 0; k < 6; ++k) w[k] = wo[k] + b * acc[k];
    if (tanR != 0.0) {
        for (int layer = 0; layer < 2; ++layer) {
            const int k = 3 * layer;
            const T ux = vfac(wo[k], c.eps_h) * wo[k + 1];
            w[k + 1] = w[k + 1] + dt * (ux * wo[k + 2] * tanR);
            w[k + 2] = w[k + 2] - dt * (ux * wo[k + 1] * tanR);
        }
    }
    filtro(w, dt, c);
    dis_implicita(wo, w, dt, c);
    coulomb(w, dt, c);
}

// ---------------------------------------------------------------- solver
struct Solver {
    lsh_params p;
    Consts c;
    Geo g;
    int nx, ny;
    size_t N;
    std::vector<double> acc[7];
    std::vector<double> slope_x[7], slope_y[7];  // second order: half minmod differences
    std::vector<double> dti;

    explicit Solver(const lsh_params& prm) : p(prm), c(make_consts(prm)), g(make_geo(prm)) {
        nx = prm.nx; ny = prm.ny; N = size_t(nx) * ny;
        for (int k = 0; k < 7; ++k) acc[k].assign(N, 0.0);
        if (prm.order == 2)
            for (int k = 0; k < 7; ++k) { slope_x[k].assign(N, 0.0); slope_y[k].assign(N, 0.0); }
        dti.assign(N, kBig);
    }

    // Face value of cell `id` on side `side` (0 W, 1 E, 2 S (toward j-1), 3 N
    // (toward j+1)).  First order (or a cell whose slopes were zeroed): the
    // cell value itself.
    void face(const double* const* W, size_t id, int side, double out[6], double& Hf) const {
        if (p.order != 2) {
            for (int k = 0; k < 6; ++k) out[k] = W[k][id];
            Hf = W[6][id];
            return;
        }
        const std::vector<double>* s = (side < 2) ? slope_x : slope_y;
        const double sg = (side & 1) ? 1.0 : -1.0;
        const double de1 = s[0][id], de2 = s[3][id], dH = s[6][id];
        out[0] = W[0][id] + sg * (de1 - de2);
        out[1] = W[1][id] + sg * s[1][id];
        out[2] = W[2][id] + sg * s[2][id];
        out[3] = W[3][id] + sg * (de2 + dH);
        out[4] = W[4][id] + sg * s[4][id];
        out[5] = W[5][id] + sg * s[5][id];
        Hf = W[6][id] + sg * dH;
    }

    static double minmod(double a, double b) {
        if (a > 0.0 && b > 0.0) return (a < b) ? a : b;
        if (a < 0.0 && b < 0.0) return (a > b) ? a : b;
        return 0.0;
    }

    // minmod slopes of (eta1, q1x, q1y, eta2, q2x, q2y, H), halved, with a
    // first-order fallback for any cell whose reconstructed depths go negative.
    void reconstruct(const double* const* W) {
        const int NX = nx, NY = ny;
#pragma omp parallel for schedule(static)
        for (int j = 0; j < NY; ++j) {
            for (int i = 0; i < NX; ++i) {
                const size_t id = size_t(j) * NX + i;
                auto pv = [&](size_t q, int k) -> double {
                    switch (k) {
                        case 0: return (W[0][q] + W[3][q]) - W[6][q];
                        case 3: return W[3][q] - W[6][q];
                        case 6: return W[6][q];
                        default: return W[k][q];
                    }
                };
                double sx[7], sy[7];
                for (int k = 0; k < 7; ++k) {
                    const double pc = pv(id, k);
                    sx[k] = (i > 0 && i < NX - 1) ? 0.5 * minmod(pc - pv(id - 1, k), pv(id + 1, k) - pc) : 0.0;
                    sy[k] = (j > 0 && j < NY - 1) ? 0.5 * minmod(pc - pv(id - NX, k), pv(id + NX, k) - pc) : 0.0;
                }
                const double h1 = W[0][id], h2 = W[3][id];
                const double dh1x = sx[0] - sx[3], dh2x = sx[3] + sx[6];
                const double dh1y = sy[0] - sy[3], dh2y = sy[3] + sy[6];
                const bool bad = (h1 + dh1x < 0.0) || (h1 - dh1x < 0.0) || (h2 + dh2x < 0.0) || (h2 - dh2x < 0.0) ||
                                 (h1 + dh1y < 0.0) || (h1 - dh1y < 0.0) || (h2 + dh2y < 0.0) || (h2 - dh2y < 0.0);
                for (int k = 0; k < 7; ++k) {
                    slope_x[k][id] = bad ? 0.0 : sx[k];
                    slope_y[k][id] = bad ? 0.0 : sy[k];
                }
            }
        }
    }

    // One colour pass over horizontal (dir 0) or vertical (dir 1) edges of
    // parity `par` (Arista_kernel.cu:651-838).  Edges of one colour touch
    // disjoint cells, so the loop is race-free.
    void pass(const double* const* W, int dir, int par, double dt) {
        const int NX = nx, NY = ny;
        const int nlines = (dir == 0) ? (NY - par) / 2 + 1 : (NX - par) / 2 + 1;  // edge rows / columns
        const int nalong = (dir == 0) ? NX : NY;
#pragma omp parallel for schedule(static)
        for (int t = 0; t < nlines; ++t) {
            const int e = par + 2 * t;  // edge row y (dir 0) or column x (dir 1)
            if ((dir == 0 && e > NY) || (dir == 1 && e > NX)) continue;
            for (int s = 0; s < nalong; ++s) {
                EdgeIn<double> in;
                size_t id0, id1 = 0;
                double bor;
                int side0, side1;
                if (dir == 0) {
                    const int x = s, y = e;
                    in.len = g.len_h[y];
                    if (y == 0) { id0 = size_t(x); in.nx = 0.0; in.ny = -1.0; in.interior = false; bor = p.borde_sup; side0 = 2; }
                    else if (y == NY) { id0 = size_t(NY - 1) * NX + x; in.nx = 0.0; in.ny = 1.0; in.interior = false; bor = p.borde_inf; side0 = 3; }
                    else { id0 = size_t(y - 1) * NX + x; id1 = id0 + NX; in.nx = 0.0; in.ny = 1.0; in.interior = true; bor = 0.0; side0 = 3; }
                    side1 = 2;
                } else {
                    const int x = e, y = s;
                    in.len = g.len_v[y];
                    if (x == 0) { id0 = size_t(y) * NX; in.nx = -1.0; in.ny = 0.0; in.interior = false; bor = p.borde_izq; side0 = 0; }
                    else if (x == NX) { id0 = size_t(y) * NX + NX - 1; in.nx = 1.0; in.ny = 0.0; in.interior = false; bor = p.borde_der; side0 = 1; }
                    else { id0 = size_t(y) * NX + x - 1; id1 = id0 + 1; in.nx = 1.0; in.ny = 0.0; in.interior = true; bor = 0.0; side0 = 1; }
                    side1 = 0;
                }
                const int row0 = int(id0 / NX);
                face(W, id0, side0, in.W0, in.H0);
                in.area0 = g.area[row0];
                in.hc0[0] = W[0][id0]; in.hc0[1] = W[3][id0];
                in.acc0h[0] = acc[0][id0]; in.acc0h[1] = acc[3][id0];
                if (in.interior) {
                    face(W, id1, side1, in.W1, in.H1);
                    in.area1 = g.area[id1 / NX];
                    in.hc1[0] = W[0][id1]; in.hc1[1] = W[3][id1];
                    in.acc1h[0] = acc[0][id1]; in.acc1h[1] = acc[3][id1];
                } else {
                    // ghost cell: normal discharge times the boundary factor (:689-695, 776-782)
                    for (int k = 0; k < 6; ++k) in.W1[k] = in.W0[k];
                    const int kn = (dir == 0) ? 2 : 1;
                    in.W1[kn] = in.W0[kn] * bor;
                    in.W1[kn + 3] = in.W0[kn + 3] * bor;
                    in.H1 = in.H0;
                    in.area1 = in.area0;
                    in.hc1[0] = in.hc1[1] = 0.0;
                    in.acc1h[0] = in.acc1h[1] = 0.0;
                }
                double d0[6], d1[6], wave;
                if (!edge_flux(in, dt, c, d0, d1, wave)) continue;
                for (int k = 0; k < 6; ++k) acc[k][id0] -= d0[k];
                acc[6][id0] += wave;
                if (in.interior) {
                    for (int k = 0; k < 6; ++k) acc[k][id1] -= d1[k];
                    acc[6][id1] += wave;
                }
            }
        }
    }

    // Second order: cell-midpoint integral of the non-conservative pressure
    // product g h d(eta) over the reconstructed cell (x and y momenta).
    void volume_integral(const double* const* W) {
        const int NX = nx, NY = ny;
#pragma omp parallel for schedule(static)
        for (int j = 0; j < NY; ++j) {
            for (int i = 0; i < NX; ++i) {
                const size_t id = size_t(j) * NX + i;
                const double gh1 = c.g * W[0][id], gh2 = c.g * W[3][id];
                const double e1x = 2.0 * slope_x[0][id], e2x = 2.0 * slope_x[3][id];
                const double e1y = 2.0 * slope_y[0][id], e2y = 2.0 * slope_y[3][id];
                acc[1][id] -= c.peso * (gh1 * e1x * g.wx[j]);
                acc[4][id] -= c.peso * (gh2 * ((1.0 - c.r) * e2x + c.r * e1x) * g.wx[j]);
                acc[2][id] -= c.peso * (gh1 * e1y * g.wy[j]);
                acc[5][id] -= c.peso * (gh2 * ((1.0 - c.r) * e2y + c.r * e1y) * g.wy[j]);
            }
        }
    }

    // One forward-Euler stage: W -> Wn with dt; returns min per-cell dt.
    double stage(const double* const* W, double* const* Wn, double dt) {
        for (int k = 0; k < 7; ++k) std::fill(acc[k].begin(), acc[k].end(), 0.0);
        if (p.order == 2) reconstruct(W);
        // ShallowWater.cu:391-427: hor-even, hor-odd, ver-even, ver-odd
        pass(W, 0, 0, dt);
        pass(W, 0, 1, dt);
        pass(W, 1, 0, dt);
        pass(W, 1, 1, dt);
        if (p.order == 2) volume_integral(W);
        const int NX = nx, NY = ny;
        double mn = kBig;
#pragma omp parallel for schedule(static) reduction(min : mn)
        for (int j = 0; j < NY; ++j) {
            for (int i = 0; i < NX; ++i) {
                const size_t id = size_t(j) * NX + i;
                double wo[6], a[7], w[6], d;
                for (int k = 0; k < 6; ++k) wo[k] = W[k][id];
                for (int k = 0; k < 7; ++k) a[k] = acc[k][id];
                volume_update(wo, a, w, d, g.area[j], g.tanR[j], dt, c);
                for (int k = 0; k < 6; ++k) Wn[k][id] = w[k];
                if (d < mn) mn = d;
            }
        }
        return mn;
    }

    double initial_dt(const double* const* W) {
        std::vector<double>& aw = acc[6];
        std::fill(aw.begin(), aw.end(), 0.0);
        const int NX = nx, NY = ny;
        for (int dir = 0; dir < 2; ++dir) {
            for (int par = 0; par < 2; ++par) {
                const int nlines = (dir == 0) ? (NY - par) / 2 + 1 : (NX - par) / 2 + 1;
                const int nalong = (dir == 0) ? NX : NY;
#pragma omp parallel for schedule(static)
                for (int t = 0; t < nlines; ++t) {
                    const int e = par + 2 * t;
                    if ((dir == 0 && e > NY) || (dir == 1 && e > NX)) continue;
                    for (int s = 0; s < nalong; ++s) {
                        size_t id0, id1 = 0;
                        double nxv, nyv, bor, len;
                        bool interior;
                        if (dir == 0) {
                            const int x = s, y = e;
                            len = g.len_h[y];
                            if (y == 0) { id0 = size_t(x); nxv = 0; nyv = -1; interior = false; bor = p.borde_sup; }
                            else if (y == NY) { id0 = size_t(NY - 1) * NX + x; nxv = 0; nyv = 1; interior = false; bor = p.borde_inf; }
                            else { id0 = size_t(y - 1) * NX + x; id1 = id0 + NX; nxv = 0; nyv = 1; interior = true; bor = 0; }
                        } else {
                            const int x = e, y = s;
                            len = g.len_v[y];
                            if (x == 0) { id0 = size_t(y) * NX; nxv = -1; nyv = 0; interior = false; bor = p.borde_izq; }
                            else if (x == NX) { id0 = size_t(y) * NX + NX - 1; nxv = 1; nyv = 0; interior = false; bor = p.borde_der; }
                            else { id0 = size_t(y) * NX + x - 1; id1 = id0 + 1; nxv = 1; nyv = 0; interior = true; bor = 0; }
                        }
                        double W0[6], W1[6];
                        for (int k = 0; k < 6; ++k) W0[k] = W[k][id0];
                        if (interior) for (int k = 0; k < 6; ++k) W1[k] = W[k][id1];
                        else {
                            for (int k = 0; k < 6; ++k) W1[k] = W0[k];
                            const int kn = (dir == 0) ? 2 : 1;
                            W1[kn] = W0[kn] * bor; W1[kn + 3] = W0[kn + 3] * bor;
                        }
                        const double wv = edge_initial_wave(W0, W1, nxv, nyv, len, c);
                        aw[id0] += wv;
                        if (interior) aw[id1] += wv;
                    }
                }
            }
        }
        double mn = kBig;
        for (int j = 0; j < NY; ++j)
            for (int i = 0; i < NX; ++i) {
                const double a = aw[size_t(j) * NX + i];
                const double d = (a < kEps) ? kBig : (2.0 * c.cfl * g.area[j]) / a;  // Volumen_kernel.cu:226
                if (d < mn) mn = d;
            }
        return mn;
    }
};

}  // namespace orc

extern "C" {

int orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

static int check_params(const lsh_params* p) {
    if (!p || p->nx < 1 || p->ny < 1 || (p->order != 1 && p->order != 2)) return LSH_ERR_INVALID;
    if (!(p->eps_h > 0) || !(p->gravity > 0) || !(p->r < 1.0) || !(p->peso > 0)) return LSH_ERR_INVALID;
    return LSH_OK;
}

// Initial dt (ShallowWater.cu:236-257) of the state W[7] (h1 q1x q1y h2 q2x q2y H).
int orc_initial_dt(const lsh_params* p, const double* const* W, double* dt0) {
    if (int s = check_params(p)) return s;
    orc::Solver S(*p);
    *dt0 = S.initial_dt(W);
    return LSH_OK;
}

// Advance W in place by up to `nsteps` steps (<= 0: unlimited) while t < t_end
// (t_end < 0: no time limit).  *dt_io is the dt of the next step on entry and
// on exit (lagged dt, Volumen_kernel.cu:256 + ShallowWater.cu:439-442); *t_io is
// the time.  eta_max / eta_time (nx*ny, may be NULL) follow
// actualizarEta1MaximaGPU (Volumen_kernel.cu:182-213), evaluated before each step.
int orc_run(const lsh_params* p, double* const* W, long long nsteps, double t_end, double* t_io,
            double* dt_io, long long* steps_done, double* eta_max, double* eta_time) {
    if (int s = check_params(p)) return s;
    orc::Solver S(*p);
    const size_t N = S.N;
    std::vector<double> tmp[6], tmp2[6];
    double* Wn[7];
    double* W2[7];
    for (int k = 0; k < 6; ++k) { tmp[k].resize(N); Wn[k] = tmp[k].data(); }
    Wn[6] = W[6];
    if (p->order == 2) {
        for (int k = 0; k < 6; ++k) { tmp2[k].resize(N); W2[k] = tmp2[k].data(); }
        W2[6] = W[6];
    }
    double t = *t_io, dt = *dt_io;
    long long n = 0;
    while ((nsteps <= 0 || n < nsteps) && (t_end < 0 || t < t_end)) {
        if (eta_max) {
            for (size_t id = 0; id < N; ++id) {
                const double v = W[0][id] - W[6][id];
                if (v > eta_max[id]) { eta_max[id] = v; if (eta_time) eta_time[id] = t; }
            }
        }
        double dtn;
        if (p->order == 1) {
            dtn = S.stage(W, Wn, dt);
            for (int k = 0; k < 6; ++k) std::memcpy(W[k], Wn[k], N * sizeof(double));
        } else {
            dtn = S.stage(W, Wn, dt);       // W1 = E(W^n), dt_next from W^n's speeds
            S.stage(Wn, W2, dt);            // W2 = E(W1)
            for (int k = 0; k < 6; ++k)
                for (size_t id = 0; id < N; ++id) W[k][id] = 0.5 * (W[k][id] + W2[k][id]);
        }
        t += dt;
        dt = dtn;
        ++n;
        if (p->dt_min > 0 && dt < p->dt_min) { *t_io = t; *dt_io = dt; if (steps_done) *steps_done = n; return LSH_ERR_STALL; }
    }
    *t_io = t;
    *dt_io = dt;
    if (steps_done) *steps_done = n;
    return LSH_OK;
}

// Elementwise access to the shared elementary functions (tests compare them
// with the C library): which 0 exp_neg, 1 cbrt_pos, 2 log_pos, 3 pow_pos(x, 1e-3).
int orc_fpmath(int which, const double* x, double* y, long long n) {
    for (long long i = 0; i < n; ++i) {
        switch (which) {
            case 0: y[i] = lshm::exp_neg(x[i]); break;
            case 1: y[i] = lshm::cbrt_pos(x[i]); break;
            case 2: y[i] = lshm::log_pos(x[i]); break;
            case 3: y[i] = lshm::pow_pos(x[i], 1.0e-3); break;
            default: return LSH_ERR_INVALID;
        }
    }
    return LSH_OK;
}

// Masks of a state: bit0 h1 >= eps_h, bit1 h2 >= eps_h, bit2 granular layer at
// rest (h2 >= eps_h and q2 == 0).
int orc_masks(const lsh_params* p, const double* const* W, uint8_t* mask) {
    const size_t N = size_t(p->nx) * p->ny;
    for (size_t id = 0; id < N; ++id) {
        uint8_t m = 0;
        if (W[0][id] >= p->eps_h) m |= 1;
        if (W[3][id] >= p->eps_h) { m |= 2; if (W[4][id] == 0.0 && W[5][id] == 0.0) m |= 4; }
        mask[id] = m;
    }
    return LSH_OK;
}

}  // extern "C"
