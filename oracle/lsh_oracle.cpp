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
    // derived on the host, identically in the CUDA library (lsh_core.cu make_consts)
    double omr;       // 1 - r
    double inv_gp;    // 1 / (g (1 - r))
    double inv_eps;   // 1 / eps_h
    double inv_peso;  // 1 / peso
    double eps_1r;    // eps_h (1 + r)
    double g_mf02;    // g mf0^2
    double g_mfs2;    // g mfs^2
    double sqrt_g;    // sqrt(g)
    int law;
    int eig_sort;
};

struct Geo {
    int nx, ny;
    std::vector<double> area;    // [ny]   cell area of row j
    std::vector<double> inv_area;  // [ny] 1 / area
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
    c.omr = 1.0 - p.r;
    c.inv_gp = 1.0 / c.gp;
    c.inv_eps = 1.0 / p.eps_h;
    c.inv_peso = 1.0 / p.peso;
    c.eps_1r = p.eps_h * (1.0 + p.r);
    c.g_mf02 = (p.gravity * p.mf0) * p.mf0;
    c.g_mfs2 = (p.gravity * p.mfs) * p.mfs;
    c.sqrt_g = std::sqrt(p.gravity);
    c.law = p.friction_law;
    c.eig_sort = p.eig_sort;
    return c;
}

static Geo make_geo(const lsh_params& p) {
    Geo g;
    g.nx = p.nx; g.ny = p.ny;
    g.area.resize(p.ny); g.len_v.resize(p.ny); g.len_h.resize(p.ny + 1);
    g.tanR.resize(p.ny); g.wx.resize(p.ny); g.wy.resize(p.ny); g.inv_area.resize(p.ny);
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
    for (int j = 0; j < p.ny; ++j) g.inv_area[j] = 1.0 / g.area[j];
    return g;
}

// ---------------------------------------------------------------- helpers
// The arithmetic below fixes every fused multiply-add (fmad) and every
// reciprocal of a constant (inv_*) explicitly; the CUDA kernels
// (landslidehysea_gb300/csrc/lsh_scheme.cuh) evaluate the same sequence.

inline double tmin(double a, double b) { return (b < a) ? b : a; }
inline double tmax(double a, double b) { return (b > a) ? b : a; }
inline double max0(double a) { return (a > 0.0) ? a : 0.0; }
inline double fmad(double a, double b, double c) { return lshm::fmad(a, b, c); }
inline double exp_neg(double x) { return lshm::exp_neg(x); }

// sqrt(2) h / sqrt(h^4 + max(h, eps_h)^4): the desingularised 1/h factor
// (Arista_kernel.cu:74,380; Volumen_kernel.cu:13,44,48).  For h > eps_h the
// expression is exactly 1/h, which is how it is evaluated there.
inline double vfac(double h, double eps_h) {
    if (h > eps_h) return 1.0 / h;
    const double h2 = h * h, m2 = eps_h * eps_h;
    return (kSqrt2 * h) / sqrt(fmad(h2, h2, m2 * m2));
}

inline double pow43(double h) { return h * lshm::cbrt_pos(h); }

inline int sgn(double x) { return (fabs(x) < kEps) ? 0 : ((x > 0) ? 1 : -1); }  // Constantes.hxx:14

struct V4 { double x, y, z, w; };

// The fixed compare-and-swap sequence of Arista_kernel.cu:193-234, including
// its (i=2, j=1) compare, which leaves the larger of y/z in y (eig_sort 0);
// with eig_sort 1 that compare is (1,2) and the sequence is a true sort.
inline void sort_eig(V4& D, int full) {
    auto cs = [](double& a, double& b) { if (a > b) { double t = b; b = a; a = t; } };
    cs(D.x, D.y); cs(D.x, D.z); cs(D.x, D.w); cs(D.y, D.z); cs(D.y, D.w);
    if (full) cs(D.y, D.z);
    else if (D.z > D.y) { double t = D.y; D.y = D.z; D.z = t; }
    cs(D.z, D.w);
}

// aproximarAutovalores1D (Arista_kernel.cu:152-237) given the two layers'
// depths, velocities (u1, u2) and the total normal discharge q:
// external u -+ sqrt(g h), internal uu -+ sqrt(g' h1 h2 F |1 - (u1-u2)^2 F / g'|).
// sqrt_h >= 0: sqrt(h1) is known and h2 == 0, so sqrt(g h) = sqrt(g) sqrt(h1).
inline V4 eig(double h1, double h2, double u1, double u2, double q, const Consts& c, double sqrt_h = -1.0) {
    const double h = h1 + h2;
    const double F = vfac(h, c.eps_h);
    const double u = q * F;
    const double cg = (sqrt_h >= 0.0) ? c.sqrt_g * sqrt_h : sqrt(c.g * h);
    const double uu = fmad(u1, h2, u2 * h1) * F;
    const double d = u1 - u2;
    const double aux = fmad(-((d * d) * F), c.inv_gp, 1.0);
    const double ci = sqrt((((c.gp * h1) * h2) * F) * fabs(aux));
    V4 D{u - cg, uu - ci, uu + ci, u + cg};
    sort_eig(D, c.eig_sort);
    return D;
}

// defTerminoFriccion (Arista_kernel.cu:11-58): friction coefficient mu.
inline double friction_mu(double h1, double u1, double h2, double u2, const Consts& c) {
    if (c.law == LSH_FRICTION_COULOMB) return c.mu;
    // Pouliquen law (the reference's #ifndef COULOMB branch)
    const double a = (10.0 * h1) * c.inv_eps;
    const double rr = 1.0 - c.r * (1.0 - exp_neg(a * a));
    const double gp = c.g * rr;
    const double fr1 = ((u1 * u1) * vfac(h1, c.eps_h)) / gp;
    const double fr2 = ((u2 * u2) * vfac(h2, c.eps_h)) / gp;
    const double fr = sqrt(fmad((1.0 - rr) * fr1, fr2, fr1 + fr2));
    const double beta = 0.136, L2 = 8.0e-4, chi = 1.0e-3;
    const double mustop = c.tan1 + (c.tan2 - c.tan1) / (1.0 + h2 / L2);
    const double mustart = c.tan3 + (c.tan4 - c.tan3) / (1.0 + h2 / L2);
    double muf;
    if (fr > beta) muf = c.tan1 + (c.tan2 - c.tan1) / (1.0 + beta * h2 / (fr * L2));
    else if (fabs(fr) < kEps) muf = c.tan3 + (c.tan4 - c.tan3) / (1.0 + h2 / L2);
    else muf = fmad(lshm::pow_pos(fr / beta, chi), mustop - mustart, mustart);
    return (muf * c.L) / c.H;
}

// 1 - r (1 - exp(-(10 h1 / eps_h)^2)) (Arista_kernel.cu:136, Volumen_kernel.cu:15)
inline double fsc_of(double h1, const Consts& c) {
    const double a = (10.0 * h1) * c.inv_eps;
    return 1.0 - c.r * (1.0 - exp_neg(a * a));
}

// ---------------------------------------------------------------- edge flux
// One face state in the edge's normal frame: depth, normal and tangential
// discharge of each layer, bottom depth.
struct Face { double h1, qn1, qt1, h2, qn2, qt2, H; };

// Inputs of one edge.  A / B are the states facing the edge (cell values at
// first order, reconstructed face values at second order; B is the ghost at a
// boundary); hc* are the cell-average depths and acc*h the partial
// accumulators (h1, h2) the positivity limiter reads.
struct EdgeIn {
    Face A, B;
    double len, area0, area1, inv_area0, inv_area1;
    bool interior;
    double hc0[2], hc1[2];
    double acc0h[2], acc1h[2];
};

// Edge output in the normal frame: per layer (mass, normal momentum,
// tangential momentum) to subtract from cell 0 (m) and cell 1 (p).
struct EdgeOut { double m[6], p[6]; double wave; };

// procesarArista (Arista_kernel.cu:324-645).  Returns false for a dry edge
// (no contribution at all, :397).
bool edge_flux(const EdgeIn& e, double dt, const Consts& c, EdgeOut& o) {
    const double eps = c.eps_h;
    double Aq1 = e.A.qn1, Aq2 = e.A.qn2, Bq1 = e.B.qn1, Bq2 = e.B.qn2;
    const double Ah1 = e.A.h1, Ah2 = e.A.h2, Bh1 = e.B.h1, Bh2 = e.B.h2;
    const double H0 = e.A.H, H1 = e.B.H;

    const double h1ij = 0.5 * (Ah1 + Bh1);
    const double h2ij = 0.5 * (Ah2 + Bh2);
    if (!((h1ij >= kEps) || (h2ij >= kEps))) return false;

    // tratamientoSecoMojado (Arista_kernel.cu:301-321)
    if ((Ah2 < eps) && (H1 - Bh2 > H0)) Bq2 = 0.0;
    if ((Bh2 < eps) && (H0 - Ah2 > H1)) Aq2 = 0.0;
    if ((Ah1 < eps) && (H1 - Bh1 - Bh2 > H0 - Ah2)) Bq1 = 0.0;
    if ((Bh1 < eps) && (H0 - Ah1 - Ah2 > H1 - Bh2)) Aq1 = 0.0;
    if ((Ah2 + Ah1 < eps) && (H1 - Bh1 - Bh2 > H0)) { Bq1 = 0.0; Bq2 = 0.0; }
    if ((Bh2 + Bh1 < eps) && (H0 - Ah1 - Ah2 > H1)) { Aq1 = 0.0; Aq2 = 0.0; }

    // Roe-type averages (Arista_kernel.cu:375-395)
    const double fA1 = vfac(Ah1, eps), fB1 = vfac(Bh1, eps);
    const double fA2 = vfac(Ah2, eps), fB2 = vfac(Bh2, eps);
    const double sa1 = sqrt(Ah1), sb1 = sqrt(Bh1);
    const double u1ij = fmad(sa1, fA1 * Aq1, sb1 * (fB1 * Bq1)) / (sa1 + sb1 + kEps);
    const double sa2 = sqrt(Ah2), sb2 = sqrt(Bh2);
    const double u2ij = fmad(sa2, fA2 * Aq2, sb2 * (fB2 * Bq2)) / (sa2 + sb2 + kEps);
    // a cell's celerity sqrt(g h) is sqrt(g) sqrt(h1) when its granular layer is empty
    const bool oneA = (Ah2 == 0.0), oneB = (Bh2 == 0.0);

    // hydrostatic reconstruction (terminosPresion1D, :94-115)
    const double Hm = tmin(H0, H1);
    const double deta1 = max0(Bh1 + Bh2 - H1 + Hm) - max0(Ah1 + Ah2 - H0 + Hm);
    const double deta2 = max0(Bh2 - H1 + Hm) - max0(Ah2 - H0 + Hm);
    const double gh1 = c.g * h1ij, gh2 = c.g * h2ij;
    V4 tp{0.0, gh1 * deta1, 0.0, gh2 * fmad(c.omr, deta2, c.r * deta1)};

    // edge Coulomb switch (terminosPresion1DMod :134-147, identityModification :259-264)
    const double mu = friction_mu(h1ij, u1ij, h2ij, u2ij, c);
    const double sc = ((fsc_of(h1ij, c) * mu) * c.g) * h2ij;
    const bool coul = fabs(h2ij * u2ij) < (c.peso * sc) * dt;
    V4 tp2 = tp;
    if (coul) tp2.w = (gh2 * c.r) * deta1;

    // eigenvalue bounds (:427-444)
    const V4 D = eig(h1ij, h2ij, u1ij, u2ij, fmad(h1ij, u1ij, h2ij * u2ij), c);
    const V4 E0 = eig(Ah1, Ah2, fA1 * Aq1, fA2 * Aq2, Aq1 + Aq2, c, oneA ? sa1 : -1.0);
    const V4 E1 = eig(Bh1, Bh2, fB1 * Bq1, fB2 * Bq2, Bq1 + Bq2, c, oneB ? sb1 : -1.0);
    const double aut1 = tmin(D.x, tmin(E0.x, E1.x));
    const double aut3 = tmax(D.w, tmax(E0.w, E1.w));
    double lmax = tmax(fabs(aut3), fabs(aut1));
    const double umax = tmax(fabs(u1ij), fabs(u2ij));
    if (umax > lmax) lmax = umax;
    double aut2 = tmax(fabs(D.y), fabs(D.z));
    if (sgn(aut1 + aut3) < 0) aut2 = -aut2;

    // PVM / IFCP coefficients (:446-465); the three parabola weights share
    // one reciprocal of (aut1-aut2)(aut1-aut3)(aut2-aut3)
    double a0, a1, a2;
    if ((fabs(aut1 - aut3) >= kEps) && (fabs(aut1 - aut2) >= kEps) && (fabs(aut2 - aut3) >= kEps)) {
        if ((h1ij >= eps) && (h2ij >= eps)) {
            const double d12 = aut1 - aut2, d13 = aut1 - aut3, d23 = aut2 - aut3;
            const double inv = 1.0 / ((d12 * d13) * d23);
            const double a = (fabs(aut1) * d23) * inv;
            const double b = -((fabs(aut2) * d13) * inv);
            const double cc = (fabs(aut3) * d12) * inv;
            a0 = fmad(a * aut2, aut3, fmad(b * aut1, aut3, (cc * aut1) * aut2));
            a1 = -fmad(a, aut2 + aut3, fmad(b, aut1 + aut3, cc * (aut1 + aut2)));
            a2 = a + b + cc;
        } else {
            const double inv = 1.0 / (aut3 - aut1);
            a0 = fmad(aut3, fabs(aut1), -(aut1 * fabs(aut3))) * inv;
            a1 = (fabs(aut3) - fabs(aut1)) * inv;
            a2 = 0.0;
        }
    } else {
        a0 = lmax; a1 = 0.0; a2 = 0.0;
    }

    // physical fluxes (getFlujo_1dC :62-92)
    const V4 FA{Aq1, (Ah1 < kEps) ? 0.0 : (fA1 * Aq1) * Aq1, Aq2, (Ah2 < kEps) ? 0.0 : (fA2 * Aq2) * Aq2};
    const V4 FB{Bq1, (Bh1 < kEps) ? 0.0 : (fB1 * Bq1) * Bq1, Bq2, (Bh2 < kEps) ? 0.0 : (fB2 * Bq2) * Bq2};
    const V4 dF{FB.x - FA.x, FB.y - FA.y, FB.z - FA.z, FB.w - FA.w};
    tp2 = V4{tp2.x + dF.x, tp2.y + dF.y, tp2.z + dF.z, tp2.w + dF.w};
    const V4 half{0.5 * (dF.x + tp.x), 0.5 * (dF.y + tp.y), 0.5 * (dF.z + tp.z), 0.5 * (dF.w + tp.w)};

    // A * tp2 (:476-482)
    const V4 At{tp2.y, fmad(gh1, tp2.z, fmad(u1ij + u1ij, tp2.y, fmad(-u1ij, u1ij, gh1) * tp2.x)), tp2.w,
                fmad(c.r * gh2, tp2.x, fmad(fmad(-u2ij, u2ij, gh2), tp2.z, (u2ij + u2ij) * tp2.w))};

    // identityModification (:239-276)
    V4 I{deta1, Bq1 - Aq1, 0.0, Bq2 - Aq2};
    if (!coul) {
        if ((Ah1 > eps) && (Bh1 > eps)) I.x = I.x - deta2;
        I.z = deta2;
    }

    // viscosity and the two one-sided fluxes (:488-504)
    const V4 Q{0.5 * fmad(a0, I.x, fmad(a1, tp2.x, a2 * At.x)), 0.5 * fmad(a0, I.y, fmad(a1, tp2.y, a2 * At.y)),
               0.5 * fmad(a0, I.z, fmad(a1, tp2.z, a2 * At.z)), 0.5 * fmad(a0, I.w, fmad(a1, tp2.w, a2 * At.w))};
    const V4 Fm{half.x + (FA.x - Q.x), half.y + (FA.y - Q.y), half.z + (FA.z - Q.z), half.w + (FA.w - Q.w)};
    const V4 Fp{half.x + (Q.x - FB.x), half.y + (Q.y - FB.y), half.z + (Q.z - FB.z), half.w + (Q.w - FB.w)};

    // upwinded tangential velocity (:506-532)
    const double u1t = (fabs(Fm.x) < kEps) ? 0.0 : ((Fm.x > 0.0) ? fA1 * e.A.qt1 : fB1 * e.B.qt1);
    const double u2t = (fabs(Fm.z) < kEps) ? 0.0 : ((Fm.z > 0.0) ? fA2 * e.A.qt2 : fB2 * e.B.qt2);
    const double s1 = Fm.x * u1t, s2 = Fm.z * u2t;

    // normal-frame fluxes times the edge length: (mass, normal, tangential);
    // the tangential part is +s for cell 0 and -s for cell 1 (:534-552)
    double M[6] = {Fm.x, Fm.y, s1, Fm.z, Fm.w, s2};
    double P[6] = {Fp.x, Fp.y, -s1, Fp.z, Fp.w, -s2};
    for (int k = 0; k < 6; ++k) { P[k] = e.len * P[k]; M[k] = e.len * M[k]; }

    // positivity limiter on the partially accumulated depths (:554-609)
    const double b0 = dt * e.inv_area0;
    const double hp00 = fmad(b0, e.acc0h[0], e.hc0[0]), hp01 = fmad(b0, e.acc0h[1], e.hc0[1]);
    double hp10 = 0.0, hp11 = 0.0;
    if (e.interior) {
        const double b1 = dt * e.inv_area1;
        hp10 = fmad(b1, e.acc1h[0], e.hc1[0]); hp11 = fmad(b1, e.acc1h[1], e.hc1[1]);
    }
    const double factor = 1.0 * c.beta;
    for (int layer = 0; layer < 2; ++layer) {
        const int k = 3 * layer;
        double dta = kBig, dtb = kBig;
        if (M[k] > 0.0) dta = ((layer ? hp01 : hp00) * e.area0) / fmad(factor, M[k], kEps);
        if (e.interior && P[k] > 0.0) dtb = ((layer ? hp11 : hp10) * e.area1) / fmad(factor, P[k], kEps);
        const double dtl = tmin(dta, dtb);
        if (!(dt <= dtl)) {
            const double alpha = dtl / (dt + kEps);
            for (int q = k; q < k + 3; ++q) { M[q] = alpha * M[q]; P[q] = alpha * P[q]; }
        }
    }

    if (lmax < eps) lmax = lmax + eps;  // :611-612
    o.wave = (e.len * lmax) * c.inv_peso;
    for (int k = 0; k < 6; ++k) { o.m[k] = c.peso * M[k]; o.p[k] = c.peso * P[k]; }
    return true;
}

// procesarAristaDeltaTInicial (Arista_kernel.cu:1040-1127): wave-speed bound
// for the initial dt.  No wet/dry fix, no dry-edge skip, and the max of the
// signed sorted external eigenvalues (:1107).
double edge_initial_wave(const Face& A, const Face& B, double len, const Consts& c) {
    const double eps = c.eps_h;
    const double h1ij = 0.5 * (A.h1 + B.h1);
    const double fA1 = vfac(A.h1, eps), fB1 = vfac(B.h1, eps);
    double sa = sqrt(A.h1), sb = sqrt(B.h1);
    const double u1ij = fmad(sa, fA1 * A.qn1, sb * (fB1 * B.qn1)) / (sa + sb + kEps);
    const double h2ij = 0.5 * (A.h2 + B.h2);
    const double fA2 = vfac(A.h2, eps), fB2 = vfac(B.h2, eps);
    sa = sqrt(A.h2); sb = sqrt(B.h2);
    const double u2ij = fmad(sa, fA2 * A.qn2, sb * (fB2 * B.qn2)) / (sa + sb + kEps);
    const V4 D = eig(h1ij, h2ij, u1ij, u2ij, fmad(h1ij, u1ij, h2ij * u2ij), c);
    double lmax = tmax(D.x, D.w);
    const double b = tmax(fabs(u1ij), fabs(u2ij));
    if (b > lmax) lmax = b;
    if (lmax < eps) lmax = lmax + eps;
    return len * lmax;
}

// ---------------------------------------------------------------- state update
// filtroEstado (Volumen_kernel.cu:92-180); its "complex" block is dead (cf = 0).
inline void filtro(double w[6], double dt, const Consts& c) {
    if (w[0] < 0.0) w[0] = 0.0;
    if (w[3] < 0.0) w[3] = 0.0;
    for (int layer = 0; layer < 2; ++layer) {
        const int k = 3 * layer;
        const double x = w[k] * c.inv_eps;
        const double x2 = x * x;
        const double d = fmad(x2, x2, kEps);
        // exp(-dt / d) is exactly 1 once dt / d < 2^-54; below this bound
        // (conservative by far more than the roundings of 1/d and dt*(1/d))
        // the factor is 1 and the division is not needed
        if (dt < d * 0x1.fp-55) continue;
        const double aux = exp_neg(dt * (1.0 / d));
        w[k + 1] = w[k + 1] * aux;
        w[k + 2] = w[k + 2] * aux;
    }
    for (int layer = 0; layer < 2; ++layer) {
        const double vmax = layer ? c.vmax2 : c.vmax1;
        if (vmax > 0.0) {
            const int k = 3 * layer;
            const double h = w[k];
            const double f = vfac(h, c.eps_h);
            double ux = f * w[k + 1], uy = f * w[k + 2];
            const double u = sqrt(fmad(ux, ux, uy * uy));
            if (u > vmax) {
                const double s = vmax / u;
                ux = ux * s; uy = uy * s;
                w[k + 1] = ux * h; w[k + 2] = uy * h;
            }
        }
    }
}

// disImplicita (Volumen_kernel.cu:31-90): semi-implicit interlayer and bottom
// friction.  Speeds of the previous state `wo` enter the coefficients.
inline void dis_implicita(const double wo[6], double w[6], double dt, const Consts& c) {
    if (w[0] < 0.0) w[0] = 0.0;
    if (w[3] < 0.0) w[3] = 0.0;
    const double eps = c.eps_h;
    const double h1 = w[0], h2 = w[3];
    const double f1 = vfac(h1, eps), f2 = vfac(h2, eps);
    double u1x = f1 * w[1], u1y = f1 * w[2], u2x = f2 * w[4], u2y = f2 * w[5];
    const double fo1 = vfac(wo[0], eps), fo2 = vfac(wo[3], eps);
    const double uo1x = fo1 * wo[1], uo1y = fo1 * wo[2], uo2x = fo2 * wo[4], uo2y = fo2 * wo[5];
    const double dx = uo1x - uo2x, dy = uo1y - uo2y;
    const double du = sqrt(fmad(dx, dx, dy * dy));
    const double u1 = sqrt(fmad(uo1x, uo1x, uo1y * uo1y));
    const double u2 = sqrt(fmad(uo2x, uo2x, uo2y * uo2y));
    if ((h1 > 0.0) && (h2 > 0.0)) {
        const double hmod = fmad(c.r, h1, h2);
        const double m = (hmod > c.eps_1r) ? hmod : c.eps_1r;
        const double hm2 = hmod * hmod, m2 = m * m;
        const double hh = hmod / sqrt(fmad(hm2, hm2, m2 * m2));
        const double k12 = ((dt * kSqrt2) * hh) * (c.mfc * du);
        const double c1 = k12 * h2;
        const double c2 = (k12 * c.r) * h1;
        const double c3 = ((dt * c.g_mfs2) * u2) / (pow43(h2) + kEps);
        const double e1 = 1.0 + c1, e2 = 1.0 + c2 + c3;
        const double det = 1.0 / fmad(e1, e2, -(c1 * c2));
        w[1] = (h1 * fmad(u1x, e2, c1 * u2x)) * det;
        w[4] = (h2 * fmad(u2x, e1, c2 * u1x)) * det;
        w[2] = (h1 * fmad(u1y, e2, c1 * u2y)) * det;
        w[5] = (h2 * fmad(u2y, e1, c2 * u1y)) * det;
    }
    // bottom friction: h u / (1 + c1) with u = vfac(h) q; above eps_h,
    // vfac(h) = 1/h and h u is q itself
    // 1 / (1 + c1) with c1 = X / Y is Y / (Y + X): one division
    if ((h1 > 0.0) && (h2 < eps)) {
        const double Y = pow43(h1) + kEps, X = (dt * c.g_mf02) * u1;
        const double inv = Y / (Y + X);
        if (h1 > eps) { w[1] = w[1] * inv; w[2] = w[2] * inv; }
        else { w[1] = (h1 * (f1 * w[1])) * inv; w[2] = (h1 * (f1 * w[2])) * inv; }
    }
    if ((h2 > 0.0) && (h1 < eps)) {
        const double Y = pow43(h2) + kEps, X = (dt * c.g_mfs2) * u2;
        const double inv = Y / (Y + X);
        if (h2 > eps) { w[4] = w[4] * inv; w[5] = w[5] * inv; }
        else { w[4] = (h2 * (f2 * w[4])) * inv; w[5] = (h2 * (f2 * w[5])) * inv; }
    }
}

// coulomb (Volumen_kernel.cu:7-26): granular stop / slow-down.
inline void coulomb(double w[6], double dt, const Consts& c) {
    if (!(w[3] > 0.0)) {  // no granular layer: the reference's factor is 0
        w[4] = w[4] * 0.0;
        w[5] = w[5] * 0.0;
        return;
    }
    double mu = c.mu;
    if (c.law != LSH_FRICTION_COULOMB) {
        const double u1 = sqrt(fmad(w[1], w[1], w[2] * w[2])) * vfac(w[0], c.eps_h);
        const double u2 = sqrt(fmad(w[4], w[4], w[5] * w[5])) * vfac(w[3], c.eps_h);
        mu = friction_mu(w[0], u1, w[3], u2, c);
    }
    const double sc = ((((fsc_of(w[0], c) * mu) * c.g) * w[3]) * dt);
    const double normq = sqrt(fmad(w[4], w[4], w[5] * w[5]));
    double aux = 0.0;
    if ((normq + sc >= kEps) && (normq >= sc)) aux = normq / (normq + sc);
    w[4] = w[4] * aux;
    w[5] = w[5] * aux;
}

// obtenerEstadoYDeltaTVolumenesGPU (Volumen_kernel.cu:231-284) for one cell:
// per-cell dt from the wave accumulator, forward Euler stage, the spherical
// metric source (new), then filtroEstado -> disImplicita -> coulomb.
// `rate` gets acc_w / area (0 below EPSILON): the step's dt is
// 2 CFL / max(rate), i.e. min over cells of 2 CFL area / acc_w
// (Volumen_kernel.cu:256) with one division per step.
inline void volume_update(const double wo[6], const double acc[7], double w[6], double& rate, double area,
                          double inv_area, double tanR, double dt, const Consts& c) {
    (void)area;
    rate = (acc[6] < kEps) ? 0.0 : acc[6] * inv_area;
    const double b = dt * inv_area;
    for (int k = 0; k < 6; ++k) w[k] = fmad(b, acc[k], wo[k]);
    if (tanR != 0.0) {
        for (int layer = 0; layer < 2; ++layer) {
            const int k = 3 * layer;
            if (wo[k] == 0.0 && wo[k + 1] == 0.0 && wo[k + 2] == 0.0) continue;  // adds exactly 0
            const double ux = vfac(wo[k], c.eps_h) * wo[k + 1];
            const double s = dt * (ux * tanR);
            w[k + 1] = fmad(s, wo[k + 2], w[k + 1]);
            w[k + 2] = fmad(-s, wo[k + 1], w[k + 2]);
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
    // (toward j+1)) in the edge frame of normal (nx, ny): normal discharge
    // q.n and tangential q_y nx - q_x ny (Arista_kernel.cu:363-371, 509-525).
    // First order (or a cell whose slopes were zeroed): the cell value itself.
    Face face(const double* const* W, size_t id, int side, double nxv, double nyv) const {
        double w[6], Hf;
        for (int k = 0; k < 6; ++k) w[k] = W[k][id];
        Hf = W[6][id];
        if (p.order == 2) {
            const std::vector<double>* s = (side < 2) ? slope_x : slope_y;
            const double sg = (side & 1) ? 1.0 : -1.0;
            const double de1 = s[0][id], de2 = s[3][id], dH = s[6][id];
            w[0] = w[0] + sg * (de1 - de2);
            w[1] = w[1] + sg * s[1][id];
            w[2] = w[2] + sg * s[2][id];
            w[3] = w[3] + sg * (de2 + dH);
            w[4] = w[4] + sg * s[4][id];
            w[5] = w[5] + sg * s[5][id];
            Hf = Hf + sg * dH;
        }
        Face f;
        f.h1 = w[0]; f.qn1 = w[1] * nxv + w[2] * nyv; f.qt1 = w[2] * nxv - w[1] * nyv;
        f.h2 = w[3]; f.qn2 = w[4] * nxv + w[5] * nyv; f.qt2 = w[5] * nxv - w[4] * nyv;
        f.H = Hf;
        return f;
    }

    // The edge of colour pass (dir, par) number (line, along): its cells,
    // outward normal of cell 0, length and boundary factor
    // (Arista_kernel.cu:651-838: vertical edge x between columns x-1 and x,
    // horizontal edge y between rows y-1 and y; row 0's outer edge is "sup").
    struct EdgeGeo { size_t id0, id1; bool interior; double nx, ny, len, bor; int side0, side1; };
    EdgeGeo edge_geo(int dir, int e, int s) const {
        EdgeGeo q;
        q.id1 = 0;
        q.bor = 0.0;
        const size_t NX = size_t(nx);
        if (dir == 0) {
            const int x = s, y = e;
            q.len = g.len_h[y]; q.nx = 0.0; q.side1 = 2;
            if (y == 0) { q.id0 = size_t(x); q.ny = -1.0; q.interior = false; q.bor = p.borde_sup; q.side0 = 2; }
            else if (y == ny) { q.id0 = size_t(ny - 1) * NX + x; q.ny = 1.0; q.interior = false; q.bor = p.borde_inf; q.side0 = 3; }
            else { q.id0 = size_t(y - 1) * NX + x; q.id1 = q.id0 + NX; q.ny = 1.0; q.interior = true; q.side0 = 3; }
        } else {
            const int x = e, y = s;
            q.len = g.len_v[y]; q.ny = 0.0; q.side1 = 0;
            if (x == 0) { q.id0 = size_t(y) * NX; q.nx = -1.0; q.interior = false; q.bor = p.borde_izq; q.side0 = 0; }
            else if (x == nx) { q.id0 = size_t(y) * NX + NX - 1; q.nx = 1.0; q.interior = false; q.bor = p.borde_der; q.side0 = 1; }
            else { q.id0 = size_t(y) * NX + x - 1; q.id1 = q.id0 + 1; q.nx = 1.0; q.interior = true; q.side0 = 1; }
        }
        return q;
    }

    // ghost face: the cell's own face with the normal discharges times the
    // boundary factor (:689-695, 776-782)
    static Face ghost(const Face& a, double bor) {
        Face b = a;
        b.qn1 = a.qn1 * bor;
        b.qn2 = a.qn2 * bor;
        return b;
    }

    // the cell value in the edge frame (the initial-dt pass is first order)
    static Face face_cell(const double* const* W, size_t id, double nxv, double nyv) {
        Face f;
        f.h1 = W[0][id]; f.qn1 = W[1][id] * nxv + W[2][id] * nyv; f.qt1 = W[2][id] * nxv - W[1][id] * nyv;
        f.h2 = W[3][id]; f.qn2 = W[4][id] * nxv + W[5][id] * nyv; f.qt2 = W[5][id] * nxv - W[4][id] * nyv;
        f.H = W[6][id];
        return f;
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
            for (int s = 0; s < nalong; ++s) {
                const EdgeGeo q = edge_geo(dir, e, s);
                EdgeIn in;
                in.len = q.len;
                in.interior = q.interior;
                const size_t row0 = q.id0 / NX;
                in.A = face(W, q.id0, q.side0, q.nx, q.ny);
                in.area0 = g.area[row0];
                in.inv_area0 = g.inv_area[row0];
                in.hc0[0] = W[0][q.id0]; in.hc0[1] = W[3][q.id0];
                in.acc0h[0] = acc[0][q.id0]; in.acc0h[1] = acc[3][q.id0];
                if (q.interior) {
                    const size_t row1 = q.id1 / NX;
                    in.B = face(W, q.id1, q.side1, q.nx, q.ny);
                    in.area1 = g.area[row1];
                    in.inv_area1 = g.inv_area[row1];
                    in.hc1[0] = W[0][q.id1]; in.hc1[1] = W[3][q.id1];
                    in.acc1h[0] = acc[0][q.id1]; in.acc1h[1] = acc[3][q.id1];
                } else {
                    in.B = ghost(in.A, q.bor);
                    in.area1 = in.area0;
                    in.inv_area1 = in.inv_area0;
                    in.hc1[0] = in.hc1[1] = 0.0;
                    in.acc1h[0] = in.acc1h[1] = 0.0;
                }
                EdgeOut o;
                if (!edge_flux(in, dt, c, o)) continue;
                // rotate the normal-frame fluxes back: x = fn nx - ft ny, y = fn ny + ft nx
                const double nxv = q.nx, nyv = q.ny;
                double d0[6], d1[6];
                for (int l = 0; l < 2; ++l) {
                    const int k = 3 * l;
                    d0[k] = o.m[k];
                    d0[k + 1] = o.m[k + 1] * nxv - o.m[k + 2] * nyv;
                    d0[k + 2] = o.m[k + 1] * nyv + o.m[k + 2] * nxv;
                    d1[k] = o.p[k];
                    d1[k + 1] = o.p[k + 1] * nxv - o.p[k + 2] * nyv;
                    d1[k + 2] = o.p[k + 1] * nyv + o.p[k + 2] * nxv;
                }
                for (int k = 0; k < 6; ++k) acc[k][q.id0] -= d0[k];
                acc[6][q.id0] += o.wave;
                if (q.interior) {
                    for (int k = 0; k < 6; ++k) acc[k][q.id1] -= d1[k];
                    acc[6][q.id1] += o.wave;
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
                acc[1][id] -= c.peso * ((gh1 * e1x) * g.wx[j]);
                acc[4][id] -= c.peso * ((gh2 * fmad(c.omr, e2x, c.r * e1x)) * g.wx[j]);
                acc[2][id] -= c.peso * ((gh1 * e1y) * g.wy[j]);
                acc[5][id] -= c.peso * ((gh2 * fmad(c.omr, e2y, c.r * e1y)) * g.wy[j]);
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
        double mx = 0.0;
#pragma omp parallel for schedule(static) reduction(max : mx)
        for (int j = 0; j < NY; ++j) {
            for (int i = 0; i < NX; ++i) {
                const size_t id = size_t(j) * NX + i;
                double wo[6], a[7], w[6], rate;
                for (int k = 0; k < 6; ++k) wo[k] = W[k][id];
                for (int k = 0; k < 7; ++k) a[k] = acc[k][id];
                volume_update(wo, a, w, rate, g.area[j], g.inv_area[j], g.tanR[j], dt, c);
                for (int k = 0; k < 6; ++k) Wn[k][id] = w[k];
                if (rate > mx) mx = rate;
            }
        }
        return dt_of(mx);
    }

    // dt from the largest acc_w / area; 1e30 when no cell has a wave speed
    double dt_of(double max_rate) const { return (max_rate > 0.0) ? (2.0 * c.cfl) / max_rate : kBig; }

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
                        const EdgeGeo q = edge_geo(dir, e, s);
                        const Face A = face_cell(W, q.id0, q.nx, q.ny);
                        const Face B = q.interior ? face_cell(W, q.id1, q.nx, q.ny) : ghost(A, q.bor);
                        const double wv = edge_initial_wave(A, B, q.len, c);
                        aw[q.id0] += wv;
                        if (q.interior) aw[q.id1] += wv;
                    }
                }
            }
        }
        double mx = 0.0;
        for (int j = 0; j < NY; ++j)
            for (int i = 0; i < NX; ++i) {
                const double a = aw[size_t(j) * NX + i];
                const double rate = (a < kEps) ? 0.0 : a * g.inv_area[j];  // Volumen_kernel.cu:226
                if (rate > mx) mx = rate;
            }
        return dt_of(mx);
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
