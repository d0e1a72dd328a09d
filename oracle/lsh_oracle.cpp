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
#include "dual.h"
#include "count.h"

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
constexpr double kReconThin = 0.5;               // second order: least face depth / cell depth

using std::fabs;
using std::sqrt;
using std::tan;

// Floating fields are T: double for the oracle, Dual for its tangent-linear
// model (the differentiable parameters r, mf0, mfs and the Coulomb angle
// carry their tangents through every derived constant).
template <class T>
struct ConstsT {
    T g, r, gp, eps_h, peso, beta, cfl, mu, mfc, mf0, mfs, vmax1, vmax2, L, H;
    T tan1, tan2, tan3, tan4;
    // derived on the host, identically in the CUDA library (lsh_setup.h make_consts)
    T omr;       // 1 - r
    T inv_gp;    // 1 / (g (1 - r))
    T inv_eps;   // 1 / eps_h
    T inv_peso;  // 1 / peso
    T eps_1r;    // eps_h (1 + r)
    T g_mf02;    // g mf0^2
    T g_mfs2;    // g mfs^2
    T sqrt_g;    // sqrt(g)
    int law;
    int eig_sort;
};
using Consts = ConstsT<double>;

struct Geo {
    int nx, ny;
    std::vector<double> area;    // [ny]   cell area of row j
    std::vector<double> inv_area;  // [ny] 1 / area
    std::vector<double> len_v;   // [ny]   length of the vertical edges of row j
    std::vector<double> len_h;   // [ny+1] length of horizontal edge row y
    std::vector<double> tanR;    // [ny]   tan(lat_j)/R, 0 for Cartesian
    std::vector<double> wx, wy;  // [ny]   second-order volume-integral weights
};

// r, mf0, mfs and tan(angle1) come in as T so the tangent-linear model can
// seed them; for T = double these are the parameters themselves.
template <class T>
static ConstsT<T> make_consts_t(const lsh_params& p, T r, T mf0, T mfs, T tan1) {
    ConstsT<T> c;
    c.g = p.gravity; c.r = r; c.gp = p.gravity * (1.0 - r);
    c.eps_h = p.eps_h; c.peso = p.peso; c.beta = p.beta; c.cfl = p.cfl;
    // defTerminoFriccion, Coulomb law (Arista_kernel.cu:11-16): |tan(angle1)| * L/H
    c.mu = fabs(tan1) * (p.L / p.H);
    c.mfc = p.mfc; c.mf0 = mf0; c.mfs = mfs; c.vmax1 = p.vmax1; c.vmax2 = p.vmax2;
    c.L = p.L; c.H = p.H;
    c.tan1 = tan1; c.tan2 = tan(p.angle2); c.tan3 = tan(p.angle3); c.tan4 = tan(p.angle4);
    c.omr = 1.0 - r;
    c.inv_gp = 1.0 / c.gp;
    c.inv_eps = 1.0 / p.eps_h;
    c.inv_peso = 1.0 / p.peso;
    c.eps_1r = p.eps_h * (1.0 + r);
    c.g_mf02 = (p.gravity * mf0) * mf0;
    c.g_mfs2 = (p.gravity * mfs) * mfs;
    c.sqrt_g = std::sqrt(p.gravity);
    c.law = p.friction_law;
    c.eig_sort = p.eig_sort;
    return c;
}

static Consts make_consts(const lsh_params& p) { return make_consts_t<double>(p, p.r, p.mf0, p.mfs, tan(p.angle1)); }

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

// the same helpers on Dual (tangent-linear model)
inline Dual tmin(const Dual& a, const Dual& b) { return (b < a) ? b : a; }
inline Dual tmax(const Dual& a, const Dual& b) { return (b > a) ? b : a; }
inline Dual max0(const Dual& a) { return (a > 0.0) ? a : Dual(0.0); }
inline Dual vfac(const Dual& h, const Dual& eps_h) {
    if (h > eps_h) return 1.0 / h;
    const Dual h2 = h * h, m2 = eps_h * eps_h;
    return (kSqrt2 * h) / sqrt(fmad(h2, h2, m2 * m2));
}
inline Dual pow43(const Dual& h) { return h * cbrt_pos(h); }
inline int sgn(const Dual& x) { return sgn(x.v); }

// ... and on Cnt (operation counting)
long long g_cnt[kCntThreads][16];
inline Cnt tmin(const Cnt& a, const Cnt& b) { return (b < a) ? b : a; }
inline Cnt tmax(const Cnt& a, const Cnt& b) { return (b > a) ? b : a; }
inline Cnt max0(const Cnt& a) { return (a > 0.0) ? a : Cnt(0.0); }
inline Cnt vfac(const Cnt& h, const Cnt& eps_h) {
    if (h > eps_h) return 1.0 / h;
    const Cnt h2 = h * h, m2 = eps_h * eps_h;
    return (kSqrt2 * h) / sqrt(fmad(h2, h2, m2 * m2));
}
inline Cnt pow43(const Cnt& h) { return h * cbrt_pos(h); }
inline int sgn(const Cnt& x) { bump(kCmp); return sgn(x.v); }
inline double pow_pos(double x, double e) { return lshm::pow_pos(x, e); }

template <class T>
struct V4 { T x, y, z, w; };

// The fixed compare-and-swap sequence of Arista_kernel.cu:193-234, including
// its (i=2, j=1) compare, which leaves the larger of y/z in y (eig_sort 0);
// with eig_sort 1 that compare is (1,2) and the sequence is a true sort.
template <class T>
inline void sort_eig(V4<T>& D, int full) {
    auto cs = [](T& a, T& b) { if (a > b) { T t = b; b = a; a = t; } };
    cs(D.x, D.y); cs(D.x, D.z); cs(D.x, D.w); cs(D.y, D.z); cs(D.y, D.w);
    if (full) cs(D.y, D.z);
    else if (D.z > D.y) { T t = D.y; D.y = D.z; D.z = t; }
    cs(D.z, D.w);
}

// aproximarAutovalores1D (Arista_kernel.cu:152-237) given the two layers'
// depths, velocities (u1, u2) and the total normal discharge q:
// external u -+ sqrt(g h), internal uu -+ sqrt(g' h1 h2 F |1 - (u1-u2)^2 F / g'|).
// sqrt_h >= 0: sqrt(h1) is known and h2 == 0, so sqrt(g h) = sqrt(g) sqrt(h1).
template <class T>
inline V4<T> eig(T h1, T h2, T u1, T u2, T q, const ConstsT<T>& c, T sqrt_h = -1.0, bool mean_u = false) {
    const T h = h1 + h2;
    const T F = vfac(h, c.eps_h);
    // mean_u (the edge average, q = h1 u1 + h2 u2): with no granular layer and
    // h > eps_h, u = q vfac(h) = (h1 u1) / h1 is u1 itself (an exact
    // restatement of Arista_kernel.cu's u = q F there)
    const T u = (mean_u && h2 == 0.0 && h > c.eps_h) ? u1 : q * F;
    const T cg = (sqrt_h >= 0.0) ? c.sqrt_g * sqrt_h : sqrt(c.g * h);
    const T uu = fmad(u1, h2, u2 * h1) * F;
    const T d = u1 - u2;
    const T aux = fmad(-((d * d) * F), c.inv_gp, 1.0);
    const T ci = sqrt((((c.gp * h1) * h2) * F) * fabs(aux));
    V4<T> D{u - cg, uu - ci, uu + ci, u + cg};
    sort_eig(D, c.eig_sort);
    return D;
}

// defTerminoFriccion (Arista_kernel.cu:11-58): friction coefficient mu.
template <class T>
inline T friction_mu(T h1, T u1, T h2, T u2, const ConstsT<T>& c) {
    if (c.law == LSH_FRICTION_COULOMB) return c.mu;
    // Pouliquen law (the reference's #ifndef COULOMB branch)
    const T a = (10.0 * h1) * c.inv_eps;
    const T rr = 1.0 - c.r * (1.0 - exp_neg(a * a));
    const T gp = c.g * rr;
    const T fr1 = ((u1 * u1) * vfac(h1, c.eps_h)) / gp;
    const T fr2 = ((u2 * u2) * vfac(h2, c.eps_h)) / gp;
    const T fr = sqrt(fmad((1.0 - rr) * fr1, fr2, fr1 + fr2));
    const double beta = 0.136, L2 = 8.0e-4, chi = 1.0e-3;
    const T mustop = c.tan1 + (c.tan2 - c.tan1) / (1.0 + h2 / L2);
    const T mustart = c.tan3 + (c.tan4 - c.tan3) / (1.0 + h2 / L2);
    T muf;
    if (fr > beta) muf = c.tan1 + (c.tan2 - c.tan1) / (1.0 + beta * h2 / (fr * L2));
    else if (fabs(fr) < kEps) muf = c.tan3 + (c.tan4 - c.tan3) / (1.0 + h2 / L2);
    else muf = fmad(pow_pos(fr / beta, chi), mustop - mustart, mustart);
    return (muf * c.L) / c.H;
}

// 1 - r (1 - exp(-(10 h1 / eps_h)^2)) (Arista_kernel.cu:136, Volumen_kernel.cu:15)
template <class T>
inline T fsc_of(T h1, const ConstsT<T>& c) {
    const T a = (10.0 * h1) * c.inv_eps;
    return 1.0 - c.r * (1.0 - exp_neg(a * a));
}

// ---------------------------------------------------------------- edge flux
// One face state in the edge's normal frame: depth, normal and tangential
// discharge of each layer, bottom depth.
template <class T>
struct Face { T h1, qn1, qt1, h2, qn2, qt2, H; };

// Inputs of one edge.  A / B are the states facing the edge (cell values at
// first order, reconstructed face values at second order; B is the ghost at a
// boundary); hc* are the cell-average depths and acc*h the partial
// accumulators (h1, h2) the positivity limiter reads.
template <class T>
struct EdgeIn {
    Face<T> A, B;
    T len, area0, area1, inv_area0, inv_area1;
    bool interior;
    T hc0[2], hc1[2];
    T acc0h[2], acc1h[2];
};

// Edge output in the normal frame: per layer (mass, normal momentum,
// tangential momentum) to subtract from cell 0 (m) and cell 1 (p).
template <class T>
struct EdgeOut { T m[6], p[6]; T wave; };

// A face pair with no granular layer (h2 = qn2 = 0 on both faces): the
// two-layer formulas then reduce to the water layer's, but their derivatives
// with respect to h2 contain sqrt'(0) and are undefined.  The derivative
// taken is that of the single-layer branch (the CUDA kernels evaluate such
// edges with a single-layer specialisation): no sensitivity to h2 or q2.
// Values are untouched, so the double oracle is unchanged.
inline void single_layer_branch(Face<double>&, Face<double>&) {}
inline void single_layer_branch(Face<Cnt>&, Face<Cnt>&) {}
inline void single_layer_branch(Face<Dual>& A, Face<Dual>& B) {
    if (A.h2 == 0.0 && B.h2 == 0.0 && A.qn2 == 0.0 && B.qn2 == 0.0) {
        A.h2.d = B.h2.d = A.qn2.d = B.qn2.d = A.qt2.d = B.qt2.d = 0.0;
    }
}

// procesarArista (Arista_kernel.cu:324-645).  Returns false for a dry edge
// (no contribution at all, :397).
template <class T>
bool edge_flux(const EdgeIn<T>& e, T dt, const ConstsT<T>& c, EdgeOut<T>& o) {
    const T eps = c.eps_h;
    T Aq1 = e.A.qn1, Aq2 = e.A.qn2, Bq1 = e.B.qn1, Bq2 = e.B.qn2;
    const T Ah1 = e.A.h1, Ah2 = e.A.h2, Bh1 = e.B.h1, Bh2 = e.B.h2;
    const T H0 = e.A.H, H1 = e.B.H;

    const T h1ij = 0.5 * (Ah1 + Bh1);
    const T h2ij = 0.5 * (Ah2 + Bh2);
    if (!((h1ij >= kEps) || (h2ij >= kEps))) return false;

    // tratamientoSecoMojado (Arista_kernel.cu:301-321)
    if ((Ah2 < eps) && (H1 - Bh2 > H0)) Bq2 = 0.0;
    if ((Bh2 < eps) && (H0 - Ah2 > H1)) Aq2 = 0.0;
    if ((Ah1 < eps) && (H1 - Bh1 - Bh2 > H0 - Ah2)) Bq1 = 0.0;
    if ((Bh1 < eps) && (H0 - Ah1 - Ah2 > H1 - Bh2)) Aq1 = 0.0;
    if ((Ah2 + Ah1 < eps) && (H1 - Bh1 - Bh2 > H0)) { Bq1 = 0.0; Bq2 = 0.0; }
    if ((Bh2 + Bh1 < eps) && (H0 - Ah1 - Ah2 > H1)) { Aq1 = 0.0; Aq2 = 0.0; }

    // Roe-type averages (Arista_kernel.cu:375-395)
    const T fA1 = vfac(Ah1, eps), fB1 = vfac(Bh1, eps);
    const T fA2 = vfac(Ah2, eps), fB2 = vfac(Bh2, eps);
    const T sa1 = sqrt(Ah1), sb1 = sqrt(Bh1);
    const T u1ij = fmad(sa1, fA1 * Aq1, sb1 * (fB1 * Bq1)) / (sa1 + sb1 + kEps);
    const T sa2 = sqrt(Ah2), sb2 = sqrt(Bh2);
    const T u2ij = fmad(sa2, fA2 * Aq2, sb2 * (fB2 * Bq2)) / (sa2 + sb2 + kEps);
    // a cell's celerity sqrt(g h) is sqrt(g) sqrt(h1) when its granular layer is empty
    const bool oneA = (Ah2 == 0.0), oneB = (Bh2 == 0.0);

    // hydrostatic reconstruction (terminosPresion1D, :94-115)
    const T Hm = tmin(H0, H1);
    const T deta1 = max0(Bh1 + Bh2 - H1 + Hm) - max0(Ah1 + Ah2 - H0 + Hm);
    const T deta2 = max0(Bh2 - H1 + Hm) - max0(Ah2 - H0 + Hm);
    const T gh1 = c.g * h1ij, gh2 = c.g * h2ij;
    V4<T> tp{0.0, gh1 * deta1, 0.0, gh2 * fmad(c.omr, deta2, c.r * deta1)};

    // edge Coulomb switch (terminosPresion1DMod :134-147, identityModification :259-264)
    const T mu = friction_mu(h1ij, u1ij, h2ij, u2ij, c);
    const T sc = ((fsc_of(h1ij, c) * mu) * c.g) * h2ij;
    const bool coul = fabs(h2ij * u2ij) < (c.peso * sc) * dt;
    V4<T> tp2 = tp;
    if (coul) tp2.w = (gh2 * c.r) * deta1;

    // eigenvalue bounds (:427-444)
    const V4<T> D = eig(h1ij, h2ij, u1ij, u2ij, fmad(h1ij, u1ij, h2ij * u2ij), c, T(-1.0), true);
    const V4<T> E0 = eig(Ah1, Ah2, fA1 * Aq1, fA2 * Aq2, Aq1 + Aq2, c, oneA ? sa1 : -1.0);
    const V4<T> E1 = eig(Bh1, Bh2, fB1 * Bq1, fB2 * Bq2, Bq1 + Bq2, c, oneB ? sb1 : -1.0);
    const T aut1 = tmin(D.x, tmin(E0.x, E1.x));
    const T aut3 = tmax(D.w, tmax(E0.w, E1.w));
    T lmax = tmax(fabs(aut3), fabs(aut1));
    const T umax = tmax(fabs(u1ij), fabs(u2ij));
    if (umax > lmax) lmax = umax;
    T aut2 = tmax(fabs(D.y), fabs(D.z));
    if (sgn(aut1 + aut3) < 0) aut2 = -aut2;

    // PVM / IFCP coefficients (:446-465); the three parabola weights share
    // one reciprocal of (aut1-aut2)(aut1-aut3)(aut2-aut3)
    T a0, a1, a2;
    if ((fabs(aut1 - aut3) >= kEps) && (fabs(aut1 - aut2) >= kEps) && (fabs(aut2 - aut3) >= kEps)) {
        if ((h1ij >= eps) && (h2ij >= eps)) {
            const T d12 = aut1 - aut2, d13 = aut1 - aut3, d23 = aut2 - aut3;
            const T inv = 1.0 / ((d12 * d13) * d23);
            const T a = (fabs(aut1) * d23) * inv;
            const T b = -((fabs(aut2) * d13) * inv);
            const T cc = (fabs(aut3) * d12) * inv;
            a0 = fmad(a * aut2, aut3, fmad(b * aut1, aut3, (cc * aut1) * aut2));
            a1 = -fmad(a, aut2 + aut3, fmad(b, aut1 + aut3, cc * (aut1 + aut2)));
            a2 = a + b + cc;
        } else {
            const T inv = 1.0 / (aut3 - aut1);
            a0 = fmad(aut3, fabs(aut1), -(aut1 * fabs(aut3))) * inv;
            a1 = (fabs(aut3) - fabs(aut1)) * inv;
            a2 = 0.0;
        }
    } else {
        a0 = lmax; a1 = 0.0; a2 = 0.0;
    }

    // physical fluxes (getFlujo_1dC :62-92)
    const V4<T> FA{Aq1, (Ah1 < kEps) ? T(0.0) : (fA1 * Aq1) * Aq1, Aq2, (Ah2 < kEps) ? T(0.0) : (fA2 * Aq2) * Aq2};
    const V4<T> FB{Bq1, (Bh1 < kEps) ? T(0.0) : (fB1 * Bq1) * Bq1, Bq2, (Bh2 < kEps) ? T(0.0) : (fB2 * Bq2) * Bq2};
    const V4<T> dF{FB.x - FA.x, FB.y - FA.y, FB.z - FA.z, FB.w - FA.w};
    tp2 = V4<T>{tp2.x + dF.x, tp2.y + dF.y, tp2.z + dF.z, tp2.w + dF.w};
    const V4<T> half{0.5 * (dF.x + tp.x), 0.5 * (dF.y + tp.y), 0.5 * (dF.z + tp.z), 0.5 * (dF.w + tp.w)};

    // A * tp2 (:476-482)
    const V4<T> At{tp2.y, fmad(gh1, tp2.z, fmad(u1ij + u1ij, tp2.y, fmad(-u1ij, u1ij, gh1) * tp2.x)), tp2.w,
                fmad(c.r * gh2, tp2.x, fmad(fmad(-u2ij, u2ij, gh2), tp2.z, (u2ij + u2ij) * tp2.w))};

    // identityModification (:239-276)
    V4<T> I{deta1, Bq1 - Aq1, 0.0, Bq2 - Aq2};
    if (!coul) {
        if ((Ah1 > eps) && (Bh1 > eps)) I.x = I.x - deta2;
        I.z = deta2;
    }

    // viscosity and the two one-sided fluxes (:488-504)
    const V4<T> Q{0.5 * fmad(a0, I.x, fmad(a1, tp2.x, a2 * At.x)), 0.5 * fmad(a0, I.y, fmad(a1, tp2.y, a2 * At.y)),
               0.5 * fmad(a0, I.z, fmad(a1, tp2.z, a2 * At.z)), 0.5 * fmad(a0, I.w, fmad(a1, tp2.w, a2 * At.w))};
    const V4<T> Fm{half.x + (FA.x - Q.x), half.y + (FA.y - Q.y), half.z + (FA.z - Q.z), half.w + (FA.w - Q.w)};
    const V4<T> Fp{half.x + (Q.x - FB.x), half.y + (Q.y - FB.y), half.z + (Q.z - FB.z), half.w + (Q.w - FB.w)};

    // upwinded tangential velocity (:506-532)
    const T u1t = (fabs(Fm.x) < kEps) ? T(0.0) : ((Fm.x > 0.0) ? fA1 * e.A.qt1 : fB1 * e.B.qt1);
    const T u2t = (fabs(Fm.z) < kEps) ? T(0.0) : ((Fm.z > 0.0) ? fA2 * e.A.qt2 : fB2 * e.B.qt2);
    const T s1 = Fm.x * u1t, s2 = Fm.z * u2t;

    // normal-frame fluxes times the edge length: (mass, normal, tangential);
    // the tangential part is +s for cell 0 and -s for cell 1 (:534-552)
    T M[6] = {Fm.x, Fm.y, s1, Fm.z, Fm.w, s2};
    T P[6] = {Fp.x, Fp.y, -s1, Fp.z, Fp.w, -s2};
    for (int k = 0; k < 6; ++k) { P[k] = e.len * P[k]; M[k] = e.len * M[k]; }

    // positivity limiter on the partially accumulated depths (:554-609)
    const T b0 = dt * e.inv_area0;
    const T hp00 = fmad(b0, e.acc0h[0], e.hc0[0]), hp01 = fmad(b0, e.acc0h[1], e.hc0[1]);
    T hp10 = 0.0, hp11 = 0.0;
    if (e.interior) {
        const T b1 = dt * e.inv_area1;
        hp10 = fmad(b1, e.acc1h[0], e.hc1[0]); hp11 = fmad(b1, e.acc1h[1], e.hc1[1]);
    }
    const T factor = 1.0 * c.beta;
    for (int layer = 0; layer < 2; ++layer) {
        const int k = 3 * layer;
        // the reference limits when dt > min(hp area / (beta M + eps)) over the
        // outflow sides; the denominators are positive, so the test is
        // dt (beta M + eps) > hp area, and the quotients are formed only for a
        // limited edge (the CUDA kernels evaluate the same sequence)
        const bool oa = (M[k] > 0.0), ob = e.interior && (P[k] > 0.0);
        const T ha = (layer ? hp01 : hp00) * e.area0, hb = (layer ? hp11 : hp10) * e.area1;
        const T da = oa ? fmad(factor, M[k], kEps) : T(1.0), db = ob ? fmad(factor, P[k], kEps) : T(1.0);
        const bool lim = (oa && !(dt * da <= ha)) || (ob && !(dt * db <= hb));
        if (lim) {
            const T dta = oa ? ha / da : T(kBig), dtb = ob ? hb / db : T(kBig);
            const T dtl = tmin(dta, dtb);
            const T alpha = dtl / (dt + kEps);
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
template <class T>
T edge_initial_wave(const Face<T>& A, const Face<T>& B, T len, const ConstsT<T>& c) {
    const T eps = c.eps_h;
    const T h1ij = 0.5 * (A.h1 + B.h1);
    const T fA1 = vfac(A.h1, eps), fB1 = vfac(B.h1, eps);
    T sa = sqrt(A.h1), sb = sqrt(B.h1);
    const T u1ij = fmad(sa, fA1 * A.qn1, sb * (fB1 * B.qn1)) / (sa + sb + kEps);
    const T h2ij = 0.5 * (A.h2 + B.h2);
    const T fA2 = vfac(A.h2, eps), fB2 = vfac(B.h2, eps);
    sa = sqrt(A.h2); sb = sqrt(B.h2);
    const T u2ij = fmad(sa, fA2 * A.qn2, sb * (fB2 * B.qn2)) / (sa + sb + kEps);
    const V4<T> D = eig(h1ij, h2ij, u1ij, u2ij, fmad(h1ij, u1ij, h2ij * u2ij), c);
    T lmax = tmax(D.x, D.w);
    const T b = tmax(fabs(u1ij), fabs(u2ij));
    if (b > lmax) lmax = b;
    if (lmax < eps) lmax = lmax + eps;
    return len * lmax;
}

// ---------------------------------------------------------------- state update
// filtroEstado (Volumen_kernel.cu:92-180); its "complex" block is dead (cf = 0).
template <class T>
inline void filtro(T w[6], T dt, const ConstsT<T>& c) {
    if (w[0] < 0.0) w[0] = 0.0;
    if (w[3] < 0.0) w[3] = 0.0;
    for (int layer = 0; layer < 2; ++layer) {
        const int k = 3 * layer;
        const T x = w[k] * c.inv_eps;
        const T x2 = x * x;
        const T d = fmad(x2, x2, kEps);
        // exp(-dt / d) is exactly 1 once dt / d < 2^-54; below this bound
        // (conservative by far more than the roundings of 1/d and dt*(1/d))
        // the factor is 1 and the division is not needed
        if (dt < d * 0x1.fp-55) continue;
        const T aux = exp_neg(dt * (1.0 / d));
        w[k + 1] = w[k + 1] * aux;
        w[k + 2] = w[k + 2] * aux;
    }
    for (int layer = 0; layer < 2; ++layer) {
        const T vmax = layer ? c.vmax2 : c.vmax1;
        if (vmax > 0.0) {
            const int k = 3 * layer;
            const T h = w[k];
            const T f = vfac(h, c.eps_h);
            T ux = f * w[k + 1], uy = f * w[k + 2];
            const T u = sqrt(fmad(ux, ux, uy * uy));
            if (u > vmax) {
                const T s = vmax / u;
                ux = ux * s; uy = uy * s;
                w[k + 1] = ux * h; w[k + 2] = uy * h;
            }
        }
    }
}

// disImplicita (Volumen_kernel.cu:31-90): semi-implicit interlayer and bottom
// friction.  Speeds of the previous state `wo` enter the coefficients.
template <class T>
inline void dis_implicita(const T wo[6], T w[6], T dt, const ConstsT<T>& c) {
    if (w[0] < 0.0) w[0] = 0.0;
    if (w[3] < 0.0) w[3] = 0.0;
    const T eps = c.eps_h;
    const T h1 = w[0], h2 = w[3];
    const T f1 = vfac(h1, eps), f2 = vfac(h2, eps);
    T u1x = f1 * w[1], u1y = f1 * w[2], u2x = f2 * w[4], u2y = f2 * w[5];
    const T fo1 = vfac(wo[0], eps), fo2 = vfac(wo[3], eps);
    const T uo1x = fo1 * wo[1], uo1y = fo1 * wo[2], uo2x = fo2 * wo[4], uo2y = fo2 * wo[5];
    const T dx = uo1x - uo2x, dy = uo1y - uo2y;
    const T du = sqrt(fmad(dx, dx, dy * dy));
    const T u1 = sqrt(fmad(uo1x, uo1x, uo1y * uo1y));
    const T u2 = sqrt(fmad(uo2x, uo2x, uo2y * uo2y));
    if ((h1 > 0.0) && (h2 > 0.0)) {
        const T hmod = fmad(c.r, h1, h2);
        const T m = (hmod > c.eps_1r) ? hmod : c.eps_1r;
        const T hm2 = hmod * hmod, m2 = m * m;
        const T hh = hmod / sqrt(fmad(hm2, hm2, m2 * m2));
        const T k12 = ((dt * kSqrt2) * hh) * (c.mfc * du);
        const T c1 = k12 * h2;
        const T c2 = (k12 * c.r) * h1;
        const T c3 = ((dt * c.g_mfs2) * u2) / (pow43(h2) + kEps);
        const T e1 = 1.0 + c1, e2 = 1.0 + c2 + c3;
        const T det = 1.0 / fmad(e1, e2, -(c1 * c2));
        w[1] = (h1 * fmad(u1x, e2, c1 * u2x)) * det;
        w[4] = (h2 * fmad(u2x, e1, c2 * u1x)) * det;
        w[2] = (h1 * fmad(u1y, e2, c1 * u2y)) * det;
        w[5] = (h2 * fmad(u2y, e1, c2 * u1y)) * det;
    }
    // bottom friction: h u / (1 + c1) with u = vfac(h) q; above eps_h,
    // vfac(h) = 1/h and h u is q itself
    // 1 / (1 + c1) with c1 = X / Y is Y / (Y + X): one division
    if ((h1 > 0.0) && (h2 < eps)) {
        const T Y = pow43(h1) + kEps, X = (dt * c.g_mf02) * u1;
        const T inv = Y / (Y + X);
        if (h1 > eps) { w[1] = w[1] * inv; w[2] = w[2] * inv; }
        else { w[1] = (h1 * (f1 * w[1])) * inv; w[2] = (h1 * (f1 * w[2])) * inv; }
    }
    if ((h2 > 0.0) && (h1 < eps)) {
        const T Y = pow43(h2) + kEps, X = (dt * c.g_mfs2) * u2;
        const T inv = Y / (Y + X);
        if (h2 > eps) { w[4] = w[4] * inv; w[5] = w[5] * inv; }
        else { w[4] = (h2 * (f2 * w[4])) * inv; w[5] = (h2 * (f2 * w[5])) * inv; }
    }
}

// coulomb (Volumen_kernel.cu:7-26): granular stop / slow-down.
template <class T>
inline void coulomb(T w[6], T dt, const ConstsT<T>& c) {
    if (!(w[3] > 0.0)) {  // no granular layer: the reference's factor is 0
        w[4] = w[4] * 0.0;
        w[5] = w[5] * 0.0;
        return;
    }
    T mu = c.mu;
    if (c.law != LSH_FRICTION_COULOMB) {
        const T u1 = sqrt(fmad(w[1], w[1], w[2] * w[2])) * vfac(w[0], c.eps_h);
        const T u2 = sqrt(fmad(w[4], w[4], w[5] * w[5])) * vfac(w[3], c.eps_h);
        mu = friction_mu(w[0], u1, w[3], u2, c);
    }
    const T sc = ((((fsc_of(w[0], c) * mu) * c.g) * w[3]) * dt);
    const T normq = sqrt(fmad(w[4], w[4], w[5] * w[5]));
    T aux = 0.0;
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
template <class T>
inline void volume_update(const T wo[6], const T acc[7], T w[6], T& rate, double area,
                          double inv_area, double tanR, T dt, const ConstsT<T>& c) {
    (void)area;
    rate = (acc[6] < kEps) ? T(0.0) : acc[6] * inv_area;
    const T b = dt * inv_area;
    for (int k = 0; k < 6; ++k) w[k] = fmad(b, acc[k], wo[k]);
    if (tanR != 0.0) {
        for (int layer = 0; layer < 2; ++layer) {
            const int k = 3 * layer;
            if (wo[k] == 0.0 && wo[k + 1] == 0.0 && wo[k + 2] == 0.0) continue;  // adds exactly 0
            const T ux = vfac(wo[k], c.eps_h) * wo[k + 1];
            const T s = dt * (ux * tanR);
            w[k + 1] = fmad(s, wo[k + 2], w[k + 1]);
            w[k + 2] = fmad(-s, wo[k + 1], w[k + 2]);
        }
    }
    filtro(w, dt, c);
    dis_implicita(wo, w, dt, c);
    coulomb(w, dt, c);
}

// ---------------------------------------------------------------- solver
template <class T>
struct Solver {
    lsh_params p;
    ConstsT<T> c;
    Geo g;
    int nx, ny;
    size_t N;
    std::vector<T> acc[7];
    std::vector<T> slope_x[7], slope_y[7];  // second order: half minmod differences
    std::vector<T> dti;

    size_t last_argmax = 0;  // cell of the largest rate of the last stage / initial pass (first on ties)
    std::vector<T> rate_buf;

    explicit Solver(const lsh_params& prm) : Solver(prm, make_consts_t<T>(prm, prm.r, prm.mf0, prm.mfs, T(tan(prm.angle1)))) {}
    Solver(const lsh_params& prm, const ConstsT<T>& cc) : p(prm), c(cc), g(make_geo(prm)) {
        nx = prm.nx; ny = prm.ny; N = size_t(nx) * ny;
        for (int k = 0; k < 7; ++k) acc[k].assign(N, 0.0);
        if (prm.order == 2)
            for (int k = 0; k < 7; ++k) { slope_x[k].assign(N, 0.0); slope_y[k].assign(N, 0.0); }
        dti.assign(N, kBig);
    }

    // Face<T> value of cell `id` on side `side` (0 W, 1 E, 2 S (toward j-1), 3 N
    // (toward j+1)) in the edge frame of normal (nx, ny): normal discharge
    // q.n and tangential q_y nx - q_x ny (Arista_kernel.cu:363-371, 509-525).
    // First order (or a cell whose slopes were zeroed): the cell value itself.
    Face<T> face(const T* const* W, size_t id, int side, T nxv, T nyv) const {
        T w[6], Hf;
        for (int k = 0; k < 6; ++k) w[k] = W[k][id];
        Hf = W[6][id];
        if (p.order == 2) {
            const std::vector<T>* s = (side < 2) ? slope_x : slope_y;
            const T sg = (side & 1) ? 1.0 : -1.0;
            const T de1 = s[0][id], de2 = s[3][id], dH = s[6][id];
            w[0] = w[0] + sg * (de1 - de2);
            w[1] = w[1] + sg * s[1][id];
            w[2] = w[2] + sg * s[2][id];
            w[3] = w[3] + sg * (de2 + dH);
            w[4] = w[4] + sg * s[4][id];
            w[5] = w[5] + sg * s[5][id];
            Hf = Hf + sg * dH;
        }
        Face<T> f;
        f.h1 = w[0]; f.qn1 = w[1] * nxv + w[2] * nyv; f.qt1 = w[2] * nxv - w[1] * nyv;
        f.h2 = w[3]; f.qn2 = w[4] * nxv + w[5] * nyv; f.qt2 = w[5] * nxv - w[4] * nyv;
        f.H = Hf;
        return f;
    }

    // The edge of colour pass (dir, par) number (line, along): its cells,
    // outward normal of cell 0, length and boundary factor
    // (Arista_kernel.cu:651-838: vertical edge x between columns x-1 and x,
    // horizontal edge y between rows y-1 and y; row 0's outer edge is "sup").
    struct EdgeGeo { size_t id0, id1; bool interior; T nx, ny, len, bor; int side0, side1; };
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
    static Face<T> ghost(const Face<T>& a, T bor) {
        Face<T> b = a;
        b.qn1 = a.qn1 * bor;
        b.qn2 = a.qn2 * bor;
        return b;
    }

    // the cell value in the edge frame (the initial-dt pass is first order)
    static Face<T> face_cell(const T* const* W, size_t id, T nxv, T nyv) {
        Face<T> f;
        f.h1 = W[0][id]; f.qn1 = W[1][id] * nxv + W[2][id] * nyv; f.qt1 = W[2][id] * nxv - W[1][id] * nyv;
        f.h2 = W[3][id]; f.qn2 = W[4][id] * nxv + W[5][id] * nyv; f.qt2 = W[5][id] * nxv - W[4][id] * nyv;
        f.H = W[6][id];
        return f;
    }

    static T minmod(T a, T b) {
        if (a > 0.0 && b > 0.0) return (a < b) ? a : b;
        if (a < 0.0 && b < 0.0) return (a > b) ? a : b;
        return 0.0;
    }

    // minmod slopes of (eta1, q1x, q1y, eta2, q2x, q2y, H), halved, with a
    // first-order fallback for any cell where a reconstructed depth would fall
    // below kReconThin times the cell's.
    void reconstruct(const T* const* W) {
        const int NX = nx, NY = ny;
#pragma omp parallel for schedule(static)
        for (int j = 0; j < NY; ++j) {
            for (int i = 0; i < NX; ++i) {
                const size_t id = size_t(j) * NX + i;
                auto pv = [&](size_t q, int k) -> T {
                    switch (k) {
                        case 0: return (W[0][q] + W[3][q]) - W[6][q];
                        case 3: return W[3][q] - W[6][q];
                        case 6: return W[6][q];
                        default: return W[k][q];
                    }
                };
                T sx[7], sy[7];
                for (int k = 0; k < 7; ++k) {
                    const T pc = pv(id, k);
                    sx[k] = (i > 0 && i < NX - 1) ? 0.5 * minmod(pc - pv(id - 1, k), pv(id + 1, k) - pc) : T(0.0);
                    sy[k] = (j > 0 && j < NY - 1) ? 0.5 * minmod(pc - pv(id - NX, k), pv(id + NX, k) - pc) : T(0.0);
                }
                const T h1 = W[0][id], h2 = W[3][id];
                const T dh1x = sx[0] - sx[3], dh2x = sx[3] + sx[6];
                const T dh1y = sy[0] - sy[3], dh2y = sy[3] + sy[6];
                // first order where a reconstructed depth would fall below half
                // the cell's (a thin face with a finite discharge has an unbounded
                // velocity, and its wave speed collapses dt)
                const T g1 = kReconThin * h1, g2 = kReconThin * h2;
                const bool bad = (h1 + dh1x < g1) || (h1 - dh1x < g1) || (h2 + dh2x < g2) || (h2 - dh2x < g2) ||
                                 (h1 + dh1y < g1) || (h1 - dh1y < g1) || (h2 + dh2y < g2) || (h2 - dh2y < g2);
                for (int k = 0; k < 7; ++k) {
                    slope_x[k][id] = bad ? T(0.0) : sx[k];
                    slope_y[k][id] = bad ? T(0.0) : sy[k];
                }
            }
        }
    }

    // One colour pass over horizontal (dir 0) or vertical (dir 1) edges of
    // parity `par` (Arista_kernel.cu:651-838).  Edges of one colour touch
    // disjoint cells, so the loop is race-free.
    void pass(const T* const* W, int dir, int par, T dt) {
        const int NX = nx, NY = ny;
        const int nlines = (dir == 0) ? (NY - par) / 2 + 1 : (NX - par) / 2 + 1;  // edge rows / columns
        const int nalong = (dir == 0) ? NX : NY;
#pragma omp parallel for schedule(static)
        for (int t = 0; t < nlines; ++t) {
            const int e = par + 2 * t;  // edge row y (dir 0) or column x (dir 1)
            for (int s = 0; s < nalong; ++s) {
                const EdgeGeo q = edge_geo(dir, e, s);
                EdgeIn<T> in;
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
                EdgeOut<T> o;
                single_layer_branch(in.A, in.B);
                if (!edge_flux(in, dt, c, o)) continue;
                // rotate the normal-frame fluxes back: x = fn nx - ft ny, y = fn ny + ft nx
                const T nxv = q.nx, nyv = q.ny;
                T d0[6], d1[6];
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
    void volume_integral(const T* const* W) {
        const int NX = nx, NY = ny;
#pragma omp parallel for schedule(static)
        for (int j = 0; j < NY; ++j) {
            for (int i = 0; i < NX; ++i) {
                const size_t id = size_t(j) * NX + i;
                const T gh1 = c.g * W[0][id], gh2 = c.g * W[3][id];
                const T e1x = 2.0 * slope_x[0][id], e2x = 2.0 * slope_x[3][id];
                const T e1y = 2.0 * slope_y[0][id], e2y = 2.0 * slope_y[3][id];
                acc[1][id] -= c.peso * ((gh1 * e1x) * g.wx[j]);
                acc[4][id] -= c.peso * ((gh2 * fmad(c.omr, e2x, c.r * e1x)) * g.wx[j]);
                acc[2][id] -= c.peso * ((gh1 * e1y) * g.wy[j]);
                acc[5][id] -= c.peso * ((gh2 * fmad(c.omr, e2y, c.r * e1y)) * g.wy[j]);
            }
        }
    }

    // One forward-Euler stage: W -> Wn with dt; returns min per-cell dt.
    T stage(const T* const* W, T* const* Wn, T dt) {
        for (int k = 0; k < 7; ++k) std::fill(acc[k].begin(), acc[k].end(), 0.0);
        if (p.order == 2) reconstruct(W);
        // ShallowWater.cu:391-427: hor-even, hor-odd, ver-even, ver-odd
        pass(W, 0, 0, dt);
        pass(W, 0, 1, dt);
        pass(W, 1, 0, dt);
        pass(W, 1, 1, dt);
        if (p.order == 2) volume_integral(W);
        const int NX = nx, NY = ny;
        rate_buf.resize(N);
#pragma omp parallel for schedule(static)
        for (int j = 0; j < NY; ++j) {
            for (int i = 0; i < NX; ++i) {
                const size_t id = size_t(j) * NX + i;
                T wo[6], a[7], w[6], rate;
                for (int k = 0; k < 6; ++k) wo[k] = W[k][id];
                for (int k = 0; k < 7; ++k) a[k] = acc[k][id];
                volume_update(wo, a, w, rate, g.area[j], g.inv_area[j], g.tanR[j], dt, c);
                for (int k = 0; k < 6; ++k) Wn[k][id] = w[k];
                rate_buf[id] = rate;
            }
        }
        // the largest rate; the first cell holding it (the maximum is exact, so
        // the order of the scan changes nothing but which of tied cells is named)
        T mx = 0.0;
        last_argmax = 0;
        for (size_t id = 0; id < N; ++id)
            if (rate_buf[id] > mx) { mx = rate_buf[id]; last_argmax = id; }
        return dt_of(mx);
    }

    // dt from the largest acc_w / area; 1e30 when no cell has a wave speed
    T dt_of(T max_rate) const { return (max_rate > 0.0) ? (2.0 * c.cfl) / max_rate : T(kBig); }

    T initial_dt(const T* const* W) {
        std::vector<T>& aw = acc[6];
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
                        const Face<T> A = face_cell(W, q.id0, q.nx, q.ny);
                        const Face<T> B = q.interior ? face_cell(W, q.id1, q.nx, q.ny) : ghost(A, q.bor);
                        const T wv = edge_initial_wave(A, B, q.len, c);
                        aw[q.id0] += wv;
                        if (q.interior) aw[q.id1] += wv;
                    }
                }
            }
        }
        T mx = 0.0;
        last_argmax = 0;
        for (int j = 0; j < NY; ++j)
            for (int i = 0; i < NX; ++i) {
                const T a = aw[size_t(j) * NX + i];
                const T rate = (a < kEps) ? T(0.0) : a * g.inv_area[j];  // Volumen_kernel.cu:226
                if (rate > mx) { mx = rate; last_argmax = size_t(j) * NX + i; }
            }
        return dt_of(mx);
    }
};

// A run of `nsteps` steps with the gauge misfit
//   J = sum_{n=1..nsteps} sum_g (eta1_n[g] - target[(n-1) ng + g])^2,  eta1 = h1 + h2 - H,
// on T = double (the forward) or T = Dual (its tangent-linear model: state,
// dt and the parameters r, mf0, mfs, angle1 carry tangents; dt is the
// state-dependent CFL step, differentiated through the argmax cell).  The
// time loop is orc_run's.  eta (nsteps * ng, may be NULL) gets the gauge
// series; a NULL target means J = 0.
// Thin-layer projection of the tangent (h_adj > 0): a layer thinner than
// h_adj is passive in the linearisation, its (h, qx, qy) tangents set to 0.
// Values are untouched, so the forward is unchanged.
inline void thin_layer_projection(double* const*, size_t, double) {}
inline void thin_layer_projection(Cnt* const*, size_t, double) {}
inline void thin_layer_projection(Dual* const* W, size_t N, double h_adj) {
    if (!(h_adj > 0.0)) return;
    for (size_t i = 0; i < N; ++i)
        for (int l = 0; l < 2; ++l)
            if (W[3 * l][i].v < h_adj) { W[3 * l][i].d = 0.0; W[3 * l + 1][i].d = 0.0; W[3 * l + 2][i].d = 0.0; }
}

template <class T>
int run_misfit(const lsh_params& p, const ConstsT<T>& c, T* const* W, long long nsteps, bool initial, T& dt,
               int ng, const int* gauges, const double* target, T& J, double* eta, double h_adj = 0.0) {
    Solver<T> S(p, c);
    const size_t N = S.N;
    thin_layer_projection(W, N, h_adj);
    std::vector<T> tmp[6], tmp2[6];
    T* Wn[7];
    T* W2[7];
    for (int k = 0; k < 6; ++k) { tmp[k].resize(N); Wn[k] = tmp[k].data(); }
    Wn[6] = W[6];
    if (p.order == 2) {
        for (int k = 0; k < 6; ++k) { tmp2[k].resize(N); W2[k] = tmp2[k].data(); }
        W2[6] = W[6];
    }
    if (initial) dt = S.initial_dt(W);
    J = 0.0;
    for (long long n = 0; n < nsteps; ++n) {
        T dtn;
        if (p.order == 1) {
            dtn = S.stage(W, Wn, dt);
            for (int k = 0; k < 6; ++k) std::copy(Wn[k], Wn[k] + N, W[k]);
        } else {
            dtn = S.stage(W, Wn, dt);
            S.stage(Wn, W2, dt);
            for (int k = 0; k < 6; ++k)
                for (size_t id = 0; id < N; ++id) W[k][id] = 0.5 * (W[k][id] + W2[k][id]);
        }
        dt = dtn;
        thin_layer_projection(W, N, h_adj);
        for (int gi = 0; gi < ng; ++gi) {
            const size_t id = size_t(gauges[gi]);
            const T e = (W[0][id] + W[3][id]) - W[6][id];
            if (eta) eta[n * ng + gi] = value(e);
            if (target) {
                const T d = e - target[n * ng + gi];
                J = fmad(d, d, J);
            }
        }
    }
    return LSH_OK;
}

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
    orc::Solver<double> S(*p);
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
    orc::Solver<double> S(*p);
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

// Forward run with the gauge misfit (run_misfit on double).  initial != 0:
// dt from the initial-dt pass of W, else *dt_io.  On exit W is the final
// state, *dt_io the next dt, *J the misfit.
int orc_misfit_run(const lsh_params* p, double* const* W, long long nsteps, int initial, double* dt_io, int ng,
                   const int* gauges, const double* target, double* J, double* eta) {
    if (int s = check_params(p)) return s;
    const orc::Consts c = orc::make_consts(*p);
    return orc::run_misfit<double>(*p, c, W, nsteps, initial != 0, *dt_io, ng, gauges, target, *J, eta);
}

// Tangent-linear model of orc_misfit_run: dW[6] (tangents of h1..q2y, in and
// out), dpar[4] the tangents of (angle1, mf0, mfs, r), *ddt_io the tangent of
// dt (in and out; ignored on entry when initial != 0).  Values of W, dt and
// J are bit-identical to orc_misfit_run's; *dJ is the directional derivative
// (h_adj > 0: of the thin-layer-projected linearisation, run_misfit).
int orc_tl_run(const lsh_params* p, double* const* W, double* const* dW, const double* dpar, long long nsteps,
               int initial, double* dt_io, double* ddt_io, int ng, const int* gauges, const double* target,
               double* J, double* dJ, double* eta, double h_adj) {
    if (int s = check_params(p)) return s;
    using orc::Dual;
    const size_t N = size_t(p->nx) * p->ny;
    std::vector<Dual> st[7];
    Dual* Wd[7];
    for (int k = 0; k < 7; ++k) {
        st[k].resize(N);
        for (size_t i = 0; i < N; ++i) st[k][i] = Dual(W[k][i], (k < 6 && dW[k]) ? dW[k][i] : 0.0);
        Wd[k] = st[k].data();
    }
    const double t1 = std::tan(p->angle1);
    const Dual tan1(t1, (1.0 + t1 * t1) * dpar[0]);
    const orc::ConstsT<Dual> c =
        orc::make_consts_t<Dual>(*p, Dual(p->r, dpar[3]), Dual(p->mf0, dpar[1]), Dual(p->mfs, dpar[2]), tan1);
    Dual dt(*dt_io, initial ? 0.0 : *ddt_io);
    Dual Jd;
    const int s = orc::run_misfit<Dual>(*p, c, Wd, nsteps, initial != 0, dt, ng, gauges, target, Jd, eta, h_adj);
    for (int k = 0; k < 6; ++k)
        for (size_t i = 0; i < N; ++i) {
            W[k][i] = st[k][i].v;
            if (dW[k]) dW[k][i] = st[k][i].d;
        }
    *dt_io = dt.v;
    *ddt_io = dt.d;
    *J = Jd.v;
    *dJ = Jd.d;
    return s;
}

// FP64 operations of `nsteps` steps from W as the oracle performs them (the
// reference scheme's arithmetic; the CUDA kernels skip some of it on dry and
// single-layer work), by kind: counts[0..9] = add/sub, mul, fma, div, sqrt,
// exp, cbrt, pow, compare, abs.  The initial-dt pass is included once.
int orc_count_ops(const lsh_params* p, const double* const* W, long long nsteps, long long* counts) {
    if (int s = check_params(p)) return s;
    using orc::Cnt;
    const size_t N = size_t(p->nx) * p->ny;
    std::vector<Cnt> st[7];
    Cnt* Wc[7];
    for (int k = 0; k < 7; ++k) {
        st[k].resize(N);
        for (size_t i = 0; i < N; ++i) st[k][i] = Cnt(W[k][i]);
        Wc[k] = st[k].data();
    }
    std::memset(orc::g_cnt, 0, sizeof(orc::g_cnt));
    const orc::ConstsT<Cnt> c = orc::make_consts_t<Cnt>(*p, Cnt(p->r), Cnt(p->mf0), Cnt(p->mfs), Cnt(std::tan(p->angle1)));
    std::memset(orc::g_cnt, 0, sizeof(orc::g_cnt));
    Cnt dt, J;
    const int s = orc::run_misfit<Cnt>(*p, c, Wc, nsteps, true, dt, 0, nullptr, nullptr, J, nullptr);
    for (int k = 0; k < orc::kNumCnt; ++k) {
        long long t = 0;
        for (int th = 0; th < orc::kCntThreads; ++th) t += orc::g_cnt[th][k];
        counts[k] = t;
    }
    return s;
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
