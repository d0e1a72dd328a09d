// lsh_scheme.cuh -- FP64 device math of the two-layer time step.
//
// One thread evaluates one edge (edge functions) or one cell (volume
// functions).  The arithmetic is the LandSlide-HySEA scheme:
//   edge flux            src/GPU/Arista_kernel.cu:324-645 (procesarArista)
//   wet/dry fix          src/GPU/Arista_kernel.cu:301-321
//   hydrostatic terms    src/GPU/Arista_kernel.cu:94-150
//   eigenvalue bounds    src/GPU/Arista_kernel.cu:152-237
//   identity mod.        src/GPU/Arista_kernel.cu:239-276
//   initial-dt wave      src/GPU/Arista_kernel.cu:1040-1127
//   state update         src/GPU/Volumen_kernel.cu:7-180, 231-284
// evaluated in double precision on structure-of-arrays state.  Conventions
// (kept identical in the CPU oracle so both are one FP64 scheme up to
// rounding): EPSILON keeps FLT_EPSILON's value; u = vfac(h) * q with
// vfac(h) = sqrt(2) h / sqrt(h^4 + max(h, eps_h)^4), h^4 = (h*h)*(h*h);
// exp, cbrt and log come from lsh_fpmath.h (IEEE basic operations only, so
// host and device give identical bits); h^(4/3) = h * cbrt(h).  The library
// is compiled with --fmad=false: no implicit a*b+c contraction, so the FP64
// operation sequence here is exactly the oracle's and results match it bit
// for bit.
#pragma once

#include <cstdint>

#include "lsh_fpmath.h"

namespace lsh {

constexpr double kEps = 1.1920928955078125e-07;  // FLT_EPSILON (Constantes.hxx:13)
constexpr double kSqrt2 = 1.41421356237309504880;
constexpr double kBig = 1e30;

// Scalars every kernel needs; passed by value (kernel parameter space).
struct Consts {
    double g, r, gp, eps_h, peso, beta, cfl, mu, mfc, mf0, mfs, vmax1, vmax2, L, H;
    double tan1, tan2, tan3, tan4;
    double borde_sup, borde_inf, borde_izq, borde_der;
    int law;
    int order;
    int nx, ny;
    int track_eta;
    int eig_sort;
};

// Per-row geometry (device arrays, ny or ny+1 entries).
struct Geo {
    const double* area;   // [ny]
    const double* len_v;  // [ny]
    const double* len_h;  // [ny+1]
    const double* tanR;   // [ny]
    const double* wx;     // [ny]
    const double* wy;     // [ny]
};

// Device-resident time record: dt and t never leave the device between steps.
struct TimeRec {
    double t;                        // simulated time
    double dt;                       // dt of the next step
    double t_end;                    // stop once t >= t_end
    double dt_min;                   // stall guard (0: off)
    unsigned long long dtmin_bits;   // running min of per-cell dt (bits of a positive double)
    long long steps;                 // steps taken
    int done;                        // 1 once t >= t_end (kernels then return at once)
    int err;                         // sticky error bits (LSH status values as bits)
};

template <class T> struct V4 { T x, y, z, w; };

__device__ __forceinline__ double tmin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double tmax(double a, double b) { return (b > a) ? b : a; }
__device__ __forceinline__ double max0(double a) { return (a > 0.0) ? a : 0.0; }

__device__ __forceinline__ double exp_neg(double x) { return lshm::exp_neg(x); }

__device__ __forceinline__ double vfac(double h, double eps_h) {
    const double m = (h > eps_h) ? h : eps_h;
    const double h2 = h * h, m2 = m * m;
    return (kSqrt2 * h) / sqrt(h2 * h2 + m2 * m2);
}

__device__ __forceinline__ double pow43(double h) { return h * lshm::cbrt_pos(h); }

__device__ __forceinline__ int sgn(double x) { return (fabs(x) < kEps) ? 0 : ((x > 0) ? 1 : -1); }

// x == +0 or -0, by bit pattern (integer pipe)
__device__ __forceinline__ bool is_zero(double x) { return (__double_as_longlong(x) << 1) == 0; }

__device__ __forceinline__ bool is_bad(double x) {
    // NaN or Inf by bit pattern (integer pipe, no FP64 compare)
    return (__double_as_longlong(x) & 0x7ff0000000000000LL) == 0x7ff0000000000000LL;
}

// Compare-and-swap sequence of Arista_kernel.cu:193-234 (with its (2,1)
// compare) or, with `full`, the same sequence made a true sort.
__device__ __forceinline__ void sort_eig(V4<double>& D, int full) {
    double t;
    if (D.x > D.y) { t = D.y; D.y = D.x; D.x = t; }
    if (D.x > D.z) { t = D.z; D.z = D.x; D.x = t; }
    if (D.x > D.w) { t = D.w; D.w = D.x; D.x = t; }
    if (D.y > D.z) { t = D.z; D.z = D.y; D.y = t; }
    if (D.y > D.w) { t = D.w; D.w = D.y; D.y = t; }
    if (full) { if (D.y > D.z) { t = D.z; D.z = D.y; D.y = t; } }
    else if (D.z > D.y) { t = D.y; D.y = D.z; D.z = t; }
    if (D.z > D.w) { t = D.w; D.w = D.z; D.z = t; }
}

// aproximarAutovalores1D: (u1, u2) velocities and the factor vfac(h1 + h2)
// already known; returns the sorted 4 estimates.
__device__ __forceinline__ V4<double> eig_core(double h1, double h2, double u1, double u2, double q,
                                               const Consts& c) {
    const double h = h1 + h2;
    const double F = vfac(h, c.eps_h);
    const double u = q * F;
    const double cg = sqrt(c.g * h);
    const double uu = (u1 * h2 + u2 * h1) * F;
    const double d = u1 - u2;
    const double aux = 1.0 - d * d * F / c.gp;
    const double ci = sqrt(c.gp * h1 * h2 * F * fabs(aux));
    V4<double> D{u - cg, uu - ci, uu + ci, u + cg};
    sort_eig(D, c.eig_sort);
    return D;
}

// defTerminoFriccion (Arista_kernel.cu:11-58)
__device__ __forceinline__ double friction_mu(double h1, double u1, double h2, double u2, const Consts& c) {
    if (c.law == 0) return c.mu;
    const double a = 10.0 * h1 / c.eps_h;
    const double rr = 1.0 - c.r * (1.0 - exp_neg(a * a));
    const double gp = c.g * rr;
    const double fr1 = u1 * u1 * vfac(h1, c.eps_h) / gp;
    const double fr2 = u2 * u2 * vfac(h2, c.eps_h) / gp;
    const double fr = sqrt(fr1 + fr2 + (1.0 - rr) * fr1 * fr2);
    const double beta = 0.136, L2 = 8.0e-4, chi = 1.0e-3;
    const double mustop = c.tan1 + (c.tan2 - c.tan1) / (1.0 + h2 / L2);
    const double mustart = c.tan3 + (c.tan4 - c.tan3) / (1.0 + h2 / L2);
    double muf;
    if (fr > beta) muf = c.tan1 + (c.tan2 - c.tan1) / (1.0 + beta * h2 / (fr * L2));
    else if (fabs(fr) < kEps) muf = c.tan3 + (c.tan4 - c.tan3) / (1.0 + h2 / L2);
    else muf = mustart + lshm::pow_pos(fr / beta, chi) * (mustop - mustart);
    return muf * c.L / c.H;
}

__device__ __forceinline__ double fsc_of(double h1, const Consts& c) {
    const double a = 10.0 * h1 / c.eps_h;
    return 1.0 - c.r * (1.0 - exp_neg(a * a));
}

// Inputs of one edge (see the CPU oracle's EdgeIn for the meaning).
struct EdgeIn {
    double W0[6], W1[6];
    double H0, H1;
    double nx, ny, len, area0, area1;
    double hc0[2], hc1[2];
    double acc0h[2], acc1h[2];
    bool interior;
};

// procesarArista: returns false for a dry edge; otherwise d0/d1 (to subtract
// from the two cells' accumulators) and the wave term.
__device__ __forceinline__ bool edge_flux(const EdgeIn& e, double dt, const Consts& c, double d0[6],
                                          double d1[6], double& wave) {
    const double nx = e.nx, ny = e.ny, eps = c.eps_h;
    V4<double> A{e.W0[0], e.W0[1] * nx + e.W0[2] * ny, e.W0[3], e.W0[4] * nx + e.W0[5] * ny};
    V4<double> B{e.W1[0], e.W1[1] * nx + e.W1[2] * ny, e.W1[3], e.W1[4] * nx + e.W1[5] * ny};
    const double H0 = e.H0, H1 = e.H1;

    // the edge is dry when both averaged depths are below EPSILON (:397); the
    // depths do not depend on the discharges, so test before any heavy work
    const double h1ij = 0.5 * (A.x + B.x);
    const double h2ij = 0.5 * (A.z + B.z);
    if (!((h1ij >= kEps) || (h2ij >= kEps))) return false;

    if ((A.z < eps) && (H1 - B.z > H0)) B.w = 0.0;
    if ((B.z < eps) && (H0 - A.z > H1)) A.w = 0.0;
    if ((A.x < eps) && (H1 - B.x - B.z > H0 - A.z)) B.y = 0.0;
    if ((B.x < eps) && (H0 - A.x - A.z > H1 - B.z)) A.y = 0.0;
    if ((A.z + A.x < eps) && (H1 - B.x - B.z > H0)) { B.y = 0.0; B.w = 0.0; }
    if ((B.z + B.x < eps) && (H0 - A.x - A.z > H1)) { A.y = 0.0; A.w = 0.0; }

    const double fA1 = vfac(A.x, eps), fB1 = vfac(B.x, eps);
    const double fA2 = vfac(A.z, eps), fB2 = vfac(B.z, eps);
    double sa = sqrt(A.x), sb = sqrt(B.x);
    const double u1ij = (sa * (fA1 * A.y) + sb * (fB1 * B.y)) / (sa + sb + kEps);
    sa = sqrt(A.z); sb = sqrt(B.z);
    const double u2ij = (sa * (fA2 * A.w) + sb * (fB2 * B.w)) / (sa + sb + kEps);

    const double Hm = tmin(H0, H1);
    const double deta1 = max0(B.x + B.z - H1 + Hm) - max0(A.x + A.z - H0 + Hm);
    const double deta2 = max0(B.z - H1 + Hm) - max0(A.z - H0 + Hm);
    const V4<double> tp{0.0, c.g * h1ij * deta1, 0.0, c.g * h2ij * ((1.0 - c.r) * deta2 + c.r * deta1)};

    const double mu = friction_mu(h1ij, u1ij, h2ij, u2ij, c);
    const double sc = fsc_of(h1ij, c) * mu * c.g * h2ij;
    const bool coul = fabs(h2ij * u2ij) < c.peso * sc * dt;
    V4<double> tp2 = tp;
    if (coul) tp2.w = c.g * h2ij * c.r * deta1;

    const V4<double> D = eig_core(h1ij, h2ij, u1ij, u2ij, h1ij * u1ij + h2ij * u2ij, c);
    const V4<double> E0 = eig_core(A.x, A.z, fA1 * A.y, fA2 * A.w, A.y + A.w, c);
    const V4<double> E1 = eig_core(B.x, B.z, fB1 * B.y, fB2 * B.w, B.y + B.w, c);
    const double aut1 = tmin(D.x, tmin(E0.x, E1.x));
    const double aut3 = tmax(D.w, tmax(E0.w, E1.w));
    double lmax = tmax(fabs(aut3), fabs(aut1));
    const double umax = tmax(fabs(u1ij), fabs(u2ij));
    if (umax > lmax) lmax = umax;
    double aut2 = tmax(fabs(D.y), fabs(D.z));
    if (sgn(aut1 + aut3) < 0) aut2 = -aut2;

    double a0, a1, a2;
    if ((fabs(aut1 - aut3) >= kEps) && (fabs(aut1 - aut2) >= kEps) && (fabs(aut2 - aut3) >= kEps)) {
        if ((h1ij >= eps) && (h2ij >= eps)) {
            const double a = fabs(aut1) / ((aut1 - aut3) * (aut1 - aut2));
            const double b = fabs(aut2) / ((aut2 - aut1) * (aut2 - aut3));
            const double cc = fabs(aut3) / ((aut3 - aut1) * (aut3 - aut2));
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

    const V4<double> FA{A.y, (A.x < kEps) ? 0.0 : (fA1 * A.y) * A.y, A.w, (A.z < kEps) ? 0.0 : (fA2 * A.w) * A.w};
    const V4<double> FB{B.y, (B.x < kEps) ? 0.0 : (fB1 * B.y) * B.y, B.w, (B.z < kEps) ? 0.0 : (fB2 * B.w) * B.w};
    const V4<double> dF{FB.x - FA.x, FB.y - FA.y, FB.z - FA.z, FB.w - FA.w};
    tp2 = V4<double>{tp2.x + dF.x, tp2.y + dF.y, tp2.z + dF.z, tp2.w + dF.w};
    const V4<double> half{0.5 * (dF.x + tp.x), 0.5 * (dF.y + tp.y), 0.5 * (dF.z + tp.z), 0.5 * (dF.w + tp.w)};

    const double ga = c.g * h1ij, gb = c.g * h2ij;
    const V4<double> At{tp2.y, (ga - u1ij * u1ij) * tp2.x + 2.0 * u1ij * tp2.y + ga * tp2.z, tp2.w,
                        c.r * gb * tp2.x + (gb - u2ij * u2ij) * tp2.z + 2.0 * u2ij * tp2.w};

    V4<double> I{deta1, B.y - A.y, 0.0, B.w - A.w};
    if (!coul) {
        if ((A.x > eps) && (B.x > eps)) I.x = I.x - deta2;
        I.z = deta2;
    }

    const V4<double> Q{0.5 * (a0 * I.x + a1 * tp2.x + a2 * At.x), 0.5 * (a0 * I.y + a1 * tp2.y + a2 * At.y),
                       0.5 * (a0 * I.z + a1 * tp2.z + a2 * At.z), 0.5 * (a0 * I.w + a1 * tp2.w + a2 * At.w)};
    const V4<double> Fm{half.x + (FA.x - Q.x), half.y + (FA.y - Q.y), half.z + (FA.z - Q.z), half.w + (FA.w - Q.w)};
    const V4<double> Fp{half.x + (Q.x - FB.x), half.y + (Q.y - FB.y), half.z + (Q.z - FB.z), half.w + (Q.w - FB.w)};

    const double ut0 = fA1 * (e.W0[2] * nx - e.W0[1] * ny), ut1 = fB1 * (e.W1[2] * nx - e.W1[1] * ny);
    const double u1t = (fabs(Fm.x) < kEps) ? 0.0 : ((Fm.x > 0.0) ? ut0 : ut1);
    const double vt0 = fA2 * (e.W0[5] * nx - e.W0[4] * ny), vt1 = fB2 * (e.W1[5] * nx - e.W1[4] * ny);
    const double u2t = (fabs(Fm.z) < kEps) ? 0.0 : ((Fm.z > 0.0) ? vt0 : vt1);

    const double s1 = Fm.x * u1t, s2 = Fm.z * u2t;
    double P[6] = {Fp.x, Fp.y * nx + s1 * ny, Fp.y * ny - s1 * nx, Fp.z, Fp.w * nx + s2 * ny, Fp.w * ny - s2 * nx};
    double M[6] = {Fm.x, Fm.y * nx - s1 * ny, Fm.y * ny + s1 * nx, Fm.z, Fm.w * nx - s2 * ny, Fm.w * ny + s2 * nx};
#pragma unroll
    for (int k = 0; k < 6; ++k) { P[k] = e.len * P[k]; M[k] = e.len * M[k]; }

    const double b0 = dt / e.area0;
    const double hp00 = e.hc0[0] + b0 * e.acc0h[0], hp01 = e.hc0[1] + b0 * e.acc0h[1];
    double hp10 = 0.0, hp11 = 0.0;
    if (e.interior) {
        const double b1 = dt / e.area1;
        hp10 = e.hc1[0] + b1 * e.acc1h[0]; hp11 = e.hc1[1] + b1 * e.acc1h[1];
    }
    const double factor = 1.0 * c.beta;
#pragma unroll
    for (int layer = 0; layer < 2; ++layer) {
        const int k = 3 * layer;
        double dta = kBig, dtb = kBig;
        if (M[k] > 0.0) dta = (layer ? hp01 : hp00) * e.area0 / (factor * M[k] + kEps);
        if (e.interior && P[k] > 0.0) dtb = (layer ? hp11 : hp10) * e.area1 / (factor * P[k] + kEps);
        const double dtl = tmin(dta, dtb);
        if (!(dt <= dtl)) {
            const double alpha = dtl / (dt + kEps);
#pragma unroll
            for (int q = 0; q < 3; ++q) { M[k + q] = alpha * M[k + q]; P[k + q] = alpha * P[k + q]; }
        }
    }

    if (lmax < eps) lmax = lmax + eps;
    wave = e.len * lmax / c.peso;
#pragma unroll
    for (int k = 0; k < 6; ++k) { d0[k] = c.peso * M[k]; d1[k] = c.peso * P[k]; }
    return true;
}

// procesarAristaDeltaTInicial: wave-speed bound for the initial dt.
__device__ __forceinline__ double edge_initial_wave(const double W0[6], const double W1[6], double nx, double ny,
                                                    double len, const Consts& c) {
    const double eps = c.eps_h;
    const V4<double> A{W0[0], W0[1] * nx + W0[2] * ny, W0[3], W0[4] * nx + W0[5] * ny};
    const V4<double> B{W1[0], W1[1] * nx + W1[2] * ny, W1[3], W1[4] * nx + W1[5] * ny};
    const double h1ij = 0.5 * (A.x + B.x);
    double sa = sqrt(A.x), sb = sqrt(B.x);
    const double u1ij = (sa * (vfac(A.x, eps) * A.y) + sb * (vfac(B.x, eps) * B.y)) / (sa + sb + kEps);
    const double h2ij = 0.5 * (A.z + B.z);
    sa = sqrt(A.z); sb = sqrt(B.z);
    const double u2ij = (sa * (vfac(A.z, eps) * A.w) + sb * (vfac(B.z, eps) * B.w)) / (sa + sb + kEps);
    const V4<double> D = eig_core(h1ij, h2ij, u1ij, u2ij, h1ij * u1ij + h2ij * u2ij, c);
    double lmax = tmax(D.x, D.w);
    const double b = tmax(fabs(u1ij), fabs(u2ij));
    if (b > lmax) lmax = b;
    if (lmax < eps) lmax = lmax + eps;
    return len * lmax;
}

// filtroEstado (Volumen_kernel.cu:92-180)
__device__ __forceinline__ void filtro(double w[6], double dt, const Consts& c) {
    if (w[0] < 0.0) w[0] = 0.0;
    if (w[3] < 0.0) w[3] = 0.0;
#pragma unroll
    for (int layer = 0; layer < 2; ++layer) {
        const int k = 3 * layer;
        const double x = w[k] / c.eps_h;
        const double x2 = x * x;
        const double aux0 = 1.0 / (x2 * x2 + kEps);
        const double aux = exp_neg(dt * aux0);
        w[k + 1] = w[k + 1] * aux;
        w[k + 2] = w[k + 2] * aux;
    }
#pragma unroll
    for (int layer = 0; layer < 2; ++layer) {
        const double vmax = layer ? c.vmax2 : c.vmax1;
        if (vmax > 0.0) {
            const int k = 3 * layer;
            const double h = w[k];
            const double f = vfac(h, c.eps_h);
            double ux = f * w[k + 1], uy = f * w[k + 2];
            const double u = sqrt(ux * ux + uy * uy);
            if (u > vmax) {
                ux = ux * (vmax / u); uy = uy * (vmax / u);
                w[k + 1] = ux * h; w[k + 2] = uy * h;
            }
        }
    }
}

// disImplicita (Volumen_kernel.cu:31-90)
__device__ __forceinline__ void dis_implicita(const double wo[6], double w[6], double dt, const Consts& c) {
    if (w[0] < 0.0) w[0] = 0.0;
    if (w[3] < 0.0) w[3] = 0.0;
    const double eps = c.eps_h;
    const double h1 = w[0], h2 = w[3];
    const double f1 = vfac(h1, eps), f2 = vfac(h2, eps);
    double u1x = f1 * w[1], u1y = f1 * w[2], u2x = f2 * w[4], u2y = f2 * w[5];
    const double fo1 = vfac(wo[0], eps), fo2 = vfac(wo[3], eps);
    const double uo1x = fo1 * wo[1], uo1y = fo1 * wo[2], uo2x = fo2 * wo[4], uo2y = fo2 * wo[5];
    const double dx = uo1x - uo2x, dy = uo1y - uo2y;
    const double du = sqrt(dx * dx + dy * dy);
    const double u1 = sqrt(uo1x * uo1x + uo1y * uo1y);
    const double u2 = sqrt(uo2x * uo2x + uo2y * uo2y);
    const double hmod = h2 + c.r * h1;
    const double mfl = eps * (1.0 + c.r);
    const double m = (hmod > mfl) ? hmod : mfl;
    const double hm2 = hmod * hmod, m2 = m * m;
    const double hmodm = sqrt(hm2 * hm2 + m2 * m2);
    if ((h1 > 0.0) && (h2 > 0.0)) {
        const double c1 = dt * kSqrt2 * h2 * hmod / hmodm * c.mfc * du;
        const double c2 = dt * c.r * kSqrt2 * h1 * hmod / hmodm * c.mfc * du;
        const double c3 = dt * c.g * c.mfs * c.mfs * u2 / (pow43(h2) + kEps);
        const double det = 1.0 / ((1.0 + c1) * (1.0 + c2 + c3) - c1 * c2);
        w[1] = h1 * (u1x * (1.0 + c2 + c3) + c1 * u2x) * det;
        w[4] = h2 * (u2x * (1.0 + c1) + c2 * u1x) * det;
        w[2] = h1 * (u1y * (1.0 + c2 + c3) + c1 * u2y) * det;
        w[5] = h2 * (u2y * (1.0 + c1) + c2 * u1y) * det;
    }
    if ((h1 > 0.0) && (h2 < eps)) {
        u1x = f1 * w[1]; u1y = f1 * w[2];
        const double c1 = dt * c.g * c.mf0 * c.mf0 * u1 / (pow43(h1) + kEps);
        w[1] = h1 * u1x / (1.0 + c1);
        w[2] = h1 * u1y / (1.0 + c1);
    }
    if ((h2 > 0.0) && (h1 < eps)) {
        u2x = f2 * w[4]; u2y = f2 * w[5];
        const double c1 = dt * c.g * c.mfs * c.mfs * u2 / (pow43(h2) + kEps);
        w[4] = h2 * u2x / (1.0 + c1);
        w[5] = h2 * u2y / (1.0 + c1);
    }
}

// coulomb (Volumen_kernel.cu:7-26)
__device__ __forceinline__ void coulomb(double w[6], double dt, const Consts& c) {
    double mu = c.mu;
    if (c.law != 0) {
        const double u1 = sqrt(w[1] * w[1] + w[2] * w[2]) * vfac(w[0], c.eps_h);
        const double u2 = sqrt(w[4] * w[4] + w[5] * w[5]) * vfac(w[3], c.eps_h);
        mu = friction_mu(w[0], u1, w[3], u2, c);
    }
    const double sc = fsc_of(w[0], c) * mu * c.g * w[3] * dt * 1.0;
    const double normq = sqrt(w[4] * w[4] + w[5] * w[5]);
    double aux = 0.0;
    if ((normq + sc >= kEps) && (w[3] > 0.0)) aux = (normq >= sc) ? normq / (normq + sc) : 0.0;
    w[4] = w[4] * aux;
    w[5] = w[5] * aux;
}

// One cell of obtenerEstadoYDeltaTVolumenesGPU (Volumen_kernel.cu:231-284),
// plus the spherical metric source (tanR = tan(lat)/R, 0 for Cartesian).
__device__ __forceinline__ void volume_update(const double wo[6], const double acc[7], double w[6], double& dti,
                                              double area, double tanR, double dt, const Consts& c) {
    dti = (acc[6] < kEps) ? kBig : (2.0 * c.cfl * area) / acc[6];
    const double b = dt / area;
#pragma unroll
    for (int k = 0; k < 6; ++k) w[k] = wo[k] + b * acc[k];
    if (tanR != 0.0) {
#pragma unroll
        for (int layer = 0; layer < 2; ++layer) {
            const int k = 3 * layer;
            const double ux = vfac(wo[k], c.eps_h) * wo[k + 1];
            w[k + 1] = w[k + 1] + dt * (ux * wo[k + 2] * tanR);
            w[k + 2] = w[k + 2] - dt * (ux * wo[k + 1] * tanR);
        }
    }
    filtro(w, dt, c);
    dis_implicita(wo, w, dt, c);
    coulomb(w, dt, c);
}

}  // namespace lsh
