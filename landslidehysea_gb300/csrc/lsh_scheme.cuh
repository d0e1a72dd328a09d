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

#if !defined(__CUDA_ARCH__)
using std::fabs;
using std::sqrt;
#endif

constexpr double kEps = 1.1920928955078125e-07;  // FLT_EPSILON (Constantes.hxx:13)
constexpr double kSqrt2 = 1.41421356237309504880;
constexpr double kBig = 1e30;

// Scalars every kernel needs; passed by value (kernel parameter space).
struct Consts {
    double g, r, gp, eps_h, peso, beta, cfl, mu, mfc, mf0, mfs, vmax1, vmax2, L, H;
    double tan1, tan2, tan3, tan4;
    // host-derived, with the same formulas as the CPU oracle's make_consts
    double omr, inv_gp, inv_eps, inv_peso, eps_1r, g_mf02, g_mfs2, sqrt_g;
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
    const double* inv_area;  // [ny]
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
    unsigned long long rmax_bits;    // running max of per-cell acc_w / area (bits of a double >= 0)
    long long steps;                 // steps taken
    int done;                        // 1 once t >= t_end (kernels then return at once)
    int err;                         // sticky error bits (LSH status values as bits)
};

struct V4 { double x, y, z, w; };

// Compares run on the integer pipe (lsh_fpmath.h: exact for non-NaN
// operands): lt_pos / gt_pos against the positive thresholds EPSILON, eps_h,
// vmax, lt / okey for operands of either sign.
using lshm::abs_bits;
using lshm::abs_lt;
using lshm::gt0;
using lshm::gt_pos;
using lshm::lt;
using lshm::lt0;
using lshm::lt_pos;
using lshm::okey;

LSH_HD double tmin(double a, double b) { return lt(b, a) ? b : a; }
LSH_HD double tmax(double a, double b) { return lt(a, b) ? b : a; }
LSH_HD double max0(double a) { return gt0(a) ? a : 0.0; }
LSH_HD double fmad(double a, double b, double c) { return lshm::fmad(a, b, c); }
LSH_HD double exp_neg(double x) { return lshm::exp_neg(x); }

// sqrt(2) h / sqrt(h^4 + max(h, eps_h)^4); exactly 1/h for h > eps_h
LSH_HD double vfac(double h, double eps_h) {
    if (gt_pos(h, eps_h)) return 1.0 / h;
    const double h2 = h * h, m2 = eps_h * eps_h;
    return (kSqrt2 * h) / sqrt(fmad(h2, h2, m2 * m2));
}

LSH_HD double pow43(double h) { return h * lshm::cbrt_pos(h); }

LSH_HD int sgn(double x) { return abs_lt(x, kEps) ? 0 : (gt0(x) ? 1 : -1); }

// x == +0 or -0, by bit pattern (integer pipe)
LSH_HD bool is_zero(double x) {
    uint32_t lo, hi;
    lshm::halves(x, lo, hi);
    return ((hi << 1) | lo) == 0u;
}

// NaN or Inf, by the exponent bits (integer pipe)
LSH_HD bool is_bad(double x) {
    uint32_t lo, hi;
    lshm::halves(x, lo, hi);
    return (hi & 0x7ff00000u) == 0x7ff00000u;
}

// Compare-and-swap sequence of Arista_kernel.cu:193-234 (with its (2,1)
// compare) or, with `full`, the same sequence made a true sort.
// The compares run on ordered keys (okey), which travel with the values.
LSH_HD void cswap(double& a, double& b, int64_t& ka, int64_t& kb) {
    if (ka > kb) {
        const double t = a; a = b; b = t;
        const int64_t k = ka; ka = kb; kb = k;
    }
}
LSH_HD void sort_eig(V4& D, int full) {
    int64_t kx = okey(D.x), ky = okey(D.y), kz = okey(D.z), kw = okey(D.w);
    cswap(D.x, D.y, kx, ky);
    cswap(D.x, D.z, kx, kz);
    cswap(D.x, D.w, kx, kw);
    cswap(D.y, D.z, ky, kz);
    cswap(D.y, D.w, ky, kw);
    if (full) cswap(D.y, D.z, ky, kz);
    else cswap(D.z, D.y, kz, ky);
    cswap(D.z, D.w, kz, kw);
}

// aproximarAutovalores1D (Arista_kernel.cu:152-237).  L2 == false: the
// granular layer is absent (h2 = 0, u2 = 0), so the internal pair is exactly
// zero and its square root is skipped.
template <bool L2>
LSH_HD V4 eig(double h1, double h2, double u1, double u2, double q, const Consts& c,
                                  double Fknown = -1.0, double sqrt_h = -1.0, bool mean_u = false) {
    const double h = L2 ? h1 + h2 : h1;
    // mean_u (the edge average, q = h1 u1 + h2 u2): with no granular layer and
    // h > eps_h, u = q vfac(h) = (h1 u1) / h1 is u1 itself -- an exact
    // restatement the CPU oracle makes too; the single-layer edge then skips
    // the division
    const bool direct = mean_u && is_zero(h2) && gt_pos(h, c.eps_h);
    double F = 0.0;
    // single layer: vfac(h1 + 0) is vfac(h1), which the caller may already hold
    if (L2 || !direct) F = (!L2 && !lt0(Fknown)) ? Fknown : vfac(h, c.eps_h);
    const double u = direct ? u1 : q * F;
    // sqrt_h >= 0: sqrt(h1) is known and h2 == 0, so sqrt(g h) = sqrt(g) sqrt(h1)
    const double cg = !lt0(sqrt_h) ? c.sqrt_g * sqrt_h : sqrt(c.g * h);
    double uu = 0.0, ci = 0.0;
    if (L2) {
        uu = fmad(u1, h2, u2 * h1) * F;
        const double d = u1 - u2;
        const double aux = fmad(-((d * d) * F), c.inv_gp, 1.0);
        ci = sqrt((((c.gp * h1) * h2) * F) * abs_bits(aux));
    }
    V4 D{u - cg, uu - ci, uu + ci, u + cg};
    sort_eig(D, c.eig_sort);
    return D;
}

// defTerminoFriccion (Arista_kernel.cu:11-58)
LSH_HD double friction_mu(double h1, double u1, double h2, double u2, const Consts& c) {
    if (c.law == 0) return c.mu;
    const double a = (10.0 * h1) * c.inv_eps;
    const double rr = 1.0 - c.r * (1.0 - exp_neg(a * a));
    const double gp = c.g * rr;
    const double fr1 = ((u1 * u1) * vfac(h1, c.eps_h)) / gp;
    const double fr2 = ((u2 * u2) * vfac(h2, c.eps_h)) / gp;
    const double fr = sqrt(fmad((1.0 - rr) * fr1, fr2, fr1 + fr2));
    const double beta = 0.136, L2c = 8.0e-4, chi = 1.0e-3;
    const double mustop = c.tan1 + (c.tan2 - c.tan1) / (1.0 + h2 / L2c);
    const double mustart = c.tan3 + (c.tan4 - c.tan3) / (1.0 + h2 / L2c);
    double muf;
    if (gt_pos(fr, beta)) muf = c.tan1 + (c.tan2 - c.tan1) / (1.0 + beta * h2 / (fr * L2c));
    else if (abs_lt(fr, kEps)) muf = c.tan3 + (c.tan4 - c.tan3) / (1.0 + h2 / L2c);
    else muf = fmad(lshm::pow_pos(fr / beta, chi), mustop - mustart, mustart);
    return (muf * c.L) / c.H;
}

LSH_HD double fsc_of(double h1, const Consts& c) {
    const double a = (10.0 * h1) * c.inv_eps;
    return 1.0 - c.r * (1.0 - exp_neg(a * a));
}

// One face state in the edge's normal frame: depth, normal and tangential
// discharge of each layer, bottom depth.
struct Face { double h1, qn1, qt1, h2, qn2, qt2, H; };

// Inputs of one edge (the CPU oracle's EdgeIn): the two facing states A, B,
// cell-average depths and partial accumulators for the positivity limiter.
struct EdgeIn {
    Face A, B;
    double len, area0, area1, inv_area0, inv_area1;
    double hc0[2], hc1[2];
    double acc0h[2], acc1h[2];
    bool interior;
};

// Normal-frame output: per layer (mass, normal momentum, tangential
// momentum) to subtract from cell 0 (m) and cell 1 (p), and the wave term.
struct EdgeOut { double m[6], p[6]; double wave; };

// The positivity limiter's inputs, read from an EdgeIn that holds them.
struct EdgeInPos {
    const EdgeIn& e;
    LSH_HD double area(int side) const { return side ? e.area1 : e.area0; }
    LSH_HD double inv_area(int side) const { return side ? e.inv_area1 : e.inv_area0; }
    LSH_HD double hc(int side, int layer) const { return side ? e.hc1[layer] : e.hc0[layer]; }
    LSH_HD double acch(int side, int layer) const { return side ? e.acc1h[layer] : e.acc0h[layer]; }
};

// procesarArista (Arista_kernel.cu:324-645), the depths already known to be
// wet (the caller skips dry edges, :397).  L2 == false: both faces have no
// granular layer (h2 = qn2 = 0); every layer-1 value is then the same as in
// the general path and every layer-2 output is zero, so that work is skipped.
// `pos` supplies the positivity limiter's inputs (cell areas, cell depths and
// the partial accumulators of the cells' depths; EdgeInPos reads them from
// `e`): a caller may load them only where the limiter needs them, so they do
// not stay live through the flux computation.
template <bool L2, class Pos>
LSH_HD void edge_flux(const EdgeIn& e, double dt, const Consts& c, EdgeOut& o, const Pos& pos) {
    const double eps = c.eps_h;
    double Aq1 = e.A.qn1, Aq2 = L2 ? e.A.qn2 : 0.0, Bq1 = e.B.qn1, Bq2 = L2 ? e.B.qn2 : 0.0;
    const double Ah1 = e.A.h1, Bh1 = e.B.h1;
    const double Ah2 = L2 ? e.A.h2 : 0.0, Bh2 = L2 ? e.B.h2 : 0.0;
    const double H0 = e.A.H, H1 = e.B.H;
    const double h1ij = 0.5 * (Ah1 + Bh1);
    const double h2ij = L2 ? 0.5 * (Ah2 + Bh2) : 0.0;

    // tratamientoSecoMojado (Arista_kernel.cu:301-321)
    if (L2) {
        if (lt_pos(Ah2, eps) && lt(H0, H1 - Bh2)) Bq2 = 0.0;
        if (lt_pos(Bh2, eps) && lt(H1, H0 - Ah2)) Aq2 = 0.0;
        if (lt_pos(Ah1, eps) && lt(H0 - Ah2, H1 - Bh1 - Bh2)) Bq1 = 0.0;
        if (lt_pos(Bh1, eps) && lt(H1 - Bh2, H0 - Ah1 - Ah2)) Aq1 = 0.0;
        if (lt_pos(Ah2 + Ah1, eps) && lt(H0, H1 - Bh1 - Bh2)) { Bq1 = 0.0; Bq2 = 0.0; }
        if (lt_pos(Bh2 + Bh1, eps) && lt(H1, H0 - Ah1 - Ah2)) { Aq1 = 0.0; Aq2 = 0.0; }
    } else {
        if (lt_pos(Ah1, eps) && lt(H0, H1 - Bh1)) Bq1 = 0.0;
        if (lt_pos(Bh1, eps) && lt(H1, H0 - Ah1)) Aq1 = 0.0;
    }

    const double fA1 = vfac(Ah1, eps), fB1 = vfac(Bh1, eps);
    const double fA2 = L2 ? vfac(Ah2, eps) : 0.0, fB2 = L2 ? vfac(Bh2, eps) : 0.0;
    const double sa1 = sqrt(Ah1), sb1 = sqrt(Bh1);
    const double u1ij = fmad(sa1, fA1 * Aq1, sb1 * (fB1 * Bq1)) / (sa1 + sb1 + kEps);
    double u2ij = 0.0;
    if (L2) {
        const double sa2 = sqrt(Ah2), sb2 = sqrt(Bh2);
        u2ij = fmad(sa2, fA2 * Aq2, sb2 * (fB2 * Bq2)) / (sa2 + sb2 + kEps);
    }
    // a face's celerity sqrt(g h) is sqrt(g) sqrt(h1) when its granular layer is empty
    const bool oneA = !L2 || is_zero(Ah2), oneB = !L2 || is_zero(Bh2);

    const double Hm = tmin(H0, H1);
    const double deta1 = L2 ? max0(Bh1 + Bh2 - H1 + Hm) - max0(Ah1 + Ah2 - H0 + Hm)
                            : max0(Bh1 - H1 + Hm) - max0(Ah1 - H0 + Hm);
    const double deta2 = L2 ? max0(Bh2 - H1 + Hm) - max0(Ah2 - H0 + Hm) : 0.0;
    const double gh1 = c.g * h1ij, gh2 = c.g * h2ij;
    const V4 tp{0.0, gh1 * deta1, 0.0, L2 ? gh2 * fmad(c.omr, deta2, c.r * deta1) : 0.0};

    bool coul = false;
    V4 tp2 = tp;
    if (L2) {
        const double mu = friction_mu(h1ij, u1ij, h2ij, u2ij, c);
        const double sc = ((fsc_of(h1ij, c) * mu) * c.g) * h2ij;
        coul = lt(abs_bits(h2ij * u2ij), (c.peso * sc) * dt);
        if (coul) tp2.w = (gh2 * c.r) * deta1;
    }

    const V4 D = eig<L2>(h1ij, h2ij, u1ij, u2ij, L2 ? fmad(h1ij, u1ij, h2ij * u2ij) : h1ij * u1ij, c, -1.0, -1.0, true);
    const V4 E0 = eig<L2>(Ah1, Ah2, fA1 * Aq1, fA2 * Aq2, L2 ? Aq1 + Aq2 : Aq1, c, fA1, oneA ? sa1 : -1.0);
    const V4 E1 = eig<L2>(Bh1, Bh2, fB1 * Bq1, fB2 * Bq2, L2 ? Bq1 + Bq2 : Bq1, c, fB1, oneB ? sb1 : -1.0);
    const double aut1 = tmin(D.x, tmin(E0.x, E1.x));
    const double aut3 = tmax(D.w, tmax(E0.w, E1.w));
    double lmax = tmax(abs_bits(aut3), abs_bits(aut1));
    const double umax = L2 ? tmax(abs_bits(u1ij), abs_bits(u2ij)) : abs_bits(u1ij);
    if (lt(lmax, umax)) lmax = umax;
    double aut2 = tmax(abs_bits(D.y), abs_bits(D.z));
    aut2 = lshm::neg_if(aut2, sgn(aut1 + aut3) < 0);

    double a0, a1, a2 = 0.0;
    if (!abs_lt(aut1 - aut3, kEps) && !abs_lt(aut1 - aut2, kEps) && !abs_lt(aut2 - aut3, kEps)) {
        if (L2 && !lt_pos(h1ij, eps) && !lt_pos(h2ij, eps)) {
            const double d12 = aut1 - aut2, d13 = aut1 - aut3, d23 = aut2 - aut3;
            const double inv = 1.0 / ((d12 * d13) * d23);
            const double a = (abs_bits(aut1) * d23) * inv;
            const double b = -((abs_bits(aut2) * d13) * inv);
            const double cc = (abs_bits(aut3) * d12) * inv;
            a0 = fmad(a * aut2, aut3, fmad(b * aut1, aut3, (cc * aut1) * aut2));
            a1 = -fmad(a, aut2 + aut3, fmad(b, aut1 + aut3, cc * (aut1 + aut2)));
            a2 = a + b + cc;
        } else {
            const double inv = 1.0 / (aut3 - aut1);
            a0 = fmad(aut3, abs_bits(aut1), -(aut1 * abs_bits(aut3))) * inv;
            a1 = (abs_bits(aut3) - abs_bits(aut1)) * inv;
        }
    } else {
        a0 = lmax; a1 = 0.0;
    }

    const double FAy = lt_pos(Ah1, kEps) ? 0.0 : (fA1 * Aq1) * Aq1, FBy = lt_pos(Bh1, kEps) ? 0.0 : (fB1 * Bq1) * Bq1;
    const double dFx = Bq1 - Aq1, dFy = FBy - FAy;
    double dFz = 0.0, dFw = 0.0, FAw = 0.0, FBw = 0.0;
    if (L2) {
        FAw = lt_pos(Ah2, kEps) ? 0.0 : (fA2 * Aq2) * Aq2;
        FBw = lt_pos(Bh2, kEps) ? 0.0 : (fB2 * Bq2) * Bq2;
        dFz = Bq2 - Aq2;
        dFw = FBw - FAw;
    }
    tp2 = V4{tp2.x + dFx, tp2.y + dFy, tp2.z + dFz, tp2.w + dFw};
    const double half_x = 0.5 * (dFx + tp.x), half_y = 0.5 * (dFy + tp.y);

    const double Atx = tp2.y;
    const double Aty = fmad(gh1, tp2.z, fmad(u1ij + u1ij, tp2.y, fmad(-u1ij, u1ij, gh1) * tp2.x));

    V4 I{deta1, Bq1 - Aq1, 0.0, Bq2 - Aq2};
    if (!coul) {
        if (gt_pos(Ah1, eps) && gt_pos(Bh1, eps)) I.x = I.x - deta2;
        I.z = deta2;
    }

    double Qx, Qy;
    if (L2) {
        Qx = 0.5 * fmad(a0, I.x, fmad(a1, tp2.x, a2 * Atx));
        Qy = 0.5 * fmad(a0, I.y, fmad(a1, tp2.y, a2 * Aty));
    } else {
        Qx = 0.5 * fmad(a0, I.x, a1 * tp2.x);
        Qy = 0.5 * fmad(a0, I.y, a1 * tp2.y);
    }
    const double Fmx = half_x + (Aq1 - Qx), Fmy = half_y + (FAy - Qy);
    const double Fpx = half_x + (Qx - Bq1), Fpy = half_y + (Qy - FBy);

    const double u1t = abs_lt(Fmx, kEps) ? 0.0 : (gt0(Fmx) ? fA1 * e.A.qt1 : fB1 * e.B.qt1);
    const double s1 = Fmx * u1t;
    double M[6] = {Fmx, Fmy, s1, 0.0, 0.0, 0.0};
    double P[6] = {Fpx, Fpy, -s1, 0.0, 0.0, 0.0};
    if (L2) {
        const double Atz = tp2.w;
        const double Atw = fmad(c.r * gh2, tp2.x, fmad(fmad(-u2ij, u2ij, gh2), tp2.z, (u2ij + u2ij) * tp2.w));
        const double Qz = 0.5 * fmad(a0, I.z, fmad(a1, tp2.z, a2 * Atz));
        const double Qw = 0.5 * fmad(a0, I.w, fmad(a1, tp2.w, a2 * Atw));
        const double half_z = 0.5 * (dFz + tp.z), half_w = 0.5 * (dFw + tp.w);
        const double Fmz = half_z + (Aq2 - Qz), Fmw = half_w + (FAw - Qw);
        const double Fpz = half_z + (Qz - Bq2), Fpw = half_w + (Qw - FBw);
        const double u2t = abs_lt(Fmz, kEps) ? 0.0 : (gt0(Fmz) ? fA2 * e.A.qt2 : fB2 * e.B.qt2);
        const double s2 = Fmz * u2t;
        M[3] = Fmz; M[4] = Fmw; M[5] = s2;
        P[3] = Fpz; P[4] = Fpw; P[5] = -s2;
    }
    constexpr int KL = L2 ? 6 : 3;
#pragma unroll
    for (int k = 0; k < KL; ++k) { P[k] = e.len * P[k]; M[k] = e.len * M[k]; }

    const double b0 = dt * pos.inv_area(0);
    const double hp00 = fmad(b0, pos.acch(0, 0), pos.hc(0, 0));
    const double hp01 = L2 ? fmad(b0, pos.acch(0, 1), pos.hc(0, 1)) : 0.0;
    double hp10 = 0.0, hp11 = 0.0;
    if (e.interior) {
        const double b1 = dt * pos.inv_area(1);
        hp10 = fmad(b1, pos.acch(1, 0), pos.hc(1, 0));
        if (L2) hp11 = fmad(b1, pos.acch(1, 1), pos.hc(1, 1));
    }
    const double factor = 1.0 * c.beta;
#pragma unroll
    for (int layer = 0; layer < (L2 ? 2 : 1); ++layer) {
        const int k = 3 * layer;
        // limited when dt exceeds the time a side takes to empty its layer,
        // hp area / (beta M + eps): tested as dt (beta M + eps) > hp area (the
        // denominator is positive), so the divisions run only on limited edges
        const bool oa = gt0(M[k]), ob = e.interior && gt0(P[k]);
        const double ha = (layer ? hp01 : hp00) * pos.area(0), hb = (layer ? hp11 : hp10) * pos.area(1);
        const double da = oa ? fmad(factor, M[k], kEps) : 1.0, db = ob ? fmad(factor, P[k], kEps) : 1.0;
        const bool lim = (oa && lt(ha, dt * da)) || (ob && lt(hb, dt * db));
        if (lim) {
            const double dta = oa ? ha / da : kBig, dtb = ob ? hb / db : kBig;
            const double dtl = tmin(dta, dtb);
            const double alpha = dtl / (dt + kEps);
#pragma unroll
            for (int q = 0; q < 3; ++q) { M[k + q] = alpha * M[k + q]; P[k + q] = alpha * P[k + q]; }
        }
    }

    if (lt_pos(lmax, eps)) lmax = lmax + eps;
    o.wave = e.len * lmax;
    if (lshm::bits_of(c.peso) != lshm::bits_of(1.0)) {
        o.wave = o.wave * c.inv_peso;
#pragma unroll
        for (int k = 0; k < 6; ++k) { M[k] = c.peso * M[k]; P[k] = c.peso * P[k]; }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) { o.m[k] = M[k]; o.p[k] = P[k]; }
}

template <bool L2>
LSH_HD void edge_flux(const EdgeIn& e, double dt, const Consts& c, EdgeOut& o) {
    edge_flux<L2>(e, dt, c, o, EdgeInPos{e});
}

// procesarAristaDeltaTInicial: wave-speed bound for the initial dt.
LSH_HD double edge_initial_wave(const Face& A, const Face& B, double len, const Consts& c) {
    const double eps = c.eps_h;
    const double h1ij = 0.5 * (A.h1 + B.h1);
    const double fA1 = vfac(A.h1, eps), fB1 = vfac(B.h1, eps);
    double sa = sqrt(A.h1), sb = sqrt(B.h1);
    const double u1ij = fmad(sa, fA1 * A.qn1, sb * (fB1 * B.qn1)) / (sa + sb + kEps);
    const double h2ij = 0.5 * (A.h2 + B.h2);
    const double fA2 = vfac(A.h2, eps), fB2 = vfac(B.h2, eps);
    sa = sqrt(A.h2); sb = sqrt(B.h2);
    const double u2ij = fmad(sa, fA2 * A.qn2, sb * (fB2 * B.qn2)) / (sa + sb + kEps);
    const V4 D = eig<true>(h1ij, h2ij, u1ij, u2ij, fmad(h1ij, u1ij, h2ij * u2ij), c);
    double lmax = tmax(D.x, D.w);
    const double b = tmax(abs_bits(u1ij), abs_bits(u2ij));
    if (lt(lmax, b)) lmax = b;
    if (lt_pos(lmax, eps)) lmax = lmax + eps;
    return len * lmax;
}

// filtroEstado (Volumen_kernel.cu:92-180).  L2 == false: h2 = q2 = 0, so
// the layer-2 damping (0 times a factor) is skipped.
template <bool L2>
LSH_HD void filtro(double w[6], double dt, const Consts& c) {
    if (lt0(w[0])) w[0] = 0.0;
    if (lt0(w[3])) w[3] = 0.0;
#pragma unroll
    for (int layer = 0; layer < (L2 ? 2 : 1); ++layer) {
        const int k = 3 * layer;
        const double x = w[k] * c.inv_eps;
        const double x2 = x * x;
        const double d = fmad(x2, x2, kEps);
        // exp(-dt/d) is exactly 1 once dt/d < 2^-54: skip the division below a
        // bound that holds with ample margin over the roundings
        if (lt_pos(dt, d * 0x1.fp-55)) continue;  // d >= EPSILON: the bound is positive
        const double aux = exp_neg(dt * (1.0 / d));
        w[k + 1] = w[k + 1] * aux;
        w[k + 2] = w[k + 2] * aux;
    }
#pragma unroll
    for (int layer = 0; layer < 2; ++layer) {
        const double vmax = layer ? c.vmax2 : c.vmax1;
        if (gt0(vmax)) {
            const int k = 3 * layer;
            const double h = w[k];
            const double f = vfac(h, c.eps_h);
            double ux = f * w[k + 1], uy = f * w[k + 2];
            const double u = sqrt(fmad(ux, ux, uy * uy));
            if (gt_pos(u, vmax)) {
                const double s = vmax / u;
                ux = ux * s; uy = uy * s;
                w[k + 1] = ux * h; w[k + 2] = uy * h;
            }
        }
    }
}

// disImplicita (Volumen_kernel.cu:31-90).  L2 == false: the new and the old
// granular layer are empty (h2 = q2 = 0): only the water-bottom branch can run.
// fo1 = vfac(wo[0]), the old state's water factor, computed by the caller.
template <bool L2>
LSH_HD void dis_implicita(const double wo[6], double w[6], double dt, const Consts& c,
                                              double fo1) {
    if (lt0(w[0])) w[0] = 0.0;
    if (lt0(w[3])) w[3] = 0.0;
    const double eps = c.eps_h;
    const double h1 = w[0], h2 = L2 ? w[3] : 0.0;
    const double uo1x = fo1 * wo[1], uo1y = fo1 * wo[2];
    const double u1 = sqrt(fmad(uo1x, uo1x, uo1y * uo1y));
    if (!L2) {
        // bottom friction h u / (1 + c1), 1/(1 + X/Y) = Y/(Y + X); above
        // eps_h, h u is q itself
        if (gt0(h1)) {
            const double Y = pow43(h1) + kEps, X = (dt * c.g_mf02) * u1;
            const double inv = Y / (Y + X);
            if (gt_pos(h1, eps)) { w[1] = w[1] * inv; w[2] = w[2] * inv; }
            else {
                const double f1 = vfac(h1, eps);
                w[1] = (h1 * (f1 * w[1])) * inv;
                w[2] = (h1 * (f1 * w[2])) * inv;
            }
        }
        return;
    }
    const double f1 = vfac(h1, eps);
    double u1x = f1 * w[1], u1y = f1 * w[2];
    const double f2 = vfac(h2, eps);
    double u2x = f2 * w[4], u2y = f2 * w[5];
    const double fo2 = vfac(wo[3], eps);
    const double uo2x = fo2 * wo[4], uo2y = fo2 * wo[5];
    const double dx = uo1x - uo2x, dy = uo1y - uo2y;
    const double du = sqrt(fmad(dx, dx, dy * dy));
    const double u2 = sqrt(fmad(uo2x, uo2x, uo2y * uo2y));
    if (gt0(h1) && gt0(h2)) {
        const double hmod = fmad(c.r, h1, h2);
        const double m = gt_pos(hmod, c.eps_1r) ? hmod : c.eps_1r;
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
    if (gt0(h1) && lt_pos(h2, eps)) {
        const double Y = pow43(h1) + kEps, X = (dt * c.g_mf02) * u1;
        const double inv = Y / (Y + X);
        if (gt_pos(h1, eps)) { w[1] = w[1] * inv; w[2] = w[2] * inv; }
        else { w[1] = (h1 * (f1 * w[1])) * inv; w[2] = (h1 * (f1 * w[2])) * inv; }
    }
    if (gt0(h2) && lt_pos(h1, eps)) {
        const double Y = pow43(h2) + kEps, X = (dt * c.g_mfs2) * u2;
        const double inv = Y / (Y + X);
        if (gt_pos(h2, eps)) { w[4] = w[4] * inv; w[5] = w[5] * inv; }
        else { w[4] = (h2 * (f2 * w[4])) * inv; w[5] = (h2 * (f2 * w[5])) * inv; }
    }
}

// coulomb (Volumen_kernel.cu:7-26)
LSH_HD void coulomb(double w[6], double dt, const Consts& c) {
    if (!gt0(w[3])) {
        w[4] = w[4] * 0.0;
        w[5] = w[5] * 0.0;
        return;
    }
    double mu = c.mu;
    if (c.law != 0) {
        const double u1 = sqrt(fmad(w[1], w[1], w[2] * w[2])) * vfac(w[0], c.eps_h);
        const double u2 = sqrt(fmad(w[4], w[4], w[5] * w[5])) * vfac(w[3], c.eps_h);
        mu = friction_mu(w[0], u1, w[3], u2, c);
    }
    const double sc = ((((fsc_of(w[0], c) * mu) * c.g) * w[3]) * dt);
    const double normq = sqrt(fmad(w[4], w[4], w[5] * w[5]));
    double aux = 0.0;
    if (!lt_pos(normq + sc, kEps) && !lt(normq, sc)) aux = normq / (normq + sc);
    w[4] = w[4] * aux;
    w[5] = w[5] * aux;
}

// One cell of obtenerEstadoYDeltaTVolumenesGPU (Volumen_kernel.cu:231-284),
// plus the spherical metric source (tanR = tan(lat)/R, 0 for Cartesian).
// `rate` gets acc_w / area (0 below EPSILON): the step's dt is
// 2 CFL / max(rate), the min over cells of 2 CFL area / acc_w
// (Volumen_kernel.cu:256) with one division per step.
// ONE: the caller has checked that the cell's granular state wo[3..5] is
// zero and its layer-2 accumulators are +0 (an accumulator never holds -0).
// Then every layer-2 value below is the +0 the general path computes
// (b * (+0) + (+-0) = +0; Coulomb's +0 * 0 = +0), so that arithmetic is
// skipped and the single-layer branch taken.
template <bool ONE = false>
LSH_HD void volume_update(const double wo[6], const double acc[7], double w[6], double& rate,
                                              double inv_area, double tanR, double dt, const Consts& c) {
    rate = lt_pos(acc[6], kEps) ? 0.0 : acc[6] * inv_area;
    const double b = dt * inv_area;
#pragma unroll
    for (int k = 0; k < (ONE ? 3 : 6); ++k) w[k] = fmad(b, acc[k], wo[k]);
    if (ONE) { w[3] = 0.0; w[4] = 0.0; w[5] = 0.0; }
    const double fo1 = vfac(wo[0], c.eps_h);
    if (!is_zero(tanR)) {
#pragma unroll
        for (int layer = 0; layer < (ONE ? 1 : 2); ++layer) {
            const int k = 3 * layer;
            if (is_zero(wo[k]) && is_zero(wo[k + 1]) && is_zero(wo[k + 2])) continue;  // adds exactly 0
            const double ux = (layer ? vfac(wo[k], c.eps_h) : fo1) * wo[k + 1];
            const double s = dt * (ux * tanR);
            w[k + 1] = fmad(s, wo[k + 2], w[k + 1]);
            w[k + 2] = fmad(-s, wo[k + 1], w[k + 2]);
        }
    }
    // single layer: the granular layer is empty before and after the Euler
    // update (h2 = q2 = 0 in both), so its friction and Coulomb terms are zeros
    if (ONE) {
        filtro<false>(w, dt, c);
        dis_implicita<false>(wo, w, dt, c, fo1);
    } else if (is_zero(wo[3]) && is_zero(wo[4]) && is_zero(wo[5]) && is_zero(w[3]) && is_zero(w[4]) && is_zero(w[5])) {
        filtro<false>(w, dt, c);
        dis_implicita<false>(wo, w, dt, c, fo1);
        w[4] = w[4] * 0.0;  // coulomb() with h2 = 0
        w[5] = w[5] * 0.0;
    } else {
        filtro<true>(w, dt, c);
        dis_implicita<true>(wo, w, dt, c, fo1);
        coulomb(w, dt, c);
    }
}

}  // namespace lsh
