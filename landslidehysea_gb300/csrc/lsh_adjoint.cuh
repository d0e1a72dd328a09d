// lsh_adjoint.cuh -- hand-written reverse-mode (adjoint) versions of the
// per-edge and per-cell operators of lsh_scheme.cuh.
//
// Each function takes the forward operator's inputs, recomputes the forward
// arithmetic (the same statements, so every comparison takes the branch the
// forward took: branch replay by exact recomputation), then walks the
// statements backwards accumulating adjoints.  Inputs are the forward
// inputs plus the adjoints of the outputs; results are ADDED to the adjoint
// outputs (callers zero them).
//
// What is differentiated: the state (h1, q1, h2, q2 of each cell), the step
// dt (the CFL step is a function of the previous state), and the constants
// the parameters enter: r (with 1 - r, g(1 - r), 1/(g(1 - r)), eps_h(1 + r)),
// the Coulomb coefficient mu = |tan(angle1)| L/H and the Manning products
// g mf0^2, g mfs^2.  Bathymetry H, geometry, g, eps_h, beta, peso, mfc and
// vmax are constants.  Coulomb law only (the Pouliquen law's mu is
// differentiable only away from its own branch points and is not covered).
//
// Conventions where the forward is not differentiable (shared with the CPU
// oracle's tangent-linear model): sqrt'(0) = 0, |x|' = sign with +1 at 0,
// min / max / minmod / clamps follow the operand the forward selected, and
// a face pair with no granular layer (the forward's single-layer edge
// branch) has no sensitivity to h2 or q2.
#pragma once

#include "lsh_passes.cuh"
#include "lsh_scheme.cuh"

namespace lsh {

// Adjoints of the parameter-carrying constants.
struct ConstBar {
    double r, omr, gp, inv_gp, mu, g_mf02, g_mfs2, eps_1r;
};

LSH_HD void cb_zero(ConstBar& b) { b.r = b.omr = b.gp = b.inv_gp = b.mu = b.g_mf02 = b.g_mfs2 = b.eps_1r = 0.0; }

LSH_HD double sgn1(double x) { return lt0(x) ? -1.0 : 1.0; }
// x * sgn1(s) as a sign-bit flip (integer pipe; the same bits)
LSH_HD double times_sgn1(double x, double s) { return lshm::neg_if(x, lt0(s)); }

// d vfac / dh
LSH_HD double vfac_d(double h, double eps_h) {
    if (gt_pos(h, eps_h)) { const double v = 1.0 / h; return -(v * v); }
    const double h2 = h * h, m2 = eps_h * eps_h;
    const double q = fmad(h2, h2, m2 * m2);
    const double s = sqrt(q);
    // d/dh [sqrt2 h q^-1/2] = sqrt2 q^-1/2 (1 - 2 h^4 / q)
    return (kSqrt2 / s) * (1.0 - (2.0 * (h2 * h2)) / q);
}

// d (h cbrt h) / dh = (4/3) cbrt h; 0 at h = 0
LSH_HD double pow43_d(double h) {
    if (!gt0(h)) return 0.0;
    const double c = lshm::cbrt_pos(h);
    return c + c / 3.0;
}

LSH_HD double sqrt_bar(double s, double sb) { return gt0(s) ? sb / (2.0 * s) : 0.0; }

// The compare-and-swap network of sort_eig on values, carrying the labels
// of the unsorted entries: after the call D[k] = entry perm[k].
LSH_HD void sort_eig_perm(double D[4], int perm[4], int full) {
    auto cs = [&](int a, int b) {
        if (lt(D[b], D[a])) {
            double t = D[b]; D[b] = D[a]; D[a] = t;
            int u = perm[b]; perm[b] = perm[a]; perm[a] = u;
        }
    };
    cs(0, 1); cs(0, 2); cs(0, 3); cs(1, 2); cs(1, 3);
    if (full) cs(1, 2);
    else if (lt(D[1], D[2])) {
        double t = D[1]; D[1] = D[2]; D[2] = t;
        int u = perm[1]; perm[1] = perm[2]; perm[2] = u;
    }
    cs(2, 3);
}

// Adjoint of eig<L2>(h1, h2, u1, u2, q, c, Fknown, sqrt_h) given the
// adjoints of its sorted outputs Db (x, y, z, w).
template <bool L2>
LSH_HD void eig_adj(double h1, double h2, double u1, double u2, double q, const Consts& c, double Fknown,
                    double sqrt_h, const V4& Db, double& h1b, double& h2b, double& u1b, double& u2b, double& qb,
                    double& Fknownb, double& sqrt_hb, ConstBar& cb, bool mean_u = false) {
    const double h = L2 ? h1 + h2 : h1;
    const bool useFk = (!L2 && !lt0(Fknown));
    // as eig: the edge average's u is u1 itself with no granular layer and h > eps_h
    const bool direct = mean_u && is_zero(h2) && gt_pos(h, c.eps_h);
    const double F = useFk ? Fknown : vfac(h, c.eps_h);
    const double u = direct ? u1 : q * F;
    const bool useSh = !lt0(sqrt_h);
    const double cg = useSh ? c.sqrt_g * sqrt_h : sqrt(c.g * h);
    double uu = 0.0, ci = 0.0, d = 0.0, aux = 0.0, P = 0.0;
    if (L2) {
        uu = fmad(u1, h2, u2 * h1) * F;
        d = u1 - u2;
        aux = fmad(-((d * d) * F), c.inv_gp, 1.0);
        P = (((c.gp * h1) * h2) * F);
        ci = sqrt(P * abs_bits(aux));
    }
    double e[4] = {u - cg, uu - ci, uu + ci, u + cg};
    int perm[4] = {0, 1, 2, 3};
    sort_eig_perm(e, perm, c.eig_sort);
    // eb[perm[k]] = 0 + Db_k: each entry takes the one sorted adjoint whose
    // label it is (selections on the integer pipe; a store through perm would
    // put eb in local memory), then the same addition to +0
    double eb[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const double v = (perm[0] == j) ? Db.x : (perm[1] == j) ? Db.y : (perm[2] == j) ? Db.z : Db.w;
        eb[j] = 0.0 + v;
    }
    const double ub = eb[0] + eb[3];
    const double cgb = eb[3] - eb[0];
    double Fb = 0.0, hb = 0.0;
    if (L2) {
        const double uub = eb[1] + eb[2];
        const double cib = eb[2] - eb[1];
        const double Xb = sqrt_bar(ci, cib);
        const double A = abs_bits(aux);
        const double Pb = Xb * A;
        const double auxb = times_sgn1(Xb * P, aux);
        cb.gp += Pb * ((h1 * h2) * F);
        h1b += Pb * ((c.gp * h2) * F);
        h2b += Pb * ((c.gp * h1) * F);
        Fb += Pb * ((c.gp * h1) * h2);
        // aux = 1 - d^2 F inv_gp
        const double db = auxb * (-2.0 * d * F * c.inv_gp);
        Fb += auxb * (-(d * d) * c.inv_gp);
        cb.inv_gp += auxb * (-((d * d) * F));
        u1b += db;
        u2b -= db;
        // uu = (u1 h2 + u2 h1) F
        const double n = fmad(u1, h2, u2 * h1);
        const double nb = uub * F;
        Fb += uub * n;
        u1b += nb * h2;
        h2b += nb * u1;
        u2b += nb * h1;
        h1b += nb * u2;
    }
    if (useSh) sqrt_hb += cgb * c.sqrt_g;
    else if (gt0(cg)) hb += (cgb * c.g) / (2.0 * cg);
    if (direct) {
        u1b += ub;
    } else {
        qb += ub * F;
        Fb += ub * q;
    }
    if (useFk) Fknownb += Fb;
    else hb += Fb * vfac_d(h, c.eps_h);
    h1b += hb;
    if (L2) h2b += hb;
}

// Adjoint-side view of an edge: adjoints of the two faces, the cell-average
// depths and the partial accumulators the limiter read.
struct FaceBar { double h1, qn1, qt1, h2, qn2, qt2; };
struct EdgeInBar {
    FaceBar A, B;
    double hc0[2], hc1[2];
    double acc0h[2], acc1h[2];
};

LSH_HD void face_bar_zero(FaceBar& f) { f.h1 = f.qn1 = f.qt1 = f.h2 = f.qn2 = f.qt2 = 0.0; }
LSH_HD void edge_bar_zero(EdgeInBar& b) {
    face_bar_zero(b.A);
    face_bar_zero(b.B);
    b.hc0[0] = b.hc0[1] = b.hc1[0] = b.hc1[1] = 0.0;
    b.acc0h[0] = b.acc0h[1] = b.acc1h[0] = b.acc1h[1] = 0.0;
}

// Adjoint of edge_flux<L2>: `ob` holds the adjoints of o.m, o.p, o.wave.
template <bool L2>
LSH_HD void edge_flux_adj(const EdgeIn& e, double dt, const Consts& c, const EdgeOut& ob, EdgeInBar& eb,
                          double& dtb, ConstBar& cb) {
    // ---------------------------------------------------------------- forward
    const double eps = c.eps_h;
    double Aq1 = e.A.qn1, Aq2 = L2 ? e.A.qn2 : 0.0, Bq1 = e.B.qn1, Bq2 = L2 ? e.B.qn2 : 0.0;
    const double Ah1 = e.A.h1, Bh1 = e.B.h1;
    const double Ah2 = L2 ? e.A.h2 : 0.0, Bh2 = L2 ? e.B.h2 : 0.0;
    const double H0 = e.A.H, H1 = e.B.H;
    const double h1ij = 0.5 * (Ah1 + Bh1);
    const double h2ij = L2 ? 0.5 * (Ah2 + Bh2) : 0.0;
    bool zA1 = false, zA2 = false, zB1 = false, zB2 = false;
    if (L2) {
        if (lt_pos(Ah2, eps) && lt(H0, H1 - Bh2)) zB2 = true;
        if (lt_pos(Bh2, eps) && lt(H1, H0 - Ah2)) zA2 = true;
        if (lt_pos(Ah1, eps) && lt(H0 - Ah2, H1 - Bh1 - Bh2)) zB1 = true;
        if (lt_pos(Bh1, eps) && lt(H1 - Bh2, H0 - Ah1 - Ah2)) zA1 = true;
        if (lt_pos(Ah2 + Ah1, eps) && lt(H0, H1 - Bh1 - Bh2)) { zB1 = true; zB2 = true; }
        if (lt_pos(Bh2 + Bh1, eps) && lt(H1, H0 - Ah1 - Ah2)) { zA1 = true; zA2 = true; }
    } else {
        if (lt_pos(Ah1, eps) && lt(H0, H1 - Bh1)) zB1 = true;
        if (lt_pos(Bh1, eps) && lt(H1, H0 - Ah1)) zA1 = true;
    }
    if (zA1) Aq1 = 0.0;
    if (zA2) Aq2 = 0.0;
    if (zB1) Bq1 = 0.0;
    if (zB2) Bq2 = 0.0;

    const double fA1 = vfac(Ah1, eps), fB1 = vfac(Bh1, eps);
    const double fA2 = L2 ? vfac(Ah2, eps) : 0.0, fB2 = L2 ? vfac(Bh2, eps) : 0.0;
    const double sa1 = sqrt(Ah1), sb1 = sqrt(Bh1);
    const double num1 = fmad(sa1, fA1 * Aq1, sb1 * (fB1 * Bq1));
    const double den1 = sa1 + sb1 + kEps;
    const double u1ij = num1 / den1;
    double sa2 = 0.0, sb2 = 0.0, num2 = 0.0, den2 = 1.0, u2ij = 0.0;
    if (L2) {
        sa2 = sqrt(Ah2); sb2 = sqrt(Bh2);
        num2 = fmad(sa2, fA2 * Aq2, sb2 * (fB2 * Bq2));
        den2 = sa2 + sb2 + kEps;
        u2ij = num2 / den2;
    }
    const bool oneA = !L2 || is_zero(Ah2), oneB = !L2 || is_zero(Bh2);

    const double Hm = tmin(H0, H1);
    const double P1 = L2 ? Bh1 + Bh2 - H1 + Hm : Bh1 - H1 + Hm;
    const double P0 = L2 ? Ah1 + Ah2 - H0 + Hm : Ah1 - H0 + Hm;
    const double deta1 = max0(P1) - max0(P0);
    const double Q1 = L2 ? Bh2 - H1 + Hm : 0.0, Q0 = L2 ? Ah2 - H0 + Hm : 0.0;
    const double deta2 = L2 ? max0(Q1) - max0(Q0) : 0.0;
    const double gh1 = c.g * h1ij, gh2 = c.g * h2ij;
    const double sw = L2 ? fmad(c.omr, deta2, c.r * deta1) : 0.0;
    const V4 tp{0.0, gh1 * deta1, 0.0, L2 ? gh2 * sw : 0.0};

    bool coul = false;
    V4 tp2 = tp;
    if (L2) {
        const double mu = friction_mu(h1ij, u1ij, h2ij, u2ij, c);
        const double sc = ((fsc_of(h1ij, c) * mu) * c.g) * h2ij;
        coul = lt(abs_bits(h2ij * u2ij), (c.peso * sc) * dt);
        if (coul) tp2.w = (gh2 * c.r) * deta1;
    }

    const double qD = L2 ? fmad(h1ij, u1ij, h2ij * u2ij) : h1ij * u1ij;
    const double uA1 = fA1 * Aq1, uA2 = fA2 * Aq2, uB1 = fB1 * Bq1, uB2 = fB2 * Bq2;
    const double qA = L2 ? Aq1 + Aq2 : Aq1, qB = L2 ? Bq1 + Bq2 : Bq1;
    const double shA = oneA ? sa1 : -1.0, shB = oneB ? sb1 : -1.0;
    const V4 D = eig<L2>(h1ij, h2ij, u1ij, u2ij, qD, c, -1.0, -1.0, true);
    const V4 E0 = eig<L2>(Ah1, Ah2, uA1, uA2, qA, c, fA1, shA);
    const V4 E1 = eig<L2>(Bh1, Bh2, uB1, uB2, qB, c, fB1, shB);
    const double m01 = tmin(E0.x, E1.x);
    const double aut1 = tmin(D.x, m01);
    const double M01 = tmax(E0.w, E1.w);
    const double aut3 = tmax(D.w, M01);
    const double lmax0 = tmax(abs_bits(aut3), abs_bits(aut1));
    const double umax = L2 ? tmax(abs_bits(u1ij), abs_bits(u2ij)) : abs_bits(u1ij);
    const bool lm_u = lt(lmax0, umax);
    double lmax = lm_u ? umax : lmax0;
    const double aut2u = tmax(abs_bits(D.y), abs_bits(D.z));
    const bool neg2 = (sgn(aut1 + aut3) < 0);
    const double aut2 = lshm::neg_if(aut2u, neg2);

    int branch;  // 0: three waves, 1: two waves, 2: degenerate (a0 = lmax)
    double a0, a1, a2 = 0.0;
    double d12 = 0.0, d13 = 0.0, d23 = 0.0, inv = 0.0, aa = 0.0, bb = 0.0, cc = 0.0;
    if (!abs_lt(aut1 - aut3, kEps) && !abs_lt(aut1 - aut2, kEps) && !abs_lt(aut2 - aut3, kEps)) {
        if (L2 && !lt_pos(h1ij, eps) && !lt_pos(h2ij, eps)) {
            branch = 0;
            d12 = aut1 - aut2; d13 = aut1 - aut3; d23 = aut2 - aut3;
            inv = 1.0 / ((d12 * d13) * d23);
            aa = (fabs(aut1) * d23) * inv;
            bb = -((fabs(aut2) * d13) * inv);
            cc = (fabs(aut3) * d12) * inv;
            a0 = fmad(aa * aut2, aut3, fmad(bb * aut1, aut3, (cc * aut1) * aut2));
            a1 = -fmad(aa, aut2 + aut3, fmad(bb, aut1 + aut3, cc * (aut1 + aut2)));
            a2 = aa + bb + cc;
        } else {
            branch = 1;
            inv = 1.0 / (aut3 - aut1);
            a0 = fmad(aut3, fabs(aut1), -(aut1 * fabs(aut3))) * inv;
            a1 = (fabs(aut3) - fabs(aut1)) * inv;
        }
    } else {
        branch = 2;
        a0 = lmax; a1 = 0.0;
    }

    const bool fAy = !lt_pos(Ah1, kEps), fBy = !lt_pos(Bh1, kEps);
    const double FAy = fAy ? uA1 * Aq1 : 0.0, FBy = fBy ? uB1 * Bq1 : 0.0;
    const double dFx = Bq1 - Aq1, dFy = FBy - FAy;
    double dFz = 0.0, dFw = 0.0, FAw = 0.0, FBw = 0.0;
    const bool fAw = L2 && !lt_pos(Ah2, kEps), fBw = L2 && !lt_pos(Bh2, kEps);
    if (L2) {
        FAw = fAw ? uA2 * Aq2 : 0.0;
        FBw = fBw ? uB2 * Bq2 : 0.0;
        dFz = Bq2 - Aq2;
        dFw = FBw - FAw;
    }
    const V4 T2{tp2.x + dFx, tp2.y + dFy, tp2.z + dFz, tp2.w + dFw};
    const double Atx = T2.y;
    const double Aty = fmad(gh1, T2.z, fmad(u1ij + u1ij, T2.y, fmad(-u1ij, u1ij, gh1) * T2.x));
    V4 I{deta1, Bq1 - Aq1, 0.0, Bq2 - Aq2};
    const bool icx = !coul && gt_pos(Ah1, eps) && gt_pos(Bh1, eps);
    if (!coul) {
        if (icx) I.x = I.x - deta2;
        I.z = deta2;
    }
    double Qx, Qy;
    if (L2) {
        Qx = 0.5 * fmad(a0, I.x, fmad(a1, T2.x, a2 * Atx));
        Qy = 0.5 * fmad(a0, I.y, fmad(a1, T2.y, a2 * Aty));
    } else {
        Qx = 0.5 * fmad(a0, I.x, a1 * T2.x);
        Qy = 0.5 * fmad(a0, I.y, a1 * T2.y);
    }
    const double half_x = 0.5 * (dFx + tp.x), half_y = 0.5 * (dFy + tp.y);
    const double Fmx = half_x + (Aq1 - Qx), Fmy = half_y + (FAy - Qy);
    const double Fpx = half_x + (Qx - Bq1), Fpy = half_y + (Qy - FBy);
    const int t1 = abs_lt(Fmx, kEps) ? 0 : (gt0(Fmx) ? 1 : 2);
    const double u1t = (t1 == 0) ? 0.0 : ((t1 == 1) ? fA1 * e.A.qt1 : fB1 * e.B.qt1);
    const double s1 = Fmx * u1t;
    double M[6] = {Fmx, Fmy, s1, 0.0, 0.0, 0.0};
    double P[6] = {Fpx, Fpy, -s1, 0.0, 0.0, 0.0};
    double Atz = 0.0, Atw = 0.0, Qz = 0.0, Qw = 0.0, Fmz = 0.0, u2t = 0.0, rgh2 = 0.0, mw = 0.0;
    int t2 = 0;
    if (L2) {
        Atz = T2.w;
        rgh2 = c.r * gh2;
        mw = fmad(-u2ij, u2ij, gh2);
        Atw = fmad(rgh2, T2.x, fmad(mw, T2.z, (u2ij + u2ij) * T2.w));
        Qz = 0.5 * fmad(a0, I.z, fmad(a1, T2.z, a2 * Atz));
        Qw = 0.5 * fmad(a0, I.w, fmad(a1, T2.w, a2 * Atw));
        const double half_z = 0.5 * (dFz + tp.z), half_w = 0.5 * (dFw + tp.w);
        Fmz = half_z + (Aq2 - Qz);
        const double Fmw = half_w + (FAw - Qw);
        const double Fpz = half_z + (Qz - Bq2), Fpw = half_w + (Qw - FBw);
        t2 = abs_lt(Fmz, kEps) ? 0 : (gt0(Fmz) ? 1 : 2);
        u2t = (t2 == 0) ? 0.0 : ((t2 == 1) ? fA2 * e.A.qt2 : fB2 * e.B.qt2);
        const double s2 = Fmz * u2t;
        M[3] = Fmz; M[4] = Fmw; M[5] = s2;
        P[3] = Fpz; P[4] = Fpw; P[5] = -s2;
    }
    constexpr int KL = L2 ? 6 : 3;
    for (int k = 0; k < KL; ++k) { P[k] = e.len * P[k]; M[k] = e.len * M[k]; }

    const double b0 = dt * e.inv_area0;
    const double hp0[2] = {fmad(b0, e.acc0h[0], e.hc0[0]), L2 ? fmad(b0, e.acc0h[1], e.hc0[1]) : 0.0};
    double b1 = 0.0, hp1[2] = {0.0, 0.0};
    if (e.interior) {
        b1 = dt * e.inv_area1;
        hp1[0] = fmad(b1, e.acc1h[0], e.hc1[0]);
        if (L2) hp1[1] = fmad(b1, e.acc1h[1], e.hc1[1]);
    }
    const double factor = 1.0 * c.beta;
    bool lim[2] = {false, false}, useA[2] = {false, false}, useB[2] = {false, false};
    double alpha[2] = {1.0, 1.0}, dta[2] = {kBig, kBig}, dtbv[2] = {kBig, kBig}, dtl[2] = {kBig, kBig};
    double Mpre[6], Ppre[6], denA[2] = {1.0, 1.0}, denB[2] = {1.0, 1.0};
    for (int k = 0; k < 6; ++k) { Mpre[k] = M[k]; Ppre[k] = P[k]; }
    for (int layer = 0; layer < (L2 ? 2 : 1); ++layer) {
        const int k = 3 * layer;
        useA[layer] = gt0(M[k]);
        useB[layer] = e.interior && gt0(P[k]);
        const double ha = hp0[layer] * e.area0, hb = hp1[layer] * e.area1;
        if (useA[layer]) denA[layer] = fmad(factor, M[k], kEps);
        if (useB[layer]) denB[layer] = fmad(factor, P[k], kEps);
        lim[layer] = (useA[layer] && lt(ha, dt * denA[layer])) || (useB[layer] && lt(hb, dt * denB[layer]));
        if (lim[layer]) {
            if (useA[layer]) dta[layer] = ha / denA[layer];
            if (useB[layer]) dtbv[layer] = hb / denB[layer];
            dtl[layer] = tmin(dta[layer], dtbv[layer]);
            alpha[layer] = dtl[layer] / (dt + kEps);
        }
    }

    // ---------------------------------------------------------------- reverse
    double mb[6], pb[6];
    for (int k = 0; k < 6; ++k) { mb[k] = ob.m[k]; pb[k] = ob.p[k]; }
    double wb = ob.wave;
    if (lshm::bits_of(c.peso) != lshm::bits_of(1.0)) {
        wb = wb * c.inv_peso;
        for (int k = 0; k < 6; ++k) { mb[k] = c.peso * mb[k]; pb[k] = c.peso * pb[k]; }
    }
    double lmaxb = e.len * wb;  // lmax (+ eps) -> wave

    double hp0b[2] = {0.0, 0.0}, hp1b[2] = {0.0, 0.0};
    for (int layer = 0; layer < (L2 ? 2 : 1); ++layer) {
        if (!lim[layer]) continue;
        const int k = 3 * layer;
        double alb = 0.0;
        for (int q = k; q < k + 3; ++q) {
            alb += mb[q] * Mpre[q] + pb[q] * Ppre[q];
            mb[q] = mb[q] * alpha[layer];
            pb[q] = pb[q] * alpha[layer];
        }
        const double dtlb = alb / (dt + kEps);
        dtb += -alb * (alpha[layer] / (dt + kEps));
        // tmin(dta, dtb) = (dtb < dta) ? dtb : dta
        if (lt(dtbv[layer], dta[layer])) {
            // dtb = hp1 area1 / (beta P + eps)
            hp1b[layer] += dtlb * (e.area1 / denB[layer]);
            pb[k] += (-dtlb * (dtbv[layer] / denB[layer])) * factor;
        } else if (useA[layer]) {
            hp0b[layer] += dtlb * (e.area0 / denA[layer]);
            mb[k] += (-dtlb * (dta[layer] / denA[layer])) * factor;
        }
    }
    // hp = b acc + hc, b = dt / area
    double b0b = 0.0, b1b = 0.0;
    for (int layer = 0; layer < (L2 ? 2 : 1); ++layer) {
        b0b += hp0b[layer] * e.acc0h[layer];
        eb.acc0h[layer] += hp0b[layer] * b0;
        eb.hc0[layer] += hp0b[layer];
        if (e.interior) {
            b1b += hp1b[layer] * e.acc1h[layer];
            eb.acc1h[layer] += hp1b[layer] * b1;
            eb.hc1[layer] += hp1b[layer];
        }
    }
    dtb += b0b * e.inv_area0 + b1b * e.inv_area1;
    for (int k = 0; k < KL; ++k) { mb[k] = mb[k] * e.len; pb[k] = pb[k] * e.len; }

    // fluxes
    double Fmxb = mb[0], Fmyb = mb[1], Fpxb = pb[0], Fpyb = pb[1];
    const double s1b = mb[2] - pb[2];
    Fmxb += s1b * u1t;
    const double u1tb = s1b * Fmx;
    double fA1b = 0.0, fB1b = 0.0, fA2b = 0.0, fB2b = 0.0;
    if (t1 == 1) { fA1b += u1tb * e.A.qt1; eb.A.qt1 += u1tb * fA1; }
    else if (t1 == 2) { fB1b += u1tb * e.B.qt1; eb.B.qt1 += u1tb * fB1; }
    double Aq1b = 0.0, Bq1b = 0.0, Aq2b = 0.0, Bq2b = 0.0, FAyb = 0.0, FByb = 0.0, FAwb = 0.0, FBwb = 0.0;
    double Qxb, Qyb, Qzb = 0.0, Qwb = 0.0, halfxb, halfyb, halfzb = 0.0, halfwb = 0.0;
    halfxb = Fmxb + Fpxb; Aq1b += Fmxb; Qxb = Fpxb - Fmxb; Bq1b -= Fpxb;
    halfyb = Fmyb + Fpyb; FAyb += Fmyb; Qyb = Fpyb - Fmyb; FByb -= Fpyb;
    if (L2) {
        double Fmzb = mb[3], Fmwb = mb[4], Fpzb = pb[3], Fpwb = pb[4];
        const double s2b = mb[5] - pb[5];
        Fmzb += s2b * u2t;
        const double u2tb = s2b * Fmz;
        if (t2 == 1) { fA2b += u2tb * e.A.qt2; eb.A.qt2 += u2tb * fA2; }
        else if (t2 == 2) { fB2b += u2tb * e.B.qt2; eb.B.qt2 += u2tb * fB2; }
        halfzb = Fmzb + Fpzb; Aq2b += Fmzb; Qzb = Fpzb - Fmzb; Bq2b -= Fpzb;
        halfwb = Fmwb + Fpwb; FAwb += Fmwb; Qwb = Fpwb - Fmwb; FBwb -= Fpwb;
    }
    // Q = 0.5 (a0 I + a1 T2 + a2 At)
    double a0b = 0.5 * (Qxb * I.x + Qyb * I.y);
    double a1b = 0.5 * (Qxb * T2.x + Qyb * T2.y);
    double a2b = 0.0;
    double Ixb = 0.5 * Qxb * a0, Iyb = 0.5 * Qyb * a0, Izb = 0.0, Iwb = 0.0;
    double T2xb = 0.5 * Qxb * a1, T2yb = 0.5 * Qyb * a1, T2zb = 0.0, T2wb = 0.0;
    double Atxb = 0.0, Atyb = 0.0, Atzb = 0.0, Atwb = 0.0;
    double u1b = 0.0, u2b = 0.0, gh1b = 0.0, gh2b = 0.0;
    if (L2) {
        a0b += 0.5 * (Qzb * I.z + Qwb * I.w);
        a1b += 0.5 * (Qzb * T2.z + Qwb * T2.w);
        a2b = 0.5 * (Qxb * Atx + Qyb * Aty + Qzb * Atz + Qwb * Atw);
        Izb = 0.5 * Qzb * a0; Iwb = 0.5 * Qwb * a0;
        T2zb = 0.5 * Qzb * a1; T2wb = 0.5 * Qwb * a1;
        Atxb = 0.5 * Qxb * a2; Atyb = 0.5 * Qyb * a2; Atzb = 0.5 * Qzb * a2; Atwb = 0.5 * Qwb * a2;
        // Atw = r gh2 T2x + (gh2 - u2^2) T2z + 2 u2 T2w
        cb.r += Atwb * (T2.x * gh2);
        gh2b += Atwb * (T2.x * c.r);
        T2xb += Atwb * rgh2;
        gh2b += Atwb * T2.z;
        u2b += Atwb * (-2.0 * u2ij * T2.z + 2.0 * T2.w);
        T2zb += Atwb * mw;
        T2wb += Atwb * (u2ij + u2ij);
        T2wb += Atzb;
        // Aty = gh1 T2z + 2 u1 T2y + (gh1 - u1^2) T2x
        gh1b += Atyb * (T2.z + T2.x);
        T2zb += Atyb * gh1;
        u1b += Atyb * (2.0 * T2.y - 2.0 * u1ij * T2.x);
        T2yb += Atyb * (u1ij + u1ij);
        T2xb += Atyb * fmad(-u1ij, u1ij, gh1);
        T2yb += Atxb;
    }
    // I
    double deta1b = Ixb, deta2b = 0.0;
    if (icx) deta2b -= Ixb;
    Bq1b += Iyb; Aq1b -= Iyb;
    if (L2) {
        if (!coul) deta2b += Izb;
        Bq2b += Iwb; Aq2b -= Iwb;
    }
    // half = 0.5 (dF + tp)
    double dFxb = 0.5 * halfxb + T2xb, dFyb = 0.5 * halfyb + T2yb, dFzb = 0.0, dFwb = 0.0;
    double tpyb = 0.5 * halfyb + T2yb, tpwb = 0.0;
    if (L2) {
        dFzb = 0.5 * halfzb + T2zb;
        dFwb = 0.5 * halfwb + T2wb;
        tpwb = 0.5 * halfwb;
        if (coul) {
            gh2b += T2wb * (c.r * deta1);
            cb.r += T2wb * (gh2 * deta1);
            deta1b += T2wb * (gh2 * c.r);
        } else {
            tpwb += T2wb;
        }
    }
    // dF
    Bq1b += dFxb; Aq1b -= dFxb;
    FByb += dFyb; FAyb -= dFyb;
    if (L2) { Bq2b += dFzb; Aq2b -= dFzb; FBwb += dFwb; FAwb -= dFwb; }
    double uA1b = 0.0, uA2b = 0.0, uB1b = 0.0, uB2b = 0.0;
    if (fAy) { uA1b += FAyb * Aq1; Aq1b += FAyb * uA1; }
    if (fBy) { uB1b += FByb * Bq1; Bq1b += FByb * uB1; }
    if (fAw) { uA2b += FAwb * Aq2; Aq2b += FAwb * uA2; }
    if (fBw) { uB2b += FBwb * Bq2; Bq2b += FBwb * uB2; }
    // PVM / IFCP coefficients
    double aut1b = 0.0, aut2b = 0.0, aut3b = 0.0;
    if (branch == 0) {
        const double ab_ = a0b * (aut2 * aut3) - a1b * (aut2 + aut3) + a2b;
        const double bb_ = a0b * (aut1 * aut3) - a1b * (aut1 + aut3) + a2b;
        const double cb_ = a0b * (aut1 * aut2) - a1b * (aut1 + aut2) + a2b;
        aut1b += a0b * (bb * aut3 + cc * aut2) - a1b * (bb + cc);
        aut2b += a0b * (aa * aut3 + cc * aut1) - a1b * (aa + cc);
        aut3b += a0b * (aa * aut2 + bb * aut1) - a1b * (aa + bb);
        double d12b = 0.0, d13b = 0.0, d23b = 0.0, invb = 0.0;
        aut1b += times_sgn1(ab_, aut1) * d23 * inv; d23b += ab_ * fabs(aut1) * inv; invb += ab_ * fabs(aut1) * d23;
        aut2b -= times_sgn1(bb_, aut2) * d13 * inv; d13b -= bb_ * fabs(aut2) * inv; invb -= bb_ * fabs(aut2) * d13;
        aut3b += times_sgn1(cb_, aut3) * d12 * inv; d12b += cb_ * fabs(aut3) * inv; invb += cb_ * fabs(aut3) * d12;
        const double Pb = -invb * (inv * inv);
        d12b += Pb * (d13 * d23); d13b += Pb * (d12 * d23); d23b += Pb * (d12 * d13);
        aut1b += d12b + d13b;
        aut2b += d23b - d12b;
        aut3b -= d13b + d23b;
    } else if (branch == 1) {
        const double n0 = fmad(aut3, fabs(aut1), -(aut1 * fabs(aut3)));
        const double n1 = fabs(aut3) - fabs(aut1);
        const double n0b = a0b * inv, n1b = a1b * inv;
        const double invb = a0b * n0 + a1b * n1;
        aut3b += n0b * (fabs(aut1) - times_sgn1(aut1, aut3)) + times_sgn1(n1b, aut3);
        aut1b += n0b * (times_sgn1(aut3, aut1) - fabs(aut3)) - times_sgn1(n1b, aut1);
        const double denb = -invb * (inv * inv);
        aut3b += denb;
        aut1b -= denb;
    } else {
        lmaxb += a0b;
    }
    // signed aut2
    const double aut2ub = lshm::neg_if(aut2b, neg2);
    V4 Db{0.0, 0.0, 0.0, 0.0}, E0b{0.0, 0.0, 0.0, 0.0}, E1b{0.0, 0.0, 0.0, 0.0};
    if (abs_lt(D.y, D.z)) Db.z += times_sgn1(aut2ub, D.z);
    else Db.y += times_sgn1(aut2ub, D.y);
    // lmax
    if (lm_u) {
        if (L2 && abs_lt(u1ij, u2ij)) u2b += times_sgn1(lmaxb, u2ij);
        else u1b += times_sgn1(lmaxb, u1ij);
    } else {
        if (abs_lt(aut3, aut1)) aut1b += times_sgn1(lmaxb, aut1);
        else aut3b += times_sgn1(lmaxb, aut3);
    }
    // aut1 = tmin(D.x, tmin(E0.x, E1.x)); aut3 = tmax(D.w, tmax(E0.w, E1.w))
    if (lt(m01, D.x)) { if (lt(E1.x, E0.x)) E1b.x += aut1b; else E0b.x += aut1b; }
    else Db.x += aut1b;
    if (lt(D.w, M01)) { if (lt(E0.w, E1.w)) E1b.w += aut3b; else E0b.w += aut3b; }
    else Db.w += aut3b;
    // eigenvalue bounds
    double h1ijb = 0.0, h2ijb = 0.0, qDb = 0.0, dummyF = 0.0, dummyS = 0.0;
    eig_adj<L2>(h1ij, h2ij, u1ij, u2ij, qD, c, -1.0, -1.0, Db, h1ijb, h2ijb, u1b, u2b, qDb, dummyF, dummyS, cb, true);
    h1ijb += qDb * u1ij;
    u1b += qDb * h1ij;
    if (L2) { h2ijb += qDb * u2ij; u2b += qDb * h2ij; }
    double Ah1b = 0.0, Ah2b = 0.0, Bh1b = 0.0, Bh2b = 0.0, qAb = 0.0, qBb = 0.0, sa1b = 0.0, sb1b = 0.0;
    double sa2b = 0.0, sb2b = 0.0;
    {
        double shb = 0.0;
        eig_adj<L2>(Ah1, Ah2, uA1, uA2, qA, c, fA1, shA, E0b, Ah1b, Ah2b, uA1b, uA2b, qAb, fA1b, shb, cb);
        if (!lt0(shA)) sa1b += shb;
        shb = 0.0;
        eig_adj<L2>(Bh1, Bh2, uB1, uB2, qB, c, fB1, shB, E1b, Bh1b, Bh2b, uB1b, uB2b, qBb, fB1b, shb, cb);
        if (!lt0(shB)) sb1b += shb;
    }
    Aq1b += qAb; Bq1b += qBb;
    if (L2) { Aq2b += qAb; Bq2b += qBb; }
    fA1b += uA1b * Aq1; Aq1b += uA1b * fA1;
    fB1b += uB1b * Bq1; Bq1b += uB1b * fB1;
    if (L2) {
        fA2b += uA2b * Aq2; Aq2b += uA2b * fA2;
        fB2b += uB2b * Bq2; Bq2b += uB2b * fB2;
    }
    // tp
    gh1b += tpyb * deta1;
    deta1b += tpyb * gh1;
    if (L2) {
        gh2b += tpwb * sw;
        const double swb = tpwb * gh2;
        cb.omr += swb * deta2;
        deta2b += swb * c.omr;
        cb.r += swb * deta1;
        deta1b += swb * c.r;
    }
    h1ijb += gh1b * c.g;
    h2ijb += gh2b * c.g;
    if (L2) {
        if (gt0(Q1)) Bh2b += deta2b;
        if (gt0(Q0)) Ah2b -= deta2b;
    }
    if (gt0(P1)) { Bh1b += deta1b; if (L2) Bh2b += deta1b; }
    if (gt0(P0)) { Ah1b -= deta1b; if (L2) Ah2b -= deta1b; }
    // Roe-type velocities
    {
        const double num1b = u1b / den1;
        const double den1b = -u1b * (u1ij / den1);
        sa1b += num1b * uA1 + den1b;
        fA1b += num1b * (sa1 * Aq1);
        Aq1b += num1b * (sa1 * fA1);
        sb1b += num1b * uB1 + den1b;
        fB1b += num1b * (sb1 * Bq1);
        Bq1b += num1b * (sb1 * fB1);
    }
    if (L2) {
        const double num2b = u2b / den2;
        const double den2b = -u2b * (u2ij / den2);
        sa2b += num2b * uA2 + den2b;
        fA2b += num2b * (sa2 * Aq2);
        Aq2b += num2b * (sa2 * fA2);
        sb2b += num2b * uB2 + den2b;
        fB2b += num2b * (sb2 * Bq2);
        Bq2b += num2b * (sb2 * fB2);
    }
    Ah1b += sqrt_bar(sa1, sa1b) + fA1b * vfac_d(Ah1, eps);
    Bh1b += sqrt_bar(sb1, sb1b) + fB1b * vfac_d(Bh1, eps);
    if (L2) {
        Ah2b += sqrt_bar(sa2, sa2b) + fA2b * vfac_d(Ah2, eps);
        Bh2b += sqrt_bar(sb2, sb2b) + fB2b * vfac_d(Bh2, eps);
    }
    Ah1b += 0.5 * h1ijb; Bh1b += 0.5 * h1ijb;
    if (L2) { Ah2b += 0.5 * h2ijb; Bh2b += 0.5 * h2ijb; }
    // wet/dry: a zeroed discharge does not depend on its input
    eb.A.h1 += Ah1b; eb.B.h1 += Bh1b;
    if (!zA1) eb.A.qn1 += Aq1b;
    if (!zB1) eb.B.qn1 += Bq1b;
    if (L2) {
        eb.A.h2 += Ah2b; eb.B.h2 += Bh2b;
        if (!zA2) eb.A.qn2 += Aq2b;
        if (!zB2) eb.B.qn2 += Bq2b;
    }
}

// Adjoint of edge_initial_wave(A, B, len, c) (no wet/dry fix, signed max).
LSH_HD void edge_initial_wave_adj(const Face& A, const Face& B, double len, const Consts& c, double wb, FaceBar& Ab,
                                  FaceBar& Bb, ConstBar& cb) {
    const double eps = c.eps_h;
    const double h1ij = 0.5 * (A.h1 + B.h1);
    const double fA1 = vfac(A.h1, eps), fB1 = vfac(B.h1, eps);
    const double sa1 = sqrt(A.h1), sb1 = sqrt(B.h1);
    const double uA1 = fA1 * A.qn1, uB1 = fB1 * B.qn1;
    const double num1 = fmad(sa1, uA1, sb1 * uB1), den1 = sa1 + sb1 + kEps;
    const double u1ij = num1 / den1;
    const double h2ij = 0.5 * (A.h2 + B.h2);
    const double fA2 = vfac(A.h2, eps), fB2 = vfac(B.h2, eps);
    const double sa2 = sqrt(A.h2), sb2 = sqrt(B.h2);
    const double uA2 = fA2 * A.qn2, uB2 = fB2 * B.qn2;
    const double num2 = fmad(sa2, uA2, sb2 * uB2), den2 = sa2 + sb2 + kEps;
    const double u2ij = num2 / den2;
    const double q = fmad(h1ij, u1ij, h2ij * u2ij);
    const V4 D = eig<true>(h1ij, h2ij, u1ij, u2ij, q, c);
    const double lm0 = tmax(D.x, D.w);
    const double bmax = tmax(fabs(u1ij), fabs(u2ij));
    // reverse
    const double lmaxb = len * wb;
    double u1b = 0.0, u2b = 0.0;
    V4 Db{0.0, 0.0, 0.0, 0.0};
    if (lt(lm0, bmax)) {
        if (abs_lt(u1ij, u2ij)) u2b += times_sgn1(lmaxb, u2ij);
        else u1b += times_sgn1(lmaxb, u1ij);
    } else {
        if (lt(D.x, D.w)) Db.w += lmaxb;
        else Db.x += lmaxb;
    }
    double h1ijb = 0.0, h2ijb = 0.0, qb = 0.0, fk = 0.0, sh = 0.0;
    eig_adj<true>(h1ij, h2ij, u1ij, u2ij, q, c, -1.0, -1.0, Db, h1ijb, h2ijb, u1b, u2b, qb, fk, sh, cb);
    h1ijb += qb * u1ij; u1b += qb * h1ij;
    h2ijb += qb * u2ij; u2b += qb * h2ij;
    const double num1b = u1b / den1, den1b = -u1b * (u1ij / den1);
    const double num2b = u2b / den2, den2b = -u2b * (u2ij / den2);
    const double sa1b = num1b * uA1 + den1b, sb1b = num1b * uB1 + den1b;
    const double sa2b = num2b * uA2 + den2b, sb2b = num2b * uB2 + den2b;
    const double uA1b = num1b * sa1, uB1b = num1b * sb1, uA2b = num2b * sa2, uB2b = num2b * sb2;
    Ab.qn1 += uA1b * fA1; Bb.qn1 += uB1b * fB1; Ab.qn2 += uA2b * fA2; Bb.qn2 += uB2b * fB2;
    Ab.h1 += sqrt_bar(sa1, sa1b) + (uA1b * A.qn1) * vfac_d(A.h1, eps) + 0.5 * h1ijb;
    Bb.h1 += sqrt_bar(sb1, sb1b) + (uB1b * B.qn1) * vfac_d(B.h1, eps) + 0.5 * h1ijb;
    Ab.h2 += sqrt_bar(sa2, sa2b) + (uA2b * A.qn2) * vfac_d(A.h2, eps) + 0.5 * h2ijb;
    Bb.h2 += sqrt_bar(sb2, sb2b) + (uB2b * B.qn2) * vfac_d(B.h2, eps) + 0.5 * h2ijb;
}

// ------------------------------------------------------------------ volume

// Bottom-friction factor block of dis_implicita: w[kq], w[kq+1] of a layer of
// depth h (> 0) with old speed un, coefficient gm (g mf^2); returns the
// adjoints into wb (in place), h (hb), un (unb), gm (gmb), dt (dtb).
LSH_HD void bottom_friction_adj(double h, double un, double gm, double dt, double eps, const double win[2],
                                double wbar[2], double& hb, double& unb, double& gmb, double& dtb) {
    const double Y = pow43(h) + kEps, X = (dt * gm) * un;
    const double inv = Y / (Y + X);
    double invb = 0.0;
    if (gt_pos(h, eps)) {
        invb = wbar[0] * win[0] + wbar[1] * win[1];
        wbar[0] = wbar[0] * inv;
        wbar[1] = wbar[1] * inv;
    } else {
        const double f = vfac(h, eps);
        double fb = 0.0;
        for (int k = 0; k < 2; ++k) {
            const double t = h * (f * win[k]);
            invb += wbar[k] * t;
            const double tb = wbar[k] * inv;
            hb += tb * (f * win[k]);
            fb += tb * (h * win[k]);
            wbar[k] = tb * (h * f);
        }
        hb += fb * vfac_d(h, eps);
    }
    const double YX = Y + X;
    const double Yb = invb * (X / (YX * YX));
    const double Xb = -invb * (Y / (YX * YX));
    hb += Yb * pow43_d(h);
    dtb += Xb * (gm * un);
    gmb += Xb * (dt * un);
    unb += Xb * (dt * gm);
}

// Adjoint of volume_update (with the order-2 pressure integral applied to
// `acc` by the caller before the call): given wb = adjoint of the new state,
// adds the adjoints of the old state (wob), of acc[0..5] (accb) and of dt.
// `rateb` is the adjoint of the cell's dt rate output.
LSH_HD void volume_update_adj(const double wo[6], const double acc[7], double inv_area, double tanR, double dt,
                              const Consts& c, const double wbar_in[6], double rateb, double wob[6], double accb[7],
                              double& dtb, ConstBar& cb) {
    const double eps = c.eps_h;
    // ---- forward, saving the state after each sub-step
    double w1[6];
    const double b = dt * inv_area;
    for (int k = 0; k < 6; ++k) w1[k] = fmad(b, acc[k], wo[k]);
    const double fo1 = vfac(wo[0], eps);
    bool sph[2] = {false, false};
    double Fs[2] = {0.0, 0.0}, uxs[2] = {0.0, 0.0}, ss[2] = {0.0, 0.0};
    if (!is_zero(tanR)) {
        for (int layer = 0; layer < 2; ++layer) {
            const int k = 3 * layer;
            if (is_zero(wo[k]) && is_zero(wo[k + 1]) && is_zero(wo[k + 2])) continue;
            sph[layer] = true;
            Fs[layer] = layer ? vfac(wo[k], eps) : fo1;
            uxs[layer] = Fs[layer] * wo[k + 1];
            ss[layer] = dt * (uxs[layer] * tanR);
            w1[k + 1] = fmad(ss[layer], wo[k + 2], w1[k + 1]);
            w1[k + 2] = fmad(-ss[layer], wo[k + 1], w1[k + 2]);
        }
    }
    const bool single = is_zero(wo[3]) && is_zero(wo[4]) && is_zero(wo[5]) && is_zero(w1[3]) && is_zero(w1[4]) &&
                        is_zero(w1[5]);
    const int nl = single ? 1 : 2;
    // filtro: clamp, damping, vmax caps
    double wc[6];
    for (int k = 0; k < 6; ++k) wc[k] = w1[k];
    const bool cl0 = lt0(wc[0]), cl3 = lt0(wc[3]);
    if (cl0) wc[0] = 0.0;
    if (cl3) wc[3] = 0.0;
    double wd[6];
    for (int k = 0; k < 6; ++k) wd[k] = wc[k];
    bool damp[2] = {false, false};
    double dd[2] = {1.0, 1.0}, xx[2] = {0.0, 0.0}, x2s[2] = {0.0, 0.0}, auxs[2] = {1.0, 1.0};
    for (int layer = 0; layer < nl; ++layer) {
        const int k = 3 * layer;
        xx[layer] = wd[k] * c.inv_eps;
        x2s[layer] = xx[layer] * xx[layer];
        dd[layer] = fmad(x2s[layer], x2s[layer], kEps);
        if (lt_pos(dt, dd[layer] * 0x1.fp-55)) continue;  // dd >= EPSILON: the bound is positive
        damp[layer] = true;
        auxs[layer] = exp_neg(dt * (1.0 / dd[layer]));
        wd[k + 1] = wd[k + 1] * auxs[layer];
        wd[k + 2] = wd[k + 2] * auxs[layer];
    }
    double wv[6];
    for (int k = 0; k < 6; ++k) wv[k] = wd[k];
    bool cap[2] = {false, false};
    double vf[2] = {0.0, 0.0}, vux[2] = {0.0, 0.0}, vuy[2] = {0.0, 0.0}, vu[2] = {0.0, 0.0}, vs[2] = {0.0, 0.0};
    for (int layer = 0; layer < 2; ++layer) {
        const double vmax = layer ? c.vmax2 : c.vmax1;
        if (!gt0(vmax)) continue;
        const int k = 3 * layer;
        const double h = wv[k];
        vf[layer] = vfac(h, eps);
        vux[layer] = vf[layer] * wv[k + 1];
        vuy[layer] = vf[layer] * wv[k + 2];
        vu[layer] = sqrt(fmad(vux[layer], vux[layer], vuy[layer] * vuy[layer]));
        if (gt_pos(vu[layer], vmax)) {
            cap[layer] = true;
            vs[layer] = vmax / vu[layer];
            wv[k + 1] = (vux[layer] * vs[layer]) * h;
            wv[k + 2] = (vuy[layer] * vs[layer]) * h;
        }
    }
    // dis_implicita (its clamps are no-ops after filtro's)
    const double h1 = wv[0], h2 = single ? 0.0 : wv[3];
    const double uo1x = fo1 * wo[1], uo1y = fo1 * wo[2];
    const double u1o = sqrt(fmad(uo1x, uo1x, uo1y * uo1y));
    const double fo2 = vfac(wo[3], eps);
    const double uo2x = fo2 * wo[4], uo2y = fo2 * wo[5];
    const double ddx = uo1x - uo2x, ddy = uo1y - uo2y;
    const double du = sqrt(fmad(ddx, ddx, ddy * ddy));
    const double u2o = sqrt(fmad(uo2x, uo2x, uo2y * uo2y));
    const bool blkA = !single && gt0(h1) && gt0(h2);
    const bool blkB = gt0(h1) && lt_pos(h2, eps);
    const bool blkC = !single && gt0(h2) && lt_pos(h1, eps);
    double wa[6];  // after block A
    for (int k = 0; k < 6; ++k) wa[k] = wv[k];
    const double f1 = vfac(h1, eps), f2 = single ? 0.0 : vfac(h2, eps);
    double hmod = 0.0, mm = 0.0, hm2 = 0.0, m2 = 0.0, Sq = 0.0, hh = 0.0, k12 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0,
           P3 = 1.0, e1 = 1.0, e2 = 1.0, det = 1.0, n1x = 0.0, n1y = 0.0, n2x = 0.0, n2y = 0.0;
    double u1x = 0.0, u1y = 0.0, u2x = 0.0, u2y = 0.0;
    if (blkA) {
        u1x = f1 * wv[1]; u1y = f1 * wv[2];
        u2x = f2 * wv[4]; u2y = f2 * wv[5];
        hmod = fmad(c.r, h1, h2);
        mm = gt_pos(hmod, c.eps_1r) ? hmod : c.eps_1r;
        hm2 = hmod * hmod; m2 = mm * mm;
        Sq = sqrt(fmad(hm2, hm2, m2 * m2));
        hh = hmod / Sq;
        k12 = ((dt * kSqrt2) * hh) * (c.mfc * du);
        c1 = k12 * h2;
        c2 = (k12 * c.r) * h1;
        P3 = pow43(h2) + kEps;
        c3 = ((dt * c.g_mfs2) * u2o) / P3;
        e1 = 1.0 + c1; e2 = 1.0 + c2 + c3;
        det = 1.0 / fmad(e1, e2, -(c1 * c2));
        n1x = fmad(u1x, e2, c1 * u2x); n2x = fmad(u2x, e1, c2 * u1x);
        n1y = fmad(u1y, e2, c1 * u2y); n2y = fmad(u2y, e1, c2 * u1y);
        wa[1] = (h1 * n1x) * det;
        wa[4] = (h2 * n2x) * det;
        wa[2] = (h1 * n1y) * det;
        wa[5] = (h2 * n2y) * det;
    }
    double wbk[6];  // after block B
    for (int k = 0; k < 6; ++k) wbk[k] = wa[k];
    if (blkB) {
        const double Y = pow43(h1) + kEps, X = (dt * c.g_mf02) * u1o;
        const double inv = Y / (Y + X);
        if (gt_pos(h1, eps)) { wbk[1] = wa[1] * inv; wbk[2] = wa[2] * inv; }
        else { wbk[1] = (h1 * (f1 * wa[1])) * inv; wbk[2] = (h1 * (f1 * wa[2])) * inv; }
    }
    double wcc[6];  // after block C (= dis_implicita's output)
    for (int k = 0; k < 6; ++k) wcc[k] = wbk[k];
    if (blkC) {
        const double Y = pow43(h2) + kEps, X = (dt * c.g_mfs2) * u2o;
        const double inv = Y / (Y + X);
        if (gt_pos(h2, eps)) { wcc[4] = wbk[4] * inv; wcc[5] = wbk[5] * inv; }
        else { wcc[4] = (h2 * (f2 * wbk[4])) * inv; wcc[5] = (h2 * (f2 * wbk[5])) * inv; }
    }

    // ---- reverse
    double g[6];
    for (int k = 0; k < 6; ++k) g[k] = wbar_in[k];
    // coulomb (or, single layer, q2 * 0)
    if (single || !gt0(wcc[3])) {
        g[4] = 0.0;
        g[5] = 0.0;
    } else {
        const double hc1 = wcc[0], hc2 = wcc[3];
        const double a = (10.0 * hc1) * c.inv_eps;
        const double ex = exp_neg(a * a);
        const double fsc = 1.0 - c.r * (1.0 - ex);
        const double sc = (((fsc * c.mu) * c.g) * hc2) * dt;
        const double nq = sqrt(fmad(wcc[4], wcc[4], wcc[5] * wcc[5]));
        const bool act = !lt_pos(nq + sc, kEps) && !lt(nq, sc);
        const double aux = act ? nq / (nq + sc) : 0.0;
        const double auxb = g[4] * wcc[4] + g[5] * wcc[5];
        g[4] = g[4] * aux;
        g[5] = g[5] * aux;
        if (act) {
            const double s2 = (nq + sc) * (nq + sc);
            const double nqb = auxb * (sc / s2);
            const double scb = -auxb * (nq / s2);
            if (gt0(nq)) { g[4] += nqb * (wcc[4] / nq); g[5] += nqb * (wcc[5] / nq); }
            const double fscb = scb * (((c.mu * c.g) * hc2) * dt);
            cb.mu += scb * (((fsc * c.g) * hc2) * dt);
            g[3] += scb * (((fsc * c.mu) * c.g) * dt);
            dtb += scb * (((fsc * c.mu) * c.g) * hc2);
            cb.r += fscb * (-(1.0 - ex));
            const double exb = fscb * c.r;
            const double ab = (exb * (-ex)) * (2.0 * a);
            g[0] += ab * (10.0 * c.inv_eps);
        }
    }
    // dis_implicita, blocks C, B, A in reverse
    double h1b = 0.0, h2b = 0.0, u1ob = 0.0, u2ob = 0.0;
    if (blkC) {
        double wbar2[2] = {g[4], g[5]};
        const double win[2] = {wbk[4], wbk[5]};
        bottom_friction_adj(h2, u2o, c.g_mfs2, dt, eps, win, wbar2, h2b, u2ob, cb.g_mfs2, dtb);
        g[4] = wbar2[0]; g[5] = wbar2[1];
    }
    if (blkB) {
        double wbar1[2] = {g[1], g[2]};
        const double win[2] = {wa[1], wa[2]};
        bottom_friction_adj(h1, u1o, c.g_mf02, dt, eps, win, wbar1, h1b, u1ob, cb.g_mf02, dtb);
        g[1] = wbar1[0]; g[2] = wbar1[1];
    }
    double uo1xb = 0.0, uo1yb = 0.0, uo2xb = 0.0, uo2yb = 0.0;
    if (blkA) {
        const double o1x = g[1], o1y = g[2], o2x = g[4], o2y = g[5];
        const double detb = (o1x * (h1 * n1x) + o2x * (h2 * n2x)) + (o1y * (h1 * n1y) + o2y * (h2 * n2y));
        const double n1xb = o1x * (h1 * det), n2xb = o2x * (h2 * det);
        const double n1yb = o1y * (h1 * det), n2yb = o2y * (h2 * det);
        h1b += (o1x * n1x + o1y * n1y) * det;
        h2b += (o2x * n2x + o2y * n2y) * det;
        double u1xb = n1xb * e2 + n2xb * c2, u1yb = n1yb * e2 + n2yb * c2;
        double u2xb = n1xb * c1 + n2xb * e1, u2yb = n1yb * c1 + n2yb * e1;
        double e1b = n2xb * u2x + n2yb * u2y;
        double e2b = n1xb * u1x + n1yb * u1y;
        double c1b = n1xb * u2x + n1yb * u2y;
        double c2b = n2xb * u1x + n2yb * u1y;
        const double den = fmad(e1, e2, -(c1 * c2));
        (void)den;
        const double denb = -detb * (det * det);
        e1b += denb * e2; e2b += denb * e1;
        c1b -= denb * c2; c2b -= denb * c1;
        c1b += e1b;
        c2b += e2b;
        const double c3b = e2b;
        const double nn = (dt * c.g_mfs2) * u2o;
        const double nnb = c3b / P3;
        const double P3b = -c3b * (c3 / P3);
        dtb += nnb * (c.g_mfs2 * u2o);
        cb.g_mfs2 += nnb * (dt * u2o);
        u2ob += nnb * (dt * c.g_mfs2);
        (void)nn;
        h2b += P3b * pow43_d(h2);
        double k12b = c2b * (c.r * h1) + c1b * h2;
        cb.r += c2b * (k12 * h1);
        h1b += c2b * (k12 * c.r);
        h2b += c1b * k12;
        dtb += k12b * ((kSqrt2 * hh) * (c.mfc * du));
        const double hhb = k12b * ((dt * kSqrt2) * (c.mfc * du));
        const double dub = k12b * ((dt * kSqrt2) * hh) * c.mfc;
        double hmodb = hhb / Sq;
        const double Sqb = -hhb * (hh / Sq);
        const double Qb = sqrt_bar(Sq, Sqb);
        const double hm2b = Qb * (2.0 * hm2), m2b = Qb * (2.0 * m2);
        hmodb += hm2b * (2.0 * hmod);
        const double mb = m2b * (2.0 * mm);
        if (gt_pos(hmod, c.eps_1r)) hmodb += mb;
        else cb.eps_1r += mb;
        cb.r += hmodb * h1;
        h1b += hmodb * c.r;
        h2b += hmodb;
        if (gt0(du)) {
            const double dxb = dub * (ddx / du), dyb = dub * (ddy / du);
            uo1xb += dxb; uo2xb -= dxb;
            uo1yb += dyb; uo2yb -= dyb;
        }
        // u1 = f1 w, u2 = f2 w (pre-block values)
        const double f1b = u1xb * wv[1] + u1yb * wv[2];
        const double f2b = u2xb * wv[4] + u2yb * wv[5];
        g[1] = u1xb * f1; g[2] = u1yb * f1;
        g[4] = u2xb * f2; g[5] = u2yb * f2;
        h1b += f1b * vfac_d(h1, eps);
        h2b += f2b * vfac_d(h2, eps);
    }
    // old speeds
    if (gt0(u1o)) { uo1xb += u1ob * (uo1x / u1o); uo1yb += u1ob * (uo1y / u1o); }
    if (!single && gt0(u2o)) { uo2xb += u2ob * (uo2x / u2o); uo2yb += u2ob * (uo2y / u2o); }
    const double fo1b = uo1xb * wo[1] + uo1yb * wo[2];
    wob[1] += uo1xb * fo1;
    wob[2] += uo1yb * fo1;
    wob[0] += fo1b * vfac_d(wo[0], eps);
    if (!single) {
        const double fo2b = uo2xb * wo[4] + uo2yb * wo[5];
        wob[4] += uo2xb * fo2;
        wob[5] += uo2yb * fo2;
        wob[3] += fo2b * vfac_d(wo[3], eps);
    }
    g[0] += h1b;
    if (!single) g[3] += h2b;
    // vmax caps
    for (int layer = 1; layer >= 0; --layer) {
        if (!cap[layer]) continue;
        const int k = 3 * layer;
        const double h = wd[k];
        const double oxb = g[k + 1], oyb = g[k + 2];
        double uxb = oxb * (vs[layer] * h), uyb = oyb * (vs[layer] * h);
        const double sb = oxb * (vux[layer] * h) + oyb * (vuy[layer] * h);
        double hb = oxb * (vux[layer] * vs[layer]) + oyb * (vuy[layer] * vs[layer]);
        const double vmax = layer ? c.vmax2 : c.vmax1;
        const double ub = -sb * (vmax / (vu[layer] * vu[layer]));
        if (gt0(vu[layer])) { uxb += ub * (vux[layer] / vu[layer]); uyb += ub * (vuy[layer] / vu[layer]); }
        const double fb = uxb * wd[k + 1] + uyb * wd[k + 2];
        g[k + 1] = uxb * vf[layer];
        g[k + 2] = uyb * vf[layer];
        hb += fb * vfac_d(h, eps);
        g[k] += hb;
    }
    // damping
    for (int layer = nl - 1; layer >= 0; --layer) {
        if (!damp[layer]) continue;
        const int k = 3 * layer;
        const double auxb = g[k + 1] * wc[k + 1] + g[k + 2] * wc[k + 2];
        g[k + 1] = g[k + 1] * auxs[layer];
        g[k + 2] = g[k + 2] * auxs[layer];
        const double invd = 1.0 / dd[layer];
        const double zb = -auxb * auxs[layer];
        dtb += zb * invd;
        const double db = -(zb * dt) * (invd * invd);
        const double x2b = db * (2.0 * x2s[layer]);
        const double xb = x2b * (2.0 * xx[layer]);
        g[k] += xb * c.inv_eps;
    }
    if (single) { g[4] = 0.0; g[5] = 0.0; }
    // clamps
    if (cl0) g[0] = 0.0;
    if (cl3) g[3] = 0.0;
    // spherical metric source
    for (int layer = 1; layer >= 0; --layer) {
        if (!sph[layer]) continue;
        const int k = 3 * layer;
        const double sb = g[k + 1] * wo[k + 2] - g[k + 2] * wo[k + 1];
        wob[k + 2] += g[k + 1] * ss[layer];
        wob[k + 1] -= g[k + 2] * ss[layer];
        dtb += sb * (uxs[layer] * tanR);
        const double uxb = sb * (dt * tanR);
        const double Fb = uxb * wo[k + 1];
        wob[k + 1] += uxb * Fs[layer];
        wob[k] += Fb * vfac_d(wo[k], eps);
    }
    // Euler stage
    double bb = 0.0;
    for (int k = 0; k < 6; ++k) {
        wob[k] += g[k];
        accb[k] += g[k] * b;
        bb += g[k] * acc[k];
    }
    dtb += bb * inv_area;
    // rate = acc_w / area (0 below EPSILON)
    if (!lt_pos(acc[6], kEps)) accb[6] += rateb * inv_area;
}

}  // namespace lsh

// ------------------------------------------------------------------ per-edge / per-cell bodies
// The same gathers and scatters as lsh_passes.cuh's forward bodies, run in
// reverse.  One thread owns one edge (cells of one colour pass are
// disjoint, so the read-modify-writes of the adjoint arrays do not race) or
// one cell.

namespace lsh {

struct AdjArgs {
    Consts c;
    Geo geo;
    const double* W[7];     // the stage's input state
    const double* sx[7];    // its slopes (order 2)
    const double* sy[7];
    const double* acc[7];   // the stage's final accumulators (before the order-2 pressure integral)
    const double* snap[2];  // acc[0], acc[3] before this edge pass (nullptr: first pass, zeros)
    double* Wbar[6];        // adjoint of the stage input (accumulated)
    double* sxb[7];         // adjoint of the slopes (order 2; [6] unused)
    double* syb[7];
    double* accb[7];        // adjoint of the accumulators
    const double* wbar[6];  // volume: adjoint of the stage output
    double* Xbar[6];        // volume MODE 2: adjoint of the step's initial state (+= wbar / 2)
    const unsigned* tape;   // reconstruction branch tape (order 2)
    long long rate_cell;    // cell holding the largest dt rate (-1: none)
    double rate_bar;        // adjoint of that rate
    double dt;
};

// Face-value adjoint to cell-state and slope adjoints (the reverse of
// face_depths + face_rest): fb is in the edge frame.
template <int DIR, int ORDER>
LSH_HD void face_scatter(const AdjArgs& a, int id, int side, bool pos_normal, const FaceBar& fb) {
    // back to x / y components (face_rest's selections reversed)
    double qx1b, qy1b, qx2b, qy2b;
    if (DIR == 1) {
        qx1b = lshm::neg_if(fb.qn1, !pos_normal); qy1b = lshm::neg_if(fb.qt1, !pos_normal);
        qx2b = lshm::neg_if(fb.qn2, !pos_normal); qy2b = lshm::neg_if(fb.qt2, !pos_normal);
    } else {
        // qn = sg qy, qt = -sg qx
        qy1b = lshm::neg_if(fb.qn1, !pos_normal); qx1b = lshm::neg_if(fb.qt1, pos_normal);
        qy2b = lshm::neg_if(fb.qn2, !pos_normal); qx2b = lshm::neg_if(fb.qt2, pos_normal);
    }
    a.Wbar[0][id] += fb.h1;
    a.Wbar[1][id] += qx1b;
    a.Wbar[2][id] += qy1b;
    a.Wbar[3][id] += fb.h2;
    a.Wbar[4][id] += qx2b;
    a.Wbar[5][id] += qy2b;
    if (ORDER == 2) {
        double* const* s = (side < 2) ? a.sxb : a.syb;
        // h1 = W0 + sg (s0 - s3), h2 = W3 + sg (s3 + s6), q = W + sg s, sg = +-1:
        // the products by sg are sign-bit flips
        const bool neg = !(side & 1);
        using lshm::neg_if;
        s[0][id] += neg_if(fb.h1, neg);
        s[3][id] += neg_if(fb.h2 - fb.h1, neg);
        s[1][id] += neg_if(qx1b, neg);
        s[2][id] += neg_if(qy1b, neg);
        s[4][id] += neg_if(qx2b, neg);
        s[5][id] += neg_if(qy2b, neg);
    }
}

// Adjoint of do_edge<DIR, FIRST, ORDER> for the edge at (x, y).
template <int DIR, bool FIRST, int ORDER>
LSH_HD void edge_adj_body(const AdjArgs& a, int x, int y, double& dtb, ConstBar& cb) {
    const int nx = a.c.nx, ny = a.c.ny;
    EdgeIn e;
    int id0, id1 = -1, side0, row0, row1 = 0;
    double bor = 0.0;
    bool pos_normal = true;
    if (DIR == 0) {
        e.len = a.geo.len_h[y];
        if (y == 0) { id0 = x; row0 = 0; pos_normal = false; bor = a.c.borde_sup; side0 = 2; }
        else if (y == ny) { id0 = (ny - 1) * nx + x; row0 = ny - 1; bor = a.c.borde_inf; side0 = 3; }
        else { id0 = (y - 1) * nx + x; id1 = id0 + nx; row0 = y - 1; row1 = y; side0 = 3; }
    } else {
        e.len = a.geo.len_v[y];
        row0 = row1 = y;
        if (x == 0) { id0 = y * nx; pos_normal = false; bor = a.c.borde_izq; side0 = 0; }
        else if (x == nx) { id0 = y * nx + nx - 1; bor = a.c.borde_der; side0 = 1; }
        else { id0 = y * nx + x - 1; id1 = id0 + 1; side0 = 1; }
    }
    e.interior = (id1 >= 0);
    // the adjoint is linear in the output adjoints: none, nothing to do
    {
        bool zero = true;
        for (int k = 0; k < 7; ++k) zero = zero && is_zero(a.accb[k][id0]);
        if (e.interior)
            for (int k = 0; k < 7; ++k) zero = zero && is_zero(a.accb[k][id1]);
        if (zero) return;
    }
    const int side1 = (DIR == 0) ? 2 : 0;
    // the forward's face construction (same helpers, host or device)
    KArgs f;
    f.c = a.c;
    for (int k = 0; k < 7; ++k) { f.W[k] = a.W[k]; f.sx[k] = a.sx[k]; f.sy[k] = a.sy[k]; }
    face_depths<ORDER>(f, id0, side0, e.A.h1, e.A.h2);
    if (e.interior) face_depths<ORDER>(f, id1, side1, e.B.h1, e.B.h2);
    else { e.B.h1 = e.A.h1; e.B.h2 = e.A.h2; }
    if (lt_pos(0.5 * (e.A.h1 + e.B.h1), kEps) && lt_pos(0.5 * (e.A.h2 + e.B.h2), kEps)) return;  // dry edge
    face_rest<DIR, ORDER>(f, id0, side0, pos_normal, e.A);
    e.area0 = a.geo.area[row0];
    e.inv_area0 = a.geo.inv_area[row0];
    e.hc0[0] = a.W[0][id0];
    e.hc0[1] = a.W[3][id0];
    if (FIRST || !a.snap[0]) { e.acc0h[0] = 0.0; e.acc0h[1] = 0.0; }
    else { e.acc0h[0] = a.snap[0][id0]; e.acc0h[1] = a.snap[1][id0]; }
    if (e.interior) {
        face_rest<DIR, ORDER>(f, id1, side1, pos_normal, e.B);
        e.area1 = a.geo.area[row1];
        e.inv_area1 = a.geo.inv_area[row1];
        e.hc1[0] = a.W[0][id1];
        e.hc1[1] = a.W[3][id1];
        if (FIRST || !a.snap[0]) { e.acc1h[0] = 0.0; e.acc1h[1] = 0.0; }
        else { e.acc1h[0] = a.snap[0][id1]; e.acc1h[1] = a.snap[1][id1]; }
    } else {
        e.B = e.A;
        e.B.qn1 = e.A.qn1 * bor;
        e.B.qn2 = e.A.qn2 * bor;
        e.area1 = e.area0;
        e.inv_area1 = e.inv_area0;
        e.hc1[0] = e.hc1[1] = 0.0;
        e.acc1h[0] = e.acc1h[1] = 0.0;
    }
    // output adjoints: acc[k][id0] -= d0[k], acc[k][id1] -= d1[k], acc[6] += wave
    EdgeOut ob;
    for (int l = 0; l < 2; ++l) {
        const int k = 3 * l;
        // negations as sign-bit flips (integer pipe; the bits of -x)
        using lshm::neg_if;
        const double g0[3] = {neg_if(a.accb[k][id0], true), neg_if(a.accb[k + 1][id0], true),
                              neg_if(a.accb[k + 2][id0], true)};
        double g1[3] = {0.0, 0.0, 0.0};
        if (e.interior) {
            g1[0] = neg_if(a.accb[k][id1], true);
            g1[1] = neg_if(a.accb[k + 1][id1], true);
            g1[2] = neg_if(a.accb[k + 2][id1], true);
        }
        ob.m[k] = g0[0];
        ob.p[k] = g1[0];
        if (DIR == 1) {
            // d[k+1] = sg m[k+1], d[k+2] = sg m[k+2]
            ob.m[k + 1] = neg_if(g0[1], !pos_normal);
            ob.m[k + 2] = neg_if(g0[2], !pos_normal);
            ob.p[k + 1] = neg_if(g1[1], !pos_normal);
            ob.p[k + 2] = neg_if(g1[2], !pos_normal);
        } else {
            // d[k+1] = -sg m[k+2], d[k+2] = sg m[k+1]
            ob.m[k + 1] = neg_if(g0[2], !pos_normal);
            ob.m[k + 2] = neg_if(g0[1], pos_normal);
            ob.p[k + 1] = neg_if(g1[2], !pos_normal);
            ob.p[k + 2] = neg_if(g1[1], pos_normal);
        }
    }
    ob.wave = 0.0;
    if (a.rate_cell >= 0) {
        if (id0 == a.rate_cell) ob.wave += a.accb[6][id0];
        if (e.interior && id1 == a.rate_cell) ob.wave += a.accb[6][id1];
    }
    EdgeInBar eb;
    edge_bar_zero(eb);
    if (is_zero(e.A.h2) && is_zero(e.B.h2) && is_zero(e.A.qn2) && is_zero(e.B.qn2))
        edge_flux_adj<false>(e, a.dt, a.c, ob, eb, dtb, cb);
    else
        edge_flux_adj<true>(e, a.dt, a.c, ob, eb, dtb, cb);
    if (!e.interior) {
        // the ghost is built from face A
        eb.A.h1 += eb.B.h1; eb.A.qt1 += eb.B.qt1; eb.A.qn1 += bor * eb.B.qn1;
        eb.A.h2 += eb.B.h2; eb.A.qt2 += eb.B.qt2; eb.A.qn2 += bor * eb.B.qn2;
    }
    face_scatter<DIR, ORDER>(a, id0, side0, pos_normal, eb.A);
    a.Wbar[0][id0] += eb.hc0[0];
    a.Wbar[3][id0] += eb.hc0[1];
    if (!FIRST && a.snap[0]) { a.accb[0][id0] += eb.acc0h[0]; a.accb[3][id0] += eb.acc0h[1]; }
    if (e.interior) {
        face_scatter<DIR, ORDER>(a, id1, side1, pos_normal, eb.B);
        a.Wbar[0][id1] += eb.hc1[0];
        a.Wbar[3][id1] += eb.hc1[1];
        if (!FIRST && a.snap[0]) { a.accb[0][id1] += eb.acc1h[0]; a.accb[3][id1] += eb.acc1h[1]; }
    }
}

// Adjoint of volume_cell<MODE> for cell id.  MODE 0 / 1: Wbar (the stage
// input's adjoint) gets the old state's part; MODE 2 also passes wbar / 2 to
// Xbar (the average with the step's initial state).  Writes accb[0..6] of the
// cell and, at order 2, the pressure integral's slope adjoints.
template <int MODE>
LSH_HD void volume_adj_body(const AdjArgs& a, int id, double& dtb, ConstBar& cb) {
    const int nx = a.c.nx;
    const int j = id / nx;
    double wo[6], acc[7], wbar[6];
    for (int k = 0; k < 6; ++k) wbar[k] = a.wbar[k][id];
    bool any = (a.rate_cell == (long long)id);
    for (int k = 0; k < 6; ++k) any |= !is_zero(wbar[k]);
    if (!any) {
        // a zero adjoint (every dry cell under the thin-layer projection):
        // zero accumulator and slope adjoints, nothing to add upstream
        if (a.c.order == 2)
            for (int k = 0; k < 7; ++k) { a.sxb[k][id] = 0.0; a.syb[k][id] = 0.0; }
        for (int k = 0; k < 7; ++k) a.accb[k][id] = 0.0;
        return;
    }
    for (int k = 0; k < 6; ++k) wo[k] = a.W[k][id];
    for (int k = 0; k < 7; ++k) acc[k] = a.acc[k][id];
    if (MODE == 2) {
        for (int k = 0; k < 6; ++k) {
            a.Xbar[k][id] += 0.5 * wbar[k];
            wbar[k] = 0.5 * wbar[k];
        }
    }
    double e1x = 0.0, e2x = 0.0, e1y = 0.0, e2y = 0.0, gh1 = 0.0, gh2 = 0.0, wx = 0.0, wy = 0.0;
    if (a.c.order == 2) {
        gh1 = a.c.g * wo[0]; gh2 = a.c.g * wo[3];
        e1x = 2.0 * a.sx[0][id]; e2x = 2.0 * a.sx[3][id];
        e1y = 2.0 * a.sy[0][id]; e2y = 2.0 * a.sy[3][id];
        wx = a.geo.wx[j]; wy = a.geo.wy[j];
        acc[1] -= a.c.peso * ((gh1 * e1x) * wx);
        acc[4] -= a.c.peso * ((gh2 * fmad(a.c.omr, e2x, a.c.r * e1x)) * wx);
        acc[2] -= a.c.peso * ((gh1 * e1y) * wy);
        acc[5] -= a.c.peso * ((gh2 * fmad(a.c.omr, e2y, a.c.r * e1y)) * wy);
    }
    double wob[6] = {0, 0, 0, 0, 0, 0}, accb[7] = {0, 0, 0, 0, 0, 0, 0};
    if (any) {
        const double rateb = (a.rate_cell == (long long)id && MODE != 2) ? a.rate_bar : 0.0;
        volume_update_adj(wo, acc, a.geo.inv_area[j], a.geo.tanR[j], a.dt, a.c, wbar, rateb, wob, accb, dtb, cb);
    }
    if (a.c.order == 2 && any) {
        // acc[1] -= peso gh1 e1x wx, acc[4] -= peso gh2 (omr e2x + r e1x) wx (y likewise)
        const double p = a.c.peso;
        const double b1 = -p * accb[1] * wx, b4 = -p * accb[4] * wx;
        const double b2 = -p * accb[2] * wy, b5 = -p * accb[5] * wy;
        const double sxw = fmad(a.c.omr, e2x, a.c.r * e1x), syw = fmad(a.c.omr, e2y, a.c.r * e1y);
        const double gh1b = b1 * e1x + b2 * e1y;
        const double gh2b = b4 * sxw + b5 * syw;
        const double e1xb = b1 * gh1 + b4 * gh2 * a.c.r, e2xb = b4 * gh2 * a.c.omr;
        const double e1yb = b2 * gh1 + b5 * gh2 * a.c.r, e2yb = b5 * gh2 * a.c.omr;
        cb.omr += b4 * gh2 * e2x + b5 * gh2 * e2y;
        cb.r += b4 * gh2 * e1x + b5 * gh2 * e1y;
        wob[0] += gh1b * a.c.g;
        wob[3] += gh2b * a.c.g;
        a.sxb[0][id] = 2.0 * e1xb;
        a.sxb[3][id] = 2.0 * e2xb;
        a.syb[0][id] = 2.0 * e1yb;
        a.syb[3][id] = 2.0 * e2yb;
    } else if (a.c.order == 2) {
        a.sxb[0][id] = 0.0; a.sxb[3][id] = 0.0; a.syb[0][id] = 0.0; a.syb[3][id] = 0.0;
    }
    if (a.c.order == 2) {
        for (int k : {1, 2, 4, 5, 6}) { a.sxb[k][id] = 0.0; a.syb[k][id] = 0.0; }
    }
    for (int k = 0; k < 6; ++k) a.Wbar[k][id] += wob[k];
    for (int k = 0; k < 7; ++k) a.accb[k][id] = accb[k];
}

// Branch tape of one cell's reconstruction (recon_cell): for variable k and
// direction d (0 x, 1 y) bits 2 (7 d + k) .. +1 hold the minmod choice (0
// zero, 1 the backward difference, 2 the forward one); bit 28: slopes zeroed
// (a reconstructed depth below kReconThin of the cell's, or the dry shortcut).
// Without bit 28, sx and sy hold the cell's slopes (recon_cell's values).
LSH_HD unsigned recon_tape_slopes(const double* const* W, int nx, int ny, int id, double sx[7], double sy[7]) {
    const int j = id / nx, i = id - j * nx;
    {
        bool dry = is_zero(W[0][id]) && is_zero(W[3][id]);
        if (dry && i > 0) dry = is_zero(W[0][id - 1]) && is_zero(W[3][id - 1]);
        if (dry && i < nx - 1) dry = is_zero(W[0][id + 1]) && is_zero(W[3][id + 1]);
        if (dry && j > 0) dry = is_zero(W[0][id - nx]) && is_zero(W[3][id - nx]);
        if (dry && j < ny - 1) dry = is_zero(W[0][id + nx]) && is_zero(W[3][id + nx]);
        if (dry) return 1u << 28;
    }
    auto rv = [&](int q, int k) -> double {
        if (k == 0) return (W[0][q] + W[3][q]) - W[6][q];
        if (k == 3) return W[3][q] - W[6][q];
        return W[k][q];
    };
    // minmod's choice (0: neither, 1: a, 2: b), on the bit patterns like minmod
    auto choice = [](double a, double b, double& v) -> unsigned {
        const uint64_t ua = lshm::bits_of(a), ub = lshm::bits_of(b);
        if (((ua << 1) != 0) && ((ub << 1) != 0) && ((ua ^ ub) >> 63) == 0) {
            if ((ua & lshm::kMag) < (ub & lshm::kMag)) { v = a; return 1u; }
            v = b;
            return 2u;
        }
        v = 0.0;
        return 0u;
    };
    unsigned t = 0;
    for (int k = 0; k < 7; ++k) {
        const double pc = rv(id, k);
        double v = 0.0;
        sx[k] = 0.0;
        sy[k] = 0.0;
        if (i > 0 && i < nx - 1) { t |= choice(pc - rv(id - 1, k), rv(id + 1, k) - pc, v) << (2 * k); sx[k] = 0.5 * v; }
        if (j > 0 && j < ny - 1) { t |= choice(pc - rv(id - nx, k), rv(id + nx, k) - pc, v) << (2 * (7 + k)); sy[k] = 0.5 * v; }
    }
    const double h1 = W[0][id], h2 = W[3][id];
    const double dh1x = sx[0] - sx[3], dh2x = sx[3] + sx[6];
    const double dh1y = sy[0] - sy[3], dh2y = sy[3] + sy[6];
    const double g1 = kReconThin * h1, g2 = kReconThin * h2;
    const int64_t k1 = okey(g1), k2 = okey(g2);
    const bool bad = okey(h1 + dh1x) < k1 || okey(h1 - dh1x) < k1 || okey(h2 + dh2x) < k2 || okey(h2 - dh2x) < k2 ||
                     okey(h1 + dh1y) < k1 || okey(h1 - dh1y) < k1 || okey(h2 + dh2y) < k2 || okey(h2 - dh2y) < k2;
    if (bad) return 1u << 28;
    return t;
}

LSH_HD unsigned recon_tape_cell(const double* const* W, int nx, int ny, int id) {
    double sx[7], sy[7];
    return recon_tape_slopes(W, nx, ny, id, sx, sy);
}

// The reconstruction of recon_cell (lsh_passes.cuh) writing its slopes and
// returning the branch tape of recon_tape_cell in one pass: the slopes are
// the halved minmod choices, the operations recon_cell performs, so they are
// bit-identical to recon_cell's.
LSH_HD unsigned recon_cell_tape(const KArgs& a, int id) {
    double sx[7], sy[7];
    const unsigned t = recon_tape_slopes(a.W, a.c.nx, a.c.ny, id, sx, sy);
    if (t & (1u << 28)) {
        // zero slopes; with slope-zero flags (as recon_cell keeps them) a cell
        // whose stored slopes are already zero skips the stores
        if (a.szero && a.szero[id]) return t;
        for (int k = 0; k < 7; ++k) { a.sxw[k][id] = 0.0; a.syw[k][id] = 0.0; }
        if (a.szero) a.szero[id] = 1;
        return t;
    }
    if (a.szero) a.szero[id] = 0;
    for (int k = 0; k < 7; ++k) {
        a.sxw[k][id] = sx[k];
        a.syw[k][id] = sy[k];
    }
    return t;
}

// Reconstruction adjoint, gathered at cell id: Wbar[id] += sum over the
// slopes that read cell id of d(slope)/d(W[id]) * slope adjoint.
LSH_HD void recon_adj_cell(const AdjArgs& a, int id) {
    const int nx = a.c.nx, ny = a.c.ny;
    const int j = id / nx, i = id - j * nx;
    double vb[7] = {0, 0, 0, 0, 0, 0, 0};
    // neighbours q whose slope in direction d reads id: (q, d, role) with role
    // 0: id is q itself, 1: id is q's backward neighbour, 2: q's forward one
    const int nq[5] = {id, id + 1, id - 1, id + nx, id - nx};
    const int nd[5] = {-1, 0, 0, 1, 1};
    const bool ok[5] = {true, i < nx - 1, i > 0, j < ny - 1, j > 0};
    // A warp none of whose cells is read by a slope with a nonzero adjoint
    // skips the sums below (integer tests only): the per-slope updates are
    // if-converted, so without the vote every warp would issue them.  In a
    // warp that runs them, a cell without such a slope adds zeros to +0 and
    // leaves below like a skipped one.
    bool need = false;
    for (int m = 0; m < 5; ++m) {
        if (!ok[m]) continue;
        const int q = nq[m];
        const unsigned t = a.tape[q];
        if (t & (1u << 28)) continue;
        for (int d = 0; d < 2; ++d) {
            if (m > 0 && nd[m] != d) continue;
            const double* const* sb = d ? a.syb : a.sxb;
            for (int k = 0; k < 6; ++k)
                if ((t >> (2 * (7 * d + k))) & 3u) need |= !is_zero(sb[k][q]);
        }
    }
    if (!warp_any(need)) return;
    for (int m = 0; m < 5; ++m) {
        if (!ok[m]) continue;
        const int q = nq[m];
        const unsigned t = a.tape[q];
        if (t & (1u << 28)) continue;
        for (int d = 0; d < 2; ++d) {
            if (m > 0 && nd[m] != d) continue;
            const double* const* sb = d ? a.syb : a.sxb;
            for (int k = 0; k < 6; ++k) {
                if (k == 6) continue;
                const unsigned ch = (t >> (2 * (7 * d + k))) & 3u;
                if (ch == 0u) continue;
                const double g = 0.5 * sb[k][q];
                if (m == 0) vb[k] += lshm::neg_if(g, ch != 1u);    // a = pc - back, b = fwd - pc
                else if (m == 1 || m == 3) { if (ch == 1u) vb[k] -= g; }  // id is q's backward neighbour
                else { if (ch == 2u) vb[k] += g; }                 // id is q's forward neighbour
            }
        }
    }
    // recon variables: eta1 = h1 + h2 - H, eta2 = h2 - H, the discharges
    // (no slope read by this cell carries an adjoint: nothing to add)
    bool any = false;
    for (int k = 0; k < 6; ++k) any |= !is_zero(vb[k]);
    if (!any) return;
    a.Wbar[0][id] += vb[0];
    a.Wbar[3][id] += vb[0] + vb[3];
    a.Wbar[1][id] += vb[1];
    a.Wbar[2][id] += vb[2];
    a.Wbar[4][id] += vb[4];
    a.Wbar[5][id] += vb[5];
}

// Adjoint of the initial-dt pass through the cell holding the largest rate:
// its (up to) four edges' wave terms, first-order faces.
LSH_HD void init_wave_adj_cell(const AdjArgs& a, int cell, double accwb, ConstBar& cb) {
    const int nx = a.c.nx, ny = a.c.ny;
    const int j = cell / nx, i = cell - j * nx;
    KArgs f;
    f.c = a.c;
    for (int k = 0; k < 7; ++k) { f.W[k] = a.W[k]; f.sx[k] = a.sx[k]; f.sy[k] = a.sy[k]; }
    for (int which = 0; which < 4; ++which) {
        const int DIRv = (which < 2) ? 0 : 1;  // 0, 1: horizontal edges y = j, j + 1; 2, 3: vertical x = i, i + 1
        const int x = (DIRv == 0) ? i : i + (which - 2);
        const int y = (DIRv == 0) ? j + which : j;
        int id0, id1 = -1;
        double bor = 0.0, len;
        bool pos_normal = true;
        if (DIRv == 0) {
            len = a.geo.len_h[y];
            if (y == 0) { id0 = x; pos_normal = false; bor = a.c.borde_sup; }
            else if (y == ny) { id0 = (ny - 1) * nx + x; bor = a.c.borde_inf; }
            else { id0 = (y - 1) * nx + x; id1 = id0 + nx; }
        } else {
            len = a.geo.len_v[y];
            if (x == 0) { id0 = y * nx; pos_normal = false; bor = a.c.borde_izq; }
            else if (x == nx) { id0 = y * nx + nx - 1; bor = a.c.borde_der; }
            else { id0 = y * nx + x - 1; id1 = id0 + 1; }
        }
        Face A, B;
        A.h1 = a.W[0][id0];
        A.h2 = a.W[3][id0];
        if (DIRv == 0) face_rest<0, 1>(f, id0, 0, pos_normal, A);
        else face_rest<1, 1>(f, id0, 0, pos_normal, A);
        if (id1 >= 0) {
            B.h1 = a.W[0][id1];
            B.h2 = a.W[3][id1];
            if (DIRv == 0) face_rest<0, 1>(f, id1, 0, pos_normal, B);
            else face_rest<1, 1>(f, id1, 0, pos_normal, B);
        } else {
            B = A;
            B.qn1 = A.qn1 * bor;
            B.qn2 = A.qn2 * bor;
        }
        FaceBar Ab, Bb;
        face_bar_zero(Ab);
        face_bar_zero(Bb);
        edge_initial_wave_adj(A, B, len, a.c, accwb, Ab, Bb, cb);
        if (id1 < 0) {
            Ab.h1 += Bb.h1; Ab.qt1 += Bb.qt1; Ab.qn1 += bor * Bb.qn1;
            Ab.h2 += Bb.h2; Ab.qt2 += Bb.qt2; Ab.qn2 += bor * Bb.qn2;
        }
        if (DIRv == 0) {
            face_scatter<0, 1>(a, id0, 0, pos_normal, Ab);
            if (id1 >= 0) face_scatter<0, 1>(a, id1, 0, pos_normal, Bb);
        } else {
            face_scatter<1, 1>(a, id0, 0, pos_normal, Ab);
            if (id1 >= 0) face_scatter<1, 1>(a, id1, 0, pos_normal, Bb);
        }
    }
}

}  // namespace lsh

namespace lsh {

// Parameter gradients from the constant adjoints: d/d(angle1, mf0, mfs, r)
// through mu = |tan angle1| L/H, g mf0^2, g mfs^2 and r's derived constants.
LSH_HD void param_grads(double angle1, double mf0, double mfs, double r, double g, double eps_h, double L,
                        double H, const ConstBar& cb, double out[4]) {
    const double t = tan(angle1);
    out[0] = cb.mu * ((t < 0.0 ? -1.0 : 1.0) * (L / H)) * (1.0 + t * t);
    out[1] = cb.g_mf02 * (2.0 * g * mf0);
    out[2] = cb.g_mfs2 * (2.0 * g * mfs);
    const double gp = g * (1.0 - r);
    out[3] = cb.r - cb.omr - g * cb.gp + cb.inv_gp * (g / (gp * gp)) + eps_h * cb.eps_1r;
}

}  // namespace lsh
