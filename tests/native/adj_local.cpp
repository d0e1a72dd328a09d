// TEST INFRASTRUCTURE: checks of the hand-written local adjoints
// (landslidehysea_gb300/csrc/lsh_adjoint.cuh) against central finite
// differences of the forward operators they reverse (lsh_scheme.cuh), both
// compiled for the host.  For random inputs x, output weights ybar and
// input directions v:  <ybar, (f(x + h v) - f(x - h v)) / 2h>  vs  <xbar, v>.
#include <cmath>
#include <cstdint>
#include <random>

#include "../../landslidehysea_gb300/csrc/lsh_adjoint.cuh"

using namespace lsh;

namespace {

int g_comp = -1;  // >= 0: check the single input component g_comp
double g_bor = 0.5;  // boundary factor of the ghost in boundary-edge checks

struct Rng {
    std::mt19937_64 g;
    explicit Rng(uint64_t s) : g(s) {}
    double u(double a, double b) { return std::uniform_real_distribution<double>(a, b)(g); }
};

Consts make_c(Rng& R, bool law0 = true) {
    Consts c{};
    c.g = 9.81; c.r = R.u(0.4, 0.6); c.gp = c.g * (1.0 - c.r); c.eps_h = 1e-5; c.peso = 1.0; c.beta = 1.0;
    c.cfl = 0.5; c.mu = std::tan(R.u(0.05, 0.3)); c.mfc = R.u(0.0, 0.02); c.mf0 = 0.025; c.mfs = 0.03;
    c.vmax1 = 0.0; c.vmax2 = 0.0; c.L = 1.0; c.H = 1.0;
    c.tan1 = c.mu; c.tan2 = c.tan3 = c.tan4 = 0.0;
    c.omr = 1.0 - c.r; c.inv_gp = 1.0 / c.gp; c.inv_eps = 1.0 / c.eps_h; c.inv_peso = 1.0;
    c.eps_1r = c.eps_h * (1.0 + c.r); c.g_mf02 = c.g * c.mf0 * c.mf0; c.g_mfs2 = c.g * c.mfs * c.mfs;
    c.sqrt_g = std::sqrt(c.g);
    c.law = law0 ? 0 : 1; c.order = 1; c.eig_sort = 0;
    return c;
}

// the differentiable inputs of an edge as a flat vector
constexpr int kEdgeVars = 12 + 8 + 1 + 8;  // faces, hc/acc, dt, constants
void edge_pack(const EdgeIn& e, double dt, const Consts& c, double* x) {
    const Face* f[2] = {&e.A, &e.B};
    int n = 0;
    for (int s = 0; s < 2; ++s) { x[n++] = f[s]->h1; x[n++] = f[s]->qn1; x[n++] = f[s]->qt1; x[n++] = f[s]->h2; x[n++] = f[s]->qn2; x[n++] = f[s]->qt2; }
    x[n++] = e.hc0[0]; x[n++] = e.hc0[1]; x[n++] = e.hc1[0]; x[n++] = e.hc1[1];
    x[n++] = e.acc0h[0]; x[n++] = e.acc0h[1]; x[n++] = e.acc1h[0]; x[n++] = e.acc1h[1];
    x[n++] = dt;
    x[n++] = c.r; x[n++] = c.omr; x[n++] = c.gp; x[n++] = c.inv_gp; x[n++] = c.mu; x[n++] = c.g_mf02; x[n++] = c.g_mfs2; x[n++] = c.eps_1r;
}
void edge_unpack(const double* x, EdgeIn& e, double& dt, Consts& c) {
    Face* f[2] = {&e.A, &e.B};
    int n = 0;
    for (int s = 0; s < 2; ++s) { f[s]->h1 = x[n++]; f[s]->qn1 = x[n++]; f[s]->qt1 = x[n++]; f[s]->h2 = x[n++]; f[s]->qn2 = x[n++]; f[s]->qt2 = x[n++]; }
    e.hc0[0] = x[n++]; e.hc0[1] = x[n++]; e.hc1[0] = x[n++]; e.hc1[1] = x[n++];
    e.acc0h[0] = x[n++]; e.acc0h[1] = x[n++]; e.acc1h[0] = x[n++]; e.acc1h[1] = x[n++];
    dt = x[n++];
    c.r = x[n++]; c.omr = x[n++]; c.gp = x[n++]; c.inv_gp = x[n++]; c.mu = x[n++]; c.g_mf02 = x[n++]; c.g_mfs2 = x[n++]; c.eps_1r = x[n++];
}
void edge_bar_pack(const EdgeInBar& b, double dtb, const ConstBar& cb, double* x) {
    const FaceBar* f[2] = {&b.A, &b.B};
    int n = 0;
    for (int s = 0; s < 2; ++s) { x[n++] = f[s]->h1; x[n++] = f[s]->qn1; x[n++] = f[s]->qt1; x[n++] = f[s]->h2; x[n++] = f[s]->qn2; x[n++] = f[s]->qt2; }
    x[n++] = b.hc0[0]; x[n++] = b.hc0[1]; x[n++] = b.hc1[0]; x[n++] = b.hc1[1];
    x[n++] = b.acc0h[0]; x[n++] = b.acc0h[1]; x[n++] = b.acc1h[0]; x[n++] = b.acc1h[1];
    x[n++] = dtb;
    x[n++] = cb.r; x[n++] = cb.omr; x[n++] = cb.gp; x[n++] = cb.inv_gp; x[n++] = cb.mu; x[n++] = cb.g_mf02; x[n++] = cb.g_mfs2; x[n++] = cb.eps_1r;
}

template <bool L2>
double edge_obj(const EdgeIn& e, double dt, const Consts& c, const EdgeOut& w) {
    EdgeOut o;
    edge_flux<L2>(e, dt, c, o);
    double s = w.wave * o.wave;
    for (int k = 0; k < 6; ++k) s += w.m[k] * o.m[k] + w.p[k] * o.p[k];
    return s;
}

}  // namespace

extern "C" {

void adjl_set_component(int k) { g_comp = k; }
void adjl_set_bor(double b) { g_bor = b; }

// One random edge check.  mode bit0: granular layer (L2), bit1: limiter
// forced active (large dt), bit2: boundary edge (no cell 1), bit3: Coulomb
// regime (slow granular layer, steep angle).  Returns |fd - adj| / scale
// over `ndir` random directions; *worst_abs gets the largest |fd - adj|.
double adjl_edge(uint64_t seed, int mode, int ndir, double* fd_out, double* adj_out) {
    Rng R(seed);
    Consts c = make_c(R);
    const bool L2 = mode & 1;
    EdgeIn e;
    e.A.h1 = R.u(2.0, 30.0); e.B.h1 = R.u(2.0, 30.0);
    e.A.H = R.u(10.0, 40.0); e.B.H = e.A.H + R.u(-3.0, 3.0);
    e.A.qn1 = R.u(-3.0, 3.0) * e.A.h1; e.B.qn1 = R.u(-3.0, 3.0) * e.B.h1;
    e.A.qt1 = R.u(-2.0, 2.0) * e.A.h1; e.B.qt1 = R.u(-2.0, 2.0) * e.B.h1;
    const double us = (mode & 8) ? 0.01 : 2.0;
    if (L2) {
        e.A.h2 = R.u(0.5, 5.0); e.B.h2 = R.u(0.5, 5.0);
        e.A.qn2 = R.u(-us, us) * e.A.h2; e.B.qn2 = R.u(-us, us) * e.B.h2;
        e.A.qt2 = R.u(-us, us) * e.A.h2; e.B.qt2 = R.u(-us, us) * e.B.h2;
        if (mode & 8) c.mu = 0.8;
    } else {
        e.A.h2 = e.B.h2 = e.A.qn2 = e.B.qn2 = e.A.qt2 = e.B.qt2 = 0.0;
    }
    e.len = R.u(10.0, 50.0);
    e.area0 = e.len * R.u(10.0, 50.0); e.area1 = e.len * R.u(10.0, 50.0);
    e.inv_area0 = 1.0 / e.area0; e.inv_area1 = 1.0 / e.area1;
    e.interior = !(mode & 4);
    e.hc0[0] = e.A.h1 * R.u(0.9, 1.1); e.hc0[1] = e.A.h2 * R.u(0.9, 1.1);
    e.hc1[0] = e.B.h1 * R.u(0.9, 1.1); e.hc1[1] = e.B.h2 * R.u(0.9, 1.1);
    e.acc0h[0] = R.u(-50, 50); e.acc0h[1] = L2 ? R.u(-10, 10) : 0.0;
    e.acc1h[0] = R.u(-50, 50); e.acc1h[1] = L2 ? R.u(-10, 10) : 0.0;
    if (!e.interior) {
        // ghost: B = A with the normal discharges times g_bor; checked as the
        // composite A -> (A, ghost(A)), as the edge kernels use it (a
        // reflecting wall, bor = -1, has zero normal mass flux, inside the
        // tangential upwinding's |F| < EPSILON dead zone: a kink FD cannot resolve)
        e.B = e.A; e.B.qn1 = g_bor * e.A.qn1; e.B.qn2 = g_bor * e.A.qn2;
        e.area1 = e.area0; e.inv_area1 = e.inv_area0;
        e.hc1[0] = e.hc1[1] = 0.0; e.acc1h[0] = e.acc1h[1] = 0.0;
    }
    double dt = (mode & 2) ? R.u(20.0, 80.0) : R.u(0.05, 0.3);
    EdgeOut w;
    for (int k = 0; k < 6; ++k) { w.m[k] = R.u(-1, 1); w.p[k] = R.u(-1, 1); }
    w.wave = R.u(-1, 1);
    EdgeInBar eb;
    edge_bar_zero(eb);
    double dtb = 0.0;
    ConstBar cb;
    cb_zero(cb);
    if (L2) edge_flux_adj<true>(e, dt, c, w, eb, dtb, cb);
    else edge_flux_adj<false>(e, dt, c, w, eb, dtb, cb);
    double x0[kEdgeVars], xb[kEdgeVars];
    edge_pack(e, dt, c, x0);
    if (!e.interior) {
        // the ghost's adjoint flows back into A
        eb.A.h1 += eb.B.h1; eb.A.qt1 += eb.B.qt1; eb.A.qn1 += g_bor * eb.B.qn1;
        eb.A.h2 += eb.B.h2; eb.A.qt2 += eb.B.qt2; eb.A.qn2 += g_bor * eb.B.qn2;
        face_bar_zero(eb.B);
    }
    edge_bar_pack(eb, dtb, cb, xb);
    double worst = 0.0;
    for (int d = 0; d < ndir; ++d) {
        double v[kEdgeVars];
        for (int k = 0; k < kEdgeVars; ++k) v[k] = R.u(-1, 1) * (std::fabs(x0[k]) + 1e-3);
        if (g_comp >= 0) for (int k = 0; k < kEdgeVars; ++k) v[k] = (k == g_comp) ? (std::fabs(x0[k]) + 1e-3) : 0.0;
        if (!L2) for (int k : {3, 4, 5, 9, 10, 11}) v[k] = 0.0;
        if (!e.interior) for (int k = 6; k < 12; ++k) v[k] = 0.0;  // B is the ghost, built by the caller
        const double h = 1e-7;
        double f[2];
        for (int s = 0; s < 2; ++s) {
            double x[kEdgeVars];
            for (int k = 0; k < kEdgeVars; ++k) x[k] = x0[k] + (s ? -h : h) * v[k];
            EdgeIn ee = e;
            double dd;
            Consts cc = c;
            edge_unpack(x, ee, dd, cc);
            if (!ee.interior) { ee.B = ee.A; ee.B.qn1 = g_bor * ee.A.qn1; ee.B.qn2 = g_bor * ee.A.qn2; }
            f[s] = L2 ? edge_obj<true>(ee, dd, cc, w) : edge_obj<false>(ee, dd, cc, w);
        }
        const double fd = (f[0] - f[1]) / (2 * h);
        double adj = 0.0;
        for (int k = 0; k < kEdgeVars; ++k) adj += xb[k] * v[k];
        const double err = std::fabs(fd - adj) / (std::fabs(fd) + std::fabs(adj) + 1e-300);
        if (err > worst) { worst = err; if (fd_out) *fd_out = fd; if (adj_out) *adj_out = adj; }
    }
    return worst;
}

// Volume update check.  mode bit0: granular layer present, bit1: spherical
// (tanR != 0), bit2: thin layers (h <= eps_h regime of vfac), bit3: vmax caps.
double adjl_volume(uint64_t seed, int mode, int ndir, double* fd_out, double* adj_out) {
    Rng R(seed);
    Consts c = make_c(R);
    if (mode & 8) { c.vmax1 = 0.5; c.vmax2 = 0.4; }
    const bool L2 = mode & 1;
    double wo[6], acc[7];
    const double hs = (mode & 4) ? 4e-6 : 1.0;
    wo[0] = R.u(2.0, 30.0) * hs; wo[1] = R.u(-2, 2) * wo[0]; wo[2] = R.u(-2, 2) * wo[0];
    if (L2) { wo[3] = R.u(0.5, 5.0) * hs; wo[4] = R.u(-1, 1) * wo[3]; wo[5] = R.u(-1, 1) * wo[3]; }
    else { wo[3] = wo[4] = wo[5] = 0.0; }
    for (int k = 0; k < 6; ++k) acc[k] = R.u(-0.1, 0.1) * (std::fabs(wo[k]) + 0.1 * hs) * 1e3;
    if (!L2) acc[3] = acc[4] = acc[5] = 0.0;
    acc[6] = R.u(1.0, 10.0);
    const double area = R.u(500, 2500), inv_area = 1.0 / area;
    const double tanR = (mode & 2) ? R.u(0.5, 2.0) * 1e-7 : 0.0;
    const double dt = R.u(0.05, 0.3);
    double wbar[6];
    for (int k = 0; k < 6; ++k) wbar[k] = R.u(-1, 1);
    const double rateb = R.u(-1, 1);
    double wob[6] = {0, 0, 0, 0, 0, 0}, accb[7] = {0, 0, 0, 0, 0, 0, 0}, dtb = 0.0;
    ConstBar cb;
    cb_zero(cb);
    volume_update_adj(wo, acc, inv_area, tanR, dt, c, wbar, rateb, wob, accb, dtb, cb);
    constexpr int NV = 6 + 7 + 1 + 8;
    double x0[NV], xb[NV];
    for (int k = 0; k < 6; ++k) { x0[k] = wo[k]; xb[k] = wob[k]; }
    for (int k = 0; k < 7; ++k) { x0[6 + k] = acc[k]; xb[6 + k] = accb[k]; }
    x0[13] = dt; xb[13] = dtb;
    const double cv[8] = {c.r, c.omr, c.gp, c.inv_gp, c.mu, c.g_mf02, c.g_mfs2, c.eps_1r};
    const double cbv[8] = {cb.r, cb.omr, cb.gp, cb.inv_gp, cb.mu, cb.g_mf02, cb.g_mfs2, cb.eps_1r};
    for (int k = 0; k < 8; ++k) { x0[14 + k] = cv[k]; xb[14 + k] = cbv[k]; }
    double worst = 0.0;
    for (int d = 0; d < ndir; ++d) {
        double v[NV];
        for (int k = 0; k < NV; ++k) v[k] = R.u(-1, 1) * (std::fabs(x0[k]) + 1e-3 * hs);
        if (g_comp >= 0) for (int k = 0; k < NV; ++k) v[k] = (k == g_comp) ? (std::fabs(x0[k]) + 1e-3 * hs) : 0.0;
        if (!L2) { v[3] = v[4] = v[5] = 0.0; v[9] = v[10] = v[11] = 0.0; }
        const double h = 1e-7;
        double f[2];
        for (int s = 0; s < 2; ++s) {
            double x[NV];
            for (int k = 0; k < NV; ++k) x[k] = x0[k] + (s ? -h : h) * v[k];
            Consts cc = c;
            cc.r = x[14]; cc.omr = x[15]; cc.gp = x[16]; cc.inv_gp = x[17]; cc.mu = x[18]; cc.g_mf02 = x[19];
            cc.g_mfs2 = x[20]; cc.eps_1r = x[21];
            double w[6], rate;
            volume_update(x, x + 6, w, rate, inv_area, tanR, x[13], cc);
            double s_ = rateb * rate;
            for (int k = 0; k < 6; ++k) s_ += wbar[k] * w[k];
            f[s] = s_;
        }
        const double fd = (f[0] - f[1]) / (2 * h);
        double adj = 0.0;
        for (int k = 0; k < NV; ++k) adj += xb[k] * v[k];
        const double err = std::fabs(fd - adj) / (std::fabs(fd) + std::fabs(adj) + 1e-300);
        if (err > worst) { worst = err; if (fd_out) *fd_out = fd; if (adj_out) *adj_out = adj; }
    }
    return worst;
}

// Initial-dt wave check (two-layer faces).
double adjl_initial_wave(uint64_t seed, int ndir, double* fd_out, double* adj_out) {
    Rng R(seed);
    Consts c = make_c(R);
    Face A, B;
    A.h1 = R.u(2, 30); B.h1 = R.u(2, 30); A.h2 = R.u(0.5, 5); B.h2 = R.u(0.5, 5);
    A.qn1 = R.u(-3, 3) * A.h1; B.qn1 = R.u(-3, 3) * B.h1; A.qn2 = R.u(-2, 2) * A.h2; B.qn2 = R.u(-2, 2) * B.h2;
    A.qt1 = A.qt2 = B.qt1 = B.qt2 = 0.0; A.H = B.H = 20.0;
    const double len = 30.0, wb = R.u(0.5, 1.5);
    FaceBar Ab, Bb;
    face_bar_zero(Ab); face_bar_zero(Bb);
    ConstBar cb;
    cb_zero(cb);
    edge_initial_wave_adj(A, B, len, c, wb, Ab, Bb, cb);
    double worst = 0.0;
    for (int d = 0; d < ndir; ++d) {
        double v[10];
        for (int k = 0; k < 10; ++k) v[k] = R.u(-1, 1);
        const double h = 1e-7;
        double f[2];
        for (int s = 0; s < 2; ++s) {
            const double sg = s ? -h : h;
            Face a = A, b = B;
            Consts cc = c;
            a.h1 += sg * v[0]; a.qn1 += sg * v[1]; a.h2 += sg * v[2]; a.qn2 += sg * v[3];
            b.h1 += sg * v[4]; b.qn1 += sg * v[5]; b.h2 += sg * v[6]; b.qn2 += sg * v[7];
            cc.gp += sg * v[8]; cc.inv_gp += sg * v[9];
            f[s] = wb * edge_initial_wave(a, b, len, cc);
        }
        const double fd = (f[0] - f[1]) / (2 * h);
        const double adj = Ab.h1 * v[0] + Ab.qn1 * v[1] + Ab.h2 * v[2] + Ab.qn2 * v[3] + Bb.h1 * v[4] + Bb.qn1 * v[5] +
                           Bb.h2 * v[6] + Bb.qn2 * v[7] + cb.gp * v[8] + cb.inv_gp * v[9];
        const double err = std::fabs(fd - adj) / (std::fabs(fd) + std::fabs(adj) + 1e-300);
        if (err > worst) { worst = err; if (fd_out) *fd_out = fd; if (adj_out) *adj_out = adj; }
    }
    return worst;
}

}  // extern "C"

extern "C" {

// The initial-dt pass's empty-edge shortcut (lsh_passes.cuh init_wave_edge):
// for two faces with zero depths and normal discharges (either sign of zero)
// the bound is exactly len * (0 + eps_h).  Returns the number of mismatches.
int adjl_initial_wave_empty(void) {
    Consts c{};
    c.g = 9.81; c.r = 0.5; c.gp = c.g * 0.5; c.inv_gp = 1.0 / c.gp; c.sqrt_g = std::sqrt(c.g);
    int bad = 0;
    const double epss[3] = {1e-5, 5e-3, 1e-3}, lens[3] = {11.1, 22.2, 37.0};
    for (double eps : epss)
        for (double len : lens)
            for (int sg = 0; sg < 4; ++sg) {
                c.eps_h = eps;
                c.inv_eps = 1.0 / eps;
                Face A{}, B{};
                if (sg & 1) { A.qn1 = -0.0; B.qn2 = -0.0; A.h1 = -0.0; }
                if (sg & 2) { A.qt1 = 3.0; B.qt2 = -2.0; }  // tangential discharge does not enter the bound
                A.H = 150.0; B.H = 120.0;
                const double w = edge_initial_wave(A, B, len, c), s = len * (0.0 + eps);
                if (lshm::bits_of(w) != lshm::bits_of(s)) ++bad;
            }
    return bad;
}

}  // extern "C"
