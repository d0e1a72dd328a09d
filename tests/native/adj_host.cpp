// TEST INFRASTRUCTURE: a host emulation of the discrete adjoint sweep, built
// from the product's own per-edge / per-cell bodies (lsh_passes.cuh forward,
// lsh_adjoint.cuh reverse) in plain loops, storing every step's state (no
// checkpointing).  It lets the CPU test suite check the adjoint arithmetic
// against the oracle's tangent-linear model; the GPU sweep (lsh_adjoint.cu)
// runs the same bodies as kernels and is checked the same way on a GPU.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/lsh.h"
#include "../../landslidehysea_gb300/csrc/lsh_adjoint.cuh"
#include "../../landslidehysea_gb300/csrc/lsh_setup.h"

using namespace lsh;

namespace lsh {
void set_last_error(const std::string&) {}
}

namespace {

using Vec = std::vector<double>;

struct Host {
    lsh_params p;
    Consts c;
    int nx, ny;
    size_t N;
    Vec geo;
    Geo G;
    explicit Host(const lsh_params& prm) : p(prm), c(make_consts(prm)), nx(prm.nx), ny(prm.ny) {
        N = size_t(nx) * ny;
        geo.assign(7 * size_t(ny + 1), 0.0);
        fill_geo(p, geo.data(), size_t(ny + 1));
        const size_t st = ny + 1;
        G.area = geo.data(); G.len_v = geo.data() + st; G.len_h = geo.data() + 2 * st; G.tanR = geo.data() + 3 * st;
        G.wx = geo.data() + 4 * st; G.wy = geo.data() + 5 * st; G.inv_area = geo.data() + 6 * st;
    }
};

// Intermediates of one forward stage.
struct Stage {
    Vec sx[7], sy[7], acc[7], snap[3][2];
    unsigned long long rmax = 0;
    long long argmax = -1;
    std::vector<unsigned> tape;
};

void arr_ptrs(Vec* v, int n, double** out) { for (int k = 0; k < n; ++k) out[k] = v[k].data(); }

// One forward stage W -> Wout (MODE 0: order 1; 1: order-2 stage 1; 2: stage 2 with Xavg).
void fwd_stage(const Host& h, const double* const* W, double* const* Wout, const double* const* Xavg, double dt, int mode,
               Stage& S) {
    const size_t N = h.N;
    for (int k = 0; k < 7; ++k) { S.sx[k].assign(N, 0.0); S.sy[k].assign(N, 0.0); S.acc[k].assign(N, 0.0); }
    TimeRec tm{};
    KArgs a;
    std::memset(&a, 0, sizeof(a));
    a.c = h.c; a.geo = h.G; a.tm = &tm;
    for (int k = 0; k < 7; ++k) { a.W[k] = W[k]; a.acc[k] = S.acc[k].data(); a.sx[k] = a.sxw[k] = S.sx[k].data(); a.sy[k] = a.syw[k] = S.sy[k].data(); }
    for (int k = 0; k < 6; ++k) { a.Wout[k] = Wout[k]; a.Xavg[k] = Xavg ? Xavg[k] : nullptr; }
    const int order = h.p.order;
    if (order == 2) {
        for (size_t id = 0; id < N; ++id) recon_cell(a, int(id));
        S.tape.resize(N);
        for (size_t id = 0; id < N; ++id) S.tape[id] = recon_tape_cell(W, h.nx, h.ny, int(id));
    }
    auto snap = [&](int s) { S.snap[s][0] = S.acc[0]; S.snap[s][1] = S.acc[3]; };
    for (int y = 0; y <= h.ny; y += 2) for (int x = 0; x < h.nx; ++x) (order == 2) ? do_edge<0, true, 2>(a, x, y, dt) : do_edge<0, true, 1>(a, x, y, dt);
    snap(0);
    for (int y = 1; y <= h.ny; y += 2) for (int x = 0; x < h.nx; ++x) (order == 2) ? do_edge<0, false, 2>(a, x, y, dt) : do_edge<0, false, 1>(a, x, y, dt);
    snap(1);
    for (int y = 0; y < h.ny; ++y) for (int x = 0; x <= h.nx; x += 2) (order == 2) ? do_edge<1, false, 2>(a, x, y, dt) : do_edge<1, false, 1>(a, x, y, dt);
    snap(2);
    for (int y = 0; y < h.ny; ++y) for (int x = 1; x <= h.nx; x += 2) (order == 2) ? do_edge<1, false, 2>(a, x, y, dt) : do_edge<1, false, 1>(a, x, y, dt);
    S.rmax = 0;
    S.argmax = -1;
    for (size_t id = 0; id < N; ++id) {
        unsigned long long b;
        if (mode == 0) b = volume_cell<0>(a, int(id), dt);
        else if (mode == 1) b = volume_cell<1>(a, int(id), dt);
        else b = volume_cell<2>(a, int(id), dt);
        if (mode != 2 && b > S.rmax) { S.rmax = b; S.argmax = (long long)id; }
    }
}

// Reverse of one stage.  wbar: adjoint of the stage output; Wbar: adjoint of
// its input (accumulated); Xbar (MODE 2): adjoint of the step's initial state.
void rev_stage(const Host& h, const double* const* W, const Stage& S, double dt, int mode, const double* const* wbar,
               double* const* Wbar, double* const* Xbar, long long rate_cell, double rate_bar, double& dtb,
               ConstBar& cb) {
    const size_t N = h.N;
    Vec accb[7], sxb[7], syb[7];
    for (int k = 0; k < 7; ++k) { accb[k].assign(N, 0.0); sxb[k].assign(N, 0.0); syb[k].assign(N, 0.0); }
    AdjArgs a;
    std::memset(&a, 0, sizeof(a));
    a.c = h.c; a.geo = h.G; a.dt = dt;
    for (int k = 0; k < 7; ++k) {
        a.W[k] = W[k]; a.sx[k] = S.sx[k].data(); a.sy[k] = S.sy[k].data(); a.acc[k] = S.acc[k].data();
        a.sxb[k] = sxb[k].data(); a.syb[k] = syb[k].data(); a.accb[k] = accb[k].data();
    }
    for (int k = 0; k < 6; ++k) { a.Wbar[k] = Wbar[k]; a.wbar[k] = wbar[k]; a.Xbar[k] = Xbar ? Xbar[k] : nullptr; }
    a.tape = S.tape.empty() ? nullptr : S.tape.data();
    a.rate_cell = rate_cell;
    a.rate_bar = rate_bar;
    const int order = h.p.order;
    for (size_t id = 0; id < N; ++id) {
        if (mode == 0) volume_adj_body<0>(a, int(id), dtb, cb);
        else if (mode == 1) volume_adj_body<1>(a, int(id), dtb, cb);
        else volume_adj_body<2>(a, int(id), dtb, cb);
    }
    a.snap[0] = S.snap[2][0].data(); a.snap[1] = S.snap[2][1].data();
    for (int y = 0; y < h.ny; ++y) for (int x = 1; x <= h.nx; x += 2) (order == 2) ? edge_adj_body<1, false, 2>(a, x, y, dtb, cb) : edge_adj_body<1, false, 1>(a, x, y, dtb, cb);
    a.snap[0] = S.snap[1][0].data(); a.snap[1] = S.snap[1][1].data();
    for (int y = 0; y < h.ny; ++y) for (int x = 0; x <= h.nx; x += 2) (order == 2) ? edge_adj_body<1, false, 2>(a, x, y, dtb, cb) : edge_adj_body<1, false, 1>(a, x, y, dtb, cb);
    a.snap[0] = S.snap[0][0].data(); a.snap[1] = S.snap[0][1].data();
    for (int y = 1; y <= h.ny; y += 2) for (int x = 0; x < h.nx; ++x) (order == 2) ? edge_adj_body<0, false, 2>(a, x, y, dtb, cb) : edge_adj_body<0, false, 1>(a, x, y, dtb, cb);
    a.snap[0] = a.snap[1] = nullptr;
    for (int y = 0; y <= h.ny; y += 2) for (int x = 0; x < h.nx; ++x) (order == 2) ? edge_adj_body<0, true, 2>(a, x, y, dtb, cb) : edge_adj_body<0, true, 1>(a, x, y, dtb, cb);
    if (order == 2)
        for (size_t id = 0; id < N; ++id) recon_adj_cell(a, int(id));
}

}  // namespace

namespace {

// The initial-dt pass over W (the host bodies of the wave pass and the
// per-cell rate): S0 gets the accumulators, the largest rate and its cell.
double initial_dt(const Host& h, const double* const* W, Stage& S0) {
    const size_t N = h.N;
    for (int k = 0; k < 7; ++k) S0.acc[k].assign(N, 0.0);
    TimeRec tm{};
    KArgs a;
    std::memset(&a, 0, sizeof(a));
    a.c = h.c; a.geo = h.G; a.tm = &tm;
    for (int k = 0; k < 7; ++k) { a.W[k] = W[k]; a.acc[k] = S0.acc[k].data(); }
    for (int y = 0; y <= h.ny; y += 2) for (int x = 0; x < h.nx; ++x) init_wave_edge<0, true>(a, x, y);
    for (int y = 1; y <= h.ny; y += 2) for (int x = 0; x < h.nx; ++x) init_wave_edge<0, false>(a, x, y);
    for (int y = 0; y < h.ny; ++y) for (int x = 0; x <= h.nx; x += 2) init_wave_edge<1, false>(a, x, y);
    for (int y = 0; y < h.ny; ++y) for (int x = 1; x <= h.nx; x += 2) init_wave_edge<1, false>(a, x, y);
    for (size_t id = 0; id < N; ++id) {
        const unsigned long long b = init_cell_rate(a, int(id));
        if (b > S0.rmax) { S0.rmax = b; S0.argmax = (long long)id; }
    }
    return dt_of(S0.rmax, 2.0 * h.c.cfl);
}

}  // namespace

extern "C" {

// The forward alone: nsteps steps of W (7 arrays, advanced in place to X_N)
// by the product's per-edge / per-cell bodies in plain loops; dts[0..nsteps]
// gets each step's dt and the one after the last.
int adjh_forward(const lsh_params* p, double* const* W, int nsteps, double* dts) {
    Host h(*p);
    const size_t N = h.N;
    Stage S0;
    dts[0] = initial_dt(h, W, S0);
    std::vector<Vec> Yv(6);
    for (int n = 0; n < nsteps; ++n) {
        Stage S1, S2;
        if (p->order == 1) {
            fwd_stage(h, W, W, nullptr, dts[n], 0, S1);
        } else {
            double* Y[7];
            for (int k = 0; k < 6; ++k) { Yv[k].assign(N, 0.0); Y[k] = Yv[k].data(); }
            Y[6] = W[6];
            fwd_stage(h, W, Y, nullptr, dts[n], 1, S1);
            fwd_stage(h, Y, W, W, dts[n], 2, S2);
        }
        dts[n + 1] = dt_of(S1.rmax, 2.0 * h.c.cfl);
    }
    return 0;
}

// Misfit J = sum_{n=1..nsteps} sum_g (eta1_n[g] - target)^2 (weight `wj`)
// plus <wfin, X_N> (wfin: 6 arrays or NULL).  W (7 arrays) is the initial
// state (unchanged).  Outputs: J (the misfit alone), grad (6 arrays: the
// gradient with respect to the initial h1..q2y), gpar (angle1, mf0, mfs, r).
int adjh_run(const lsh_params* p, const double* const* W0, int nsteps, int ng, const int* gauges, const double* target,
             double wj, const double* const* wfin, double* J, double* const* grad, double* gpar, double h_adj) {
    Host h(*p);
    const size_t N = h.N;
    std::vector<Vec> X(size_t(nsteps + 1) * 7);
    auto Xs = [&](int n, int k) -> Vec& { return X[size_t(n) * 7 + k]; };
    for (int k = 0; k < 7; ++k) Xs(0, k).assign(W0[k], W0[k] + N);
    std::vector<double> dts(nsteps + 1, 0.0);
    std::vector<Stage> S1(nsteps), S2(nsteps);
    std::vector<Vec> Ys(size_t(nsteps) * 6);
    // initial dt: the initial wave pass (on the host bodies)
    Stage S0;
    {
        const double* Wp[7];
        for (int k = 0; k < 7; ++k) Wp[k] = Xs(0, k).data();
        dts[0] = initial_dt(h, Wp, S0);
    }
    double Jv = 0.0;
    std::vector<double> eta(size_t(nsteps) * ng);
    for (int n = 0; n < nsteps; ++n) {
        double* Xn[7];
        double* Xn1[7];
        for (int k = 0; k < 7; ++k) { Xn[k] = Xs(n, k).data(); Xs(n + 1, k).assign(N, 0.0); Xn1[k] = Xs(n + 1, k).data(); }
        std::memcpy(Xn1[6], Xn[6], N * sizeof(double));
        const double dt = dts[n];
        if (p->order == 1) {
            for (int k = 0; k < 6; ++k) std::memcpy(Xn1[k], Xn[k], N * sizeof(double));
            // order 1 updates in place: run it on the copy
            fwd_stage(h, Xn1, Xn1, nullptr, dt, 0, S1[n]);
            // the in-place update reads W as it writes: volume_cell reads only its own cell, so equal
        } else {
            double* Y[7];
            for (int k = 0; k < 6; ++k) { Ys[size_t(n) * 6 + k].assign(N, 0.0); Y[k] = Ys[size_t(n) * 6 + k].data(); }
            Y[6] = Xn[6];
            fwd_stage(h, Xn, Y, nullptr, dt, 1, S1[n]);
            fwd_stage(h, Y, Xn1, Xn, dt, 2, S2[n]);
        }
        dts[n + 1] = dt_of(S1[n].rmax, 2.0 * h.c.cfl);
        for (int g = 0; g < ng; ++g) {
            const int id = gauges[g];
            const double e = (Xn1[0][id] + Xn1[3][id]) - Xn1[6][id];
            eta[size_t(n) * ng + g] = e;
            if (target) { const double d = e - target[size_t(n) * ng + g]; Jv = fmad(d, d, Jv); }
        }
    }
    *J = Jv;
    // reverse sweep
    Vec Xb[6], Xbn[6], Yb[6];
    for (int k = 0; k < 6; ++k) { Xb[k].assign(N, 0.0); if (wfin && wfin[k]) Xb[k].assign(wfin[k], wfin[k] + N); }
    ConstBar cb;
    cb_zero(cb);
    // the misfit's adjoint at X_m (m >= 1), then the thin-layer projection of X_m
    auto misfit_and_project = [&](int m) {
        if (target && wj != 0.0 && m >= 1) {
            for (int g = 0; g < ng; ++g) {
                const int id = gauges[g];
                const double d = eta[size_t(m - 1) * ng + g] - target[size_t(m - 1) * ng + g];
                Xb[0][id] += wj * 2.0 * d;
                Xb[3][id] += wj * 2.0 * d;
            }
        }
        if (h_adj > 0.0)
            for (size_t i = 0; i < N; ++i)
                for (int l = 0; l < 2; ++l)
                    if (Xs(m, 3 * l)[i] < h_adj) Xb[3 * l][i] = Xb[3 * l + 1][i] = Xb[3 * l + 2][i] = 0.0;
    };
    misfit_and_project(nsteps);
    double dtb_next = 0.0;  // adjoint of dt_{n+1}
    for (int n = nsteps - 1; n >= 0; --n) {
        const double dt = dts[n];
        double dtb = 0.0;
        // d dt_{n+1} / d R = -dt_{n+1} / R at the stage-1 argmax cell
        long long rc = -1;
        double rb = 0.0;
        if (S1[n].argmax >= 0 && dtb_next != 0.0) {
            const double R = lshm::from_bits(S1[n].rmax);
            rc = S1[n].argmax;
            rb = -dtb_next * (dts[n + 1] / R);
        }
        for (int k = 0; k < 6; ++k) Xbn[k].assign(N, 0.0);
        double* Xbnp[6];
        const double* Xbp[6];
        for (int k = 0; k < 6; ++k) { Xbnp[k] = Xbn[k].data(); Xbp[k] = Xb[k].data(); }
        const double* Xn[7];
        for (int k = 0; k < 7; ++k) Xn[k] = Xs(n, k).data();
        if (p->order == 1) {
            rev_stage(h, Xn, S1[n], dt, 0, Xbp, Xbnp, nullptr, rc, rb, dtb, cb);
        } else {
            const double* Y[7];
            for (int k = 0; k < 6; ++k) Y[k] = Ys[size_t(n) * 6 + k].data();
            Y[6] = Xn[6];
            double* Ybp[6];
            for (int k = 0; k < 6; ++k) { Yb[k].assign(N, 0.0); Ybp[k] = Yb[k].data(); }
            rev_stage(h, Y, S2[n], dt, 2, Xbp, Ybp, Xbnp, -1, 0.0, dtb, cb);
            const double* Ybc[6];
            for (int k = 0; k < 6; ++k) Ybc[k] = Yb[k].data();
            rev_stage(h, Xn, S1[n], dt, 1, Ybc, Xbnp, nullptr, rc, rb, dtb, cb);
        }
        for (int k = 0; k < 6; ++k) Xb[k].swap(Xbn[k]);
        dtb_next = dtb;
        if (n >= 1) misfit_and_project(n);
    }
    // dt_0 from the initial pass
    if (S0.argmax >= 0 && dtb_next != 0.0) {
        const double R = lshm::from_bits(S0.rmax);
        const double rb = -dtb_next * (dts[0] / R);
        const int cell = int(S0.argmax);
        const int j = cell / h.nx;
        AdjArgs a;
        std::memset(&a, 0, sizeof(a));
        a.c = h.c; a.geo = h.G;
        for (int k = 0; k < 7; ++k) a.W[k] = Xs(0, k).data();
        for (int k = 0; k < 6; ++k) a.Wbar[k] = Xb[k].data();
        init_wave_adj_cell(a, cell, rb * h.G.inv_area[j], cb);
    }
    misfit_and_project(0);
    for (int k = 0; k < 6; ++k) std::memcpy(grad[k], Xb[k].data(), N * sizeof(double));
    param_grads(p->angle1, p->mf0, p->mfs, p->r, p->gravity, p->eps_h, p->L, p->H, cb, gpar);
    return 0;
}

}  // extern "C"

extern "C" {

// Slopes of recon_cell (the forward) against recon_cell_tape (the adjoint's
// recomputation): the number of cells where any slope differs in any bit.
long long adjh_recon_check(const lsh_params* p, const double* const* W) {
    Host h(*p);
    const size_t N = h.N;
    Vec a[14], b[14];
    for (int k = 0; k < 14; ++k) { a[k].assign(N, -1.0); b[k].assign(N, -2.0); }
    KArgs ka, kb;
    std::memset(&ka, 0, sizeof(ka));
    std::memset(&kb, 0, sizeof(kb));
    ka.c = kb.c = h.c;
    for (int k = 0; k < 7; ++k) {
        ka.W[k] = kb.W[k] = W[k];
        ka.sxw[k] = a[k].data(); ka.syw[k] = a[7 + k].data();
        kb.sxw[k] = b[k].data(); kb.syw[k] = b[7 + k].data();
    }
    long long bad = 0;
    for (size_t id = 0; id < N; ++id) {
        recon_cell(ka, int(id));
        (void)recon_cell_tape(kb, int(id));
        for (int k = 0; k < 14; ++k)
            if (lshm::bits_of(a[k][id]) != lshm::bits_of(b[k][id])) { ++bad; break; }
    }
    return bad;
}

}  // extern "C"
