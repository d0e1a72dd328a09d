// lsh_passes.cuh -- per-edge and per-cell device functions of the step,
// shared by the single-grid kernels (lsh_core.cu) and the batched ensemble
// kernels (lsh_batch.cu), so both evaluate exactly the same arithmetic.
#pragma once

#if defined(__CUDACC__)
#include <cuda_runtime.h>
#endif

#include "../../include/lsh.h"
#include "lsh_scheme.cuh"

namespace lsh {

constexpr unsigned long long kRateInitBits = 0ULL;  // +0.0
constexpr int kEdgeBlock = 128;
constexpr int kCellBlock = 256;
constexpr double kReconThin = 0.5;  // second order: least face depth / cell depth

// Sticky error bit: an atomic OR on the device, a plain OR in host code.
LSH_HD void err_or(int* word, int bit) {
#if defined(__CUDA_ARCH__)
    atomicOr(word, bit);
#else
    *word |= bit;
#endif
}

// p on every active lane of the warp (the thread's own p in host code).
LSH_HD bool warp_all(bool p) {
#if defined(__CUDA_ARCH__)
    return __all_sync(__activemask(), p);
#else
    return p;
#endif
}

// p on some active lane of the warp (the thread's own p in host code).
LSH_HD bool warp_any(bool p) {
#if defined(__CUDA_ARCH__)
    return __any_sync(__activemask(), p);
#else
    return p;
#endif
}

struct KArgs {
    Consts c;
    Geo geo;
    const double* W[7];   // input state (face values are W + slopes at order 2)
    double* Wout[6];      // output state of the volume kernel
    const double* Xavg[6];  // order 2, stage 2: the step's initial state for the average
    double* acc[7];
    const double* sx[7];
    const double* sy[7];
    double* sxw[7];       // reconstruction kernel outputs
    double* syw[7];
    double* eta_max;
    double* eta_time;
    TimeRec* tm;
    unsigned char* szero;  // per cell: 1 when the stored slopes are all zero (may be null)
    // the adjoint's recomputation (null otherwise): an edge pass after the
    // first copies acc[0], acc[3] of its non-dry edges' cells, as the pass
    // before left them, to snap[0], snap[1] -- the partial sums its limiter
    // reads, which the reverse sweep needs at exactly those cells
    double* snap[2];
    unsigned* tape;       // the recomputation's reconstruction branch tape (kOpReconTape; null otherwise)
};

// Depths of a face (first order: the cell's; second order: reconstructed).
template <int ORDER>
LSH_HD void face_depths(const KArgs& a, int id, int side, double& h1, double& h2) {
    h1 = a.W[0][id];
    h2 = a.W[3][id];
    if (ORDER == 2) {
        const double* const* s = (side < 2) ? a.sx : a.sy;
        const double d1 = s[0][id] - s[3][id], d2 = s[3][id] + s[6][id];
        // side & 1: the +slope face (E or N); the sign is a sign-bit flip
        const bool neg = !(side & 1);
        h1 = h1 + lshm::neg_if(d1, neg);
        h2 = h2 + lshm::neg_if(d2, neg);
    }
}

// The rest of a face in the edge frame.  DIR 1 (vertical edge, normal
// (sg, 0)): qn = sg qx, qt = sg qy; DIR 0 (horizontal, normal (0, sg)):
// qn = sg qy, qt = -sg qx (Arista_kernel.cu:363-371, 509-525) -- selections
// and negations, no FP64 arithmetic.
template <int DIR, int ORDER>
LSH_HD void face_rest(const KArgs& a, int id, int side, bool pos_normal, lsh::Face& f) {
    double qx1 = a.W[1][id], qy1 = a.W[2][id], qx2 = a.W[4][id], qy2 = a.W[5][id], H = a.W[6][id];
    if (ORDER == 2) {
        const double* const* s = (side < 2) ? a.sx : a.sy;
        using lshm::neg_if;
        const bool neg = !(side & 1);
        qx1 = qx1 + neg_if(s[1][id], neg);
        qy1 = qy1 + neg_if(s[2][id], neg);
        qx2 = qx2 + neg_if(s[4][id], neg);
        qy2 = qy2 + neg_if(s[5][id], neg);
        H = H + neg_if(s[6][id], neg);
    }
    using lshm::neg_if;
    if (DIR == 1) {
        f.qn1 = neg_if(qx1, !pos_normal); f.qt1 = neg_if(qy1, !pos_normal);
        f.qn2 = neg_if(qx2, !pos_normal); f.qt2 = neg_if(qy2, !pos_normal);
    } else {
        f.qn1 = neg_if(qy1, !pos_normal); f.qt1 = neg_if(qx1, pos_normal);
        f.qn2 = neg_if(qy2, !pos_normal); f.qt2 = neg_if(qx2, pos_normal);
    }
    f.H = H;
}

// The accumulator update of one edge: subtract the first KL flux terms of
// each cell (KL = 3: layer 1 only, the layer-2 terms being zeros) and add the
// wave term.  The first pass of a stage writes instead of accumulating:
// every cell meets exactly one hor-even edge.
template <bool FIRST, int KL>
LSH_HD void scatter_edge(const KArgs& a, int id0, int id1, bool interior, const double d0[6], const double d1[6],
                         double wave) {
    if (FIRST) {
#pragma unroll
        for (int k = 0; k < 6; ++k) a.acc[k][id0] = (k < KL) ? 0.0 - d0[k] : 0.0;
        a.acc[6][id0] = 0.0 + wave;
        if (interior) {
#pragma unroll
            for (int k = 0; k < 6; ++k) a.acc[k][id1] = (k < KL) ? 0.0 - d1[k] : 0.0;
            a.acc[6][id1] = 0.0 + wave;
        }
    } else {
#pragma unroll
        for (int k = 0; k < KL; ++k) a.acc[k][id0] -= d0[k];
        a.acc[6][id0] += wave;
        if (interior) {
#pragma unroll
            for (int k = 0; k < KL; ++k) a.acc[k][id1] -= d1[k];
            a.acc[6][id1] += wave;
        }
    }
}

// The positivity limiter's inputs of one edge, loaded from the state and the
// accumulators where the limiter reads them: cell areas by row, cell depths
// h1, h2, and the depths' partial accumulators (zero in the first pass); a
// boundary edge's outer side mirrors the cell's area with zero depths.
template <bool FIRST>
struct LazyPos {
    const KArgs& a;
    int id0, id1, row0, row1;
    LSH_HD double area(int side) const { return a.geo.area[(side && id1 >= 0) ? row1 : row0]; }
    LSH_HD double inv_area(int side) const { return a.geo.inv_area[(side && id1 >= 0) ? row1 : row0]; }
    LSH_HD double hc(int side, int layer) const {
        if (side && id1 < 0) return 0.0;
        return a.W[layer ? 3 : 0][side ? id1 : id0];
    }
    LSH_HD double acch(int side, int layer) const {
        if (FIRST || (side && id1 < 0)) return 0.0;
        return a.acc[layer ? 3 : 0][side ? id1 : id0];
    }
};

// One edge: gather both sides, evaluate, scatter to the accumulators.
// dir 0: horizontal edge row y between rows y-1 and y, column x.
// dir 1: vertical edge column x between columns x-1 and x, row y.
template <int DIR, bool FIRST, int ORDER>
LSH_HD void do_edge(const KArgs& a, int x, int y, double dt) {
    const int nx = a.c.nx, ny = a.c.ny;
    lsh::EdgeIn e;
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
    const int side1 = (DIR == 0) ? 2 : 0;
    // Both cells empty (h1 = h2 = 0) with zero stored slopes (second order:
    // the slope-zero flags): every face depth is exactly 0, so the dry test
    // below would find the edge dry.  Integer tests only, and no slope loads:
    // most edges of a flooded-coast grid are such edges.
    if (ORDER == 1 || a.szero) {
        using lsh::is_zero;
        bool empty = is_zero(a.W[0][id0]) && is_zero(a.W[3][id0]) && (ORDER == 1 || a.szero[id0]);
        if (empty && e.interior) empty = is_zero(a.W[0][id1]) && is_zero(a.W[3][id1]) && (ORDER == 1 || a.szero[id1]);
        if (empty) {
            if (FIRST) {
#pragma unroll
                for (int k = 0; k < 7; ++k) a.acc[k][id0] = 0.0;
                if (e.interior) {
#pragma unroll
                    for (int k = 0; k < 7; ++k) a.acc[k][id1] = 0.0;
                }
            }
            return;
        }
    }
    face_depths<ORDER>(a, id0, side0, e.A.h1, e.A.h2);
    if (e.interior) face_depths<ORDER>(a, id1, side1, e.B.h1, e.B.h2);
    else { e.B.h1 = e.A.h1; e.B.h2 = e.A.h2; }
    // dry edge (Arista_kernel.cu:397): nothing to add; the first pass still
    // writes the zeros that initialise the accumulators
    if (lshm::lt_pos(0.5 * (e.A.h1 + e.B.h1), lsh::kEps) && lshm::lt_pos(0.5 * (e.A.h2 + e.B.h2), lsh::kEps)) {
        if (FIRST) {
#pragma unroll
            for (int k = 0; k < 7; ++k) a.acc[k][id0] = 0.0;
            if (e.interior) {
#pragma unroll
                for (int k = 0; k < 7; ++k) a.acc[k][id1] = 0.0;
            }
        }
        return;
    }
    if (!FIRST && a.snap[0]) {
        a.snap[0][id0] = a.acc[0][id0];
        a.snap[1][id0] = a.acc[3][id0];
        if (e.interior) {
            a.snap[0][id1] = a.acc[0][id1];
            a.snap[1][id1] = a.acc[3][id1];
        }
    }
    face_rest<DIR, ORDER>(a, id0, side0, pos_normal, e.A);
    if (e.interior) {
        face_rest<DIR, ORDER>(a, id1, side1, pos_normal, e.B);
    } else {
        // ghost: the cell's face with the normal discharges times the boundary factor
        e.B = e.A;
        e.B.qn1 = e.A.qn1 * bor;
        e.B.qn2 = e.A.qn2 * bor;
    }
    // the limiter's inputs are loaded where it reads them (LazyPos), not kept
    // live through the flux computation
    const LazyPos<FIRST> pos{a, id0, id1, row0, row1};
    lsh::EdgeOut o;
    using lsh::is_zero;
    const bool single = is_zero(e.A.h2) && is_zero(e.B.h2) && is_zero(e.A.qn2) && is_zero(e.B.qn2);
    if (single)
        lsh::edge_flux<false>(e, dt, a.c, o, pos);
    else
        lsh::edge_flux<true>(e, dt, a.c, o, pos);
    // back to x/y: DIR 1: (qx, qy) = sg (fn, ft); DIR 0: qx = -sg ft, qy = sg fn
    double d0[6], d1[6];
#pragma unroll
    for (int l = 0; l < 2; ++l) {
        const int k = 3 * l;
        d0[k] = o.m[k];
        d1[k] = o.p[k];
        using lshm::neg_if;
        if (DIR == 1) {
            d0[k + 1] = neg_if(o.m[k + 1], !pos_normal);
            d0[k + 2] = neg_if(o.m[k + 2], !pos_normal);
            d1[k + 1] = neg_if(o.p[k + 1], !pos_normal);
            d1[k + 2] = neg_if(o.p[k + 2], !pos_normal);
        } else {
            d0[k + 1] = neg_if(o.m[k + 2], pos_normal);
            d0[k + 2] = neg_if(o.m[k + 1], !pos_normal);
            d1[k + 1] = neg_if(o.p[k + 2], pos_normal);
            d1[k + 2] = neg_if(o.p[k + 1], !pos_normal);
        }
    }
    // A single-layer edge's layer-2 terms are zeros, and an accumulator never
    // holds -0 (the first pass writes 0 - d, which is +0 for d = +-0, and
    // x - y is -0 only for x = -0): subtracting them leaves the accumulator's
    // bits as they are.  A warp whose edges are all single-layer skips that
    // arithmetic and its loads, and the first pass stores the +0 it would
    // compute.
    if (warp_all(single)) scatter_edge<FIRST, 3>(a, id0, id1, e.interior, d0, d1, o.wave);
    else scatter_edge<FIRST, 6>(a, id0, id1, e.interior, d0, d1, o.wave);
}

// minmod: the operand of smaller magnitude when both are nonzero with one
// sign (b on a tie), else 0 -- on the bit patterns (integer pipe); for
// operands that are not NaN the same as the compares
//   a > 0 && b > 0 ? (a < b ? a : b) : a < 0 && b < 0 ? (a > b ? a : b) : 0
LSH_HD double minmod(double a, double b) {
    const uint64_t ua = lshm::bits_of(a), ub = lshm::bits_of(b);
    const bool nonzero = ((ua << 1) != 0) && ((ub << 1) != 0);
    const bool same = ((ua ^ ub) >> 63) == 0;
    if (!(nonzero && same)) return 0.0;
    return ((ua & lshm::kMag) < (ub & lshm::kMag)) ? a : b;
}

LSH_HD double recon_var(const KArgs& a, int id, int k) {
    if (k == 0) return (a.W[0][id] + a.W[3][id]) - a.W[6][id];
    if (k == 3) return a.W[3][id] - a.W[6][id];
    return a.W[k][id];
}

// One cell of the second-order reconstruction, its inputs read through an
// accessor w(k, di, dj) = W[k] at cell (i + di, j + dj): global memory
// (recon_cell) or a shared-memory tile (k_recon).  Neighbours are read only
// inside the grid.
template <class Acc>
LSH_HD void recon_cell_from(const KArgs& a, int id, int i, int j, const Acc& w) {
    const int nx = a.c.nx, ny = a.c.ny;
    // A cell whose own and 4 neighbours' depths are all zero only meets dry
    // edges (a dry cell's faces always have zero depth: any nonzero depth
    // slope would make one face negative and trigger the fallback), so its
    // slopes are never read: store zeros and skip the FP64 work.
    {
        using lsh::is_zero;
        bool dry = is_zero(w(0, 0, 0)) && is_zero(w(3, 0, 0));
        if (dry && i > 0) dry = is_zero(w(0, -1, 0)) && is_zero(w(3, -1, 0));
        if (dry && i < nx - 1) dry = is_zero(w(0, 1, 0)) && is_zero(w(3, 1, 0));
        if (dry && j > 0) dry = is_zero(w(0, 0, -1)) && is_zero(w(3, 0, -1));
        if (dry && j < ny - 1) dry = is_zero(w(0, 0, 1)) && is_zero(w(3, 0, 1));
        if (dry) {
            // zero slopes; a cell whose stored slopes are already zero (and stays
            // dry, the common case far from the flow) skips the 14 stores
            if (a.szero && a.szero[id]) return;
#pragma unroll
            for (int k = 0; k < 7; ++k) { a.sxw[k][id] = 0.0; a.syw[k][id] = 0.0; }
            if (a.szero) a.szero[id] = 1;
            return;
        }
    }
    // the reconstructed variables: eta1 = h1 + h2 - H, eta2 = h2 - H, the discharges, H
    auto rv = [&](int k, int di, int dj) -> double {
        if (k == 0) return (w(0, di, dj) + w(3, di, dj)) - w(6, di, dj);
        if (k == 3) return w(3, di, dj) - w(6, di, dj);
        return w(k, di, dj);
    };
    const bool inx = (i > 0 && i < nx - 1), iny = (j > 0 && j < ny - 1);
    auto slope_x = [&](int k) {
        const double pc = rv(k, 0, 0);
        return inx ? 0.5 * minmod(pc - rv(k, -1, 0), rv(k, 1, 0) - pc) : 0.0;
    };
    auto slope_y = [&](int k) {
        const double pc = rv(k, 0, 0);
        return iny ? 0.5 * minmod(pc - rv(k, 0, -1), rv(k, 0, 1) - pc) : 0.0;
    };
    // No granular layer anywhere in the stencil (h2 = q2 = 0 at the cell and
    // the neighbours it reads): eta2 = 0 - H, whose differences are exactly
    // the negated differences of H, so its slope is the negated H slope, or
    // +0 where minmod gives 0; the q2 slopes are minmod's 0, so +0; and the
    // fallback's h2 tests, 0 +- 0 against 0.5 * 0, never fire.  A warp whose
    // cells all qualify skips that FP64 work and gets the same bits.
    bool one = true;
    {
        using lsh::is_zero;
        auto nolayer = [&](int di, int dj) {
            return is_zero(w(3, di, dj)) && is_zero(w(4, di, dj)) && is_zero(w(5, di, dj));
        };
        one = nolayer(0, 0);
        if (one && i > 0) one = nolayer(-1, 0);
        if (one && i < nx - 1) one = nolayer(1, 0);
        if (one && j > 0) one = nolayer(0, -1);
        if (one && j < ny - 1) one = nolayer(0, 1);
    }
    double sx[7], sy[7];
    const bool fast = warp_all(one);
    if (fast) {
        sx[0] = slope_x(0); sy[0] = slope_y(0);
        sx[1] = slope_x(1); sy[1] = slope_y(1);
        sx[2] = slope_x(2); sy[2] = slope_y(2);
        sx[6] = slope_x(6); sy[6] = slope_y(6);
        sx[3] = lsh::is_zero(sx[6]) ? 0.0 : lshm::neg_if(sx[6], true);
        sy[3] = lsh::is_zero(sy[6]) ? 0.0 : lshm::neg_if(sy[6], true);
        sx[4] = sx[5] = sy[4] = sy[5] = 0.0;
    } else {
#pragma unroll
        for (int k = 0; k < 7; ++k) { sx[k] = slope_x(k); sy[k] = slope_y(k); }
    }
    const double h1 = w(0, 0, 0), h2 = w(3, 0, 0);
    const double dh1x = sx[0] - sx[3], dh1y = sy[0] - sy[3];
    // first order where a reconstructed depth would fall below kReconThin of
    // the cell's: a thin face with a finite discharge has an unbounded
    // velocity, whose wave speed would collapse dt
    // (the compares on the integer pipe)
    const double g1 = kReconThin * h1;
    using lshm::okey;
    const int64_t k1 = okey(g1);
    bool bad = okey(h1 + dh1x) < k1 || okey(h1 - dh1x) < k1 || okey(h1 + dh1y) < k1 || okey(h1 - dh1y) < k1;
    if (!fast) {
        const double dh2x = sx[3] + sx[6], dh2y = sy[3] + sy[6];
        const int64_t k2 = okey(kReconThin * h2);
        bad = bad || okey(h2 + dh2x) < k2 || okey(h2 - dh2x) < k2 || okey(h2 + dh2y) < k2 || okey(h2 - dh2y) < k2;
    }
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        a.sxw[k][id] = bad ? 0.0 : sx[k];
        a.syw[k][id] = bad ? 0.0 : sy[k];
    }
    if (a.szero) a.szero[id] = 0;  // conservative: only the dry path marks zeros
}

// One cell of the second-order reconstruction from global memory.
LSH_HD void recon_cell(const KArgs& a, int id) {
    const int nx = a.c.nx;
    const int j = id / nx, i = id - j * nx;
    recon_cell_from(a, id, i, j, [&](int k, int di, int dj) -> double { return a.W[k][id + di + dj * nx]; });
}

#if defined(__CUDACC__)
// Block max of the per-cell rates (non-negative doubles order like their bit
// patterns), then one 64-bit atomicMax per block.
template <int BLOCK>
__device__ __forceinline__ void block_max_bits(unsigned long long v, unsigned long long* target) {
    __shared__ unsigned long long red[BLOCK / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
        v = (w > v) ? w : v;
    }
    // linear thread index (blocks may be 2-D; warps are x-fastest)
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = (lane < BLOCK / 32) ? red[lane] : kRateInitBits;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
            v = (w > v) ? w : v;
        }
        if (lane == 0) atomicMax(target, v);
    }
}
#endif

// One cell of the Euler-stage update (k_volume); returns the bits of the
// cell's acc_w / area for the dt reduction.
// MODE 0: order 1, in place.  MODE 1: order 2 stage 1 (W -> Wout).
// MODE 2: order 2 stage 2, Wout = (Xavg + E(W)) / 2.
template <int MODE>
LSH_HD unsigned long long volume_cell(const KArgs& a, int id, double dt) {
    const int nx = a.c.nx;
    const int j = id / nx;
    double wo[6], acc[7], w[6], rate;
#pragma unroll
    for (int k = 0; k < 6; ++k) wo[k] = a.W[k][id];
#pragma unroll
    for (int k = 0; k < 7; ++k) acc[k] = a.acc[k][id];
    if (MODE != 2 && a.c.track_eta) {
        // actualizarEta1MaximaGPU (Volumen_kernel.cu:182-213): state before the step
        const double v = wo[0] - a.W[6][id];
        if (lshm::lt(a.eta_max[id], v)) { a.eta_max[id] = v; a.eta_time[id] = a.tm->t; }
    }
    // a dry, still cell with nothing flowing in maps to itself through the
    // whole update (dt contribution 1e30; its second-order pressure
    // integral is g*0*... = 0): skip the FP64 work
    bool still = true;
#pragma unroll
    for (int k = 0; k < 6; ++k) still &= lsh::is_zero(wo[k]);
#pragma unroll
    for (int k = 0; k < 7; ++k) still &= lsh::is_zero(acc[k]);
    if (still) {
#pragma unroll
        for (int k = 0; k < 6; ++k) w[k] = wo[k];
        rate = 0.0;
    } else {
        // The cell has no granular layer and receives none: wo[3..5] zero and
        // acc[3..5] +0 (bit patterns).  With finite slopes its layer-2
        // pressure term is g (+-0) (finite) = +-0, leaving acc[4], acc[5] at
        // +0, and volume_update<true> gives the general path's bits.  A warp
        // whose cells all qualify takes that path (if-converted per-lane
        // selects would still issue the FP64 work).
        using lsh::is_zero;
        bool one = is_zero(wo[3]) && is_zero(wo[4]) && is_zero(wo[5]) && lshm::bits_of(acc[3]) == 0 &&
                   lshm::bits_of(acc[4]) == 0 && lshm::bits_of(acc[5]) == 0;
        double s0x = 0.0, s3x = 0.0, s0y = 0.0, s3y = 0.0;
        if (a.c.order == 2) {
            s0x = a.sx[0][id]; s3x = a.sx[3][id]; s0y = a.sy[0][id]; s3y = a.sy[3][id];
            one = one && !lsh::is_bad(s0x) && !lsh::is_bad(s3x) && !lsh::is_bad(s0y) && !lsh::is_bad(s3y);
        }
        if (warp_all(one)) {
            if (a.c.order == 2) {
                const double gh1 = a.c.g * wo[0];
                const double wx = a.geo.wx[j], wy = a.geo.wy[j];
                acc[1] -= a.c.peso * ((gh1 * (2.0 * s0x)) * wx);
                acc[2] -= a.c.peso * ((gh1 * (2.0 * s0y)) * wy);
            }
            lsh::volume_update<true>(wo, acc, w, rate, a.geo.inv_area[j], a.geo.tanR[j], dt, a.c);
        } else {
            if (a.c.order == 2) {
                // cell-midpoint integral of g h d(eta) over the reconstructed cell
                const double gh1 = a.c.g * wo[0], gh2 = a.c.g * wo[3];
                const double e1x = 2.0 * s0x, e2x = 2.0 * s3x;
                const double e1y = 2.0 * s0y, e2y = 2.0 * s3y;
                const double wx = a.geo.wx[j], wy = a.geo.wy[j];
                acc[1] -= a.c.peso * ((gh1 * e1x) * wx);
                acc[4] -= a.c.peso * ((gh2 * lsh::fmad(a.c.omr, e2x, a.c.r * e1x)) * wx);
                acc[2] -= a.c.peso * ((gh1 * e1y) * wy);
                acc[5] -= a.c.peso * ((gh2 * lsh::fmad(a.c.omr, e2y, a.c.r * e1y)) * wy);
            }
            lsh::volume_update(wo, acc, w, rate, a.geo.inv_area[j], a.geo.tanR[j], dt, a.c);
        }
    }
    // A still cell whose output is the very bits already stored where it goes
    // skips the stores: order 1 updates in place (w == wo); stage 2 writes back
    // into the step's initial state, and the average of two equal zeros is
    // that zero.
    bool keep = false;
    if (MODE == 0 && still) {
        keep = true;
#pragma unroll
        for (int k = 0; k < 6; ++k) keep &= (a.Wout[k] == a.W[k]);
    }
    if (MODE == 2) {
        // the TVD-RK2 average 0.5 (x + w).  Where both terms are zero (every dry
        // cell) it is the AND of their patterns (+0 unless both are -0: the sum
        // of opposite zeros is +0).  A warp whose cells all have only zero terms
        // takes the AND as a whole: a per-variable select is if-converted, and
        // its predicated-off FP64 instructions still hold the FP64 pipe.
        double x[6];
        bool z = true;
        keep = still;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            x[k] = a.Xavg[k][id];
            z &= lsh::is_zero(x[k]) && lsh::is_zero(w[k]);
            keep &= (a.Wout[k] == a.Xavg[k]) && (lshm::bits_of(x[k]) == lshm::bits_of(w[k]));
        }
        if (warp_all(z)) {
#pragma unroll
            for (int k = 0; k < 6; ++k) w[k] = lshm::from_bits(lshm::bits_of(x[k]) & lshm::bits_of(w[k]));
        } else {
#pragma unroll
            for (int k = 0; k < 6; ++k) w[k] = 0.5 * (x[k] + w[k]);
        }
    }
    if (keep) return (unsigned long long)lshm::bits_of(rate);
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 6; ++k) { a.Wout[k][id] = w[k]; bad |= lsh::is_bad(w[k]); }
    if (bad) err_or(&a.tm->err, 1 << LSH_ERR_NUMERIC);
    return (unsigned long long)lshm::bits_of(rate);
}

// dt from the largest acc_w / area: 2 CFL / max rate, 1e30 when no cell has a wave speed
LSH_HD double dt_of(unsigned long long rmax_bits, double two_cfl) {
    const double m = lshm::from_bits(rmax_bits);
    return (m > 0.0) ? two_cfl / m : lsh::kBig;
}

// One edge of the initial-dt pass (procesarAristasDeltaTInicialGPU,
// Arista_kernel.cu:1129-1308): its wave-speed bound into acc[6].
template <int DIR, bool FIRST>
LSH_HD void init_wave_edge(const KArgs& a, int x, int y) {
    const int nx = a.c.nx, ny = a.c.ny;
    int id0, id1 = -1;
    double bor = 0.0, len;
    bool pos_normal = true;
    if (DIR == 0) {
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
    lsh::Face A, B;
    A.h1 = a.W[0][id0];
    A.h2 = a.W[3][id0];
    face_rest<DIR, 1>(a, id0, 0, pos_normal, A);
    if (id1 >= 0) {
        B.h1 = a.W[0][id1];
        B.h2 = a.W[3][id1];
        face_rest<DIR, 1>(a, id1, 0, pos_normal, B);
    } else {
        B = A;
        B.qn1 = A.qn1 * bor;
        B.qn2 = A.qn2 * bor;
    }
    // both faces empty and still: every term of the bound is an exact zero and
    // lmax = 0 + eps_h, so the wave is len * eps_h without the FP64 work
    using lsh::is_zero;
    const bool empty = is_zero(A.h1) && is_zero(A.h2) && is_zero(B.h1) && is_zero(B.h2) && is_zero(A.qn1) &&
                       is_zero(A.qn2) && is_zero(B.qn1) && is_zero(B.qn2);
    const double wv = empty ? len * (0.0 + a.c.eps_h) : lsh::edge_initial_wave(A, B, len, a.c);
    if (FIRST) {
        a.acc[6][id0] = 0.0 + wv;
        if (id1 >= 0) a.acc[6][id1] = 0.0 + wv;
    } else {
        a.acc[6][id0] += wv;
        if (id1 >= 0) a.acc[6][id1] += wv;
    }

}

// acc_w / area of one cell after the initial wave pass (obtenerDeltaTVolumenesGPU)
LSH_HD unsigned long long init_cell_rate(const KArgs& a, int id) {
    const int j = id / a.c.nx;
    const double w = a.acc[6][id];
    const double rate = (w < lsh::kEps) ? 0.0 : w * a.geo.inv_area[j];
    return (unsigned long long)lshm::bits_of(rate);
}

}  // namespace lsh
