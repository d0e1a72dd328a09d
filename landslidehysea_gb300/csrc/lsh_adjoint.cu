// lsh_adjoint.cu -- the discrete adjoint of the time loop on the GPU (C ABI
// in include/lsh.h, lsh_adjoint_*).
//
// Gradient of  J = w * sum_{n=1..N} sum_g (eta1_n[g] - target[n][g])^2 + <bar_final, X_N>
// (eta1 = h1 + h2 - H at the gauge cells after each step) with respect to
// the initial state (h1, q1, h2, q2 of every cell) and to the Coulomb angle,
// the Manning coefficients mf0, mfs and the density ratio r.  The step's dt
// is the CFL step of the previous state and is differentiated as such.
//
// lsh_adjoint_forward runs the N steps once, recording dt, the largest
// rate's bits and the gauge series, and stores the checkpoints of the
// binomial schedule's first descent (lsh_revolve.h) in as many state slots
// as the memory budget allows.  lsh_adjoint_gradient then walks the schedule
// backwards.  Reversing step n recomputes it from X_n with the very kernels
// of the forward (lsh_kernels.cuh), keeping what the adjoint reads: slopes,
// accumulators after each colour pass, the stage-1 state, the
// reconstruction's branch tape.  The adjoint kernels then run each stage's
// operators in reverse: volume update, the four colour passes (last first),
// reconstruction.  They use the hand-written bodies of lsh_adjoint.cuh.
// Every branch (wet/dry, Coulomb stop, limiter, eigenvalue order, minmod)
// takes the forward's direction, because the recomputation is bit-identical.
// Parameter and dt adjoints are summed per block, then in a fixed order:
// the gradient is bit-reproducible.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/lsh.h"
#include "lsh_adjoint.cuh"
#include "lsh_kernels.cuh"
#include "lsh_revolve.h"
#include "lsh_setup.h"

using lsh::AdjArgs;
using lsh::ConstBar;
using lsh::Consts;
using lsh::Geo;

namespace {

constexpr int kAdjEdgeBlock = 128;
constexpr int kAdjCellBlock = 128;
// Blocks per SM the edge and volume adjoint kernels are compiled for (their
// register budget).  One edge or cell per thread: the hardware balances the
// wet region's blocks across SMs.
#ifndef LSH_ADJ_MINBLOCKS
#define LSH_ADJ_MINBLOCKS 4
#endif
// The edge adjoint alone.  Its FP64 unit is busy about 40% of the time with
// the adjoint nonzero over a wet channel, but spills, not warps, limit it:
// a reverse sweep of 200 steps of the 1024^2 fjord (s, blocks of 128 per SM:
// registers, stack frame) took 0.89 at 2 (255, 64-96 B), 0.83 at 3 (168,
// 448 B), 0.84 at 4 (128, 640-700 B), 0.87 at 5, 0.89 at 6 and 0.90 at 8
// (64, 1 KB).
#ifndef LSH_ADJ_EDGE_MINB
#define LSH_ADJ_EDGE_MINB LSH_ADJ_MINBLOCKS
#endif

// 2-D tiles, as the forward kernels use: a warp covers a compact patch of
// the grid, so fewer warps straddle a wet/dry boundary and run half empty.
// Horizontal edges: 16 along x by 8 edge rows (warps of 16 x 2); vertical
// edges: 8 edge columns by 16 rows (warps of 8 x 4); cells: 16 x 8.
dim3 adj_edge_block(int dir) { return dir == 0 ? dim3(16, 8) : dim3(8, 16); }
dim3 adj_edge_grid(int nx, int ny, int dir, int par) {
    if (dir == 0) {
        const int nl = (ny - par) / 2 + 1;
        return dim3((unsigned)((nx + 15) / 16), (unsigned)((nl + 7) / 8));
    }
    const int nl = (nx - par) / 2 + 1;
    return dim3((unsigned)((nl + 7) / 8), (unsigned)((ny + 15) / 16));
}
dim3 adj_cell_block() { return dim3(16, 8); }
dim3 adj_cell_grid(int nx, int ny) { return dim3((unsigned)((nx + 15) / 16), (unsigned)((ny + 7) / 8)); }
long long blocks_of(dim3 g) { return (long long)g.x * g.y; }
constexpr int kRed = 9;        // dt adjoint + the 8 constant adjoints
constexpr int kPartSlots = 11;  // partial-sum launches per reversed step (2 stages x 5, + initial dt)

// ------------------------------------------------------------------ device helpers

// Block sums of the 9 partials into out[0..8].  The partials start at +0
// and stay +0 where nothing contributed, so an all-zero block writes +0 and
// an all-zero component of a warp keeps its +0 without the FP64 shuffle
// tree: the same sums, without the adds over the dry region.
template <int BLOCK>
__device__ void block_sum9(double v[kRed], double* out) {
    __shared__ double sh[BLOCK / 32][kRed];
    // linear thread index (blocks are 2-D; warps are x-fastest)
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    bool nz = false;
#pragma unroll
    for (int k = 0; k < kRed; ++k) nz |= !lsh::is_zero(v[k]);
    if (!__syncthreads_or(nz)) {
        if (tid < kRed) out[tid] = 0.0;
        return;
    }
#pragma unroll
    for (int k = 0; k < kRed; ++k) {
        if (__any_sync(0xffffffffu, !lsh::is_zero(v[k]))) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
        }
    }
    const int lane = tid & 31, warp = tid >> 5;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < kRed; ++k) sh[warp][k] = v[k];
    }
    __syncthreads();
    if (tid < kRed) {
        double s = 0.0;
        for (int w = 0; w < BLOCK / 32; ++w) s += sh[w][tid];
        out[tid] = s;
    }
}

__device__ void pack9(double dtb, const ConstBar& cb, double v[kRed]) {
    v[0] = dtb; v[1] = cb.r; v[2] = cb.omr; v[3] = cb.gp; v[4] = cb.inv_gp;
    v[5] = cb.mu; v[6] = cb.g_mf02; v[7] = cb.g_mfs2; v[8] = cb.eps_1r;
}

// Where the stage-1 dt rate peaks and the adjoint of that rate.
struct RateSel {
    long long cell;
    double bar;
};

// One edge per thread over a 2-D tile (adj_edge_block); one partial-sum row
// per block.
template <int DIR, bool FIRST, int ORDER>
__global__ void __launch_bounds__(kAdjEdgeBlock, LSH_ADJ_EDGE_MINB) k_adj_edges(AdjArgs a, const RateSel* rs, int par, double* part) {
    a.rate_cell = rs ? rs->cell : -1;
    a.rate_bar = rs ? rs->bar : 0.0;
    const int nx = a.c.nx, ny = a.c.ny;
    const int u = blockIdx.x * blockDim.x + threadIdx.x, w = blockIdx.y * blockDim.y + threadIdx.y;
    double dtb = 0.0;
    ConstBar cb;
    lsh::cb_zero(cb);
    if (DIR == 0) {
        // u: x along the edge row, w: edge row index t (y = par + 2 t)
        if (u < nx && w < (ny - par) / 2 + 1) lsh::edge_adj_body<0, FIRST, ORDER>(a, u, par + 2 * w, dtb, cb);
    } else {
        // u: edge column index t (x = par + 2 t), w: row y
        if (u < (nx - par) / 2 + 1 && w < ny) lsh::edge_adj_body<1, false, ORDER>(a, par + 2 * u, w, dtb, cb);
    }
    double v[kRed];
    pack9(dtb, cb, v);
    block_sum9<kAdjEdgeBlock>(v, part + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * kRed);
}

// One cell per thread over 16 x 8 tiles.
template <int MODE>
__global__ void __launch_bounds__(kAdjCellBlock, LSH_ADJ_MINBLOCKS) k_adj_volume(AdjArgs a, const RateSel* rs, double* part) {
    a.rate_cell = rs ? rs->cell : -1;
    a.rate_bar = rs ? rs->bar : 0.0;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    double dtb = 0.0;
    ConstBar cb;
    lsh::cb_zero(cb);
    if (i < a.c.nx && j < a.c.ny) lsh::volume_adj_body<MODE>(a, j * a.c.nx + i, dtb, cb);
    double v[kRed];
    pack9(dtb, cb, v);
    block_sum9<kAdjCellBlock>(v, part + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * kRed);
}

__global__ void __launch_bounds__(kAdjCellBlock) k_adj_recon(AdjArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < a.c.nx && j < a.c.ny) lsh::recon_adj_cell(a, j * a.c.nx + i);
}

// The recomputation's reconstruction: slopes (bit-identical to k_recon's)
// and the branch tape the reconstruction adjoint replays.
// The reconstruction with its branch tape, in the step's cell tiles (so it
// can take part in the overlapped passes through `d`).
__global__ void __launch_bounds__(kCellBlock, 8) k_recon_tape(KArgs a, unsigned* tape, Dep d = Dep{}) {
    if (d.done || d.wait) {
        const int y0 = blockIdx.y * kCellBY;
        dep_begin(d, a.tm, max(y0 - 1, 0), min(y0 + kCellBY, a.c.ny - 1));
    }
    const int id = cell_of_thread(a.c.nx, a.c.ny);
    if (id >= 0) tape[id] = lsh::recon_cell_tape(a, id);
    dep_end(d);
}

// Max and arg-max (lowest cell on ties) of acc_w / area (0 below EPSILON).
__global__ void __launch_bounds__(kCellBlock) k_adj_rate_max(const double* acc6, Geo geo, int nx, long long N,
                                                             unsigned long long* rmax) {
    unsigned long long bits = 0;
    for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < N; id += (long long)gridDim.x * blockDim.x) {
        const double w = acc6[id];
        const double rate = (w < lsh::kEps) ? 0.0 : w * geo.inv_area[id / nx];
        const unsigned long long b = lshm::bits_of(rate);
        bits = (b > bits) ? b : bits;
    }
    lsh::block_max_bits<kCellBlock>(bits, rmax);
}

__global__ void __launch_bounds__(kCellBlock) k_adj_argmax(const double* acc6, Geo geo, int nx, long long N,
                                                           const unsigned long long* rmax, long long* cell) {
    const unsigned long long m = *rmax;
    for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < N; id += (long long)gridDim.x * blockDim.x) {
        const double w = acc6[id];
        const double rate = (w < lsh::kEps) ? 0.0 : w * geo.inv_area[id / nx];
        if (m != 0 && lshm::bits_of(rate) == m) atomicMin((unsigned long long*)cell, (unsigned long long)id);
    }
}

// dt' = 2 CFL / R: the adjoint of the largest rate R is -dt'bar dt' / R (the
// volume adjoint turns it into acc_w's, times 1 / area, at the arg-max cell).
__global__ void k_adj_ratebar(const unsigned long long* rmax, const long long* cell, const double* red,
                              const double* dt_next, RateSel* out) {
    const double R = lshm::from_bits(*rmax);
    const long long c = *cell;
    const double dtb = red[0];
    if (!(R > 0.0) || c < 0 || c == 0x7fffffffffffffffLL || dtb == 0.0) {
        out->cell = -1;
        out->bar = 0.0;
        return;
    }
    out->cell = c;
    out->bar = -dtb * (*dt_next / R);
}

// The misfit's adjoint at the state after a step: 2 w (eta - target) at each gauge.
__global__ void k_adj_gauges(double* hb1, double* hb2, const int* gauges, int ng, const double* eta, const double* tgt,
                             double w) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const int id = gauges[g];
    // several gauges may share a cell: one thread adds them all, in order
    if (g > 0) {
        for (int h = 0; h < g; ++h)
            if (gauges[h] == id) return;
    }
    double s = 0.0;
    for (int h = g; h < ng; ++h)
        if (gauges[h] == id) s += w * (2.0 * (eta[h] - tgt[h]));
    hb1[id] += s;
    hb2[id] += s;
}

// Thin-layer projection: the adjoint of a layer thinner than h_adj (in the
// state the adjoint belongs to) is zeroed; the tangent-linear model zeroes
// the same tangents, so the pair stays transposes of each other.
__global__ void __launch_bounds__(kCellBlock) k_adj_project(double* b0, double* b1, double* b2,
                                                            double* b3, double* b4, double* b5, const double* h1,
                                                            const double* h2, long long N, double h_adj) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
        if (h1[i] < h_adj) { b0[i] = 0.0; b1[i] = 0.0; b2[i] = 0.0; }
        if (h2[i] < h_adj) { b3[i] = 0.0; b4[i] = 0.0; b5[i] = 0.0; }
    }
}

__global__ void k_adj_init(AdjArgs a, const RateSel* rs, double* part) {
    double v[kRed] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (threadIdx.x == 0 && rs->cell >= 0) {
        ConstBar cb;
        lsh::cb_zero(cb);
        // rate = acc_w / area at the arg-max cell
        lsh::init_wave_adj_cell(a, (int)rs->cell, rs->bar * a.geo.inv_area[rs->cell / a.c.nx], cb);
        pack9(0.0, cb, v);
    }
    block_sum9<32>(v, part);
}

// Sum the step's partials in a fixed order: red[0] = the dt adjoint of the
// step's input dt; red[1..8] += the constant adjoints.  Warp k sums
// component k (lane-strided, then a shuffle tree): deterministic.
__global__ void __launch_bounds__(32 * kRed) k_adj_reduce(const double* part, int nparts, double* red) {
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double s = 0.0;
    for (int i = lane; i < nparts; i += 32) s += part[(size_t)i * kRed + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) {
        if (k == 0) red[0] = s;
        else red[k] += s;
    }
}

// First level of the partial sums: block b adds rows [b chunk, (b+1) chunk)
// into row b of out (warp k: component k, lane-strided then a shuffle tree),
// a fixed order, so the total stays bit-reproducible.
__global__ void __launch_bounds__(32 * kRed) k_adj_reduce_rows(const double* part, long long nparts, long long chunk,
                                                               double* out) {
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long r0 = (long long)blockIdx.x * chunk;
    const long long r1 = (r0 + chunk < nparts) ? r0 + chunk : nparts;
    double s = 0.0;
    for (long long i = r0 + lane; i < r1; i += 32) s += part[(size_t)i * kRed + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) out[(size_t)blockIdx.x * kRed + k] = s;
}

__global__ void k_set_dt(lsh::TimeRec* tm, const double* dt) {
    tm->dt = *dt;
    tm->rmax_bits = kRateInitBits;
    tm->done = 0;
    tm->err = 0;
    tm->t_end = INFINITY;
}

__global__ void k_record(const lsh::TimeRec* tm, double* dt_out) { *dt_out = tm->dt; }

__global__ void k_gauge_eta(const double* h1, const double* h2, const double* H, const int* gauges, int ng, double* eta) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const int id = gauges[g];
    eta[g] = (h1[id] + h2[id]) - H[id];
}

__global__ void k_init_cell(long long* cell) { *cell = 0x7fffffffffffffffLL; }

int afail(cudaError_t e, const char* what) {
    lsh::set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    (void)cudaGetLastError();
    return (e == cudaErrorMemoryAllocation) ? LSH_ERR_GPU_OOM : LSH_ERR_CUDA;
}

#define A_CUDA(call)                                        \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return afail(e_, #call);     \
    } while (0)

}  // namespace

// ------------------------------------------------------------------ object

struct lsh_adjoint {
    lsh_params p;
    Consts c;
    int device = 0;
    int sms = 152;
    cudaStream_t stream = nullptr;
    size_t N = 0, npad = 0;
    int order = 1;
    // one slab for the working arrays
    void* slab = nullptr;
    double* X[7] = {};         // current state (X[6] = H)
    double* Y[6] = {};         // stage-1 output (order 2)
    double* s1x[7] = {}, *s1y[7] = {}, *s2x[7] = {}, *s2y[7] = {};
    double* acc1[7] = {}, *acc2[7] = {};
    double* snap1[3][2] = {}, *snap2[3][2] = {};
    double* Xb[6] = {}, *Xbn[6] = {}, *Yb[6] = {};
    double* sxb[7] = {}, *syb[7] = {}, *accb[7] = {};
    double* eta_dummy = nullptr;
    unsigned* tape1 = nullptr, *tape2 = nullptr;
    unsigned char* szero1 = nullptr, *szero2 = nullptr;  // slope-zero flags of s1x/s1y and s2x/s2y
    unsigned* dep_ctr = nullptr;    // pass-overlap counters of one step (13 segments of dep_stride)
    int dep_stride = 0;             // 0: the passes run fully ordered
    double* geo_buf = nullptr;
    Geo geo{};
    lsh::TimeRec* tm = nullptr;
    unsigned long long* rmax = nullptr;  // scratch for the arg-max
    long long* argmax = nullptr;
    RateSel* rsel = nullptr;
    double* part = nullptr;    // part_rows x kRed partial sums
    long long part_rows = 0;
    double* part2 = nullptr;   // 128 x kRed first-level sums
    double* red = nullptr;     // kRed
    // checkpoints
    double* slots = nullptr;
    int n_slots = 0;
    double budget = 180e9;
    // the recorded forward
    int nsteps = 0;
    double* d_dts = nullptr;               // nsteps + 1
    int ng = 0;
    int* d_gauges = nullptr;
    double* d_eta = nullptr;               // nsteps * ng
    double* d_tgt = nullptr;               // nsteps * ng
    bool have_target = false;
    double misfit_weight = 1.0;
    double h_adj = 0.0;       // thin-layer projection threshold (0: the exact adjoint)
    double* hN[2] = {};       // h1, h2 of the recorded run's final state
    std::vector<double> h_dts;
    std::vector<double> h_eta;  // the gauge series, nsteps x ng
    double h_red[kRed] = {};    // dt and constant adjoints after the sweep
    bool in_batch = false;      // a member of an lsh_adjoint_batch (destroyed with it)
    bool have_forward = false;
    bool spine_stored = false;  // slots 1.. hold the first descent (until a reverse sweep reuses them)
    int cur_step = -1;          // step of the state in X
    int grid = 0;
    lsh_adjoint_stats stats{};
    std::vector<int> spine;  // steps stored in slots 1, 2, ... by the forward sweep
};

namespace {

KArgs fwd_args(const lsh_adjoint* A, const double* const* W, double* const* Wout, const double* const* Xavg,
               double* const* acc, double* const* sx, double* const* sy) {
    KArgs a;
    std::memset(&a, 0, sizeof(a));
    a.c = A->c;
    a.geo = A->geo;
    for (int k = 0; k < 7; ++k) {
        a.W[k] = W[k];
        a.acc[k] = acc[k];
        a.sx[k] = sx ? sx[k] : nullptr;
        a.sy[k] = sy ? sy[k] : nullptr;
        a.sxw[k] = sx ? sx[k] : nullptr;
        a.syw[k] = sy ? sy[k] : nullptr;
    }
    for (int k = 0; k < 6; ++k) { a.Wout[k] = Wout ? Wout[k] : nullptr; a.Xavg[k] = Xavg ? Xavg[k] : nullptr; }
    a.eta_max = A->eta_dummy;
    a.eta_time = A->eta_dummy;
    a.tm = A->tm;
    // each stage's slope set has its own flags (the edges' empty-cell test reads them)
    a.szero = (sx == A->s1x) ? A->szero1 : (sx == A->s2x) ? A->szero2 : nullptr;
    return a;
}

dim3 grid_h(const lsh_adjoint* A, int par) { return edge_grid_h(A->p.nx, A->p.ny, par); }
dim3 grid_v(const lsh_adjoint* A, int par) { return edge_grid_v(A->p.nx, A->p.ny, par); }
unsigned cell_blocks(const lsh_adjoint* A) { return unsigned((A->N + kCellBlock - 1) / kCellBlock); }

// The four colour passes of one stage; snaps (may be null) get acc[0], acc[3]
// after the first three.
template <int ORDER>
void fwd_passes(const lsh_adjoint* A, const KArgs& a, double* snaps[3][2], double* const* acc, cudaStream_t s) {
    const size_t bytes = A->N * sizeof(double);
    k_edges_h<true, ORDER><<<grid_h(A, 0), edge_block_h(), 0, s>>>(a, 0);
    if (snaps) { cudaMemcpyAsync(snaps[0][0], acc[0], bytes, cudaMemcpyDeviceToDevice, s); cudaMemcpyAsync(snaps[0][1], acc[3], bytes, cudaMemcpyDeviceToDevice, s); }
    k_edges_h<false, ORDER><<<grid_h(A, 1), edge_block_h(), 0, s>>>(a, 1);
    if (snaps) { cudaMemcpyAsync(snaps[1][0], acc[0], bytes, cudaMemcpyDeviceToDevice, s); cudaMemcpyAsync(snaps[1][1], acc[3], bytes, cudaMemcpyDeviceToDevice, s); }
    k_edges_v<ORDER><<<grid_v(A, 0), edge_block_v(), 0, s>>>(a, 0);
    if (snaps) { cudaMemcpyAsync(snaps[2][0], acc[0], bytes, cudaMemcpyDeviceToDevice, s); cudaMemcpyAsync(snaps[2][1], acc[3], bytes, cudaMemcpyDeviceToDevice, s); }
    k_edges_v<ORDER><<<grid_v(A, 1), edge_block_v(), 0, s>>>(a, 1);
}

// One forward step X -> X (the product's step: the same kernels and order),
// with the time record's dt; k_advance leaves the next dt in the record.
void fwd_step(const lsh_adjoint* A, cudaStream_t s) {
    const dim3 nbc = cell_grid(A->p.nx, A->p.ny);
    double* const* X = A->X;
    if (A->dep_ctr) {
        // the product's overlapped step (lsh_kernels.cuh)
        double* Y7[7];
        for (int k = 0; k < 6; ++k) Y7[k] = A->Y[k];
        Y7[6] = A->X[6];
        const KArgs a1 = (A->order == 1) ? fwd_args(A, X, X, nullptr, A->acc1, nullptr, nullptr)
                                         : fwd_args(A, X, A->Y, nullptr, A->acc1, A->s1x, A->s1y);
        const KArgs a2 = (A->order == 1) ? a1 : fwd_args(A, Y7, X, X, A->acc2, A->s2x, A->s2y);
        enqueue_step_overlap(A->p.nx, A->p.ny, A->order, a1, a2, A->dep_ctr, A->dep_stride, A->tm, 2.0 * A->c.cfl, s);
        return;
    }
    if (A->order == 1) {
        const KArgs a = fwd_args(A, X, X, nullptr, A->acc1, nullptr, nullptr);
        fwd_passes<1>(A, a, nullptr, A->acc1, s);
        k_volume<0><<<nbc, cell_block(), 0, s>>>(a);
    } else {
        double* Y7[7];
        for (int k = 0; k < 6; ++k) Y7[k] = A->Y[k];
        Y7[6] = A->X[6];
        const KArgs a1 = fwd_args(A, X, A->Y, nullptr, A->acc1, A->s1x, A->s1y);
        k_recon<<<nbc, cell_block(), 0, s>>>(a1);
        fwd_passes<2>(A, a1, nullptr, A->acc1, s);
        k_volume<1><<<nbc, cell_block(), 0, s>>>(a1);
        const KArgs a2 = fwd_args(A, Y7, X, X, A->acc2, A->s2x, A->s2y);
        k_recon<<<nbc, cell_block(), 0, s>>>(a2);
        fwd_passes<2>(A, a2, nullptr, A->acc2, s);
        k_volume<2><<<nbc, cell_block(), 0, s>>>(a2);
    }
    k_advance<<<1, 1, 0, s>>>(A->tm, 2.0 * A->c.cfl);
}

AdjArgs adj_args(const lsh_adjoint* A, const double* const* W, const double* const* sx, const double* const* sy,
                 double* const* acc, double* const* Wbar, const double* const* wbar, double* const* Xbar,
                 const unsigned* tape, double dt) {
    AdjArgs a;
    std::memset(&a, 0, sizeof(a));
    a.c = A->c;
    a.geo = A->geo;
    for (int k = 0; k < 7; ++k) {
        a.W[k] = W[k];
        a.sx[k] = sx ? sx[k] : nullptr;
        a.sy[k] = sy ? sy[k] : nullptr;
        a.acc[k] = acc ? acc[k] : nullptr;
        a.sxb[k] = A->sxb[k];
        a.syb[k] = A->syb[k];
        a.accb[k] = A->accb[k];
    }
    for (int k = 0; k < 6; ++k) {
        a.Wbar[k] = Wbar[k];
        a.wbar[k] = wbar ? wbar[k] : nullptr;
        a.Xbar[k] = Xbar ? Xbar[k] : nullptr;
    }
    a.tape = tape;
    a.rate_cell = -1;
    a.dt = dt;
    return a;
}

// Reverse of one stage: volume (MODE), passes last-first, reconstruction.
// Each launch writes one partial-sum row per block at A->part + *nparts;
// *nparts advances by the blocks launched.
template <int ORDER, int MODE>
void rev_stage(lsh_adjoint* A, AdjArgs a, double* snaps[3][2], const RateSel* rs, long long* nparts, cudaStream_t s) {
    const int nx = A->p.nx, ny = A->p.ny;
    dim3 g = adj_cell_grid(nx, ny);
    k_adj_volume<MODE><<<g, adj_cell_block(), 0, s>>>(a, rs, A->part + *nparts * kRed);
    *nparts += blocks_of(g);
    a.snap[0] = snaps[2][0]; a.snap[1] = snaps[2][1];
    g = adj_edge_grid(nx, ny, 1, 1);
    k_adj_edges<1, false, ORDER><<<g, adj_edge_block(1), 0, s>>>(a, rs, 1, A->part + *nparts * kRed);
    *nparts += blocks_of(g);
    a.snap[0] = snaps[1][0]; a.snap[1] = snaps[1][1];
    g = adj_edge_grid(nx, ny, 1, 0);
    k_adj_edges<1, false, ORDER><<<g, adj_edge_block(1), 0, s>>>(a, rs, 0, A->part + *nparts * kRed);
    *nparts += blocks_of(g);
    a.snap[0] = snaps[0][0]; a.snap[1] = snaps[0][1];
    g = adj_edge_grid(nx, ny, 0, 1);
    k_adj_edges<0, false, ORDER><<<g, adj_edge_block(0), 0, s>>>(a, rs, 1, A->part + *nparts * kRed);
    *nparts += blocks_of(g);
    a.snap[0] = a.snap[1] = nullptr;
    g = adj_edge_grid(nx, ny, 0, 0);
    k_adj_edges<0, true, ORDER><<<g, adj_edge_block(0), 0, s>>>(a, rs, 0, A->part + *nparts * kRed);
    *nparts += blocks_of(g);
    if (ORDER == 2) k_adj_recon<<<adj_cell_grid(nx, ny), adj_cell_block(), 0, s>>>(a);
}

void zero6(double* const* v, size_t N, cudaStream_t s) {
    for (int k = 0; k < 6; ++k) cudaMemsetAsync(v[k], 0, N * sizeof(double), s);
}

// The misfit's adjoint at X_m (m >= 1: the gauges after step m - 1) added to
// A->Xb, then the thin-layer projection with the depths h1, h2 of X_m.
void misfit_and_project(lsh_adjoint* A, int m, const double* h1, const double* h2, cudaStream_t s) {
    if (m >= 1 && A->have_target && A->ng > 0 && A->misfit_weight != 0.0)
        k_adj_gauges<<<(A->ng + 127) / 128, 128, 0, s>>>(A->Xb[0], A->Xb[3], A->d_gauges, A->ng,
                                                         A->d_eta + (size_t)(m - 1) * A->ng,
                                                         A->d_tgt + (size_t)(m - 1) * A->ng, A->misfit_weight);
    if (A->h_adj > 0.0)
        k_adj_project<<<A->grid, kCellBlock, 0, s>>>(A->Xb[0], A->Xb[1], A->Xb[2], A->Xb[3], A->Xb[4], A->Xb[5],
                                                     h1, h2, (long long)A->N, A->h_adj);
}

struct Ops : lsh::RevolveOps {
    lsh_adjoint* A;
    int status = 0;
    explicit Ops(lsh_adjoint* a) : A(a) {}
    double* slot(int k, int v) const { return A->slots + ((size_t)k * 6 + v) * A->npad; }
    int advance(int from, int to) override {
        for (int n = from; n < to; ++n) {
            k_set_dt<<<1, 1, 0, A->stream>>>(A->tm, A->d_dts + n);
            fwd_step(A, A->stream);
            A->stats.recompute_steps += 1;
        }
        A_CUDA(cudaGetLastError());
        return 0;
    }
    int store(int k) override {
        for (int v = 0; v < 6; ++v)
            A_CUDA(cudaMemcpyAsync(slot(k, v), A->X[v], A->N * sizeof(double), cudaMemcpyDeviceToDevice, A->stream));
        return 0;
    }
    int restore(int k, int) override {
        for (int v = 0; v < 6; ++v)
            A_CUDA(cudaMemcpyAsync(A->X[v], slot(k, v), A->N * sizeof(double), cudaMemcpyDeviceToDevice, A->stream));
        return 0;
    }
    int reverse_step(int n) override;
};

// Adjoint of step n; the current state is X_n, A->Xb holds the adjoint of
// X_{n+1}, A->red[0] the adjoint of dt_{n+1}.  Leaves the adjoint of X_n in
// A->Xb and of dt_n in A->red[0].
int Ops::reverse_step(int n) {
    cudaStream_t s = A->stream;
    const size_t N = A->N;
    const unsigned nb = cell_blocks(A);
    const dim3 nbc = cell_grid(A->p.nx, A->p.ny);
    const int G = A->grid;
    // recompute step n's intermediates
    k_set_dt<<<1, 1, 0, s>>>(A->tm, A->d_dts + n);
    double* const* X = A->X;
    const double dt = A->h_dts[n];
    if (A->dep_ctr) {
        // overlapped passes; the edge passes take the accumulator snapshots
        // themselves, at the cells the reverse sweep reads them
        unsigned* c = A->dep_ctr;
        const int st = A->dep_stride, nx = A->p.nx, ny = A->p.ny;
        if (A->order == 1) {
            const KArgs a = fwd_args(A, X, nullptr, nullptr, A->acc1, nullptr, nullptr);
            enqueue_stage_overlap<1, -1>(nx, ny, a, s, Dep{}, c, st, true, A->snap1);
        } else {
            double* Y7[7];
            for (int k = 0; k < 6; ++k) Y7[k] = A->Y[k];
            Y7[6] = A->X[6];
            const KArgs a1 = fwd_args(A, X, A->Y, nullptr, A->acc1, A->s1x, A->s1y);
            Dep r1;
            r1.done = c;
            launch_pass(false, nbc, cell_block(), s, k_recon_tape, a1, A->tape1, r1);
            Dep pr;
            pr.wait = c; pr.target = nbc.x; pr.kind = kDepCell; pr.ntiles = (int)nbc.y;
            const Dep v1 = enqueue_stage_overlap<2, 1>(nx, ny, a1, s, pr, c + st, st, false, A->snap1);
            const KArgs a2 = fwd_args(A, Y7, nullptr, nullptr, A->acc2, A->s2x, A->s2y);
            Dep r2 = v1;
            r2.done = c + 6 * st;
            launch_pass(true, nbc, cell_block(), s, k_recon_tape, a2, A->tape2, r2);
            Dep pr2;
            pr2.wait = c + 6 * st; pr2.target = nbc.x; pr2.kind = kDepCell; pr2.ntiles = (int)nbc.y;
            enqueue_stage_overlap<2, -1>(nx, ny, a2, s, pr2, c + 7 * st, st, true, A->snap2);
        }
        // ordered after the passes (a stream operation waits for them all)
        cudaMemsetAsync(c, 0, size_t(13) * st * sizeof(unsigned), s);
    } else if (A->order == 1) {
        const KArgs a = fwd_args(A, X, nullptr, nullptr, A->acc1, nullptr, nullptr);
        fwd_passes<1>(A, a, A->snap1, A->acc1, s);
    } else {
        double* Y7[7];
        for (int k = 0; k < 6; ++k) Y7[k] = A->Y[k];
        Y7[6] = A->X[6];
        const KArgs a1 = fwd_args(A, X, A->Y, nullptr, A->acc1, A->s1x, A->s1y);
        k_recon_tape<<<nbc, cell_block(), 0, s>>>(a1, A->tape1);
        fwd_passes<2>(A, a1, A->snap1, A->acc1, s);
        k_volume<1><<<nbc, cell_block(), 0, s>>>(a1);
        const KArgs a2 = fwd_args(A, Y7, nullptr, nullptr, A->acc2, A->s2x, A->s2y);
        k_recon_tape<<<nbc, cell_block(), 0, s>>>(a2, A->tape2);
        fwd_passes<2>(A, a2, A->snap2, A->acc2, s);
    }
    // the stage-1 rate's arg-max and the adjoint of the rate
    cudaMemsetAsync(A->rmax, 0, sizeof(unsigned long long), s);
    k_init_cell<<<1, 1, 0, s>>>(A->argmax);
    k_adj_rate_max<<<G, kCellBlock, 0, s>>>(A->acc1[6], A->geo, A->p.nx, (long long)N, A->rmax);
    k_adj_argmax<<<G, kCellBlock, 0, s>>>(A->acc1[6], A->geo, A->p.nx, (long long)N, A->rmax, A->argmax);
    k_adj_ratebar<<<1, 1, 0, s>>>(A->rmax, A->argmax, A->red, A->d_dts + n + 1, A->rsel);
    zero6(A->Xbn, N, s);
    long long nparts = 0;
    if (A->order == 1) {
        AdjArgs a = adj_args(A, X, nullptr, nullptr, A->acc1, A->Xbn, A->Xb, nullptr, nullptr, dt);
        rev_stage<1, 0>(A, a, A->snap1, A->rsel, &nparts, s);
    } else {
        double* Y7[7];
        for (int k = 0; k < 6; ++k) Y7[k] = A->Y[k];
        Y7[6] = A->X[6];
        zero6(A->Yb, N, s);
        AdjArgs a2 = adj_args(A, Y7, A->s2x, A->s2y, A->acc2, A->Yb, A->Xb, A->Xbn, A->tape2, dt);
        rev_stage<2, 2>(A, a2, A->snap2, nullptr, &nparts, s);
        AdjArgs a1 = adj_args(A, X, A->s1x, A->s1y, A->acc1, A->Xbn, A->Yb, nullptr, A->tape1, dt);
        rev_stage<2, 1>(A, a1, A->snap1, A->rsel, &nparts, s);
    }
    {
        constexpr int kRows = 128;
        const long long chunk = (nparts + kRows - 1) / kRows;
        k_adj_reduce_rows<<<kRows, 32 * kRed, 0, s>>>(A->part, nparts, chunk, A->part2);
        k_adj_reduce<<<1, 32 * kRed, 0, s>>>(A->part2, kRows, A->red);
    }
    for (int k = 0; k < 6; ++k) std::swap(A->Xb[k], A->Xbn[k]);
    if (n >= 1) misfit_and_project(A, n, A->X[0], A->X[3], s);
    A->stats.reversed_steps += 1;
    A_CUDA(cudaGetLastError());
    return 0;
}

// ------------------------------------------------------------------ phases
//
// lsh_adjoint_forward and lsh_adjoint_gradient run these for one adjoint;
// lsh_adjoint_batch_* runs them for every member in lockstep, so that each
// member's stream holds a few steps of work at a time and the members'
// kernels overlap.  All of it is asynchronous on A->stream except the copies
// into pageable host memory, which wait for the stream to reach them.

// The initial-dt wave pass over X (the same kernels as lsh_set_state).
void init_wave_pass(const lsh_adjoint* A, const KArgs& a, cudaStream_t s) {
    const int nx = A->p.nx, ny = A->p.ny;
    launch_init_wave(a, nx, ny, s);
}

// The steps after which the forward sweep stores a checkpoint: the binomial
// schedule's first descent over [0, nsteps) with `slots` slots, slot 0
// holding X_0.
std::vector<int> spine_steps(int nsteps, int slots) {
    std::vector<int> v;
    int a = 0, free = slots - 1;
    while (nsteps - a > 1 && free > 0) {
        const int m = a + (int)lsh::revolve_split(nsteps - a, free + 1);
        v.push_back(m);
        a = m;
        --free;
    }
    return v;
}

double slot_bytes_of(const lsh_adjoint* A) { return 6.0 * A->npad * sizeof(double); }

// The per-step records for nsteps and `want` checkpoint slots.  On
// LSH_ERR_GPU_OOM no slots are held.
int fwd_alloc(lsh_adjoint* A, int nsteps, int want) {
    if (nsteps != A->nsteps) {
        cudaFree(A->d_dts); cudaFree(A->d_eta); cudaFree(A->d_tgt);
        A->d_dts = nullptr; A->d_eta = nullptr; A->d_tgt = nullptr;
        A->nsteps = 0;
        A_CUDA(cudaMalloc(&A->d_dts, sizeof(double) * (nsteps + 1)));
        if (A->ng > 0) {
            A_CUDA(cudaMalloc(&A->d_eta, sizeof(double) * (size_t)nsteps * A->ng));
            A_CUDA(cudaMalloc(&A->d_tgt, sizeof(double) * (size_t)nsteps * A->ng));
        }
        A->nsteps = nsteps;
    }
    if (want != A->n_slots) {
        cudaFree(A->slots);
        A->slots = nullptr;
        A->n_slots = 0;
        A_CUDA(cudaMalloc(&A->slots, (size_t)want * (size_t)slot_bytes_of(A)));
        A->n_slots = want;
    }
    return 0;
}

// Uploads X_0 and the target, runs the initial-dt pass, stores X_0 in slot 0.
int fwd_begin(lsh_adjoint* A, const double* const host_state[LSH_NVARS], const double* target) {
    cudaStream_t s = A->stream;
    const size_t N = A->N;
    A->have_forward = false;
    A->spine_stored = false;
    A->cur_step = -1;
    A->have_target = (target != nullptr) && A->ng > 0;
    if (A->have_target)
        A_CUDA(cudaMemcpyAsync(A->d_tgt, target, sizeof(double) * (size_t)A->nsteps * A->ng, cudaMemcpyHostToDevice, s));
    for (int k = 0; k < 7; ++k)
        A_CUDA(cudaMemcpyAsync(A->X[k], host_state[k], N * sizeof(double), cudaMemcpyHostToDevice, s));
    lsh::TimeRec init{};
    init.t_end = INFINITY;
    A_CUDA(cudaMemcpyAsync(A->tm, &init, sizeof(init), cudaMemcpyHostToDevice, s));
    const KArgs a = fwd_args(A, A->X, nullptr, nullptr, A->acc1, nullptr, nullptr);
    init_wave_pass(A, a, s);
    k_cell_dt<<<cell_grid(A->p.nx, A->p.ny), cell_block(), 0, s>>>(a);
    k_init_finish<<<1, 1, 0, s>>>(A->tm, 2.0 * A->c.cfl);
    k_record<<<1, 1, 0, s>>>(A->tm, A->d_dts);
    A_CUDA(cudaGetLastError());
    A->stats = lsh_adjoint_stats{};
    A->stats.slots = A->n_slots;
    A->stats.nsteps = A->nsteps;
    A->stats.slot_bytes = slot_bytes_of(A);
    A->spine.clear();
    Ops ops(A);
    return ops.store(0);
}

// Step n -> n + 1 with its dt and gauge records.
int fwd_record_step(lsh_adjoint* A, int n) {
    cudaStream_t s = A->stream;
    fwd_step(A, s);
    k_record<<<1, 1, 0, s>>>(A->tm, A->d_dts + n + 1);
    if (A->ng > 0)
        k_gauge_eta<<<(A->ng + 127) / 128, 128, 0, s>>>(A->X[0], A->X[3], A->X[6], A->d_gauges, A->ng,
                                                       A->d_eta + (size_t)n * A->ng);
    A->stats.forward_steps += 1;
    A_CUDA(cudaGetLastError());
    return 0;
}

// After step N: the final depths (the projection at N reads them), then the
// dt and gauge records into host memory.
int fwd_end(lsh_adjoint* A) {
    cudaStream_t s = A->stream;
    const size_t N = A->N;
    A_CUDA(cudaMemcpyAsync(A->hN[0], A->X[0], N * sizeof(double), cudaMemcpyDeviceToDevice, s));
    A_CUDA(cudaMemcpyAsync(A->hN[1], A->X[3], N * sizeof(double), cudaMemcpyDeviceToDevice, s));
    A->h_dts.resize(A->nsteps + 1);
    A->h_eta.resize((size_t)A->nsteps * A->ng);
    A_CUDA(cudaMemcpyAsync(A->h_dts.data(), A->d_dts, sizeof(double) * (A->nsteps + 1), cudaMemcpyDeviceToHost, s));
    if (A->ng > 0)
        A_CUDA(cudaMemcpyAsync(A->h_eta.data(), A->d_eta, sizeof(double) * A->h_eta.size(), cudaMemcpyDeviceToHost, s));
    return 0;
}

// Waits for the forward run; the misfit and the gauge series.
int fwd_host(lsh_adjoint* A, const double* target, double* misfit, double* gauge_series) {
    A_CUDA(cudaStreamSynchronize(A->stream));
    double J = 0.0;
    if (A->have_target)
        for (size_t i = 0; i < A->h_eta.size(); ++i) { const double d = A->h_eta[i] - target[i]; J = lshm::fmad(d, d, J); }
    if (misfit) *misfit = J;
    if (gauge_series && A->ng > 0) std::memcpy(gauge_series, A->h_eta.data(), sizeof(double) * A->h_eta.size());
    A->have_forward = true;
    A->spine_stored = true;
    A->cur_step = A->nsteps;
    return 0;
}

// The adjoint at X_N: the final state's cotangent (bar_final: 6 host arrays,
// entries may be null), the misfit at N, the projection.
int grad_begin(lsh_adjoint* A, double misfit_weight, const double* const bar_final[6]) {
    cudaStream_t s = A->stream;
    const size_t N = A->N;
    A->misfit_weight = misfit_weight;
    for (int k = 0; k < 6; ++k) {
        if (bar_final && bar_final[k]) A_CUDA(cudaMemcpyAsync(A->Xb[k], bar_final[k], N * sizeof(double), cudaMemcpyHostToDevice, s));
        else A_CUDA(cudaMemsetAsync(A->Xb[k], 0, N * sizeof(double), s));
    }
    A_CUDA(cudaMemsetAsync(A->red, 0, sizeof(double) * kRed, s));
    misfit_and_project(A, A->nsteps, A->hN[0], A->hN[1], s);
    A->stats.recompute_steps = 0;
    A->stats.reversed_steps = 0;
    A->spine_stored = false;  // the sweep reuses the slots
    A->cur_step = -1;
    A_CUDA(cudaGetLastError());
    return 0;
}

// After the sweep (`cur`: the step of the state in X): the adjoint of dt_0
// through the initial-dt pass of X_0, the misfit-free projection at X_0.
int grad_tail(lsh_adjoint* A, int cur) {
    cudaStream_t s = A->stream;
    const size_t N = A->N;
    if (cur != 0) {
        Ops ops(A);
        if (int st = ops.restore(0, 0)) return st;
    }
    A->cur_step = 0;
    const KArgs a = fwd_args(A, A->X, nullptr, nullptr, A->acc1, nullptr, nullptr);
    init_wave_pass(A, a, s);
    const int G = A->grid;
    cudaMemsetAsync(A->rmax, 0, sizeof(unsigned long long), s);
    k_init_cell<<<1, 1, 0, s>>>(A->argmax);
    k_adj_rate_max<<<G, kCellBlock, 0, s>>>(A->acc1[6], A->geo, A->p.nx, (long long)N, A->rmax);
    k_adj_argmax<<<G, kCellBlock, 0, s>>>(A->acc1[6], A->geo, A->p.nx, (long long)N, A->rmax, A->argmax);
    k_adj_ratebar<<<1, 1, 0, s>>>(A->rmax, A->argmax, A->red, A->d_dts, A->rsel);
    AdjArgs aa = adj_args(A, A->X, nullptr, nullptr, nullptr, A->Xb, nullptr, nullptr, nullptr, A->h_dts[0]);
    k_adj_init<<<1, 32, 0, s>>>(aa, A->rsel, A->part);
    k_adj_reduce<<<1, 32 * kRed, 0, s>>>(A->part, 1, A->red);
    misfit_and_project(A, 0, A->X[0], A->X[3], s);
    A_CUDA(cudaGetLastError());
    return 0;
}

// The state gradient (6 host arrays, entries may be null) and the reduced
// dt and constant adjoints into host memory; returns after the copies.
int grad_copy(lsh_adjoint* A, double* const grad_state[6]) {
    cudaStream_t s = A->stream;
    for (int k = 0; k < 6; ++k)
        if (grad_state && grad_state[k])
            A_CUDA(cudaMemcpyAsync(grad_state[k], A->Xb[k], A->N * sizeof(double), cudaMemcpyDeviceToHost, s));
    A_CUDA(cudaMemcpyAsync(A->h_red, A->red, sizeof(A->h_red), cudaMemcpyDeviceToHost, s));
    A_CUDA(cudaStreamSynchronize(s));
    return 0;
}

// d/d(angle1, mf0, mfs, r) from the constant adjoints.
void grad_params_of(const lsh_adjoint* A, double gp[4]) {
    const double* red = A->h_red;
    ConstBar cb{red[1], red[2], red[3], red[4], red[5], red[6], red[7], red[8]};
    lsh::param_grads(A->p.angle1, A->p.mf0, A->p.mfs, A->p.r, A->p.gravity, A->p.eps_h, A->p.L, A->p.H, cb, gp);
}

// The schedule's operations applied to every member in turn: one schedule,
// one slot count, every member's state at the same step.
struct BatchOps : lsh::RevolveOps {
    std::vector<Ops> ops;
    int advance(int from, int to) override {
        for (int n = from; n < to; ++n)
            for (auto& o : ops)
                if (int st = o.advance(n, n + 1)) return st;
        return 0;
    }
    int store(int k) override {
        for (auto& o : ops)
            if (int st = o.store(k)) return st;
        return 0;
    }
    int restore(int k, int step) override {
        for (auto& o : ops)
            if (int st = o.restore(k, step)) return st;
        return 0;
    }
    int reverse_step(int n) override {
        for (auto& o : ops)
            if (int st = o.reverse_step(n)) return st;
        return 0;
    }
};

}  // namespace

struct lsh_adjoint_batch {
    std::vector<lsh_adjoint*> m;
    double budget = -1.0;  // < 0: 180 GB, capped by free memory at the forward run
    int nsteps = 0;
    int n_slots = 0;
    bool have_forward = false;
    lsh_adjoint_stats stats{};
};

// ------------------------------------------------------------------ C ABI

extern "C" {

int lsh_adjoint_create(const lsh_params* params, int device, int n_gauges, const int* gauge_cells, lsh_adjoint** out) {
    if (!out || !params || n_gauges < 0 || (n_gauges > 0 && !gauge_cells)) return LSH_ERR_INVALID;
    *out = nullptr;
    if (const char* why = lsh::params_problem(params)) { lsh::set_last_error(why); return LSH_ERR_INVALID; }
    if (params->friction_law != LSH_FRICTION_COULOMB) {
        lsh::set_last_error("lsh_adjoint: the Coulomb friction law only");
        return LSH_ERR_INVALID;
    }
    const long long N = (long long)params->nx * params->ny;
    for (int g = 0; g < n_gauges; ++g)
        if (gauge_cells[g] < 0 || gauge_cells[g] >= N) { lsh::set_last_error("lsh_adjoint: gauge cell out of range"); return LSH_ERR_INVALID; }
    if (lsh_check_device() != 0) return LSH_ERR_NO_DEVICE;
    lsh_adjoint* A = new (std::nothrow) lsh_adjoint();
    if (!A) return LSH_ERR_HOST_OOM;
    auto bail = [&](int st) { lsh_adjoint_destroy(A); return st; };
    A->p = *params;
    A->p.track_eta_max = 0;
    A->c = lsh::make_consts(A->p);
    A->order = params->order;
    A->N = (size_t)N;
    A->npad = (A->N + 31) & ~size_t(31);
    if (device >= 0) { cudaError_t e = cudaSetDevice(device); if (e != cudaSuccess) return bail(afail(e, "cudaSetDevice")); }
    cudaGetDevice(&A->device);
    cudaDeviceGetAttribute(&A->sms, cudaDevAttrMultiProcessorCount, A->device);
    A->grid = 2 * A->sms;
    { cudaError_t e = cudaStreamCreateWithFlags(&A->stream, cudaStreamNonBlocking); if (e != cudaSuccess) return bail(afail(e, "cudaStreamCreate")); }
    // working arrays: X 7, Y 6, s1/s2 28, acc 14, snaps 12, Xb/Xbn/Yb 18, sxb/syb/accb 21, eta dummy 1, hN 2
    const int narr = 7 + 6 + 28 + 14 + 12 + 18 + 21 + 1 + 2;
    const size_t geo_n = 7 * size_t(params->ny + 1);
    A->dep_stride = dep_stride_for(params->nx, params->ny);
    const size_t bytes = (size_t(narr) * A->npad + ((geo_n + 31) & ~size_t(31))) * sizeof(double) +
                         2 * A->npad * sizeof(unsigned) + 2 * A->npad + size_t(13) * A->dep_stride * sizeof(unsigned);
    { cudaError_t e = cudaMalloc(&A->slab, bytes); if (e != cudaSuccess) return bail(afail(e, "cudaMalloc adjoint work arrays")); }
    {
        // zero the work arrays and wait: the geometry and gauge copies below go
        // through the legacy default stream, which does not order against
        // this non-blocking stream
        cudaError_t e = cudaMemsetAsync(A->slab, 0, bytes, A->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(A->stream);
        if (e != cudaSuccess) return bail(afail(e, "zeroing the adjoint work arrays"));
    }
    double* cur = static_cast<double*>(A->slab);
    auto take = [&](double*& p) { p = cur; cur += A->npad; };
    for (int k = 0; k < 7; ++k) take(A->X[k]);
    for (int k = 0; k < 6; ++k) take(A->Y[k]);
    for (int k = 0; k < 7; ++k) { take(A->s1x[k]); take(A->s1y[k]); take(A->s2x[k]); take(A->s2y[k]); }
    for (int k = 0; k < 7; ++k) { take(A->acc1[k]); take(A->acc2[k]); }
    for (int q = 0; q < 3; ++q) for (int v = 0; v < 2; ++v) { take(A->snap1[q][v]); take(A->snap2[q][v]); }
    for (int k = 0; k < 6; ++k) { take(A->Xb[k]); take(A->Xbn[k]); take(A->Yb[k]); }
    for (int k = 0; k < 7; ++k) { take(A->sxb[k]); take(A->syb[k]); take(A->accb[k]); }
    take(A->eta_dummy);
    take(A->hN[0]);
    take(A->hN[1]);
    A->geo_buf = cur;
    cur += (geo_n + 31) & ~size_t(31);
    A->tape1 = reinterpret_cast<unsigned*>(cur);
    A->tape2 = A->tape1 + A->npad;
    A->szero1 = reinterpret_cast<unsigned char*>(A->tape2 + A->npad);  // zeroed with the slab
    A->szero2 = A->szero1 + A->npad;
    if (A->dep_stride) A->dep_ctr = reinterpret_cast<unsigned*>(A->szero2 + A->npad);  // zeroed with the slab
    {
        std::vector<double> g(geo_n, 0.0);
        const size_t st = size_t(params->ny + 1);
        lsh::fill_geo(A->p, g.data(), st);
        cudaError_t e = cudaMemcpy(A->geo_buf, g.data(), geo_n * sizeof(double), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return bail(afail(e, "geometry"));
        A->geo.area = A->geo_buf; A->geo.len_v = A->geo_buf + st; A->geo.len_h = A->geo_buf + 2 * st;
        A->geo.tanR = A->geo_buf + 3 * st; A->geo.wx = A->geo_buf + 4 * st; A->geo.wy = A->geo_buf + 5 * st;
        A->geo.inv_area = A->geo_buf + 6 * st;
    }
    {
        cudaError_t e = cudaMalloc(&A->tm, sizeof(lsh::TimeRec));
        if (e == cudaSuccess) e = cudaMalloc(&A->rmax, sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMalloc(&A->argmax, sizeof(long long));
        if (e == cudaSuccess) e = cudaMalloc(&A->rsel, sizeof(RateSel));
        // partial-sum rows of one reversed step: 2 volume + 8 edge launches (+1 for dt_0)
        long long ecap = 0;
        for (int dir = 0; dir < 2; ++dir)
            for (int par = 0; par < 2; ++par)
                ecap = std::max(ecap, blocks_of(adj_edge_grid(params->nx, params->ny, dir, par)));
        const long long vcap = blocks_of(adj_cell_grid(params->nx, params->ny));
        A->part_rows = std::max<long long>((long long)kPartSlots * A->grid, 2 * vcap + 8 * ecap + 1);
        if (e == cudaSuccess) e = cudaMalloc(&A->part, sizeof(double) * kRed * A->part_rows);
        if (e == cudaSuccess) e = cudaMalloc(&A->part2, sizeof(double) * kRed * 128);
        if (e == cudaSuccess) e = cudaMalloc(&A->red, sizeof(double) * kRed);
        if (e == cudaSuccess && n_gauges > 0) e = cudaMalloc(&A->d_gauges, sizeof(int) * n_gauges);
        if (e != cudaSuccess) return bail(afail(e, "cudaMalloc adjoint scalars"));
    }
    A->ng = n_gauges;
    if (n_gauges > 0) { cudaError_t e = cudaMemcpy(A->d_gauges, gauge_cells, sizeof(int) * n_gauges, cudaMemcpyHostToDevice); if (e != cudaSuccess) return bail(afail(e, "gauges")); }
    // default checkpoint budget: 180 GB, capped by what is free (leaving 4 GB)
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    A->budget = std::min(180e9, std::max(0.0, (double)fr - 4e9));
    A->stats.slot_bytes = 6.0 * A->npad * sizeof(double);
    { cudaError_t e = cudaStreamSynchronize(A->stream); if (e != cudaSuccess) return bail(afail(e, "init")); }
    *out = A;
    return LSH_OK;
}

static void destroy_adjoint(lsh_adjoint* A) {
    if (A->stream) cudaStreamSynchronize(A->stream);
    cudaFree(A->slab);
    cudaFree(A->tm); cudaFree(A->rmax); cudaFree(A->argmax); cudaFree(A->rsel); cudaFree(A->part); cudaFree(A->part2); cudaFree(A->red);
    cudaFree(A->d_gauges); cudaFree(A->d_eta); cudaFree(A->d_tgt); cudaFree(A->d_dts);
    cudaFree(A->slots);
    if (A->stream) cudaStreamDestroy(A->stream);
    (void)cudaGetLastError();
    delete A;
}

int lsh_adjoint_destroy(lsh_adjoint* A) {
    if (!A) return LSH_OK;
    if (A->in_batch) {
        lsh::set_last_error("lsh_adjoint_destroy: a batch member is destroyed with its batch");
        return LSH_ERR_INVALID;
    }
    destroy_adjoint(A);
    return LSH_OK;
}

int lsh_adjoint_set_thin_layer(lsh_adjoint* A, double h_adj) {
    if (!A || !(h_adj >= 0.0)) return LSH_ERR_INVALID;
    A->h_adj = h_adj;
    return LSH_OK;
}

int lsh_adjoint_set_budget(lsh_adjoint* A, double bytes) {
    if (!A || !(bytes >= 0.0)) return LSH_ERR_INVALID;
    A->budget = bytes;
    return LSH_OK;
}

int lsh_adjoint_forward(lsh_adjoint* A, const double* const host_state[LSH_NVARS], int nsteps, const double* target,
                        double* misfit, double* gauge_series) {
    if (!A || !host_state || nsteps < 1) return LSH_ERR_INVALID;
    for (int k = 0; k < LSH_NVARS; ++k) if (!host_state[k]) return LSH_ERR_INVALID;
    const auto t0 = std::chrono::steady_clock::now();
    int want = (int)std::min<double>((double)nsteps, std::floor(A->budget / slot_bytes_of(A)));
    if (want < 1) { lsh::set_last_error("lsh_adjoint: the checkpoint budget holds no state"); return LSH_ERR_INVALID; }
    int st = fwd_alloc(A, nsteps, want);
    while (st == LSH_ERR_GPU_OOM && want > 1) {
        want /= 2;
        st = fwd_alloc(A, nsteps, want);
    }
    if (st) return st;
    if ((st = fwd_begin(A, host_state, target))) return st;
    // the schedule's first descent, with the gauge series and dt records
    Ops ops(A);
    int a = 0, slot = 0;
    for (const int m : spine_steps(nsteps, A->n_slots)) {
        for (int n = a; n < m; ++n)
            if ((st = fwd_record_step(A, n))) return st;
        if ((st = ops.store(++slot))) return st;
        A->spine.push_back(m);
        a = m;
    }
    for (int n = a; n < nsteps; ++n)
        if ((st = fwd_record_step(A, n))) return st;
    if ((st = fwd_end(A))) return st;
    if ((st = fwd_host(A, target, misfit, gauge_series))) return st;
    A->stats.ms_forward = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return LSH_OK;
}

int lsh_adjoint_gradient(lsh_adjoint* A, double misfit_weight, const double* const bar_final[6], double* grad_state[6],
                         double grad_params[4]) {
    if (!A || !A->have_forward) return LSH_ERR_INVALID;
    const auto t0 = std::chrono::steady_clock::now();
    const bool pre = A->spine_stored;
    Ops ops(A);
    ops.cur = A->cur_step;
    if (int st = grad_begin(A, misfit_weight, bar_final)) return st;
    if (int st = lsh::revolve_reverse(ops, 0, A->nsteps, 0, A->n_slots - 1, pre)) return st;
    if (int st = grad_tail(A, ops.cur)) return st;
    if (int st = grad_copy(A, grad_state)) return st;
    double gp[4];
    grad_params_of(A, gp);
    if (grad_params) for (int k = 0; k < 4; ++k) grad_params[k] = gp[k];
    A->stats.ms_gradient = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return LSH_OK;
}

int lsh_adjoint_get_times(lsh_adjoint* A, double* t_out) {
    if (!A || !t_out || !A->have_forward) return LSH_ERR_INVALID;
    double t = 0.0;
    for (int n = 0; n < A->nsteps; ++n) {
        t += A->h_dts[n];
        t_out[n] = t;
    }
    return LSH_OK;
}

int lsh_adjoint_get_state(lsh_adjoint* A, double* const host_state[6]) {
    if (!A || !host_state || A->cur_step != A->nsteps) return LSH_ERR_INVALID;
    for (int k = 0; k < 6; ++k)
        if (host_state[k])
            A_CUDA(cudaMemcpyAsync(host_state[k], A->X[k], A->N * sizeof(double), cudaMemcpyDeviceToHost, A->stream));
    A_CUDA(cudaStreamSynchronize(A->stream));
    return LSH_OK;
}

int lsh_adjoint_get_stats(lsh_adjoint* A, lsh_adjoint_stats* out) {
    if (!A || !out) return LSH_ERR_INVALID;
    *out = A->stats;
    return LSH_OK;
}

int lsh_revolve_plan(int nsteps, int slots, long long* forward_steps, long long* optimal) {
    if (nsteps < 1 || slots < 1) return LSH_ERR_INVALID;
    // run the schedule with counting operations (no device work)
    struct Count : lsh::RevolveOps {
        long long fw = 0;
        int next = 0;
        std::vector<int> slot_step;
        int bad = 0;
        int advance(int from, int to) override { fw += to - from; return 0; }
        int store(int k) override {
            if (k >= (int)slot_step.size()) slot_step.resize(k + 1, -1);
            slot_step[k] = cur;
            return 0;
        }
        int restore(int k, int step) override {
            if (k >= (int)slot_step.size() || slot_step[k] != step) bad = 1;
            return 0;
        }
        int reverse_step(int step) override {
            if (step != next || cur != step) bad = 1;
            --next;
            return 0;
        }
    } c;
    c.slot_step.assign(1, 0);
    c.cur = 0;
    // the first descent, as lsh_adjoint_forward runs it
    int a = 0, free = slots - 1, slot = 0;
    while (nsteps - a > 1 && free > 0) {
        const int m = a + (int)lsh::revolve_split(nsteps - a, free + 1);
        c.cur = m;
        ++slot;
        c.store(slot);
        a = m;
        --free;
    }
    const long long descent = a;  // the spine's advances, counted as the schedule counts them
    c.cur = nsteps;
    c.next = nsteps - 1;
    if (lsh::revolve_reverse(c, 0, nsteps, 0, slots - 1, true)) return LSH_ERR_INVALID;
    if (c.bad || c.next != -1) return LSH_ERR_INVALID;
    if (forward_steps) *forward_steps = descent + c.fw;
    if (optimal) *optimal = lsh::revolve_cost(nsteps, slots);
    return LSH_OK;
}

// ------------------------------------------------------------------ batch

int lsh_adjoint_batch_create(int n, const lsh_params* params, const int* n_gauges, const int* const* gauge_cells,
                             int device, lsh_adjoint_batch** out) {
    if (!out || n < 1 || !params) return LSH_ERR_INVALID;
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        const int ng = n_gauges ? n_gauges[i] : 0;
        if (ng < 0 || (ng > 0 && (!gauge_cells || !gauge_cells[i]))) {
            lsh::set_last_error("lsh_adjoint_batch_create: member " + std::to_string(i) + ": gauges");
            return LSH_ERR_INVALID;
        }
        if (const char* why = lsh::params_problem(&params[i])) {
            lsh::set_last_error("lsh_adjoint_batch_create: member " + std::to_string(i) + ": " + why);
            return LSH_ERR_INVALID;
        }
    }
    lsh_adjoint_batch* B = new (std::nothrow) lsh_adjoint_batch();
    if (!B) return LSH_ERR_HOST_OOM;
    for (int i = 0; i < n; ++i) {
        lsh_adjoint* A = nullptr;
        const int ng = n_gauges ? n_gauges[i] : 0;
        const int st = lsh_adjoint_create(&params[i], device, ng, ng > 0 ? gauge_cells[i] : nullptr, &A);
        if (st != LSH_OK) {
            lsh_adjoint_batch_destroy(B);
            return st;
        }
        A->in_batch = true;
        A->budget = 0.0;  // until the batch's forward run sets the slot count
        B->m.push_back(A);
    }
    *out = B;
    return LSH_OK;
}

int lsh_adjoint_batch_destroy(lsh_adjoint_batch* B) {
    if (!B) return LSH_OK;
    for (lsh_adjoint* A : B->m) destroy_adjoint(A);
    delete B;
    return LSH_OK;
}

int lsh_adjoint_batch_set_thin_layer(lsh_adjoint_batch* B, double h_adj) {
    if (!B || !(h_adj >= 0.0)) return LSH_ERR_INVALID;
    for (lsh_adjoint* A : B->m) A->h_adj = h_adj;
    return LSH_OK;
}

int lsh_adjoint_batch_set_budget(lsh_adjoint_batch* B, double bytes) {
    if (!B || !(bytes >= 0.0)) return LSH_ERR_INVALID;
    B->budget = bytes;
    return LSH_OK;
}

int lsh_adjoint_batch_forward(lsh_adjoint_batch* B, const double* const* host_states, int nsteps,
                              const double* const* targets, double* misfits, double* const* gauge_series) {
    if (!B || !host_states || nsteps < 1) return LSH_ERR_INVALID;
    const int n = (int)B->m.size();
    for (int i = 0; i < n * LSH_NVARS; ++i) if (!host_states[i]) return LSH_ERR_INVALID;
    const auto t0 = std::chrono::steady_clock::now();
    B->have_forward = false;
    // one slot count for all: with a common step count, equal counts
    // minimise the members' summed recomputation under a joint budget
    double per_slot = 0.0;
    for (lsh_adjoint* A : B->m) per_slot += slot_bytes_of(A);
    double budget = B->budget;
    if (budget < 0.0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        budget = std::min(180e9, std::max(0.0, (double)fr - 4e9));
    }
    int want = (int)std::min<double>((double)nsteps, std::floor(budget / per_slot));
    if (want < 1) { lsh::set_last_error("lsh_adjoint_batch: the checkpoint budget holds no batch state"); return LSH_ERR_INVALID; }
    for (;;) {
        int st = 0;
        for (lsh_adjoint* A : B->m)
            if ((st = fwd_alloc(A, nsteps, want))) break;
        if (st == 0) break;
        if (st != LSH_ERR_GPU_OOM || want == 1) return st;
        for (lsh_adjoint* A : B->m) { cudaFree(A->slots); A->slots = nullptr; A->n_slots = 0; }
        want /= 2;
    }
    B->nsteps = nsteps;
    B->n_slots = want;
    // a member run on its own keeps the batch's slot count
    for (lsh_adjoint* A : B->m) A->budget = want * slot_bytes_of(A);
    for (int i = 0; i < n; ++i)
        if (int st = fwd_begin(B->m[i], host_states + (size_t)i * LSH_NVARS, targets ? targets[i] : nullptr)) return st;
    BatchOps ops;
    for (lsh_adjoint* A : B->m) ops.ops.emplace_back(A);
    int a = 0, slot = 0;
    auto run = [&](int to) -> int {
        for (int s = a; s < to; ++s)
            for (lsh_adjoint* A : B->m)
                if (int st = fwd_record_step(A, s)) return st;
        return 0;
    };
    const std::vector<int> spine = spine_steps(nsteps, want);
    for (const int m : spine) {
        if (int st = run(m)) return st;
        if (int st = ops.store(++slot)) return st;
        a = m;
    }
    if (int st = run(nsteps)) return st;
    for (lsh_adjoint* A : B->m) if (int st = fwd_end(A)) return st;
    for (int i = 0; i < n; ++i) {
        lsh_adjoint* A = B->m[i];
        A->spine = spine;
        if (int st = fwd_host(A, targets ? targets[i] : nullptr, misfits ? misfits + i : nullptr,
                              gauge_series ? gauge_series[i] : nullptr))
            return st;
    }
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    B->stats = lsh_adjoint_stats{};
    B->stats.slots = want;
    B->stats.nsteps = nsteps;
    B->stats.forward_steps = B->m[0]->stats.forward_steps;
    B->stats.ms_forward = ms;
    B->stats.slot_bytes = per_slot;
    for (lsh_adjoint* A : B->m) A->stats.ms_forward = ms;
    B->have_forward = true;
    return LSH_OK;
}

int lsh_adjoint_batch_gradient(lsh_adjoint_batch* B, const double* misfit_weights, double* const* grad_states,
                               double* grad_params) {
    if (!B || !B->have_forward) return LSH_ERR_INVALID;
    const int n = (int)B->m.size();
    // the members must still hold the batch's run: same steps, slots and step
    const lsh_adjoint* A0 = B->m[0];
    for (lsh_adjoint* A : B->m)
        if (!A->have_forward || A->nsteps != B->nsteps || A->n_slots != B->n_slots || A->cur_step != A0->cur_step ||
            A->spine_stored != A0->spine_stored) {
            lsh::set_last_error("lsh_adjoint_batch_gradient: a member was run on its own since the batch's forward run");
            return LSH_ERR_INVALID;
        }
    const auto t0 = std::chrono::steady_clock::now();
    const bool pre = A0->spine_stored;
    BatchOps ops;
    for (lsh_adjoint* A : B->m) ops.ops.emplace_back(A);
    ops.cur = A0->cur_step;
    for (int i = 0; i < n; ++i)
        if (int st = grad_begin(B->m[i], misfit_weights ? misfit_weights[i] : 1.0, nullptr)) return st;
    if (int st = lsh::revolve_reverse(ops, 0, B->nsteps, 0, B->n_slots - 1, pre)) return st;
    for (lsh_adjoint* A : B->m) if (int st = grad_tail(A, ops.cur)) return st;
    for (int i = 0; i < n; ++i) {
        lsh_adjoint* A = B->m[i];
        if (int st = grad_copy(A, grad_states ? grad_states + (size_t)i * 6 : nullptr)) return st;
        double gp[4];
        grad_params_of(A, gp);
        if (grad_params) for (int k = 0; k < 4; ++k) grad_params[(size_t)i * 4 + k] = gp[k];
    }
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    B->stats.recompute_steps = B->m[0]->stats.recompute_steps;
    B->stats.reversed_steps = B->m[0]->stats.reversed_steps;
    B->stats.ms_gradient = ms;
    for (lsh_adjoint* A : B->m) A->stats.ms_gradient = ms;
    return LSH_OK;
}

int lsh_adjoint_batch_get_stats(lsh_adjoint_batch* B, lsh_adjoint_stats* out) {
    if (!B || !out) return LSH_ERR_INVALID;
    *out = B->stats;
    return LSH_OK;
}

int lsh_adjoint_batch_member(lsh_adjoint_batch* B, int i, lsh_adjoint** out) {
    if (!B || !out || i < 0 || i >= (int)B->m.size()) return LSH_ERR_INVALID;
    *out = B->m[i];
    return LSH_OK;
}

}  // extern "C"
