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
#include "lsh_queue.cuh"
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
// per block.  With `d` the block waits for the producer pass's rows over the
// cell rows its edges touch, and counts itself done (the overlapped reverse
// step; `tm` takes a timed-out wait's bit).
template <int DIR, bool FIRST, int ORDER>
__global__ void __launch_bounds__(kAdjEdgeBlock, LSH_ADJ_EDGE_MINB)
    k_adj_edges(AdjArgs a, const RateSel* rs, int par, double* part, Dep d, lsh::TimeRec* tm) {
    if (d.done || d.wait) {
        // horizontal: edge rows par + 2 w, w in [8 by, 8 by + 7], touch cell rows
        // y - 1 and y; vertical: rows [16 by, 16 by + 15]
        const int r0 = (DIR == 0) ? par + 16 * (int)blockIdx.y - 1 : 16 * (int)blockIdx.y;
        const int r1 = (DIR == 0) ? par + 16 * (int)blockIdx.y + 14 : 16 * (int)blockIdx.y + 15;
        dep_begin(d, tm, max(r0, 0), min(r1, a.c.ny - 1));
    }
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
    dep_end(d);
}

// One cell per thread over 16 x 8 tiles.  MODE 1 (the stage-1 volume of a
// second-order step) overwrites the slope adjoints that the stage-2
// reconstruction adjoint reads one row around each cell, so with `d` it
// waits for one row more on each side.
template <int MODE>
__global__ void __launch_bounds__(kAdjCellBlock, LSH_ADJ_MINBLOCKS)
    k_adj_volume(AdjArgs a, const RateSel* rs, double* part, Dep d, lsh::TimeRec* tm) {
    if (d.done || d.wait) {
        const int y0 = 8 * (int)blockIdx.y, ext = (MODE == 1) ? 1 : 0;
        dep_begin(d, tm, max(y0 - ext, 0), min(y0 + 7 + ext, a.c.ny - 1));
    }
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
    dep_end(d);
}

// Gathers the slope adjoints one cell around: with `d` it waits for the rows
// around its tile.
__global__ void __launch_bounds__(kAdjCellBlock) k_adj_recon(AdjArgs a, Dep d, lsh::TimeRec* tm) {
    if (d.done || d.wait) {
        const int y0 = 8 * (int)blockIdx.y;
        dep_begin(d, tm, max(y0 - 1, 0), min(y0 + 8, a.c.ny - 1));
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < a.c.nx && j < a.c.ny) lsh::recon_adj_cell(a, j * a.c.nx + i);
    dep_end(d);
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
__device__ __forceinline__ void ratebar_body(const unsigned long long* rmax, const long long* cell, const double* red,
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

__global__ void k_adj_ratebar(const unsigned long long* rmax, const long long* cell, const double* red,
                              const double* dt_next, RateSel* out) {
    ratebar_body(rmax, cell, red, dt_next, out);
}

// The misfit's adjoint at the state after a step: 2 w (eta - target) at each gauge.
__device__ __forceinline__ void gauge_add(double* hb1, double* hb2, const int* gauges, int ng, const double* eta,
                                          const double* tgt, double w, int g) {
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

__global__ void k_adj_gauges(double* hb1, double* hb2, const int* gauges, int ng, const double* eta, const double* tgt,
                             double w) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < ng) gauge_add(hb1, hb2, gauges, ng, eta, tgt, w, g);
}

// Thin-layer projection: the adjoint of a layer thinner than h_adj (in the
// state the adjoint belongs to) is zeroed; the tangent-linear model zeroes
// the same tangents, so the pair stays transposes of each other.
__device__ __forceinline__ void project_cells(double* b0, double* b1, double* b2, double* b3, double* b4, double* b5,
                                              const double* h1, const double* h2, long long N, double h_adj,
                                              long long start, long long stride) {
    for (long long i = start; i < N; i += stride) {
        if (h1[i] < h_adj) { b0[i] = 0.0; b1[i] = 0.0; b2[i] = 0.0; }
        if (h2[i] < h_adj) { b3[i] = 0.0; b4[i] = 0.0; b5[i] = 0.0; }
    }
}

__global__ void __launch_bounds__(kCellBlock) k_adj_project(double* b0, double* b1, double* b2,
                                                            double* b3, double* b4, double* b5, const double* h1,
                                                            const double* h2, long long N, double h_adj) {
    project_cells(b0, b1, b2, b3, b4, b5, h1, h2, N, h_adj, (long long)blockIdx.x * blockDim.x + threadIdx.x,
                  (long long)gridDim.x * blockDim.x);
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
__device__ __forceinline__ void reduce_body(const double* part, int nparts, double* red) {
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

__global__ void __launch_bounds__(32 * kRed) k_adj_reduce(const double* part, int nparts, double* red) {
    reduce_body(part, nparts, red);
}

// First level of the partial sums: block b adds rows [b chunk, (b+1) chunk)
// into row b of out (warp k: component k, lane-strided then a shuffle tree),
// a fixed order, so the total stays bit-reproducible.
constexpr int kReduceRows = 128;  // first-level rows of a step's partial sums

__device__ __forceinline__ void reduce_rows_body(const double* part, long long nparts, long long chunk, double* out,
                                                 unsigned b) {
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long r0 = (long long)b * chunk;
    const long long r1 = (r0 + chunk < nparts) ? r0 + chunk : nparts;
    double s = 0.0;
    for (long long i = r0 + lane; i < r1; i += 32) s += part[(size_t)i * kRed + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) out[(size_t)b * kRed + k] = s;
}

__global__ void __launch_bounds__(32 * kRed) k_adj_reduce_rows(const double* part, long long nparts, long long chunk,
                                                               double* out) {
    reduce_rows_body(part, nparts, chunk, out, blockIdx.x);
}

// A replayed step's time record: the recorded dt.  A timed-out wait's bit
// stays (the host reads it after the run, and later waits give up at once).
__device__ __forceinline__ void set_dt_body(lsh::TimeRec* tm, const double* dt) {
    tm->dt = *dt;
    tm->rmax_bits = kRateInitBits;
    tm->done = 0;
    tm->err &= 1 << LSH_ERR_TIMEOUT;
    tm->t_end = INFINITY;
}

__global__ void k_set_dt(lsh::TimeRec* tm, const double* dt) { set_dt_body(tm, dt); }

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
    bool own_stream = true;    // false: a batch's stream, destroyed with the batch
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
    bool ordered = false;           // lsh_adjoint_set_ordered: no pass overlap
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

// The counters of the overlapped passes, or null when they run in full order.
unsigned* overlap_ctr(const lsh_adjoint* A) { return A->ordered ? nullptr : A->dep_ctr; }

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
    if (overlap_ctr(A)) {
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
    k_adj_volume<MODE><<<g, adj_cell_block(), 0, s>>>(a, rs, A->part + *nparts * kRed, Dep{}, nullptr);
    *nparts += blocks_of(g);
    a.snap[0] = snaps[2][0]; a.snap[1] = snaps[2][1];
    g = adj_edge_grid(nx, ny, 1, 1);
    k_adj_edges<1, false, ORDER><<<g, adj_edge_block(1), 0, s>>>(a, rs, 1, A->part + *nparts * kRed, Dep{}, nullptr);
    *nparts += blocks_of(g);
    a.snap[0] = snaps[1][0]; a.snap[1] = snaps[1][1];
    g = adj_edge_grid(nx, ny, 1, 0);
    k_adj_edges<1, false, ORDER><<<g, adj_edge_block(1), 0, s>>>(a, rs, 0, A->part + *nparts * kRed, Dep{}, nullptr);
    *nparts += blocks_of(g);
    a.snap[0] = snaps[0][0]; a.snap[1] = snaps[0][1];
    g = adj_edge_grid(nx, ny, 0, 1);
    k_adj_edges<0, false, ORDER><<<g, adj_edge_block(0), 0, s>>>(a, rs, 1, A->part + *nparts * kRed, Dep{}, nullptr);
    *nparts += blocks_of(g);
    a.snap[0] = a.snap[1] = nullptr;
    g = adj_edge_grid(nx, ny, 0, 0);
    k_adj_edges<0, true, ORDER><<<g, adj_edge_block(0), 0, s>>>(a, rs, 0, A->part + *nparts * kRed, Dep{}, nullptr);
    *nparts += blocks_of(g);
    if (ORDER == 2) k_adj_recon<<<adj_cell_grid(nx, ny), adj_cell_block(), 0, s>>>(a, Dep{}, nullptr);
}


// The same passes as overlapped launches: each after the first is a
// programmatic dependent launch whose blocks wait only for the rows of the
// pass before that they read or overwrite (lsh_kernels.cuh's Dep, with the
// adjoint's block heights).  `prev` is the Dep of the pass before this stage
// (wait null: this stage starts the chain); `seg` the next free counter
// segment.  Returns the Dep of this stage's last pass for the next one.
template <int ORDER, int MODE>
Dep rev_stage_overlap(lsh_adjoint* A, AdjArgs a, double* snaps[3][2], const RateSel* rs, long long* nparts,
                      cudaStream_t s, Dep prev, unsigned*& seg, bool last) {
    const int nx = A->p.nx, ny = A->p.ny, st = A->dep_stride;
    // the Dep a consumer of a pass on grid g, of kind k and block height h, waits with
    auto waits_on = [](const unsigned* done, dim3 g, int kind, int span) {
        Dep w;
        w.wait = done; w.target = g.x; w.kind = kind; w.ntiles = (int)g.y; w.span = span;
        return w;
    };
    const int npass = (ORDER == 2) ? 6 : 5;
    int k = 0;
    auto done_of = [&](Dep d) {
        ++k;
        d.done = (last && k == npass) ? nullptr : seg;
        return d;
    };
    dim3 g = adj_cell_grid(nx, ny);
    Dep d = done_of(prev);
    launch_pass(prev.wait != nullptr, g, adj_cell_block(), s, k_adj_volume<MODE>, a, rs, A->part + *nparts * kRed, d,
                A->tm);
    *nparts += blocks_of(g);
    Dep w = waits_on(d.done, g, kDepCell, 8);
    seg += st;
    // colour passes, last first: v1, v0 (block rows of 16), h1, h0 (8 edge lines)
    const int dirs[4] = {1, 1, 0, 0}, pars[4] = {1, 0, 1, 0};
    for (int c = 0; c < 4; ++c) {
        const int dir = dirs[c], par = pars[c];
        a.snap[0] = (c < 3) ? snaps[2 - c][0] : nullptr;
        a.snap[1] = (c < 3) ? snaps[2 - c][1] : nullptr;
        g = adj_edge_grid(nx, ny, dir, par);
        d = done_of(w);
        double* part = A->part + *nparts * kRed;
        if (c < 2) launch_pass(true, g, adj_edge_block(1), s, k_adj_edges<1, false, ORDER>, a, rs, par, part, d, A->tm);
        else if (c == 2) launch_pass(true, g, adj_edge_block(0), s, k_adj_edges<0, false, ORDER>, a, rs, par, part, d, A->tm);
        else launch_pass(true, g, adj_edge_block(0), s, k_adj_edges<0, true, ORDER>, a, rs, par, part, d, A->tm);
        *nparts += blocks_of(g);
        w = waits_on(d.done, g, dir ? kDepV : (par ? kDepH1 : kDepH0), dir ? 16 : 8);
        seg += st;
    }
    a.snap[0] = a.snap[1] = nullptr;
    if (ORDER == 2) {
        g = adj_cell_grid(nx, ny);
        d = done_of(w);
        launch_pass(true, g, adj_cell_block(), s, k_adj_recon, a, d, A->tm);
        w = waits_on(d.done, g, kDepCell, 8);
        seg += st;
    }
    return w;
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
    if (overlap_ctr(A)) {
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
        if (overlap_ctr(A)) {
            unsigned* seg = A->dep_ctr;
            rev_stage_overlap<1, 0>(A, a, A->snap1, A->rsel, &nparts, s, Dep{}, seg, true);
        } else {
            rev_stage<1, 0>(A, a, A->snap1, A->rsel, &nparts, s);
        }
    } else {
        double* Y7[7];
        for (int k = 0; k < 6; ++k) Y7[k] = A->Y[k];
        Y7[6] = A->X[6];
        zero6(A->Yb, N, s);
        AdjArgs a2 = adj_args(A, Y7, A->s2x, A->s2y, A->acc2, A->Yb, A->Xb, A->Xbn, A->tape2, dt);
        AdjArgs a1 = adj_args(A, X, A->s1x, A->s1y, A->acc1, A->Xbn, A->Yb, nullptr, A->tape1, dt);
        if (overlap_ctr(A)) {
            // both stages as one chain of overlapped passes
            unsigned* seg = A->dep_ctr;
            const Dep w = rev_stage_overlap<2, 2>(A, a2, A->snap2, nullptr, &nparts, s, Dep{}, seg, false);
            rev_stage_overlap<2, 1>(A, a1, A->snap1, A->rsel, &nparts, s, w, seg, true);
        } else {
            rev_stage<2, 2>(A, a2, A->snap2, nullptr, &nparts, s);
            rev_stage<2, 1>(A, a1, A->snap1, A->rsel, &nparts, s);
        }
    }
    // ordered after the chain: its counters back to zero
    if (overlap_ctr(A)) cudaMemsetAsync(A->dep_ctr, 0, size_t(13) * A->dep_stride * sizeof(unsigned), s);
    {
        const long long chunk = (nparts + kReduceRows - 1) / kReduceRows;
        k_adj_reduce_rows<<<kReduceRows, 32 * kRed, 0, s>>>(A->part, nparts, chunk, A->part2);
        k_adj_reduce<<<1, 32 * kRed, 0, s>>>(A->part2, kReduceRows, A->red);
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

// After the stream has drained: LSH_ERR_TIMEOUT when a pass's bounded wait
// gave up during the run (the replayed steps keep that bit).
int check_waits(const lsh_adjoint* A) {
    lsh::TimeRec tm{};
    A_CUDA(cudaMemcpy(&tm, A->tm, sizeof(tm), cudaMemcpyDeviceToHost));
    if (tm.err & (1 << LSH_ERR_TIMEOUT)) {
        lsh::set_last_error("adjoint: a pass waited for its producer rows past the time limit");
        return LSH_ERR_TIMEOUT;
    }
    return 0;
}

// Waits for the forward run; the misfit and the gauge series.
int fwd_host(lsh_adjoint* A, const double* target, double* misfit, double* gauge_series) {
    A_CUDA(cudaStreamSynchronize(A->stream));
    if (int st = check_waits(A)) return st;
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
    return check_waits(A);
}

// d/d(angle1, mf0, mfs, r) from the constant adjoints.
void grad_params_of(const lsh_adjoint* A, double gp[4]) {
    const double* red = A->h_red;
    ConstBar cb{red[1], red[2], red[3], red[4], red[5], red[6], red[7], red[8]};
    lsh::param_grads(A->p.angle1, A->p.mf0, A->p.mfs, A->p.r, A->p.gravity, A->p.eps_h, A->p.L, A->p.H, cb, gp);
}

// ------------------------------------------------------------------ batched adjoint
//
// lsh_adjoint_batch_* walks one checkpoint schedule for all members, and
// each operation of the schedule is one set of launches for all members of
// an order (a group), with no per-member kernel sequence:
//   forward step   one persistent queue launch (lsh_queue.cuh: every
//                  member's tiles of every pass), the clock kernel, and a
//                  record kernel (dt, gauges);
//   reversed step  the recomputation as one queue launch (reconstruction
//                  with its branch tape, the edge passes taking their
//                  snapshots), then the whole adjoint step as ONE persistent
//                  launch of k_adjb_reverse, then the partial sums and the
//                  misfit, each one launch over all members.
// k_adjb_reverse pulls (pass, member, tile) items in pass order: the
// adjoint's zeroing, the stage-1 rate's max and arg-max (each waiting for all
// of the member's items of the pass before), the rate's adjoint (one item
// per member), then each stage's volume, four colour and reconstruction
// adjoints, last stage first.  Its tiles are the single adjoint kernels'
// 128-thread blocks and each writes its partial-sum row where that kernel's
// block does, so every member's gradient is bit-identical to a run of its
// own.  An item waits only for the rows of its member that it reads or
// overwrites in the pass it depends on, with bounded waits as in the queue.

struct ReconTape {
    static constexpr bool kOn = true;
    __device__ static unsigned run(const KArgs& a, int id) { return lsh::recon_cell_tape(a, id); }
};

constexpr int kRThreads = kAdjCellBlock;  // the adjoint kernels' block size
constexpr int kRMaxPasses = 16;
// CTAs per SM of the reverse queue (its register budget: 40 at 12) and the
// items a CTA takes per queue fetch.  Unlike the one-kernel-per-pass path,
// the queue wants many resident CTAs: each item's waits, argument copy and
// barriers leave its CTA idle, and the others fill that time.  The
// 64-member calibration's reverse sweep (100 steps), s, by CTAs per SM /
// fetch: 2/2 8.79, 3/2 7.02, 4/1 6.44, 4/2 6.23, 4/4 6.14, 5/4 5.69,
// 6/4 5.33, 7/4 5.15, 8/4 4.96, 10/4 4.75, 12/4 4.63, 12/8 4.67, 14/4 4.60,
// 16/2 4.56, 16/4 4.74, 16/8 4.95.
#ifndef LSH_ADJB_MINB
#define LSH_ADJB_MINB 12
#endif
#ifndef LSH_ADJB_FETCH
#define LSH_ADJB_FETCH 4
#endif
constexpr int kRVars = 10;                // AdjArgs variants of a step (per Xb / Xbn parity)

// Tilings: horizontal edges of parity 0 / 1 (16 columns x 8 edge lines),
// vertical edges of parity 0 / 1 (8 edge columns x 16 rows), cells (16 x 8),
// one item per member.
enum RKind : int { kRH0 = 0, kRH1 = 1, kRV0 = 2, kRV1 = 3, kRCell = 4, kRMember = 5, kRKinds = 6 };
enum ROp : int {
    kRZero = 0, kRRateMax, kRArgMax, kRRateBar, kRVol0, kRVol1, kRVol2, kREV1, kREV0, kREH1, kREH0, kRRecon
};

struct RPass {
    int op, kind, var;
    int prod;   // the pass whose rows it waits for (-1: none)
    int fprod;  // the pass all of whose items of the member it waits for (-1: none)
    int rate;   // 1: reads the stage-1 rate selection
    int parts;  // 1: writes one partial-sum row per item
    int item_off, ctr_off;
};

// Per member: what the rate items, the partial sums and the waits use.
struct RMember {
    unsigned long long* rmax;
    long long* argmax;
    RateSel* rsel;
    const double* red;   // red[0]: the adjoint of the next step's dt
    const double* dts;   // the recorded dt of every step
    double* part;        // partial-sum rows
    lsh::TimeRec* tm;
};

struct RPlan {
    int n, npass, total_items;
    RPass pass[kRMaxPasses];
    const int* tile_pre;  // [kind][n + 1]
    const int* row_pre;   // [kind][n + 1]
    const int* tiles_x;   // [kind][n]
    const int* part_off;  // [pass][n]: the member's first partial row of the pass
    const AdjArgs* args;  // [parity][kRVars][n]
    const RMember* mem;   // [n]
    unsigned* ctr;
    unsigned* head;
    int* abort_flag;
};

// Forward record of a step: dt and the gauges.
struct FMember {
    const lsh::TimeRec* tm;
    double* dts;
    const double* h1;
    const double* h2;
    const double* H;
    const int* gauges;
    int ng;
    double* eta;
};

// The misfit's adjoint and the thin-layer projection after a reversed step.
struct RMis {
    double* b[6];          // the adjoint at the step's state
    const double* h1;      // that state's depths
    const double* h2;
    const int* gauges;
    int ng;                // 0: no misfit term
    const double* eta;     // [nsteps][ng]
    const double* tgt;
    double w, h_adj;
    long long N;
};

struct RRed {
    const double* part;
    long long nparts;
    double* part2;
    double* red;
};

void adj_tiles(int nx, int ny, int kind, int& tx, int& ty) {
    if (kind == kRMember) { tx = ty = 1; return; }
    const dim3 g = (kind == kRCell) ? adj_cell_grid(nx, ny) : adj_edge_grid(nx, ny, kind >= kRV0 ? 1 : 0, kind & 1);
    tx = (int)g.x;
    ty = (int)g.y;
}

// Cell rows an item reads or overwrites.  The stage-1 volume adjoint (kRVol1)
// overwrites the slope adjoints that the stage-2 reconstruction adjoint reads
// one row around each cell, so it covers one row more on each side.
__device__ __forceinline__ void r_item_rows(int op, int kind, int ty, int ny, int& r0, int& r1) {
    if (kind == kRH0 || kind == kRH1) { const int y0 = kind + 16 * ty; r0 = y0 - 1; r1 = y0 + 14; }
    else if (kind == kRV0 || kind == kRV1) { r0 = 16 * ty; r1 = r0 + 15; }
    else if (op == kRRecon || op == kRVol1) { r0 = 8 * ty - 1; r1 = 8 * ty + 8; }
    else { r0 = 8 * ty; r1 = r0 + 7; }
    r0 = max(r0, 0);
    r1 = min(r1, ny - 1);
}

// Tile rows of a pass of `kind` that touch cell rows [r0, r1].
__device__ __forceinline__ void r_producer_rows(int kind, int r0, int r1, int& t0, int& t1) {
    if (kind == kRV0 || kind == kRV1) { t0 = r0 / 16; t1 = r1 / 16; }
    else if (kind == kRCell) { t0 = r0 / 8; t1 = r1 / 8; }
    else if (kind == kRMember) { t0 = 0; t1 = 0; }
    else {
        // horizontal edge row y = p + 2 t touches cell rows y - 1 and y
        const int p = kind;
        t0 = (max(r0 - p + 1, 0) / 2) / 8;
        t1 = (max(r1 + 1 - p, 0) / 2) / 8;
    }
}

template <int DIR, bool FIRST, int ORDER, int PAR>
__device__ __forceinline__ void r_edges(const AdjArgs& a, int tx, int ty, double* part) {
    const int nx = a.c.nx, ny = a.c.ny, tid = threadIdx.x;
    double dtb = 0.0;
    ConstBar cb;
    lsh::cb_zero(cb);
    if (DIR == 0) {
        const int u = tx * 16 + (tid & 15), w = ty * 8 + (tid >> 4);
        if (u < nx && w < (ny - PAR) / 2 + 1) lsh::edge_adj_body<0, FIRST, ORDER>(a, u, PAR + 2 * w, dtb, cb);
    } else {
        const int u = tx * 8 + (tid & 7), w = ty * 16 + (tid >> 3);
        if (u < (nx - PAR) / 2 + 1 && w < ny) lsh::edge_adj_body<1, false, ORDER>(a, PAR + 2 * u, w, dtb, cb);
    }
    double v[kRed];
    pack9(dtb, cb, v);
    block_sum9<kRThreads>(v, part);
}

template <int MODE>
__device__ __forceinline__ void r_volume(const AdjArgs& a, int tx, int ty, double* part) {
    const int tid = threadIdx.x, i = tx * 16 + (tid & 15), j = ty * 8 + (tid >> 4);
    double dtb = 0.0;
    ConstBar cb;
    lsh::cb_zero(cb);
    if (i < a.c.nx && j < a.c.ny) lsh::volume_adj_body<MODE>(a, j * a.c.nx + i, dtb, cb);
    double v[kRed];
    pack9(dtb, cb, v);
    block_sum9<kRThreads>(v, part);
}

// Max (ARG false) or arg-max (ARG true) of the stage-1 rate over a cell tile.
template <bool ARG>
__device__ __forceinline__ void r_rate(const AdjArgs& a, const RMember& M, int tx, int ty) {
    const int tid = threadIdx.x, i = tx * 16 + (tid & 15), j = ty * 8 + (tid >> 4);
    const bool in = (i < a.c.nx && j < a.c.ny);
    const long long id = (long long)j * a.c.nx + i;
    unsigned long long b = 0;
    if (in) {
        const double w = a.acc[6][id];
        const double rate = (w < lsh::kEps) ? 0.0 : w * a.geo.inv_area[j];
        b = lshm::bits_of(rate);
    }
    if (!ARG) {
        lsh::block_max_bits<kRThreads>(b, M.rmax);
    } else {
        const unsigned long long m = *M.rmax;
        if (in && m != 0 && b == m) atomicMin((unsigned long long*)M.argmax, (unsigned long long)id);
    }
}

template <int ORDER>
__global__ void __launch_bounds__(kRThreads, LSH_ADJB_MINB) k_adjb_reverse(RPlan P, int parity, int step) {
    __shared__ __align__(16) unsigned long long sargs[(sizeof(AdjArgs) + 7) / 8];
    __shared__ int s_first, s_pass, s_scen, s_tile, s_ntx, s_copy, s_lo, s_hi, s_key;
    AdjArgs& a = *reinterpret_cast<AdjArgs*>(sargs);
    const int tid = threadIdx.x;
    // thread 0's: the producer rows and the full passes last found complete,
    // and the (member, rate) its patched dt and rate selection belong to
    WaitCache wc;
    int full_pass = -1, full_scen = -1, patch_scen = -1, patch_rate = -1;
    if (tid == 0) { s_lo = 0; s_hi = 0; s_key = -1; }
    for (;;) {
        if (tid == 0) s_first = (int)atomicAdd(P.head, (unsigned)LSH_ADJB_FETCH);
        __syncthreads();
        const int first = s_first;
        if (first >= P.total_items) break;
        const int last = min(first + LSH_ADJB_FETCH, P.total_items);
        for (int it = first; it < last; ++it) {
            if (tid == 0) {
                if (it < s_lo || it >= s_hi) {
                    int p = 0;
                    while (p + 1 < P.npass && it >= P.pass[p + 1].item_off) ++p;
                    const int kind = P.pass[p].kind;
                    const int* tp = P.tile_pre + kind * (P.n + 1);
                    const int l = it - P.pass[p].item_off;
                    int lo = 0, hi = P.n - 1;  // the member: the last one whose first tile is <= l
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (tp[mid] <= l) lo = mid;
                        else hi = mid - 1;
                    }
                    s_pass = p;
                    s_scen = lo;
                    s_lo = P.pass[p].item_off + tp[lo];
                    s_hi = P.pass[p].item_off + tp[lo + 1];
                    s_ntx = P.tiles_x[kind * P.n + lo];
                }
                s_tile = it - s_lo;
                const int key = (parity * kRVars + P.pass[s_pass].var) * P.n + s_scen;
                s_copy = (key != s_key);
                s_key = key;
            }
            __syncthreads();
            const int p = s_pass, s = s_scen, t = s_tile, ntx = s_ntx;
            const RPass ps = P.pass[p];
            if (s_copy) {
                const unsigned long long* src =
                    reinterpret_cast<const unsigned long long*>(P.args + (parity * kRVars + ps.var) * P.n + s);
                for (int k = tid; k < (int)((sizeof(AdjArgs) + 7) / 8); k += kRThreads) sargs[k] = src[k];
                __syncthreads();
            }
            const int ty = t / ntx, tx = t - ty * ntx;
            const RMember& M = P.mem[s];
            if (tid == 0) {
                bool gave_up = false;
                unsigned long long start = 0;
                if (ps.prod >= 0) {
                    const RPass pp = P.pass[ps.prod];
                    int r0, r1, t0, t1;
                    r_item_rows(ps.op, ps.kind, ty, a.c.ny, r0, r1);
                    r_producer_rows(pp.kind, r0, r1, t0, t1);
                    const int rbase = P.row_pre[pp.kind * (P.n + 1) + s];
                    const int nrows = P.row_pre[pp.kind * (P.n + 1) + s + 1] - rbase;
                    t0 = max(t0, 0);
                    t1 = min(t1, nrows - 1);
                    if (!wc.covers(ps.prod, s, t0, t1)) {
                        gave_up = queue_wait(P.ctr + pp.ctr_off + rbase, t0, t1,
                                             (unsigned)P.tiles_x[pp.kind * P.n + s], P.abort_flag, start);
                        if (!gave_up) wc.set(ps.prod, s, t0, t1);
                    }
                }
                if (!gave_up && ps.fprod >= 0 && !(ps.fprod == full_pass && s == full_scen)) {
                    const RPass pp = P.pass[ps.fprod];
                    const int rbase = P.row_pre[pp.kind * (P.n + 1) + s];
                    const int nrows = P.row_pre[pp.kind * (P.n + 1) + s + 1] - rbase;
                    gave_up = queue_wait(P.ctr + pp.ctr_off + rbase, 0, nrows - 1, (unsigned)P.tiles_x[pp.kind * P.n + s],
                                         P.abort_flag, start);
                    if (!gave_up) { full_pass = ps.fprod; full_scen = s; }
                }
                if (gave_up) atomicOr(&M.tm->err, 1 << LSH_ERR_TIMEOUT);
                // the step's dt and, for the stage-1 passes, the rate selection
                // (final once the pass may run: it waits for the rate item)
                if (s_copy || s != patch_scen || ps.rate != patch_rate) {
                    a.dt = M.dts[step];
                    if (ps.rate) { a.rate_cell = M.rsel->cell; a.rate_bar = M.rsel->bar; }
                    else { a.rate_cell = -1; a.rate_bar = 0.0; }
                    patch_scen = s;
                    patch_rate = ps.rate;
                }
            }
            __syncthreads();
            double* part = ps.parts ? M.part + ((size_t)P.part_off[p * P.n + s] + t) * kRed : nullptr;
            switch (ps.op) {
                case kRZero: {
                    const int i = tx * 16 + (tid & 15), j = ty * 8 + (tid >> 4);
                    if (i < a.c.nx && j < a.c.ny) {
                        const int id = j * a.c.nx + i;
                        for (int k = 0; k < 6; ++k) a.Wbar[k][id] = 0.0;
                        if (a.Xbar[0])
                            for (int k = 0; k < 6; ++k) a.Xbar[k][id] = 0.0;
                    }
                    break;
                }
                case kRRateMax: r_rate<false>(a, M, tx, ty); break;
                case kRArgMax: r_rate<true>(a, M, tx, ty); break;
                case kRRateBar:
                    if (tid == 0) ratebar_body(M.rmax, M.argmax, M.red, M.dts + step + 1, M.rsel);
                    break;
                case kREV1: r_edges<1, false, ORDER, 1>(a, tx, ty, part); break;
                case kREV0: r_edges<1, false, ORDER, 0>(a, tx, ty, part); break;
                case kREH1: r_edges<0, false, ORDER, 1>(a, tx, ty, part); break;
                case kREH0: r_edges<0, true, ORDER, 0>(a, tx, ty, part); break;
                default:
                    if constexpr (ORDER == 1) {
                        r_volume<0>(a, tx, ty, part);
                    } else {
                        if (ps.op == kRVol2) r_volume<2>(a, tx, ty, part);
                        else if (ps.op == kRVol1) r_volume<1>(a, tx, ty, part);
                        else {
                            const int i = tx * 16 + (tid & 15), j = ty * 8 + (tid >> 4);
                            if (i < a.c.nx && j < a.c.ny) lsh::recon_adj_cell(a, j * a.c.nx + i);
                        }
                    }
                    break;
            }
            __syncthreads();  // the tile's writes are done, and sargs may be refilled
            if (tid == 0) queue_done(P.ctr + ps.ctr_off + P.row_pre[ps.kind * (P.n + 1) + s] + ty);
        }
    }
}

// Every member's time record for step `step` (k_set_dt), and the arg-max
// scratch reset.
__global__ void k_adjb_pre(const RMember* t, int n, int step) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const RMember M = t[s];
    set_dt_body(M.tm, M.dts + step);
    *M.rmax = 0ull;
    *M.argmax = 0x7fffffffffffffffLL;
}

// After a forward step: its dt and gauge records (k_record, k_gauge_eta); one block per member.
__global__ void k_adjb_record(const FMember* t, int step) {
    const FMember f = t[blockIdx.x];
    if (threadIdx.x == 0) f.dts[step + 1] = f.tm->dt;
    for (int g = threadIdx.x; g < f.ng; g += blockDim.x) {
        const int id = f.gauges[g];
        f.eta[(size_t)step * f.ng + g] = (f.h1[id] + f.h2[id]) - f.H[id];
    }
}

// The queues' counters and heads back to zero.
__global__ void k_adjb_reset(unsigned* c1, int n1, unsigned* h1, unsigned* c2, int n2, unsigned* h2) {
    const int gid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    if (gid == 0) { *h1 = 0u; *h2 = 0u; }
    for (int i = gid; i < n1; i += stride) c1[i] = 0u;
    for (int i = gid; i < n2; i += stride) c2[i] = 0u;
}

__global__ void __launch_bounds__(32 * kRed) k_adjb_reduce_rows(const RRed* t) {
    const RRed r = t[blockIdx.y];
    reduce_rows_body(r.part, r.nparts, (r.nparts + kReduceRows - 1) / kReduceRows, r.part2, blockIdx.x);
}

__global__ void __launch_bounds__(32 * kRed) k_adjb_reduce(const RRed* t) {
    const RRed r = t[blockIdx.x];
    reduce_body(r.part2, kReduceRows, r.red);
}

__global__ void k_adjb_gauges(const RMis* t, int m) {
    const RMis& r = t[blockIdx.y];
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= r.ng) return;
    gauge_add(r.b[0], r.b[3], r.gauges, r.ng, r.eta + (size_t)(m - 1) * r.ng, r.tgt + (size_t)(m - 1) * r.ng, r.w, g);
}

__global__ void __launch_bounds__(kCellBlock) k_adjb_project(const RMis* t) {
    const RMis& r = t[blockIdx.y];
    if (!(r.h_adj > 0.0)) return;
    project_cells(r.b[0], r.b[1], r.b[2], r.b[3], r.b[4], r.b[5], r.h1, r.h2, r.N, r.h_adj,
                  (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
}

// The members of one order, with their queues and tables.
struct AdjGroup {
    int order = 1;
    std::vector<lsh_adjoint*> m;
    KArgs* d_kargs = nullptr;  // [2][n] the forward step, then [8][n] the recomputation
    void* qmem_fwd = nullptr;
    void* qmem_rec = nullptr;
    void* rmem = nullptr;      // the reverse plan's tables and counters
    void* tables = nullptr;    // AdjArgs [2][kRVars][n], RMember [n], FMember [n], RMis [2][n], RRed [n]
    BPlan fwd{}, rec{};
    int nctr_fwd = 0, nctr_rec = 0;
    RPlan rev{};
    int nctr_rev = 0;
    AdjArgs* d_aargs = nullptr;
    RMember* d_mem = nullptr;
    FMember* d_fmem = nullptr;
    RMis* d_mis = nullptr;
    RRed* d_red = nullptr;
    int max_ng = 0;
    unsigned proj_blocks = 1;
    int parity = 0;            // Xb / Xbn as the AdjArgs of parity 0 hold them, or swapped (1)
};

void free_group(AdjGroup& g) {
    cudaFree(g.d_kargs); cudaFree(g.qmem_fwd); cudaFree(g.qmem_rec); cudaFree(g.rmem); cudaFree(g.tables);
    g = AdjGroup{};
}

// The reverse plan (order 2: 16 passes, order 1: 9).
int build_rplan(AdjGroup& g) {
    const int n = (int)g.m.size();
    struct Spec { int op, kind, var, prod, fprod, rate, parts; };
    std::vector<Spec> sp;
    if (g.order == 2) {
        sp = {{kRZero, kRCell, 5, -1, -1, 0, 0},   {kRRateMax, kRCell, 0, -1, -1, 0, 0},
              {kRArgMax, kRCell, 0, -1, 1, 0, 0},  {kRRateBar, kRMember, 0, -1, 2, 0, 0},
              {kRVol2, kRCell, 5, 0, -1, 0, 1},    {kREV1, kRV1, 6, 4, -1, 0, 1},
              {kREV0, kRV0, 7, 5, -1, 0, 1},       {kREH1, kRH1, 8, 6, -1, 0, 1},
              {kREH0, kRH0, 9, 7, -1, 0, 1},       {kRRecon, kRCell, 5, 8, -1, 0, 0},
              {kRVol1, kRCell, 0, 9, 3, 1, 1},     {kREV1, kRV1, 1, 10, -1, 1, 1},
              {kREV0, kRV0, 2, 11, -1, 1, 1},      {kREH1, kRH1, 3, 12, -1, 1, 1},
              {kREH0, kRH0, 4, 13, -1, 1, 1},      {kRRecon, kRCell, 0, 14, -1, 0, 0}};
    } else {
        sp = {{kRZero, kRCell, 0, -1, -1, 0, 0},  {kRRateMax, kRCell, 0, -1, -1, 0, 0},
              {kRArgMax, kRCell, 0, -1, 1, 0, 0}, {kRRateBar, kRMember, 0, -1, 2, 0, 0},
              {kRVol0, kRCell, 0, 0, 3, 1, 1},    {kREV1, kRV1, 1, 4, -1, 1, 1},
              {kREV0, kRV0, 2, 5, -1, 1, 1},      {kREH1, kRH1, 3, 6, -1, 1, 1},
              {kREH0, kRH0, 4, 7, -1, 1, 1}};
    }
    std::vector<int> tile_pre(size_t(kRKinds) * (n + 1)), row_pre(size_t(kRKinds) * (n + 1)), tiles_x(size_t(kRKinds) * n);
    long long kind_tiles[kRKinds], kind_rows[kRKinds];
    for (int k = 0; k < kRKinds; ++k) {
        long long tsum = 0, rsum = 0;
        for (int s = 0; s < n; ++s) {
            int tx, ty;
            adj_tiles(g.m[s]->p.nx, g.m[s]->p.ny, k, tx, ty);
            tile_pre[k * (n + 1) + s] = (int)tsum;
            row_pre[k * (n + 1) + s] = (int)rsum;
            tiles_x[k * n + s] = tx;
            tsum += (long long)tx * ty;
            rsum += ty;
        }
        tile_pre[k * (n + 1) + n] = (int)tsum;
        row_pre[k * (n + 1) + n] = (int)rsum;
        kind_tiles[k] = tsum;
        kind_rows[k] = rsum;
    }
    RPlan& P = g.rev;
    P = RPlan{};
    P.n = n;
    P.npass = (int)sp.size();
    std::vector<int> part_off(sp.size() * n, 0);
    std::vector<long long> part_run(n, 0);
    long long items = 0, ctrs = 0;
    for (int i = 0; i < P.npass; ++i) {
        RPass& q = P.pass[i];
        q.op = sp[i].op; q.kind = sp[i].kind; q.var = sp[i].var; q.prod = sp[i].prod; q.fprod = sp[i].fprod;
        q.rate = sp[i].rate; q.parts = sp[i].parts;
        q.item_off = (int)items;
        q.ctr_off = (int)ctrs;
        items += kind_tiles[q.kind];
        ctrs += kind_rows[q.kind];
        for (int s = 0; s < n; ++s) {
            part_off[(size_t)i * n + s] = (int)part_run[s];
            if (q.parts) part_run[s] += tile_pre[q.kind * (n + 1) + s + 1] - tile_pre[q.kind * (n + 1) + s];
        }
    }
    for (int s = 0; s < n; ++s)
        if (part_run[s] > g.m[s]->part_rows) { lsh::set_last_error("batched adjoint: partial-sum rows"); return LSH_ERR_INVALID; }
    if (items > 0x7fffffffLL - 1024 || ctrs > 0x7fffffffLL) {
        lsh::set_last_error("batched adjoint too large for one step's work queue");
        return LSH_ERR_INVALID;
    }
    P.total_items = (int)items;
    g.nctr_rev = (int)ctrs;
    const size_t nints = tile_pre.size() + row_pre.size() + tiles_x.size() + part_off.size();
    const size_t ibytes = (nints * sizeof(int) + 255) & ~size_t(255);
    A_CUDA(cudaMalloc(&g.rmem, ibytes + size_t(ctrs) * sizeof(unsigned) + 256));
    int* ti = static_cast<int*>(g.rmem);
    std::vector<int> all;
    all.reserve(nints);
    all.insert(all.end(), tile_pre.begin(), tile_pre.end());
    all.insert(all.end(), row_pre.begin(), row_pre.end());
    all.insert(all.end(), tiles_x.begin(), tiles_x.end());
    all.insert(all.end(), part_off.begin(), part_off.end());
    A_CUDA(cudaMemcpy(ti, all.data(), nints * sizeof(int), cudaMemcpyHostToDevice));
    P.tile_pre = ti;
    P.row_pre = ti + tile_pre.size();
    P.tiles_x = P.row_pre + row_pre.size();
    P.part_off = P.tiles_x + tiles_x.size();
    char* rest = static_cast<char*>(g.rmem) + ibytes;
    P.ctr = reinterpret_cast<unsigned*>(rest);
    P.head = P.ctr + ctrs;
    P.abort_flag = reinterpret_cast<int*>(P.head + 1);
    A_CUDA(cudaMemset(rest, 0, size_t(ctrs) * sizeof(unsigned) + 256));
    P.args = g.d_aargs;
    P.mem = g.d_mem;
    // the partial-sum tables of the reduction
    std::vector<RRed> red(n);
    for (int s = 0; s < n; ++s) red[s] = RRed{g.m[s]->part, part_run[s], g.m[s]->part2, g.m[s]->red};
    A_CUDA(cudaMemcpy(g.d_red, red.data(), sizeof(RRed) * n, cudaMemcpyHostToDevice));
    return LSH_OK;
}

// The group's queues and tables (pointers that live as long as the members).
int build_group(AdjGroup& g) {
    const int n = (int)g.m.size();
    std::vector<int> nx(n), ny(n);
    std::vector<KArgs> ka(size_t(10) * n);
    for (int s = 0; s < n; ++s) {
        lsh_adjoint* A = g.m[s];
        nx[s] = A->p.nx;
        ny[s] = A->p.ny;
        double* const* X = A->X;
        double* Y7[7];
        for (int k = 0; k < 6; ++k) Y7[k] = A->Y[k];
        Y7[6] = A->X[6];
        // the forward step: stage 1 (X -> Y, or X -> X), stage 2 (Y -> X, averaged with X)
        const KArgs a1 = (g.order == 1) ? fwd_args(A, X, X, nullptr, A->acc1, nullptr, nullptr)
                                        : fwd_args(A, X, A->Y, nullptr, A->acc1, A->s1x, A->s1y);
        ka[s] = a1;
        ka[n + s] = (g.order == 1) ? a1 : fwd_args(A, Y7, X, X, A->acc2, A->s2x, A->s2y);
        // the recomputation: per stage the plain arguments (with the branch
        // tape), then the three snapshot-taking edge passes
        KArgs r1 = (g.order == 1) ? fwd_args(A, X, nullptr, nullptr, A->acc1, nullptr, nullptr)
                                  : fwd_args(A, X, A->Y, nullptr, A->acc1, A->s1x, A->s1y);
        r1.tape = A->tape1;
        KArgs r2 = r1;
        if (g.order == 2) {
            r2 = fwd_args(A, Y7, nullptr, nullptr, A->acc2, A->s2x, A->s2y);
            r2.tape = A->tape2;
        }
        for (int st = 0; st < 2; ++st) {
            const KArgs& base = st ? r2 : r1;
            double* const (*snaps)[2] = st ? A->snap2 : A->snap1;
            ka[size_t(2 + 4 * st) * n + s] = base;
            for (int k = 0; k < 3; ++k) {
                KArgs v = base;
                v.snap[0] = snaps[k][0];
                v.snap[1] = snaps[k][1];
                ka[size_t(2 + 4 * st + 1 + k) * n + s] = v;
            }
        }
        g.max_ng = std::max(g.max_ng, A->ng);
        g.proj_blocks = std::max(g.proj_blocks, (unsigned)A->grid);
    }
    A_CUDA(cudaMalloc(&g.d_kargs, sizeof(KArgs) * ka.size()));
    A_CUDA(cudaMemcpy(g.d_kargs, ka.data(), sizeof(KArgs) * ka.size(), cudaMemcpyHostToDevice));
    // tables
    size_t off = 0;
    auto carve = [&](size_t bytes) { const size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
    const size_t o_a = carve(sizeof(AdjArgs) * 2 * kRVars * n), o_m = carve(sizeof(RMember) * n),
                 o_f = carve(sizeof(FMember) * n), o_mis = carve(sizeof(RMis) * 2 * n), o_r = carve(sizeof(RRed) * n);
    A_CUDA(cudaMalloc(&g.tables, off));
    char* tb = static_cast<char*>(g.tables);
    g.d_aargs = reinterpret_cast<AdjArgs*>(tb + o_a);
    g.d_mem = reinterpret_cast<RMember*>(tb + o_m);
    g.d_fmem = reinterpret_cast<FMember*>(tb + o_f);
    g.d_mis = reinterpret_cast<RMis*>(tb + o_mis);
    g.d_red = reinterpret_cast<RRed*>(tb + o_r);
    // the forward step's queue
    std::vector<QPassSpec> fp, rp;
    const int stages = (g.order == 2) ? 2 : 1;
    for (int st = 0; st < stages; ++st) {
        if (g.order == 2) fp.push_back({kOpRecon, kBCell, st});
        fp.push_back({kOpH0, kBH0, st});
        fp.push_back({kOpH1, kBH1, st});
        fp.push_back({kOpV0, kBV0, st});
        fp.push_back({kOpV1, kBV1, st});
        fp.push_back({(g.order == 1) ? kOpVol0 : (st == 0 ? kOpVol1 : kOpVol2), kBCell, st});
    }
    if (int st = build_queue_plan(nx, ny, fp, g.d_kargs, &g.qmem_fwd, g.fwd, g.nctr_fwd)) return st;
    // the recomputation's queue (variables 0..7 of its table)
    for (int st = 0; st < stages; ++st) {
        const int v = 4 * st;
        if (g.order == 2) rp.push_back({kOpReconTape, kBCell, v});
        rp.push_back({kOpH0, kBH0, v});
        rp.push_back({kOpH1, kBH1, v + 1});
        rp.push_back({kOpV0, kBV0, v + 2});
        rp.push_back({kOpV1, kBV1, v + 3});
        if (g.order == 2 && st == 0) rp.push_back({kOpVol1, kBCell, v});
    }
    if (int st = build_queue_plan(nx, ny, rp, g.d_kargs + 2 * n, &g.qmem_rec, g.rec, g.nctr_rec)) return st;
    return build_rplan(g);
}

// The per-run tables: the records' pointers (after fwd_alloc) and, at the
// start of a reverse sweep, the adjoint arguments of both parities and the
// misfit terms.
int group_tables(AdjGroup& g, bool sweep) {
    const int n = (int)g.m.size();
    std::vector<RMember> mem(n);
    std::vector<FMember> fm(n);
    for (int s = 0; s < n; ++s) {
        lsh_adjoint* A = g.m[s];
        mem[s] = RMember{A->rmax, A->argmax, A->rsel, A->red, A->d_dts, A->part, A->tm};
        fm[s] = FMember{A->tm, A->d_dts, A->X[0], A->X[3], A->X[6], A->d_gauges, A->ng, A->d_eta};
    }
    A_CUDA(cudaMemcpy(g.d_mem, mem.data(), sizeof(RMember) * n, cudaMemcpyHostToDevice));
    A_CUDA(cudaMemcpy(g.d_fmem, fm.data(), sizeof(FMember) * n, cudaMemcpyHostToDevice));
    if (!sweep) return LSH_OK;
    std::vector<AdjArgs> aa(size_t(2) * kRVars * n);
    std::vector<RMis> mis(size_t(2) * n);
    for (int par = 0; par < 2; ++par) {
        for (int s = 0; s < n; ++s) {
            lsh_adjoint* A = g.m[s];
            double* Xb[6], *Xbn[6];
            for (int k = 0; k < 6; ++k) {
                Xb[k] = par ? A->Xbn[k] : A->Xb[k];
                Xbn[k] = par ? A->Xb[k] : A->Xbn[k];
            }
            double* Y7[7];
            for (int k = 0; k < 6; ++k) Y7[k] = A->Y[k];
            Y7[6] = A->X[6];
            AdjArgs st[2];
            // stage 1 (order 1: the step) and stage 2
            if (g.order == 1) {
                st[0] = adj_args(A, A->X, nullptr, nullptr, A->acc1, Xbn, Xb, nullptr, nullptr, 0.0);
                st[1] = st[0];
            } else {
                st[0] = adj_args(A, A->X, A->s1x, A->s1y, A->acc1, Xbn, A->Yb, nullptr, A->tape1, 0.0);
                st[1] = adj_args(A, Y7, A->s2x, A->s2y, A->acc2, A->Yb, Xb, Xbn, A->tape2, 0.0);
            }
            for (int h = 0; h < 2; ++h) {
                double* const (*snaps)[2] = h ? A->snap2 : A->snap1;
                // variables: base, then the edge passes v1, v0, h1 (snapshots 2, 1, 0), h0 (none)
                for (int v = 0; v < 5; ++v) {
                    AdjArgs x = st[h];
                    x.snap[0] = x.snap[1] = nullptr;
                    if (v >= 1 && v <= 3) { x.snap[0] = snaps[3 - v][0]; x.snap[1] = snaps[3 - v][1]; }
                    aa[(size_t(par) * kRVars + 5 * h + v) * n + s] = x;
                }
            }
            RMis r{};
            for (int k = 0; k < 6; ++k) r.b[k] = Xb[k];
            r.h1 = A->X[0];
            r.h2 = A->X[3];
            r.gauges = A->d_gauges;
            r.ng = (A->have_target && A->ng > 0 && A->misfit_weight != 0.0) ? A->ng : 0;
            r.eta = A->d_eta;
            r.tgt = A->d_tgt;
            r.w = A->misfit_weight;
            r.h_adj = A->h_adj;
            r.N = (long long)A->N;
            mis[size_t(par) * n + s] = r;
        }
    }
    A_CUDA(cudaMemcpy(g.d_aargs, aa.data(), sizeof(AdjArgs) * aa.size(), cudaMemcpyHostToDevice));
    A_CUDA(cudaMemcpy(g.d_mis, mis.data(), sizeof(RMis) * mis.size(), cudaMemcpyHostToDevice));
    g.parity = 0;
    return LSH_OK;
}

#ifndef LSH_ADJB_FWD_CTAS
#define LSH_ADJB_FWD_CTAS 20  // forward queue CTAs per SM (at most kBMaxCtas)
#endif
#ifndef LSH_ADJB_FWD_FETCH
#define LSH_ADJB_FWD_FETCH 2
#endif
constexpr int kAdjbFwdCtas = LSH_ADJB_FWD_CTAS;
constexpr int kAdjbFwdFetch = LSH_ADJB_FWD_FETCH;

// Forward step n -> n + 1 of every member (RECORD: with its dt and gauge records).
void group_forward(AdjGroup& g, int sms, int n, bool record, cudaStream_t s) {
    const int nm = (int)g.m.size();
    if (!record) k_adjb_pre<<<(nm + 127) / 128, 128, 0, s>>>(g.d_mem, nm, n);
    const int grid = sms * kAdjbFwdCtas;
    if (g.order == 1) k_batch_step<1><<<grid, kBThreads, 0, s>>>(g.fwd, kAdjbFwdFetch);
    else k_batch_step<2><<<grid, kBThreads, 0, s>>>(g.fwd, kAdjbFwdFetch);
    const int adv = std::max(1, std::min((std::max(g.nctr_fwd, nm) + 255) / 256, 2 * sms));
    k_batch_advance<<<adv, 256, 0, s>>>(g.d_kargs, nm, g.fwd.ctr, g.nctr_fwd, g.fwd.head);
    if (record) k_adjb_record<<<nm, 128, 0, s>>>(g.d_fmem, n);
}

// The adjoint of step n for every member (Ops::reverse_step, batched).
void group_reverse(AdjGroup& g, int sms, int n, cudaStream_t s) {
    const int nm = (int)g.m.size();
    k_adjb_pre<<<(nm + 127) / 128, 128, 0, s>>>(g.d_mem, nm, n);
    const int grid = sms * kAdjbFwdCtas;
    if (g.order == 1) k_batch_step<1, ReconTape><<<grid, kBThreads, 0, s>>>(g.rec, kAdjbFwdFetch);
    else k_batch_step<2, ReconTape><<<grid, kBThreads, 0, s>>>(g.rec, kAdjbFwdFetch);
    const int rgrid = sms * LSH_ADJB_MINB;
    if (g.order == 1) k_adjb_reverse<1><<<rgrid, kRThreads, 0, s>>>(g.rev, g.parity, n);
    else k_adjb_reverse<2><<<rgrid, kRThreads, 0, s>>>(g.rev, g.parity, n);
    const int rst = std::max(1, std::min((std::max(g.nctr_rec, g.nctr_rev) + 255) / 256, 2 * sms));
    k_adjb_reset<<<rst, 256, 0, s>>>(g.rec.ctr, g.nctr_rec, g.rec.head, g.rev.ctr, g.nctr_rev, g.rev.head);
    k_adjb_reduce_rows<<<dim3(kReduceRows, nm), 32 * kRed, 0, s>>>(g.d_red);
    k_adjb_reduce<<<nm, 32 * kRed, 0, s>>>(g.d_red);
    // the new adjoint is in Xbn: swap, as Ops::reverse_step does
    for (lsh_adjoint* A : g.m) {
        for (int k = 0; k < 6; ++k) std::swap(A->Xb[k], A->Xbn[k]);
        A->stats.reversed_steps += 1;
    }
    g.parity ^= 1;
    if (n >= 1) {
        if (g.max_ng > 0) k_adjb_gauges<<<dim3((g.max_ng + 127) / 128, nm), 128, 0, s>>>(g.d_mis + (size_t)g.parity * nm, n);
        k_adjb_project<<<dim3(g.proj_blocks, nm), kCellBlock, 0, s>>>(g.d_mis + (size_t)g.parity * nm);
    }
}

}  // namespace

struct lsh_adjoint_batch {
    std::vector<lsh_adjoint*> m;
    std::vector<AdjGroup> groups;  // the members by order
    cudaStream_t stream = nullptr; // every member's stream
    int sms = 152;
    double budget = -1.0;  // < 0: 180 GB, capped by free memory at the forward run
    int nsteps = 0;
    int n_slots = 0;
    bool have_forward = false;
    lsh_adjoint_stats stats{};
};

namespace {

// The schedule's operations for the whole batch: one schedule, one slot
// count, every member's state at the same step; each operation one set of
// launches per group.
struct BatchOps : lsh::RevolveOps {
    lsh_adjoint_batch* B;
    explicit BatchOps(lsh_adjoint_batch* b) : B(b) {}
    int advance(int from, int to) override {
        for (int n = from; n < to; ++n)
            for (AdjGroup& g : B->groups) {
                group_forward(g, B->sms, n, false, B->stream);
                for (lsh_adjoint* A : g.m) A->stats.recompute_steps += 1;
            }
        A_CUDA(cudaGetLastError());
        return 0;
    }
    int store(int k) override {
        for (lsh_adjoint* A : B->m)
            if (int st = Ops(A).store(k)) return st;
        return 0;
    }
    int restore(int k, int step) override {
        for (lsh_adjoint* A : B->m)
            if (int st = Ops(A).restore(k, step)) return st;
        return 0;
    }
    int reverse_step(int n) override {
        for (AdjGroup& g : B->groups) group_reverse(g, B->sms, n, B->stream);
        A_CUDA(cudaGetLastError());
        return 0;
    }
};

}  // namespace

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
    if (A->stream && A->own_stream) cudaStreamDestroy(A->stream);
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

int lsh_adjoint_set_ordered(lsh_adjoint* A, int ordered) {
    if (!A) return LSH_ERR_INVALID;
    A->ordered = (ordered != 0);
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
    // one stream for all members, so that their own operations (uploads,
    // checkpoint copies) and the batch's launches stay in order
    B->sms = B->m[0]->sms;
    {
        cudaError_t e = cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { const int st = afail(e, "cudaStreamCreate"); lsh_adjoint_batch_destroy(B); return st; }
    }
    for (lsh_adjoint* A : B->m) {
        cudaStreamSynchronize(A->stream);
        cudaStreamDestroy(A->stream);
        A->stream = B->stream;
        A->own_stream = false;
    }
    for (int order = 1; order <= 2; ++order) {
        AdjGroup g;
        g.order = order;
        for (lsh_adjoint* A : B->m)
            if (A->order == order) g.m.push_back(A);
        if (g.m.empty()) continue;
        B->groups.push_back(g);
        if (int st = build_group(B->groups.back())) {
            lsh_adjoint_batch_destroy(B);
            return st;
        }
    }
    *out = B;
    return LSH_OK;
}

int lsh_adjoint_batch_destroy(lsh_adjoint_batch* B) {
    if (!B) return LSH_OK;
    if (B->stream) cudaStreamSynchronize(B->stream);
    for (AdjGroup& g : B->groups) free_group(g);
    for (lsh_adjoint* A : B->m) destroy_adjoint(A);
    if (B->stream) cudaStreamDestroy(B->stream);
    (void)cudaGetLastError();
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
    for (AdjGroup& g : B->groups)
        if (int st = group_tables(g, false)) return st;
    for (int i = 0; i < n; ++i)
        if (int st = fwd_begin(B->m[i], host_states + (size_t)i * LSH_NVARS, targets ? targets[i] : nullptr)) return st;
    BatchOps ops(B);
    int a = 0, slot = 0;
    auto run = [&](int to) -> int {
        for (int s = a; s < to; ++s)
            for (AdjGroup& g : B->groups) {
                group_forward(g, B->sms, s, true, B->stream);
                for (lsh_adjoint* A : g.m) A->stats.forward_steps += 1;
            }
        A_CUDA(cudaGetLastError());
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
    BatchOps ops(B);
    ops.cur = A0->cur_step;
    for (int i = 0; i < n; ++i)
        if (int st = grad_begin(B->m[i], misfit_weights ? misfit_weights[i] : 1.0, nullptr)) return st;
    for (AdjGroup& g : B->groups)
        if (int st = group_tables(g, true)) return st;
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
