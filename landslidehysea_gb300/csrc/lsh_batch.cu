// lsh_batch.cu -- batched ensemble: many scenarios on uneven grids advanced
// together on one GPU (C ABI in include/lsh.h, lsh_batch_*).
//
// Every scenario keeps its own parameters, geometry, state and device clock
// (t, dt), in one slab.  A step runs the same passes as the single-grid path
// (reconstruction, 4 colour edge passes, Euler stage; twice at second
// order), with the same device code (lsh_passes.cuh), but the whole step of
// every scenario is ONE persistent launch: CTAs of 64 threads pull work items
// -- (pass, scenario, 2-D tile of the single-grid shapes) -- from a device
// queue, in pass order.  An item waits only for the rows of its own scenario
// that the pass before it writes (per-row completion counters, as the
// single-grid path's overlapped launches do), so a pass of one scenario runs
// while other scenarios, or other rows, are still in the pass before: no
// whole-grid barrier between passes.  Items of one pass touch disjoint cells
// of their scenario, so which CTA takes an item, and when, changes no bit:
// every scenario is bit-identical to its single-grid run.  A small kernel
// then advances every scenario's clock and resets the queue and counters, so
// a run of steps is one CUDA graph launch.  The CTA count per SM and the
// items taken per queue fetch are picked by lsh_batch_autotune, which times
// candidates on the live batch.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/lsh.h"
#include "lsh_passes.cuh"
#include "lsh_setup.h"

using lsh::KArgs;
using lsh::kCellBlock;
using lsh::kEdgeBlock;
using lsh::kRateInitBits;

namespace {

constexpr int kBatchGraphSteps = 8;
constexpr int kBThreads = 64;    // threads per persistent CTA
constexpr int kBMaxCtas = 20;    // CTAs per SM the step kernel is compiled for (48 registers)
constexpr int kMaxPasses = 12;

// Tilings of a scenario's passes, 64-thread tiles of the single-grid shapes:
// horizontal edges of parity 0 / 1 (16 columns x 4 edge lines), vertical
// edges of parity 0 / 1 (8 edge columns x 8 rows), cells (16 x 4).
enum BKind : int { kBH0 = 0, kBH1 = 1, kBV0 = 2, kBV1 = 3, kBCell = 4, kBKinds = 5 };
constexpr int kTileHX = 16, kTileHY = 4, kTileVX = 8, kTileVY = 8, kTileCX = 16, kTileCY = 4;
// What a pass does.
enum BOp : int { kOpH0 = 0, kOpH1 = 1, kOpV0 = 2, kOpV1 = 3, kOpRecon = 4, kOpVol0 = 5, kOpVol1 = 6, kOpVol2 = 7 };

struct BPass {
    int op;        // BOp
    int kind;      // BKind of its tiles
    int stage;     // arguments: args[s] (stage 1) or args[n + s] (stage 2)
    int prod;      // the pass whose writes it reads (-1: the step's first pass)
    int item_off;  // first item of the pass in the step's queue
    int ctr_off;   // first counter of the pass
};

// Everything the step kernel needs, passed by value.
struct BPlan {
    int n;                  // scenarios
    int npass;
    int total_items;
    BPass pass[kMaxPasses];
    const int* tile_pre;    // [kind][n + 1]: first tile of each scenario (prefix sums)
    const int* row_pre;     // [kind][n + 1]: first tile row of each scenario
    const int* tiles_x;     // [kind][n]: tiles per tile row
    const KArgs* args;      // [n] stage 1, [n, 2n) stage 2 (second order)
    unsigned* ctr;          // completion counters: per pass, per scenario tile row
    unsigned* head;         // the step's queue head
    int* abort_flag;        // set when a wait gives up; later waits give up at once
};

// Cell rows an item of `op` reads (tile row ty of a scenario with ny rows).
__device__ __forceinline__ void item_rows(int op, int ty, int ny, int& r0, int& r1) {
    if (op == kOpH0 || op == kOpH1) {
        const int y0 = op + 2 * kTileHY * ty;  // first edge row (parity op)
        r0 = y0 - 1; r1 = y0 + 2 * (kTileHY - 1);
    } else if (op == kOpV0 || op == kOpV1) {
        r0 = kTileVY * ty; r1 = r0 + kTileVY - 1;
    } else if (op == kOpRecon) {
        r0 = kTileCY * ty - 1; r1 = kTileCY * ty + kTileCY;
    } else {
        r0 = kTileCY * ty; r1 = r0 + kTileCY - 1;
    }
    r0 = max(r0, 0);
    r1 = min(r1, ny - 1);
}

// Tile rows of a pass of `kind` that write cell rows [r0, r1].
__device__ __forceinline__ void producer_rows(int kind, int r0, int r1, int& t0, int& t1) {
    if (kind == kBV0 || kind == kBV1) { t0 = r0 / kTileVY; t1 = r1 / kTileVY; }
    else if (kind == kBCell) { t0 = r0 / kTileCY; t1 = r1 / kTileCY; }
    else {
        // horizontal edge row y = p + 2 t writes cell rows y - 1 and y
        const int p = kind;
        t0 = (max(r0 - p + 1, 0) / 2) / kTileHY;
        t1 = (max(r1 + 1 - p, 0) / 2) / kTileHY;
    }
}

// One item's work: the single-grid kernels' per-thread bodies on one tile.
template <int ORDER, int OP>
__device__ __forceinline__ void item_work(const KArgs& a, int tx, int ty, double dt) {
    const int nx = a.c.nx, ny = a.c.ny, tid = threadIdx.x;
    if (OP == kOpH0 || OP == kOpH1) {
        const int par = OP;
        const int x = tx * kTileHX + tid % kTileHX, line = ty * kTileHY + tid / kTileHX;
        if (x < nx && line < (ny - par) / 2 + 1) lsh::do_edge<0, OP == kOpH0, ORDER>(a, x, par + 2 * line, dt);
    } else if (OP == kOpV0 || OP == kOpV1) {
        const int par = OP - kOpV0;
        const int x = par + 2 * (tx * kTileVX + tid % kTileVX), y = ty * kTileVY + tid / kTileVX;
        if (x <= nx && y < ny) lsh::do_edge<1, false, ORDER>(a, x, y, dt);
    } else {
        const int i = tx * kTileCX + tid % kTileCX, j = ty * kTileCY + tid / kTileCX;
        const bool in = (i < nx && j < ny);
        if (OP == kOpRecon) {
            if (in) lsh::recon_cell(a, j * nx + i);
        } else {
            constexpr int MODE = OP - kOpVol0;
            unsigned long long bits = kRateInitBits;
            if (in) bits = lsh::volume_cell<MODE>(a, j * nx + i, dt);
            if (MODE != 2) lsh::block_max_bits<kBThreads>(bits, &a.tm->rmax_bits);
        }
    }
}

// The whole step of every scenario.  Items are dequeued in pass order, and an
// item waits only for items of earlier passes, which running CTAs took
// before it: the earliest unfinished item always has its inputs, so the
// queue drains whatever the number of resident CTAs.  Waits are bounded
// (~2 s of %globaltimer); one that runs out sets LSH_ERR_TIMEOUT on its
// scenario and the batch's abort flag, and later waits give up at once.
template <int ORDER>
__global__ void __launch_bounds__(kBThreads, kBMaxCtas) k_batch_step(BPlan P, int fetch) {
    __shared__ __align__(16) unsigned long long sargs[(sizeof(KArgs) + 7) / 8];
    __shared__ int s_first, s_pass, s_scen, s_tile, s_ntx, s_copy;
    // the last decoded (pass, scenario): its items [s_lo, s_hi) of the queue,
    // and the arguments held in sargs (stage * n + scenario, -1: none).
    // Consecutive items of the queue share them, so most items skip the
    // scenario search and the argument copy.
    __shared__ int s_lo, s_hi, s_args_key;
    const KArgs& a = *reinterpret_cast<const KArgs*>(sargs);
    const int tid = threadIdx.x;
    if (tid == 0) { s_lo = 0; s_hi = 0; s_args_key = -1; }
    for (;;) {
        if (tid == 0) s_first = (int)atomicAdd(P.head, (unsigned)fetch);
        __syncthreads();
        const int first = s_first;
        if (first >= P.total_items) break;
        const int last = min(first + fetch, P.total_items);
        for (int it = first; it < last; ++it) {
            if (tid == 0) {
                if (it < s_lo || it >= s_hi) {
                    int p = 0;
                    while (p + 1 < P.npass && it >= P.pass[p + 1].item_off) ++p;
                    const int kind = P.pass[p].kind;
                    const int* tp = P.tile_pre + kind * (P.n + 1);
                    const int l = it - P.pass[p].item_off;
                    int lo = 0, hi = P.n - 1;  // the scenario: the last one whose first tile is <= l
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
                const int key = P.pass[s_pass].stage * P.n + s_scen;
                s_copy = (key != s_args_key);
                s_args_key = key;
            }
            __syncthreads();
            const int p = s_pass, s = s_scen, t = s_tile, ntx = s_ntx;
            const BPass ps = P.pass[p];
            if (s_copy) {
                const unsigned long long* src = reinterpret_cast<const unsigned long long*>(P.args + ps.stage * P.n + s);
                for (int k = tid; k < (int)((sizeof(KArgs) + 7) / 8); k += kBThreads) sargs[k] = src[k];
                __syncthreads();
            }
            const int ty = t / ntx, tx = t - ty * ntx;
            const bool live = !a.tm->done;  // uniform: the clock changes between steps only
            if (live && ps.prod >= 0 && tid == 0) {
                const BPass pp = P.pass[ps.prod];
                int r0, r1, t0, t1;
                item_rows(ps.op, ty, a.c.ny, r0, r1);
                producer_rows(pp.kind, r0, r1, t0, t1);
                const int rbase = P.row_pre[pp.kind * (P.n + 1) + s];
                const int nrows = P.row_pre[pp.kind * (P.n + 1) + s + 1] - rbase;
                t0 = max(t0, 0);
                t1 = min(t1, nrows - 1);
                const unsigned target = (unsigned)P.tiles_x[pp.kind * P.n + s];
                const unsigned* c = P.ctr + pp.ctr_off + rbase;
                volatile int* abort_flag = P.abort_flag;
                unsigned long long start = 0;
                bool gave_up = false;
                for (int r = t0; r <= t1 && !gave_up; ++r) {
                    unsigned ns = 32;
                    for (;;) {
                        unsigned v;
                        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(c + r) : "memory");
                        if (v >= target) break;
                        if (*abort_flag) { gave_up = true; break; }
                        unsigned long long now;
                        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
                        if (start == 0) start = now;
                        else if (now - start > 2000000000ull) { atomicExch(P.abort_flag, 1); gave_up = true; break; }
                        __nanosleep(ns);
                        if (ns < 1024) ns *= 2;
                    }
                }
                if (gave_up) atomicOr(&a.tm->err, 1 << LSH_ERR_TIMEOUT);
            }
            __syncthreads();
            if (live) {
                const double dt = a.tm->dt;
                switch (ps.op) {
                    case kOpH0: item_work<ORDER, kOpH0>(a, tx, ty, dt); break;
                    case kOpH1: item_work<ORDER, kOpH1>(a, tx, ty, dt); break;
                    case kOpV0: item_work<ORDER, kOpV0>(a, tx, ty, dt); break;
                    case kOpV1: item_work<ORDER, kOpV1>(a, tx, ty, dt); break;
                    default:
                        if constexpr (ORDER == 1) {
                            item_work<ORDER, kOpVol0>(a, tx, ty, dt);
                        } else {
                            if (ps.op == kOpRecon) item_work<ORDER, kOpRecon>(a, tx, ty, dt);
                            else if (ps.op == kOpVol1) item_work<ORDER, kOpVol1>(a, tx, ty, dt);
                            else item_work<ORDER, kOpVol2>(a, tx, ty, dt);
                        }
                        break;
                }
            }
            __syncthreads();  // the tile's writes are done, and sargs may be refilled
            if (tid == 0) {
                // release: the barrier above orders the tile's writes before it
                unsigned* c = P.ctr + ps.ctr_off + P.row_pre[ps.kind * (P.n + 1) + s] + ty;
                asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(c) : "memory");
            }
        }
    }
}

// Every scenario's clock (k_advance of the single-grid path); the queue head
// and the completion counters back to zero for the next step.
__global__ void k_batch_advance(const KArgs* __restrict__ args, int n, unsigned* ctr, int n_ctr, unsigned* head) {
    const int gid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    if (gid == 0) *head = 0u;
    for (int i = gid; i < n_ctr; i += stride) ctr[i] = 0u;
    for (int s = gid; s < n; s += stride) {
        lsh::TimeRec* tm = args[s].tm;
        if (tm->done) continue;
        tm->t += tm->dt;
        tm->steps += 1;
        const double nd = lsh::dt_of(tm->rmax_bits, 2.0 * args[s].c.cfl);
        tm->dt = nd;
        tm->rmax_bits = kRateInitBits;
        if (tm->t >= tm->t_end) tm->done = 1;
        if (tm->dt_min > 0.0 && nd < tm->dt_min) { tm->err |= 1 << LSH_ERR_STALL; tm->done = 1; }
        if (tm->err) tm->done = 1;
    }
}

// Initial dt of one scenario (set_state): wave pass, rate max, dt.
template <int DIR, bool FIRST>
__global__ void __launch_bounds__(kEdgeBlock) k_batch_init_wave(const KArgs* args, int s, int par) {
    const KArgs& a = args[s];
    const int nx = a.c.nx, ny = a.c.ny;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nlines = (DIR == 0) ? (ny - par) / 2 + 1 : (nx - par) / 2 + 1;
    const int nalong = (DIR == 0) ? nx : ny;
    for (int bl = blockIdx.y; bl < ((DIR == 0) ? nlines : nalong); bl += gridDim.y) {
        if (DIR == 0) { if (tid >= nx) return; lsh::init_wave_edge<0, FIRST>(a, tid, par + 2 * bl); }
        else { if (tid >= nlines) return; lsh::init_wave_edge<1, FIRST>(a, par + 2 * tid, bl); }
    }
}

__global__ void __launch_bounds__(kCellBlock) k_batch_init_cells(const KArgs* args, int s) {
    const KArgs& a = args[s];
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long bits = kRateInitBits;
    if (id < a.c.nx * a.c.ny) {
        bits = lsh::init_cell_rate(a, id);
        a.eta_max[id] = a.W[0][id] + a.W[3][id] - a.W[6][id];
        a.eta_time[id] = 0.0;
    }
    lsh::block_max_bits<kCellBlock>(bits, &a.tm->rmax_bits);
}

__global__ void k_batch_init_finish(const KArgs* args, int s) {
    lsh::TimeRec* tm = args[s].tm;
    tm->dt = lsh::dt_of(tm->rmax_bits, 2.0 * args[s].c.cfl);
    tm->rmax_bits = kRateInitBits;
    tm->t = 0.0;
    tm->steps = 0;
    tm->done = 0;
    tm->err = 0;
}

int bfail(cudaError_t e, const char* what) {
    lsh::set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    (void)cudaGetLastError();
    return (e == cudaErrorMemoryAllocation) ? LSH_ERR_GPU_OOM : LSH_ERR_CUDA;
}

#define B_CUDA(call)                                         \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return bfail(e_, #call);      \
    } while (0)

}  // namespace

// ------------------------------------------------------------------ batch object

struct lsh_batch {
    int n = 0;
    int order = 1;
    int device = 0;
    int sms = 152;
    cudaStream_t stream = nullptr;
    std::vector<lsh_params> params;
    std::vector<size_t> base;       // first cell of each scenario in the slab arrays
    size_t total = 0;
    void* slab = nullptr;
    KArgs* d_args = nullptr;        // [n] (stage 1), [n, 2n) (stage 2)
    std::vector<KArgs> h_args;
    lsh::TimeRec* d_tm = nullptr;   // [n]
    void* d_plan_mem = nullptr;     // the plan's tables, counters, queue head and abort flag
    BPlan plan{};
    int n_ctr = 0;                  // completion counters of one step
    lsh_tune tune{};
    cudaGraphExec_t graph = nullptr;
    long long launches = 0;
};

namespace {

constexpr int kernels_per_step = 2;  // the step kernel and the clock kernel

// Tiles of scenario `p` in each tiling: (tiles per row, tile rows).
void scenario_tiles(const lsh_params& p, int kind, int& tx, int& ty) {
    const int nx = p.nx, ny = p.ny;
    if (kind == kBH0 || kind == kBH1) {
        tx = (nx + kTileHX - 1) / kTileHX;
        ty = ((ny - kind) / 2 + 1 + kTileHY - 1) / kTileHY;
    } else if (kind == kBV0 || kind == kBV1) {
        tx = ((nx - (kind - kBV0)) / 2 + 1 + kTileVX - 1) / kTileVX;
        ty = (ny + kTileVY - 1) / kTileVY;
    } else {
        tx = (nx + kTileCX - 1) / kTileCX;
        ty = (ny + kTileCY - 1) / kTileCY;
    }
}

// The step's passes, their items and counters, and the device tables.
int build_plan(lsh_batch* b) {
    const int n = b->n;
    std::vector<int> tile_pre(size_t(kBKinds) * (n + 1)), row_pre(size_t(kBKinds) * (n + 1)), tiles_x(size_t(kBKinds) * n);
    long long kind_tiles[kBKinds], kind_rows[kBKinds];
    for (int k = 0; k < kBKinds; ++k) {
        long long tsum = 0, rsum = 0;
        for (int s = 0; s < n; ++s) {
            int tx, ty;
            scenario_tiles(b->params[s], k, tx, ty);
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
    // the passes of a step, each reading what the one before it wrote
    struct P { int op, kind, stage; };
    std::vector<P> passes;
    const int stages = (b->order == 2) ? 2 : 1;
    for (int st = 0; st < stages; ++st) {
        if (b->order == 2) passes.push_back({kOpRecon, kBCell, st});
        passes.push_back({kOpH0, kBH0, st});
        passes.push_back({kOpH1, kBH1, st});
        passes.push_back({kOpV0, kBV0, st});
        passes.push_back({kOpV1, kBV1, st});
        passes.push_back({(b->order == 1) ? kOpVol0 : (st == 0 ? kOpVol1 : kOpVol2), kBCell, st});
    }
    BPlan& P0 = b->plan;
    P0 = BPlan{};
    P0.n = n;
    P0.npass = (int)passes.size();
    long long items = 0, ctrs = 0;
    for (int i = 0; i < P0.npass; ++i) {
        BPass& q = P0.pass[i];
        q.op = passes[i].op;
        q.kind = passes[i].kind;
        q.stage = passes[i].stage;
        q.prod = i - 1;
        q.item_off = (int)items;
        q.ctr_off = (int)ctrs;
        items += kind_tiles[q.kind];
        ctrs += kind_rows[q.kind];
    }
    if (items > 0x7fffffffLL - 1024 || ctrs > 0x7fffffffLL) {
        lsh::set_last_error("batch too large for one step's work queue");
        return LSH_ERR_INVALID;
    }
    P0.total_items = (int)items;
    b->n_ctr = (int)ctrs;
    // one allocation: tables, counters, queue head, abort flag
    const size_t tbytes = (tile_pre.size() + row_pre.size() + tiles_x.size()) * sizeof(int);
    const size_t bytes = ((tbytes + 255) & ~size_t(255)) + size_t(ctrs) * sizeof(unsigned) + 256;
    if (b->d_plan_mem) { cudaFree(b->d_plan_mem); b->d_plan_mem = nullptr; }
    B_CUDA(cudaMalloc(&b->d_plan_mem, bytes));
    int* ti = static_cast<int*>(b->d_plan_mem);
    B_CUDA(cudaMemcpy(ti, tile_pre.data(), tile_pre.size() * sizeof(int), cudaMemcpyHostToDevice));
    B_CUDA(cudaMemcpy(ti + tile_pre.size(), row_pre.data(), row_pre.size() * sizeof(int), cudaMemcpyHostToDevice));
    B_CUDA(cudaMemcpy(ti + tile_pre.size() + row_pre.size(), tiles_x.data(), tiles_x.size() * sizeof(int),
                      cudaMemcpyHostToDevice));
    P0.tile_pre = ti;
    P0.row_pre = ti + tile_pre.size();
    P0.tiles_x = ti + tile_pre.size() + row_pre.size();
    char* rest = static_cast<char*>(b->d_plan_mem) + ((tbytes + 255) & ~size_t(255));
    P0.ctr = reinterpret_cast<unsigned*>(rest);
    P0.head = reinterpret_cast<unsigned*>(rest + size_t(ctrs) * sizeof(unsigned));
    P0.abort_flag = reinterpret_cast<int*>(P0.head + 1);
    B_CUDA(cudaMemset(rest, 0, size_t(ctrs) * sizeof(unsigned) + 256));
    P0.args = b->d_args;
    return LSH_OK;
}

void enqueue_batch_step(lsh_batch* b, cudaStream_t s) {
    const int grid = std::max(1, b->sms * std::min(std::max(b->tune.ctas_per_sm, 1), kBMaxCtas));
    const int fetch = std::max(1, b->tune.items_per_fetch);
    if (b->order == 1) k_batch_step<1><<<grid, kBThreads, 0, s>>>(b->plan, fetch);
    else k_batch_step<2><<<grid, kBThreads, 0, s>>>(b->plan, fetch);
    const int adv = std::max(1, std::min((std::max(b->n_ctr, b->n) + 255) / 256, 2 * b->sms));
    k_batch_advance<<<adv, 256, 0, s>>>(b->d_args, b->n, b->plan.ctr, b->n_ctr, b->plan.head);
}

int build_graph(lsh_batch* b) {
    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    cudaStream_t cap = nullptr;
    B_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        for (int i = 0; i < kBatchGraphSteps; ++i) enqueue_batch_step(b, cap);
        e = cudaStreamEndCapture(cap, &g);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) return bfail(e, "batch graph capture");
    return LSH_OK;
}

}  // namespace

extern "C" {

int lsh_batch_create(const lsh_params* params, int n, int device, lsh_batch** out) {
    if (!out || !params || n < 1) return LSH_ERR_INVALID;
    *out = nullptr;
    for (int s = 0; s < n; ++s) {
        if (const char* why = lsh::params_problem(params + s)) {
            lsh::set_last_error("scenario " + std::to_string(s) + ": " + why);
            return LSH_ERR_INVALID;
        }
        if (params[s].order != params[0].order) { lsh::set_last_error("all scenarios of a batch must share the order"); return LSH_ERR_INVALID; }
    }
    if (lsh_check_device() != 0) return LSH_ERR_NO_DEVICE;
    lsh_batch* b = new (std::nothrow) lsh_batch();
    if (!b) return LSH_ERR_HOST_OOM;
    b->n = n;
    b->order = params[0].order;
    b->params.assign(params, params + n);
    auto bail = [&](int st) { lsh_batch_destroy(b); return st; };
    if (device >= 0) { cudaError_t e = cudaSetDevice(device); if (e != cudaSuccess) return bail(bfail(e, "cudaSetDevice")); }
    cudaGetDevice(&b->device);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    { cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking); if (e != cudaSuccess) return bail(bfail(e, "cudaStreamCreate")); }

    // slab: per scenario (padded to 32 doubles) X 7, Y 6, acc 7, eta 2, slopes 14 (order 2), geometry 7*(ny+1)
    b->base.resize(n);
    size_t cells = 0, geo = 0;
    std::vector<size_t> geo_off(n);
    for (int s = 0; s < n; ++s) {
        b->base[s] = cells;
        cells += (size_t(params[s].nx) * params[s].ny + 31) & ~size_t(31);
        geo_off[s] = geo;
        geo += (size_t(7) * (params[s].ny + 1) + 31) & ~size_t(31);
    }
    b->total = cells;
    const int arrays = 7 + 6 + 7 + 2 + ((b->order == 2) ? 14 : 0);
    // order 2: one slope-zero flag byte per cell after the geometry
    const size_t flag_bytes = (b->order == 2) ? ((cells + 7) & ~size_t(7)) : 0;
    const size_t bytes = (size_t(arrays) * cells + geo) * sizeof(double) + flag_bytes;
    { cudaError_t e = cudaMalloc(&b->slab, bytes); if (e != cudaSuccess) return bail(bfail(e, "cudaMalloc batch slab")); }
    { cudaError_t e = cudaMalloc(&b->d_tm, sizeof(lsh::TimeRec) * n); if (e != cudaSuccess) return bail(bfail(e, "cudaMalloc")); }
    const int nargs = (b->order == 2) ? 2 * n : n;
    { cudaError_t e = cudaMalloc(&b->d_args, sizeof(KArgs) * nargs); if (e != cudaSuccess) return bail(bfail(e, "cudaMalloc")); }

    double* slab = static_cast<double*>(b->slab);
    auto arr = [&](int k) { return slab + size_t(k) * cells; };
    double* geo_base = slab + size_t(arrays) * cells;
    unsigned char* flags = reinterpret_cast<unsigned char*>(geo_base + geo);
    // no slope is known to be zero yet (ordered before the blocking copies below)
    if (flag_bytes) cudaMemset(flags, 0, flag_bytes);
    b->h_args.assign(nargs, KArgs{});
    for (int s = 0; s < n; ++s) {
        const lsh_params& p = params[s];
        std::vector<double> g(size_t(7) * (p.ny + 1), 0.0);
        lsh::fill_geo(p, g.data(), size_t(p.ny + 1));
        double* gd = geo_base + geo_off[s];
        { cudaError_t e = cudaMemcpy(gd, g.data(), g.size() * sizeof(double), cudaMemcpyHostToDevice); if (e != cudaSuccess) return bail(bfail(e, "geometry")); }
        KArgs a;
        std::memset(&a, 0, sizeof(a));
        a.c = lsh::make_consts(p);
        const size_t st = p.ny + 1;
        a.geo.area = gd; a.geo.len_v = gd + st; a.geo.len_h = gd + 2 * st; a.geo.tanR = gd + 3 * st;
        a.geo.wx = gd + 4 * st; a.geo.wy = gd + 5 * st; a.geo.inv_area = gd + 6 * st;
        const size_t o = b->base[s];
        for (int k = 0; k < 7; ++k) { a.W[k] = arr(k) + o; a.acc[k] = arr(13 + k) + o; }
        for (int k = 0; k < 6; ++k) a.Wout[k] = arr(k) + o;
        a.eta_max = arr(20) + o;
        a.eta_time = arr(21) + o;
        if (b->order == 2) {
            for (int k = 0; k < 7; ++k) {
                a.sx[k] = a.sxw[k] = arr(22 + k) + o;
                a.sy[k] = a.syw[k] = arr(29 + k) + o;
            }
            for (int k = 0; k < 6; ++k) a.Wout[k] = arr(7 + k) + o;  // stage 1: X -> Y
            a.szero = flags + o;  // both stages share the slopes and their flags
        }
        a.tm = b->d_tm + s;
        b->h_args[s] = a;
        if (b->order == 2) {
            KArgs a2 = a;  // stage 2: Y -> X, average with X
            for (int k = 0; k < 6; ++k) { a2.W[k] = arr(7 + k) + o; a2.Wout[k] = arr(k) + o; a2.Xavg[k] = arr(k) + o; }
            a2.W[6] = arr(6) + o;
            b->h_args[n + s] = a2;
        }
    }
    { cudaError_t e = cudaMemcpy(b->d_args, b->h_args.data(), sizeof(KArgs) * nargs, cudaMemcpyHostToDevice); if (e != cudaSuccess) return bail(bfail(e, "args")); }
    std::vector<lsh::TimeRec> tms(n);
    for (int s = 0; s < n; ++s) { tms[s] = lsh::TimeRec{}; tms[s].t_end = INFINITY; tms[s].dt_min = params[s].dt_min; tms[s].done = 1; }
    { cudaError_t e = cudaMemcpy(b->d_tm, tms.data(), sizeof(lsh::TimeRec) * n, cudaMemcpyHostToDevice); if (e != cudaSuccess) return bail(bfail(e, "time")); }
    b->tune = lsh_tune{16, 1, 0.0};
    if (int st = build_plan(b)) return bail(st);
    *out = b;
    return LSH_OK;
}

int lsh_batch_destroy(lsh_batch* b) {
    if (!b) return LSH_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->d_plan_mem) cudaFree(b->d_plan_mem);
    if (b->d_args) cudaFree(b->d_args);
    if (b->d_tm) cudaFree(b->d_tm);
    if (b->slab) cudaFree(b->slab);
    if (b->stream) cudaStreamDestroy(b->stream);
    (void)cudaGetLastError();
    delete b;
    return LSH_OK;
}

int lsh_batch_set_state(lsh_batch* b, int s, const double* const host_state[LSH_NVARS], double* dt0_out) {
    if (!b || s < 0 || s >= b->n || !host_state) return LSH_ERR_INVALID;
    const lsh_params& p = b->params[s];
    const size_t N = size_t(p.nx) * p.ny;
    const KArgs& a = b->h_args[s];
    for (int k = 0; k < 7; ++k) {
        if (!host_state[k]) return LSH_ERR_INVALID;
        B_CUDA(cudaMemcpyAsync(const_cast<double*>(a.W[k]), host_state[k], N * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    }
    lsh::TimeRec init{};
    init.t_end = INFINITY;
    init.dt_min = p.dt_min;
    B_CUDA(cudaMemcpyAsync(a.tm, &init, sizeof(init), cudaMemcpyHostToDevice, b->stream));
    const int nx = p.nx, ny = p.ny;
    cudaStream_t st = b->stream;
    k_batch_init_wave<0, true><<<dim3((nx + kEdgeBlock - 1) / kEdgeBlock, std::min(ny / 2 + 1, 65535)), kEdgeBlock, 0, st>>>(b->d_args, s, 0);
    k_batch_init_wave<0, false><<<dim3((nx + kEdgeBlock - 1) / kEdgeBlock, std::min((ny - 1) / 2 + 1, 65535)), kEdgeBlock, 0, st>>>(b->d_args, s, 1);
    k_batch_init_wave<1, false><<<dim3((nx / 2 + 1 + kEdgeBlock - 1) / kEdgeBlock, std::min(ny, 65535)), kEdgeBlock, 0, st>>>(b->d_args, s, 0);
    k_batch_init_wave<1, false><<<dim3(((nx - 1) / 2 + 1 + kEdgeBlock - 1) / kEdgeBlock, std::min(ny, 65535)), kEdgeBlock, 0, st>>>(b->d_args, s, 1);
    k_batch_init_cells<<<unsigned((N + kCellBlock - 1) / kCellBlock), kCellBlock, 0, st>>>(b->d_args, s);
    k_batch_init_finish<<<1, 1, 0, st>>>(b->d_args, s);
    b->launches += 6;
    B_CUDA(cudaGetLastError());
    lsh::TimeRec out{};
    B_CUDA(cudaMemcpyAsync(&out, a.tm, sizeof(out), cudaMemcpyDeviceToHost, st));
    B_CUDA(cudaStreamSynchronize(st));
    if (dt0_out) *dt0_out = out.dt;
    return LSH_OK;
}

int lsh_batch_step(lsh_batch* b, int nsteps) {
    if (!b || nsteps < 0) return LSH_ERR_INVALID;
    if (!b->graph) { if (int s = build_graph(b)) return s; }
    const int full = nsteps / kBatchGraphSteps, rest = nsteps % kBatchGraphSteps;
    for (int i = 0; i < full; ++i) B_CUDA(cudaGraphLaunch(b->graph, b->stream));
    for (int i = 0; i < rest; ++i) enqueue_batch_step(b, b->stream);
    B_CUDA(cudaGetLastError());
    b->launches += (long long)nsteps * kernels_per_step;
    return LSH_OK;
}

int lsh_batch_synchronize(lsh_batch* b) {
    if (!b) return LSH_ERR_INVALID;
    B_CUDA(cudaStreamSynchronize(b->stream));
    std::vector<lsh::TimeRec> tms(b->n);
    B_CUDA(cudaMemcpy(tms.data(), b->d_tm, sizeof(lsh::TimeRec) * b->n, cudaMemcpyDeviceToHost));
    for (const auto& t : tms)
        if (t.err)
            for (int s = 1; s < 31; ++s)
                if (t.err & (1 << s)) return s;
    return LSH_OK;
}

int lsh_batch_get_state(lsh_batch* b, int s, double* const host_state[LSH_NVARS]) {
    if (!b || s < 0 || s >= b->n || !host_state) return LSH_ERR_INVALID;
    const size_t N = size_t(b->params[s].nx) * b->params[s].ny;
    const KArgs& a = b->h_args[s];
    for (int k = 0; k < 7; ++k)
        if (host_state[k]) B_CUDA(cudaMemcpyAsync(host_state[k], a.W[k], N * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    B_CUDA(cudaStreamSynchronize(b->stream));
    return LSH_OK;
}

int lsh_batch_get_time(lsh_batch* b, int s, double* t, double* dt, long long* steps) {
    if (!b || s < 0 || s >= b->n) return LSH_ERR_INVALID;
    lsh::TimeRec out{};
    B_CUDA(cudaMemcpyAsync(&out, b->d_tm + s, sizeof(out), cudaMemcpyDeviceToHost, b->stream));
    B_CUDA(cudaStreamSynchronize(b->stream));
    if (t) *t = out.t;
    if (dt) *dt = out.dt;
    if (steps) *steps = out.steps;
    return LSH_OK;
}

int lsh_batch_set_tune(lsh_batch* b, const lsh_tune* tune) {
    if (!b || !tune || tune->ctas_per_sm < 1 || tune->ctas_per_sm > kBMaxCtas || tune->items_per_fetch < 1 ||
        tune->items_per_fetch > 64)
        return LSH_ERR_INVALID;
    B_CUDA(cudaStreamSynchronize(b->stream));
    b->tune = *tune;
    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    return LSH_OK;
}

int lsh_batch_get_tune(lsh_batch* b, lsh_tune* tune) {
    if (!b || !tune) return LSH_ERR_INVALID;
    *tune = b->tune;
    return LSH_OK;
}

// Time each candidate configuration on `trial_steps` live steps of the batch
// (CUDA events around one graph-replayed run); keep the fastest.  The steps
// taken while tuning are real steps of the simulation.
int lsh_batch_autotune(lsh_batch* b, int trial_steps, lsh_tune* best_out) {
    if (!b || trial_steps < 1) return LSH_ERR_INVALID;
    static const int ctas[] = {8, 12, 16, 20};
    static const int fetches[] = {1, 2, 4};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    lsh_tune best = b->tune;
    best.ms_per_step = INFINITY;
    for (int c : ctas) {
        for (int f : fetches) {
            lsh_tune t{c, f, 0.0};
            if (int s = lsh_batch_set_tune(b, &t)) { cudaEventDestroy(e0); cudaEventDestroy(e1); return s; }
            if (int s = lsh_batch_step(b, 1)) { cudaEventDestroy(e0); cudaEventDestroy(e1); return s; }  // warm-up
            cudaEventRecord(e0, b->stream);
            if (int s = lsh_batch_step(b, trial_steps)) { cudaEventDestroy(e0); cudaEventDestroy(e1); return s; }
            cudaEventRecord(e1, b->stream);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            t.ms_per_step = ms / trial_steps;
            if (t.ms_per_step < best.ms_per_step) best = t;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (int s = lsh_batch_set_tune(b, &best)) return s;
    b->tune.ms_per_step = best.ms_per_step;
    if (best_out) *best_out = best;
    return LSH_OK;
}

int lsh_batch_get_launch_count(lsh_batch* b, long long* launches) {
    if (!b || !launches) return LSH_ERR_INVALID;
    *launches = b->launches;
    return LSH_OK;
}

}  // extern "C"
