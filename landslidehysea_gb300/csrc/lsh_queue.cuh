// lsh_queue.cuh -- the device work queue of the batched paths: one
// persistent launch runs a sequence of passes (reconstruction, the four
// colour edge passes, the Euler stage) over many scenarios of uneven grids.
//
// CTAs of 64 threads pull items -- (pass, scenario, 2-D tile of the
// single-grid shapes) -- from one queue, in pass order.  An item waits only
// for the rows of its own scenario that the pass before it wrote (per-row
// completion counters, as the single-grid path's overlapped launches use),
// so a pass of one scenario runs while other scenarios, or other rows, are
// still in the pass before: no whole-grid barrier between passes.  Items of
// one pass touch disjoint cells of their scenario, so which CTA takes an
// item, and when, changes no bit: every scenario is bit-identical to its
// single-grid run.  The ensemble (lsh_batch.cu) runs a time step this way;
// the batched adjoint (lsh_adjoint.cu) runs its forward steps and the
// recomputation of a reversed step (reconstruction with its branch tape,
// edge passes with their snapshots) this way too.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/lsh.h"
#include "lsh_passes.cuh"
#include "lsh_setup.h"

// Internal linkage: every translation unit that includes this header gets
// its own copy of the kernels.
namespace {

using lsh::KArgs;
using lsh::kRateInitBits;

// No branch tape: the forward step's kernels.
struct NoTape {
    static constexpr bool kOn = false;
    __device__ static unsigned run(const KArgs&, int) { return 0u; }
};

constexpr int kBThreads = 64;    // threads per persistent CTA
// CTAs per SM the step kernel is compiled for (its register budget: 48 at 20)
#ifndef LSH_BATCH_MAXCTAS
#define LSH_BATCH_MAXCTAS 20
#endif
constexpr int kBMaxCtas = LSH_BATCH_MAXCTAS;
constexpr int kMaxPasses = 12;

// Tilings of a scenario's passes, 64-thread tiles of the single-grid shapes:
// horizontal edges of parity 0 / 1 (16 columns x 4 edge lines), vertical
// edges of parity 0 / 1 (8 edge columns x 8 rows), cells (16 x 4).
enum BKind : int { kBH0 = 0, kBH1 = 1, kBV0 = 2, kBV1 = 3, kBCell = 4, kBKinds = 5 };
constexpr int kTileHX = 16, kTileHY = 4, kTileVX = 8, kTileVY = 8, kTileCX = 16, kTileCY = 4;
// What a pass does.
// kOpReconTape: the reconstruction that also stores the adjoint's branch
// tape (a.tape); only a kernel instantiated with a tape policy runs it.
enum BOp : int {
    kOpH0 = 0, kOpH1 = 1, kOpV0 = 2, kOpV1 = 3, kOpRecon = 4, kOpVol0 = 5, kOpVol1 = 6, kOpVol2 = 7, kOpReconTape = 8
};

struct BPass {
    int op;        // BOp
    int kind;      // BKind of its tiles
    int var;       // its arguments: args[var * n + s] (the stage, or a stage with snapshot outputs)
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
    const KArgs* args;      // [var][n]: [n] stage 1, [n, 2n) stage 2, ...
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
    } else if (op == kOpRecon || op == kOpReconTape) {
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

// Waits (one thread) until counters c[t0..t1] reach `target`.  Bounded:
// after ~2 s of %globaltimer from `start` (0: from the first miss) it sets
// *abort_flag and gives up, as does every later wait that finds the flag
// set.  Returns true when it gave up.
__device__ __forceinline__ bool queue_wait(const unsigned* c, int t0, int t1, unsigned target, int* abort_flag,
                                           unsigned long long& start) {
    volatile int* abort_v = abort_flag;
    for (int r = t0; r <= t1; ++r) {
        unsigned ns = 32;
        for (;;) {
            unsigned v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(c + r) : "memory");
            if (v >= target) break;
            if (*abort_v) return true;
            unsigned long long now;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
            if (start == 0) start = now;
            else if (now - start > 2000000000ull) { atomicExch(abort_flag, 1); return true; }
            __nanosleep(ns);
            if (ns < 1024) ns *= 2;
        }
    }
    return false;
}

// The producer rows a CTA's thread 0 last found complete: (pass, scenario,
// tile rows [t0, t1]).  Counters only grow within a launch, so an item whose
// wait falls inside that range needs no new acquire: the earlier acquire,
// followed by the block barrier, already orders its reads after the
// producers' writes.  Consecutive items of one tile row share their waits.
struct WaitCache {
    int pass = -1, scen = -1, t0 = 0, t1 = -1;
    __device__ bool covers(int p, int s, int a, int b) const { return p == pass && s == scen && a >= t0 && b <= t1; }
    __device__ void set(int p, int s, int a, int b) { pass = p; scen = s; t0 = a; t1 = b; }
};

// Marks n items of counter row c done: a release add, ordered after the
// items' writes by the block barrier before it (one thread).
__device__ __forceinline__ void queue_done(unsigned* c, unsigned n = 1u) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(c), "r"(n) : "memory");
}

// One item's work: the single-grid kernels' per-thread bodies on one tile.
// Returns the thread's dt-rate bits for the Euler stages that take the rate
// maximum (kOpVol0, kOpVol1), kRateInitBits otherwise; the caller reduces them.
template <int ORDER, int OP, class TAPE>
__device__ __forceinline__ unsigned long long item_work(const KArgs& a, int tx, int ty, double dt) {
    const int nx = a.c.nx, ny = a.c.ny, tid = threadIdx.x;
    if constexpr (OP == kOpH0 || OP == kOpH1) {
        const int par = OP;
        const int x = tx * kTileHX + tid % kTileHX, line = ty * kTileHY + tid / kTileHX;
        if (x < nx && line < (ny - par) / 2 + 1) lsh::do_edge<0, OP == kOpH0, ORDER>(a, x, par + 2 * line, dt);
    } else if constexpr (OP == kOpV0 || OP == kOpV1) {
        const int par = OP - kOpV0;
        const int x = par + 2 * (tx * kTileVX + tid % kTileVX), y = ty * kTileVY + tid / kTileVX;
        if (x <= nx && y < ny) lsh::do_edge<1, false, ORDER>(a, x, y, dt);
    } else {
        const int i = tx * kTileCX + tid % kTileCX, j = ty * kTileCY + tid / kTileCX;
        const bool in = (i < nx && j < ny);
        if constexpr (OP == kOpRecon) {
            if (in) lsh::recon_cell(a, j * nx + i);
        } else if constexpr (OP == kOpReconTape) {
            if constexpr (TAPE::kOn)
                if (in) a.tape[j * nx + i] = TAPE::run(a, j * nx + i);
        } else {
            constexpr int MODE = OP - kOpVol0;
            unsigned long long bits = kRateInitBits;
            if (in) bits = lsh::volume_cell<MODE>(a, j * nx + i, dt);
            return (MODE != 2) ? bits : kRateInitBits;
        }
    }
    return kRateInitBits;
}

// A run of tiles tx0 .. tx0 + run - 1 of one tile row; the largest rate bits.
template <int ORDER, int OP, class TAPE>
__device__ __forceinline__ unsigned long long run_work(const KArgs& a, int tx0, int run, int ty, double dt) {
    unsigned long long bits = kRateInitBits;
    for (int j = 0; j < run; ++j) {
        const unsigned long long b = item_work<ORDER, OP, TAPE>(a, tx0 + j, ty, dt);
        bits = (b > bits) ? b : bits;
    }
    return bits;
}

// The whole step of every scenario.  Items are dequeued in pass order, and an
// item waits only for items of earlier passes, which running CTAs took
// before it: the earliest unfinished item always has its inputs, so the
// queue drains whatever the number of resident CTAs.  A CTA takes `fetch`
// consecutive items at a time and works them in runs: the items of one tile
// row of one (pass, scenario) share their wait, their barriers and one
// counter add, and an Euler stage's rate maximum is reduced once per run.
// Waits are bounded (~2 s of %globaltimer); one that runs out sets
// LSH_ERR_TIMEOUT on its scenario and the batch's abort flag, and later
// waits give up at once.
template <int ORDER, class TAPE = NoTape>
__global__ void __launch_bounds__(kBThreads, kBMaxCtas) k_batch_step(BPlan P, int fetch) {
    __shared__ __align__(16) unsigned long long sargs[(sizeof(KArgs) + 7) / 8];
    __shared__ int s_first, s_pass, s_scen, s_tile, s_ntx, s_copy, s_run;
    // the last decoded (pass, scenario): its items [s_lo, s_hi) of the queue,
    // and the arguments held in sargs (var * n + scenario, -1: none).
    // Consecutive items of the queue share them, so most runs skip the
    // scenario search and the argument copy.
    __shared__ int s_lo, s_hi, s_args_key;
    const KArgs& a = *reinterpret_cast<const KArgs*>(sargs);
    const int tid = threadIdx.x;
    WaitCache wc;  // thread 0's
    if (tid == 0) { s_lo = 0; s_hi = 0; s_args_key = -1; }
    for (;;) {
        if (tid == 0) s_first = (int)atomicAdd(P.head, (unsigned)fetch);
        __syncthreads();
        const int first = s_first;
        if (first >= P.total_items) break;
        const int last = min(first + fetch, P.total_items);
        for (int it = first; it < last;) {
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
                // the run: the fetched items left in this tile row of this (pass, scenario)
                s_run = min(min(last, s_hi) - it, s_ntx - s_tile % s_ntx);
                const int key = P.pass[s_pass].var * P.n + s_scen;
                s_copy = (key != s_args_key);
                s_args_key = key;
            }
            __syncthreads();
            const int p = s_pass, s = s_scen, t = s_tile, ntx = s_ntx, run = s_run;
            const BPass ps = P.pass[p];
            if (s_copy) {
                const unsigned long long* src = reinterpret_cast<const unsigned long long*>(P.args + ps.var * P.n + s);
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
                if (!wc.covers(ps.prod, s, t0, t1)) {
                    unsigned long long start = 0;
                    const bool gave_up = queue_wait(P.ctr + pp.ctr_off + rbase, t0, t1,
                                                    (unsigned)P.tiles_x[pp.kind * P.n + s], P.abort_flag, start);
                    if (gave_up) atomicOr(&a.tm->err, 1 << LSH_ERR_TIMEOUT);
                    else wc.set(ps.prod, s, t0, t1);
                }
            }
            __syncthreads();
            if (live) {
                const double dt = a.tm->dt;
                unsigned long long bits = kRateInitBits;
                switch (ps.op) {
                    case kOpH0: run_work<ORDER, kOpH0, TAPE>(a, tx, run, ty, dt); break;
                    case kOpH1: run_work<ORDER, kOpH1, TAPE>(a, tx, run, ty, dt); break;
                    case kOpV0: run_work<ORDER, kOpV0, TAPE>(a, tx, run, ty, dt); break;
                    case kOpV1: run_work<ORDER, kOpV1, TAPE>(a, tx, run, ty, dt); break;
                    default:
                        if constexpr (ORDER == 1) {
                            bits = run_work<ORDER, kOpVol0, TAPE>(a, tx, run, ty, dt);
                        } else {
                            if (ps.op == kOpRecon) run_work<ORDER, kOpRecon, TAPE>(a, tx, run, ty, dt);
                            else if (TAPE::kOn && ps.op == kOpReconTape) run_work<ORDER, kOpReconTape, TAPE>(a, tx, run, ty, dt);
                            else if (ps.op == kOpVol1) bits = run_work<ORDER, kOpVol1, TAPE>(a, tx, run, ty, dt);
                            else run_work<ORDER, kOpVol2, TAPE>(a, tx, run, ty, dt);
                        }
                        break;
                }
                if (ps.op == kOpVol0 || ps.op == kOpVol1) lsh::block_max_bits<kBThreads>(bits, &a.tm->rmax_bits);
            }
            __syncthreads();  // the run's writes are done, and sargs may be refilled
            if (tid == 0) {
                // release: the barrier above orders the run's writes before it
                queue_done(P.ctr + ps.ctr_off + P.row_pre[ps.kind * (P.n + 1) + s] + ty, (unsigned)run);
            }
            it += run;
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


// Tiles of a scenario with nx x ny cells in each tiling: (tiles per row, tile rows).
inline void queue_tiles(int nx, int ny, int kind, int& tx, int& ty) {
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

struct QPassSpec {
    int op, kind, var;
};

// The plan of a chain of passes (each reading what the one before it wrote)
// over scenarios of nx[s] x ny[s] cells: its items, counters and device
// tables, in one allocation *mem (freed by the caller; a previous one is
// freed here).  Synchronous.  Returns LSH_OK or an LSH_ERR_* code.
inline int build_queue_plan(const std::vector<int>& nx, const std::vector<int>& ny, const std::vector<QPassSpec>& passes,
                            const KArgs* d_args, void** mem, BPlan& P0, int& n_ctr) {
    const int n = (int)nx.size();
    if ((int)passes.size() > kMaxPasses) { lsh::set_last_error("queue plan: too many passes"); return LSH_ERR_INVALID; }
    std::vector<int> tile_pre(size_t(kBKinds) * (n + 1)), row_pre(size_t(kBKinds) * (n + 1)), tiles_x(size_t(kBKinds) * n);
    long long kind_tiles[kBKinds], kind_rows[kBKinds];
    for (int k = 0; k < kBKinds; ++k) {
        long long tsum = 0, rsum = 0;
        for (int s = 0; s < n; ++s) {
            int tx, ty;
            queue_tiles(nx[s], ny[s], k, tx, ty);
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
    P0 = BPlan{};
    P0.n = n;
    P0.npass = (int)passes.size();
    long long items = 0, ctrs = 0;
    for (int i = 0; i < P0.npass; ++i) {
        BPass& q = P0.pass[i];
        q.op = passes[i].op;
        q.kind = passes[i].kind;
        q.var = passes[i].var;
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
    n_ctr = (int)ctrs;
    // one allocation: tables, counters, queue head, abort flag
    const size_t tbytes = (tile_pre.size() + row_pre.size() + tiles_x.size()) * sizeof(int);
    const size_t bytes = ((tbytes + 255) & ~size_t(255)) + size_t(ctrs) * sizeof(unsigned) + 256;
    if (*mem) { cudaFree(*mem); *mem = nullptr; }
    auto fail = [](cudaError_t e, const char* what) {
        lsh::set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
        (void)cudaGetLastError();
        return (e == cudaErrorMemoryAllocation) ? LSH_ERR_GPU_OOM : LSH_ERR_CUDA;
    };
    cudaError_t e = cudaMalloc(mem, bytes);
    if (e != cudaSuccess) { *mem = nullptr; return fail(e, "cudaMalloc queue plan"); }
    int* ti = static_cast<int*>(*mem);
    if ((e = cudaMemcpy(ti, tile_pre.data(), tile_pre.size() * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(ti + tile_pre.size(), row_pre.data(), row_pre.size() * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(ti + tile_pre.size() + row_pre.size(), tiles_x.data(), tiles_x.size() * sizeof(int),
                        cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(e, "queue plan tables");
    P0.tile_pre = ti;
    P0.row_pre = ti + tile_pre.size();
    P0.tiles_x = ti + tile_pre.size() + row_pre.size();
    char* rest = static_cast<char*>(*mem) + ((tbytes + 255) & ~size_t(255));
    P0.ctr = reinterpret_cast<unsigned*>(rest);
    P0.head = reinterpret_cast<unsigned*>(rest + size_t(ctrs) * sizeof(unsigned));
    P0.abort_flag = reinterpret_cast<int*>(P0.head + 1);
    if ((e = cudaMemset(rest, 0, size_t(ctrs) * sizeof(unsigned) + 256)) != cudaSuccess) return fail(e, "queue plan counters");
    P0.args = d_args;
    return LSH_OK;
}

}  // namespace
