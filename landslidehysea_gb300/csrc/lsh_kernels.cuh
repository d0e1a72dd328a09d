// lsh_kernels.cuh -- the step's kernels (thin launches of the per-edge and
// per-cell bodies of lsh_passes.cuh), shared by the single-grid context
// (lsh_core.cu) and the adjoint's forward recomputation (lsh_adjoint.cu), so
// both run the same device code.  Internal linkage: each translation unit
// that includes this header gets its own copy.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <utility>

#include "../../include/lsh.h"
#include "lsh_passes.cuh"

namespace {

using lsh::KArgs;
using lsh::TimeRec;
using lsh::kCellBlock;
using lsh::kEdgeBlock;
using lsh::kRateInitBits;

// Thread-block shapes of the edge passes (x along threadIdx.x, lines along
// threadIdx.y; kEdgeTile threads, below): a warp spans LSH_EDGE_H_BX cells of an
// edge row, or LSH_EDGE_V_BX edge columns (2 LSH_EDGE_V_BX cells) of a row,
// and 32 / BX lines, so fewer warps straddle a wet/dry front than with
// one-line warps, while each row segment stays one contiguous load.
#ifndef LSH_EDGE_H_BX
#define LSH_EDGE_H_BX 16
#endif
#ifndef LSH_EDGE_V_BX
#define LSH_EDGE_V_BX 8
#endif
// Blocks per SM the edge and cell kernels are compiled for: a register cap
// of 65536 / (threads * MINB).  The FP64 unit returns results through the
// short scoreboard, and the edge passes also wait on their loads; at the
// compiler's choice (128-168 registers, 3 blocks of 128) too few warps were
// resident to cover both.  Measured on the 2048^2 fjord, ms per step
// (threads x blocks per SM: registers):
//   before the empty-edge test: 128x3 2.46, 128x4 (128) 2.33, 128x5 (96) 2.26, 128x6 2.27;
//   after it: 128x5 2.09, 128x6 (85) 2.03, 128x7 (73) 2.01, 64x12 (85) 2.03,
//   64x14 (73) 2.00, 64x16 (64) 1.98-1.99, 64x20 (48) 2.00, 64x24 (40) 2.13, 256x2 2.40.
// With the passes overlapped (programmatic dependent launches, below) the
// SMs hold blocks of two or three passes at once, and more resident warps
// pay again (steps 5-148, ms per step; edge threads x blocks, then cell
// blocks of 256 per SM): 64x12 1.814, 64x16 1.666, 64x20 1.608, 64x24 1.690,
// 64x28 1.721, 128x8 1.640, 128x10 1.611, 128x12 1.639; with 64x20: cells
// at the compiler's choice (62-64 registers) 1.608, 5 blocks 1.587,
// 6 blocks (40 registers) 1.582; 64x24 with 6 cell blocks 1.666.
// The spills stay in L1.  1: the compiler's choice.
#ifndef LSH_EDGE_MINB
#define LSH_EDGE_MINB 20
#endif
#ifndef LSH_CELL_MINB
#define LSH_CELL_MINB 6
#endif
// Threads per edge-pass block (a tile of LSH_EDGE_H_BX x threads / BX).
#ifndef LSH_EDGE_THREADS
#define LSH_EDGE_THREADS 64
#endif
constexpr int kEdgeTile = LSH_EDGE_THREADS;
#if LSH_EDGE_MINB > 1
#define LSH_EDGE_BOUNDS __launch_bounds__(kEdgeTile, LSH_EDGE_MINB)
#else
#define LSH_EDGE_BOUNDS __launch_bounds__(kEdgeTile)
#endif
#if LSH_CELL_MINB > 1
#define LSH_CELL_BOUNDS __launch_bounds__(kCellBlock, LSH_CELL_MINB)
#else
#define LSH_CELL_BOUNDS __launch_bounds__(kCellBlock)
#endif
// The reconstruction alone: 8 blocks of 256 (32 registers) hide its load
// latency best (2048^2 step: 1.940 ms at the compiler's 48 registers, 1.929
// at 6 blocks, 1.921 at 8).
#ifndef LSH_RECON_MINB
#define LSH_RECON_MINB 8
#endif
#if LSH_RECON_MINB > 1
#define LSH_RECON_BOUNDS __launch_bounds__(kCellBlock, LSH_RECON_MINB)
#else
#define LSH_RECON_BOUNDS __launch_bounds__(kCellBlock)
#endif
constexpr int kEdgeHBX = LSH_EDGE_H_BX, kEdgeHBY = kEdgeTile / LSH_EDGE_H_BX;
constexpr int kEdgeVBX = LSH_EDGE_V_BX, kEdgeVBY = kEdgeTile / LSH_EDGE_V_BX;
#ifndef LSH_CELL_BX
#define LSH_CELL_BX 16
#endif
constexpr int kCellBX = LSH_CELL_BX, kCellBY = kCellBlock / LSH_CELL_BX;

// ---------------------------------------------------------------- pass overlap
// The passes of a step run as consecutive kernels.  Each kernel's blocks end
// unevenly (wet tiles carry all the FP64 work), so a whole-grid boundary
// leaves SMs idle while the last wet tiles finish.  With `Dep` set, a pass is
// launched as a programmatic dependent of the one before it: its blocks may
// be scheduled once every block of that pass has started, and each of them
// waits only for the producer's row tiles that wrote the cell rows it reads.
// Every block of a pass adds 1 to its row tile's counter when its writes are
// done (a release add after the block's barrier); a consumer's thread 0 spins on the counters
// it needs with acquire loads, then the block synchronises.  The producer's
// blocks have all started before a consumer block can be scheduled, so a
// waiting block never keeps a producer block off the GPU.  Which rows a pass
// reads and writes:
//   horizontal edges, parity p, block row by: edge rows p + 2t,
//     t in [4 by, 4 by + 3] (kEdgeHBY = 4 lines), cells rows y - 1 and y;
//   vertical edges, block row by: cell rows [8 by, 8 by + 7];
//   cell kernels, block row by: cell rows [16 by, 16 by + 15] (the
//     reconstruction also reads the rows above and below).
// The counters are zeroed by the clock kernel at the end of the step.
enum DepKind : int { kDepH0 = 0, kDepH1 = 1, kDepV = 2, kDepCell = 3 };
struct Dep {
    const unsigned* wait = nullptr;  // producer pass's counters per block row (null: no wait)
    unsigned* done = nullptr;        // this pass's counters per block row (null: none)
    unsigned target = 0;             // producer blocks per block row (its gridDim.x)
    int kind = 0;                    // producer tiling (DepKind)
    int ntiles = 0;                  // producer block rows (its gridDim.y)
    int span = 0;                    // producer block height: cell rows, or edge lines for kDepH*
                                     // (0: the step kernels' blocks)
};

// Producer block rows that wrote cell rows [r0, r1].
__device__ __forceinline__ void dep_tiles(const Dep& d, int r0, int r1, int& t0, int& t1) {
    if (d.kind == kDepV) {
        const int b = d.span ? d.span : kEdgeVBY;
        t0 = r0 / b; t1 = r1 / b;
    } else if (d.kind == kDepCell) {
        const int b = d.span ? d.span : kCellBY;
        t0 = r0 / b; t1 = r1 / b;
    } else {
        // horizontal edge row y = p + 2 t writes cell rows y - 1 and y: the
        // edge rows touching [r0, r1] are [r0, r1 + 1]
        const int b = d.span ? d.span : kEdgeHBY;
        const int p = d.kind;
        const int lo = max(r0 - p + 1, 0) / 2, hi = (r1 + 1 - p) / 2;
        t0 = lo / b;
        t1 = max(hi, 0) / b;
    }
    t0 = max(t0, 0);
    t1 = min(t1, d.ntiles - 1);
}

// Start of a dependent pass's block: let the next pass be scheduled, then
// wait (thread 0, bounded) for the producer rows [r0, r1].  A wait that runs
// past ~2 s, or finds another block's wait already timed out, sets
// LSH_ERR_TIMEOUT in the time record and gives up (the step is then reported
// as failed and the clock kernel stops further steps).  Uniform per block.
__device__ __forceinline__ void dep_begin(const Dep& d, TimeRec* tm, int r0, int r1) {
    if (d.done) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (!d.wait) return;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        int t0, t1;
        dep_tiles(d, r0, r1, t0, t1);
        const int tbit = 1 << LSH_ERR_TIMEOUT;
        volatile int* err = &tm->err;
        unsigned long long start = 0;
        for (int t = t0; t <= t1; ++t) {
            unsigned ns = 32;
            for (;;) {
                unsigned v;
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(d.wait + t) : "memory");
                if (v >= d.target) break;
                if (*err & tbit) { t = t1; break; }
                unsigned long long now;
                asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
                if (start == 0) start = now;
                else if (now - start > 2000000000ull) { atomicOr(&tm->err, tbit); t = t1; break; }
                __nanosleep(ns);
                if (ns < 1024) ns *= 2;
            }
        }
    }
    __syncthreads();
}

// End of a pass's block: its writes are done; count it in its block row.
// The barrier orders every thread's writes before thread 0's add, whose
// release semantics (cumulative, GPU scope) publish them with it.
__device__ __forceinline__ void dep_end(const Dep& d) {
    if (!d.done) return;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0)
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(d.done + blockIdx.y) : "memory");
}

// Horizontal edges of parity `par`: x along threadIdx.x, edge rows par, par+2, ... along threadIdx.y / blocks.y.
// With `d` set the grid covers every line at once (gridDim.y * kEdgeHBY >= lines).
template <bool FIRST, int ORDER>
__global__ void LSH_EDGE_BOUNDS k_edges_h(KArgs a, int par, Dep d = Dep{}) {
    if (a.tm->done) return;
    const int nx = a.c.nx, ny = a.c.ny;
    if (d.done || d.wait) {
        const int y0 = par + 2 * (blockIdx.y * kEdgeHBY);
        dep_begin(d, a.tm, max(y0 - 1, 0), min(y0 + 2 * (kEdgeHBY - 1), ny - 1));
    }
    const int x = blockIdx.x * kEdgeHBX + threadIdx.x;
    if (x < nx) {
        const double dt = a.tm->dt;
        const int nlines = (ny - par) / 2 + 1;
        for (int t = blockIdx.y * kEdgeHBY + threadIdx.y; t < nlines; t += gridDim.y * kEdgeHBY)
            lsh::do_edge<0, FIRST, ORDER>(a, x, par + 2 * t, dt);
    }
    dep_end(d);
}

// Vertical edges of parity `par`: edge columns par, par+2, ... along threadIdx.x, rows along threadIdx.y / blocks.y.
template <int ORDER>
__global__ void LSH_EDGE_BOUNDS k_edges_v(KArgs a, int par, Dep d = Dep{}) {
    if (a.tm->done) return;
    const int nx = a.c.nx, ny = a.c.ny;
    if (d.done || d.wait) {
        const int y0 = blockIdx.y * kEdgeVBY;
        dep_begin(d, a.tm, y0, min(y0 + kEdgeVBY - 1, ny - 1));
    }
    const int t = blockIdx.x * kEdgeVBX + threadIdx.x;
    const int x = par + 2 * t;
    if (x <= nx) {
        const double dt = a.tm->dt;
        for (int y = blockIdx.y * kEdgeVBY + threadIdx.y; y < ny; y += gridDim.y * kEdgeVBY)
            lsh::do_edge<1, false, ORDER>(a, x, y, dt);
    }
    dep_end(d);
}

// Launch shapes of the two edge passes: one edge per thread.  (Blocks that
// walk several bands of lines measured slower, 2.19 ms per 2048^2 step with
// 2 bands against 1.98: a block holding several wet bands runs them one
// after the other.)
inline dim3 edge_block_h() { return dim3(kEdgeHBX, kEdgeHBY); }
inline dim3 edge_block_v() { return dim3(kEdgeVBX, kEdgeVBY); }
inline dim3 edge_grid_h(int nx, int ny, int par) {
    const int nlines = (ny - par) / 2 + 1;
    return dim3((nx + kEdgeHBX - 1) / kEdgeHBX, std::min((nlines + kEdgeHBY - 1) / kEdgeHBY, 65535));
}
inline dim3 edge_grid_v(int nx, int ny, int par) {
    const int nlines = (nx - par) / 2 + 1;
    return dim3((nlines + kEdgeVBX - 1) / kEdgeVBX, std::min((ny + kEdgeVBY - 1) / kEdgeVBY, 65535));
}

// Cell kernels: blocks of kCellBlock threads shaped LSH_CELL_BX x
// (kCellBlock / LSH_CELL_BX) over (x, y); LSH_CELL_BX = kCellBlock is one
// row segment per block.
inline dim3 cell_block() { return dim3(kCellBX, kCellBY); }
inline dim3 cell_grid(int nx, int ny) { return dim3((nx + kCellBX - 1) / kCellBX, (ny + kCellBY - 1) / kCellBY); }
// The cell of this thread, or -1 outside the grid.
__device__ __forceinline__ int cell_of_thread(int nx, int ny) {
    const int x = blockIdx.x * kCellBX + threadIdx.x, y = blockIdx.y * kCellBY + threadIdx.y;
    return (x < nx && y < ny) ? y * nx + x : -1;
}

// Second order: halved minmod slopes of (eta1, q1x, q1y, eta2, q2x, q2y, H)
// with a first-order fallback where a reconstructed depth would fall below
// kReconThin of the cell depth.
//
// (A variant that staged the block's 16 x 16 cells and a halo in shared
// memory, the depths first and the other variables only for tiles with a
// wet cell, measured 2.00 ms per 2048^2 step against 1.97 for this one: the
// stencil's neighbour loads already hit in L1.)
__global__ void LSH_RECON_BOUNDS k_recon(KArgs a, Dep d = Dep{}) {
    if (a.tm->done) return;
    if (d.done || d.wait) {
        const int y0 = blockIdx.y * kCellBY;
        dep_begin(d, a.tm, max(y0 - 1, 0), min(y0 + kCellBY, a.c.ny - 1));
    }
    const int id = cell_of_thread(a.c.nx, a.c.ny);
    if (id >= 0) lsh::recon_cell(a, id);
    dep_end(d);
}

// MODE 0: order 1, in place; per-cell dt min.  MODE 1: order 2 stage 1
// (W -> Wout), per-cell dt min.  MODE 2: order 2 stage 2, Wout = (Xavg + E(W)) / 2.
template <int MODE>
__global__ void LSH_CELL_BOUNDS k_volume(KArgs a, Dep d = Dep{}) {
    if (a.tm->done) return;
    if (d.done || d.wait) {
        const int y0 = blockIdx.y * kCellBY;
        dep_begin(d, a.tm, y0, min(y0 + kCellBY - 1, a.c.ny - 1));
    }
    const int id = cell_of_thread(a.c.nx, a.c.ny);
    const double dt = a.tm->dt;
    unsigned long long bits = kRateInitBits;
    if (id >= 0) bits = lsh::volume_cell<MODE>(a, id, dt);
    if (MODE != 2) lsh::block_max_bits<kCellBlock>(bits, &a.tm->rmax_bits);
    dep_end(d);
}


// Advance the device clock: t += dt, dt = min per-cell dt (ShallowWater.cu:436-442).
// With `ctr`, its threads also zero the n_ctr pass-overlap counters of the step.
__global__ void k_advance(TimeRec* tm, double two_cfl, unsigned* ctr = nullptr, int n_ctr = 0) {
    for (int i = threadIdx.x; i < n_ctr; i += blockDim.x) ctr[i] = 0u;
    if (threadIdx.x != 0 || tm->done) return;
    tm->t += tm->dt;
    tm->steps += 1;
    const double nd = lsh::dt_of(tm->rmax_bits, two_cfl);
    tm->dt = nd;
    tm->rmax_bits = kRateInitBits;
    if (tm->t >= tm->t_end) tm->done = 1;
    if (tm->dt_min > 0.0 && nd < tm->dt_min) { tm->err |= 1 << LSH_ERR_STALL; tm->done = 1; }
    if (tm->err) tm->done = 1;
}

// Initial-dt edge pass (procesarAristasDeltaTInicialGPU), writing acc[6]:
// the step's edge tiles (edge_block_h/v, edge_grid_h/v).
template <int DIR, bool FIRST>
__global__ void LSH_EDGE_BOUNDS k_init_wave(KArgs a, int par) {
    const int nx = a.c.nx, ny = a.c.ny;
    if (DIR == 0) {
        const int x = blockIdx.x * kEdgeHBX + threadIdx.x;
        if (x >= nx) return;
        const int nlines = (ny - par) / 2 + 1;
        for (int t = blockIdx.y * kEdgeHBY + threadIdx.y; t < nlines; t += gridDim.y * kEdgeHBY)
            lsh::init_wave_edge<0, FIRST>(a, x, par + 2 * t);
    } else {
        const int t = blockIdx.x * kEdgeVBX + threadIdx.x;
        const int x = par + 2 * t;
        if (x > nx) return;
        for (int y = blockIdx.y * kEdgeVBY + threadIdx.y; y < ny; y += gridDim.y * kEdgeVBY)
            lsh::init_wave_edge<1, FIRST>(a, x, y);
    }
}

// The four passes of the initial-dt wave sum, in the reference's order (the
// first writes acc[6], the others add).
inline void launch_init_wave(const KArgs& a, int nx, int ny, cudaStream_t s) {
    k_init_wave<0, true><<<edge_grid_h(nx, ny, 0), edge_block_h(), 0, s>>>(a, 0);
    k_init_wave<0, false><<<edge_grid_h(nx, ny, 1), edge_block_h(), 0, s>>>(a, 1);
    k_init_wave<1, false><<<edge_grid_v(nx, ny, 0), edge_block_v(), 0, s>>>(a, 0);
    k_init_wave<1, false><<<edge_grid_v(nx, ny, 1), edge_block_v(), 0, s>>>(a, 1);
}

// Per-cell rate of the initial wave pass (obtenerDeltaTVolumenesGPU) and its max.
__global__ void __launch_bounds__(kCellBlock) k_cell_dt(KArgs a) {
    const int id = cell_of_thread(a.c.nx, a.c.ny);
    unsigned long long bits = kRateInitBits;
    if (id >= 0) bits = lsh::init_cell_rate(a, id);
    lsh::block_max_bits<kCellBlock>(bits, &a.tm->rmax_bits);
}

__global__ void k_init_finish(TimeRec* tm, double two_cfl) {
    tm->dt = lsh::dt_of(tm->rmax_bits, two_cfl);
    tm->rmax_bits = kRateInitBits;
    tm->t = 0.0;
    tm->steps = 0;
    tm->done = 0;
    tm->err = 0;
}

// eta1 max initial value h1 + h2 - H, time 0 (Problema.cxx:542-546)
__global__ void __launch_bounds__(kCellBlock) k_init_eta(KArgs a) {
    const int id = cell_of_thread(a.c.nx, a.c.ny);
    if (id < 0) return;
    a.eta_max[id] = a.W[0][id] + a.W[3][id] - a.W[6][id];
    a.eta_time[id] = 0.0;
}

// ---------------------------------------------------------------- overlapped launches

// Counters per pass of a step when the passes can overlap: one per block row
// of the edge and cell kernels, rounded up; 0 when a grid would need more
// block rows than a launch holds (the passes then run fully ordered).
inline int dep_stride_for(int nx, int ny) {
    const int rows = std::max({(int)edge_grid_h(nx, ny, 0).y, (int)edge_grid_v(nx, ny, 0).y, (int)cell_grid(nx, ny).y});
    const bool fits = (long long)((ny / 2 + 1 + kEdgeHBY - 1) / kEdgeHBY) <= 65535 &&
                      (long long)((ny + kEdgeVBY - 1) / kEdgeVBY) <= 65535;
    return fits ? ((rows + 63) & ~63) : 0;
}

// Launch `kernel` on `s`; `dependent`: as a programmatic dependent of the
// kernel before it on the stream (it may start once that kernel's blocks
// have all started; its blocks order themselves through the pass counters).
template <class... P, class... A>
inline void launch_pass(bool dependent, dim3 grid, dim3 block, cudaStream_t s, void (*kernel)(P...), A&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = dependent ? at : nullptr;
    cfg.numAttrs = dependent ? 1 : 0;
    (void)cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

// The passes of one stage with overlap on an nx x ny grid: `prev` is the
// producer of the first edge pass (the reconstruction at order 2, nothing
// at order 1: then h0 is the step's first kernel); counters seg[0..4 st)
// for h0, h1, v0, v1 and the volume update (`last`: the volume's counters
// are not needed).  MODE < 0: no volume update (the stage ends after its
// edge passes).  Returns the producer description for a pass that reads
// this stage's volume output.
// snaps (may be null): for the adjoint's recomputation, the three passes
// after the first copy the partial sums they read to snaps[0], [1], [2].
template <int ORDER, int MODE>
inline Dep enqueue_stage_overlap(int nx, int ny, const KArgs& a, cudaStream_t s, Dep prev, unsigned* seg, int st,
                                 bool last, double* const (*snaps)[2] = nullptr) {
    KArgs as[3] = {a, a, a};
    if (snaps)
        for (int i = 0; i < 3; ++i) { as[i].snap[0] = snaps[i][0]; as[i].snap[1] = snaps[i][1]; }
    const dim3 gh0 = edge_grid_h(nx, ny, 0), gh1 = edge_grid_h(nx, ny, 1);
    const dim3 gv0 = edge_grid_v(nx, ny, 0), gv1 = edge_grid_v(nx, ny, 1), gc = cell_grid(nx, ny);
    Dep d0 = prev;
    d0.done = seg;
    launch_pass(prev.wait != nullptr, gh0, edge_block_h(), s, k_edges_h<true, ORDER>, a, 0, d0);
    Dep d1;
    d1.wait = seg; d1.done = seg + st; d1.target = gh0.x; d1.kind = kDepH0; d1.ntiles = (int)gh0.y;
    launch_pass(true, gh1, edge_block_h(), s, k_edges_h<false, ORDER>, as[0], 1, d1);
    Dep d2;
    d2.wait = seg + st; d2.done = seg + 2 * st; d2.target = gh1.x; d2.kind = kDepH1; d2.ntiles = (int)gh1.y;
    launch_pass(true, gv0, edge_block_v(), s, k_edges_v<ORDER>, as[1], 0, d2);
    Dep d3;
    d3.wait = seg + 2 * st; d3.done = (MODE < 0 && last) ? nullptr : seg + 3 * st; d3.target = gv0.x;
    d3.kind = kDepV; d3.ntiles = (int)gv0.y;
    launch_pass(true, gv1, edge_block_v(), s, k_edges_v<ORDER>, as[2], 1, d3);
    Dep next;
    if (MODE < 0) {
        next.wait = seg + 3 * st; next.target = gv1.x; next.kind = kDepV; next.ntiles = (int)gv1.y;
        return next;
    }
    Dep d4;
    d4.wait = seg + 3 * st; d4.done = last ? nullptr : seg + 4 * st; d4.target = gv1.x; d4.kind = kDepV;
    d4.ntiles = (int)gv1.y;
    launch_pass(true, gc, cell_block(), s, k_volume<(MODE < 0 ? 0 : MODE)>, a, d4);
    next.wait = seg + 4 * st; next.target = gc.x; next.kind = kDepCell; next.ntiles = (int)gc.y;
    return next;
}

// One whole time step with overlapped passes, counters c[0 .. 13 st):
// order 1 from a1 (in place); order 2 stage 1 from a1 (X -> Y), stage 2 from
// a2 (Y -> X with the average).  The clock kernel closes the step as a
// plain launch and zeroes the counters.  Returns the kernels launched.
inline int enqueue_step_overlap(int nx, int ny, int order, const KArgs& a1, const KArgs& a2, unsigned* c, int st,
                                TimeRec* tm, double two_cfl, cudaStream_t s) {
    const int nk = (order == 1) ? 6 : 13;
    if (order == 1) {
        enqueue_stage_overlap<1, 0>(nx, ny, a1, s, Dep{}, c, st, true);
    } else {
        const dim3 nbc = cell_grid(nx, ny);
        Dep r1;
        r1.done = c;
        launch_pass(false, nbc, cell_block(), s, k_recon, a1, r1);
        Dep pr;
        pr.wait = c; pr.target = nbc.x; pr.kind = kDepCell; pr.ntiles = (int)nbc.y;
        const Dep v1 = enqueue_stage_overlap<2, 1>(nx, ny, a1, s, pr, c + st, st, false);
        Dep r2 = v1;
        r2.done = c + 6 * st;
        launch_pass(true, nbc, cell_block(), s, k_recon, a2, r2);
        Dep pr2;
        pr2.wait = c + 6 * st; pr2.target = nbc.x; pr2.kind = kDepCell; pr2.ntiles = (int)nbc.y;
        enqueue_stage_overlap<2, 2>(nx, ny, a2, s, pr2, c + 7 * st, st, true);
    }
    // a plain launch: waits for the whole step, then zeroes the counters
    k_advance<<<1, 256, 0, s>>>(tm, two_cfl, c, nk * st);
    return nk;
}

}  // namespace
