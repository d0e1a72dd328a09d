// lsh_kernels.cuh -- the step's kernels (thin launches of the per-edge and
// per-cell bodies of lsh_passes.cuh), shared by the single-grid context
// (lsh_core.cu) and the adjoint's forward recomputation (lsh_adjoint.cu), so
// both run the same device code.  Internal linkage: each translation unit
// that includes this header gets its own copy.
#pragma once

#include <cuda_runtime.h>

#include "../../include/lsh.h"
#include "lsh_passes.cuh"

namespace {

using lsh::KArgs;
using lsh::TimeRec;
using lsh::kCellBlock;
using lsh::kEdgeBlock;
using lsh::kRateInitBits;

// Horizontal edges of parity `par`: x along threads, edge rows along blocks.
template <bool FIRST, int ORDER>
__global__ void __launch_bounds__(kEdgeBlock) k_edges_h(KArgs a, int par) {
    if (a.tm->done) return;
    const int nx = a.c.nx, ny = a.c.ny;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nx) return;
    const double dt = a.tm->dt;
    const int nlines = (ny - par) / 2 + 1;
    for (int t = blockIdx.y; t < nlines; t += gridDim.y) lsh::do_edge<0, FIRST, ORDER>(a, x, par + 2 * t, dt);
}

// Vertical edges of parity `par`: edge columns along threads, rows along blocks.
template <int ORDER>
__global__ void __launch_bounds__(kEdgeBlock) k_edges_v(KArgs a, int par) {
    if (a.tm->done) return;
    const int nx = a.c.nx, ny = a.c.ny;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int x = par + 2 * t;
    if (x > nx) return;
    const double dt = a.tm->dt;
    for (int y = blockIdx.y; y < ny; y += gridDim.y) lsh::do_edge<1, false, ORDER>(a, x, y, dt);
}

// Second order: halved minmod slopes of (eta1, q1x, q1y, eta2, q2x, q2y, H)
// with a first-order fallback where a reconstructed depth would fall below
// kReconThin of the cell depth.
__global__ void __launch_bounds__(kCellBlock) k_recon(KArgs a) {
    if (a.tm->done) return;
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= a.c.nx * a.c.ny) return;
    lsh::recon_cell(a, id);
}

// MODE 0: order 1, in place; per-cell dt min.  MODE 1: order 2 stage 1
// (W -> Wout), per-cell dt min.  MODE 2: order 2 stage 2, Wout = (Xavg + E(W)) / 2.
template <int MODE>
__global__ void __launch_bounds__(kCellBlock) k_volume(KArgs a) {
    if (a.tm->done) return;
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    const double dt = a.tm->dt;
    unsigned long long bits = kRateInitBits;
    if (id < a.c.nx * a.c.ny) bits = lsh::volume_cell<MODE>(a, id, dt);
    if (MODE != 2) lsh::block_max_bits<kCellBlock>(bits, &a.tm->rmax_bits);
}


// Advance the device clock: t += dt, dt = min per-cell dt (ShallowWater.cu:436-442).
__global__ void k_advance(TimeRec* tm, double two_cfl) {
    if (tm->done) return;
    tm->t += tm->dt;
    tm->steps += 1;
    const double nd = lsh::dt_of(tm->rmax_bits, two_cfl);
    tm->dt = nd;
    tm->rmax_bits = kRateInitBits;
    if (tm->t >= tm->t_end) tm->done = 1;
    if (tm->dt_min > 0.0 && nd < tm->dt_min) { tm->err |= 1 << LSH_ERR_STALL; tm->done = 1; }
    if (tm->err) tm->done = 1;
}

// Initial-dt edge pass (procesarAristasDeltaTInicialGPU), writing acc[6].
template <int DIR, bool FIRST>
__global__ void __launch_bounds__(kEdgeBlock) k_init_wave(KArgs a, int par) {
    const int nx = a.c.nx, ny = a.c.ny;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nlines = (DIR == 0) ? (ny - par) / 2 + 1 : (nx - par) / 2 + 1;
    const int nalong = (DIR == 0) ? nx : ny;
    // DIR 0: threads along x, lines along blocks.y; DIR 1: threads along edge columns
    for (int bl = blockIdx.y; bl < ((DIR == 0) ? nlines : nalong); bl += gridDim.y) {
        if (DIR == 0) { if (tid >= nx) return; lsh::init_wave_edge<0, FIRST>(a, tid, par + 2 * bl); }
        else { if (tid >= nlines) return; lsh::init_wave_edge<1, FIRST>(a, par + 2 * tid, bl); }
    }
}

// Per-cell rate of the initial wave pass (obtenerDeltaTVolumenesGPU) and its max.
__global__ void __launch_bounds__(kCellBlock) k_cell_dt(KArgs a) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long bits = kRateInitBits;
    if (id < a.c.nx * a.c.ny) bits = lsh::init_cell_rate(a, id);
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
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= a.c.nx * a.c.ny) return;
    a.eta_max[id] = a.W[0][id] + a.W[3][id] - a.W[6][id];
    a.eta_time[id] = 0.0;
}

}  // namespace
