// lsh_core.cu -- sm_103a kernels and the C ABI (include/lsh.h) of the
// two-layer finite-volume time step.
//
// Layout in HBM: FP64 structure-of-arrays, one array of nx*ny doubles per
// variable (h1 q1x q1y h2 q2x q2y H), row-major (cell j*nx + i).  The step:
//   order 1 (the reference scheme, ShallowWater.cu:391-442):
//     4 colour passes over edges (hor-even, hor-odd, ver-even, ver-odd),
//     accumulating into 7 SoA accumulators; the first pass writes instead of
//     accumulating, which replaces the reference's two cudaMemset per step;
//     then one volume kernel updates the state IN PLACE (each thread owns
//     one cell), folds the per-cell dt into a block min and one 64-bit
//     atomicMin on the bit pattern of the (positive) double, and a 1-thread
//     kernel advances t and dt on the device.  No host sync per step, no
//     texture copy-back (ShallowWater.cu:447-454), so a run of steps is one
//     CUDA graph launch.
//   order 2: minmod reconstruction kernel + the same 4 passes on face values
//     + volume kernel, twice (Heun / TVD-RK2), the second volume kernel
//     averaging with the step's initial state.
// The FP64 math lives in lsh_scheme.cuh.

#include <cuda_runtime.h>

#include <algorithm>
#include <utility>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/lsh.h"
#include "lsh_passes.cuh"
#include "lsh_scheme.cuh"
#include "lsh_setup.h"
#include "lsh_kernels.cuh"

using lsh::Consts;
using lsh::EdgeIn;
using lsh::Geo;
using lsh::TimeRec;

namespace {

using lsh::kCellBlock;
using lsh::kEdgeBlock;
using lsh::kRateInitBits;
using lsh::KArgs;
using lsh::dt_of;
using lsh::do_edge;
using lsh::face_rest;
constexpr int kGraphChunk = 16;

thread_local std::string g_last_error;

// FP64 throughput probe: 8 independent DFMA chains per thread.
__global__ void k_fp64_probe(double* out, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3 + k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    if (s == 12345.678) out[0] = s;  // keeps the chains live; never true in practice
}

// h1 - H at the listed cells (lsh_get_gauge_eta); NaN for a cell off the grid.
__global__ void k_gauge_eta(const double* __restrict__ h1, const double* __restrict__ H, const int* cells, int n,
                            long long N, double* out) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const int c = cells[g];
    out[g] = (c >= 0 && c < N) ? h1[c] - H[c] : __longlong_as_double(0x7ff8000000000000LL);
}

}  // namespace

// ------------------------------------------------------------------ context

struct lsh_ctx {
    lsh_params p;
    Consts c;
    int device = 0;
    cudaStream_t own = nullptr;     // created by the library; used for graph capture
    cudaStream_t stream = nullptr;  // where work runs (own, or the caller's)
    size_t N = 0;
    void* slab = nullptr;           // one device allocation for every array
    double* X[7] = {};              // state (X[6] = H)
    double* Y[6] = {};              // order-2 stage buffer
    double* acc[7] = {};
    double* sx[7] = {};
    double* sy[7] = {};
    double* eta_max = nullptr;
    double* eta_time = nullptr;
    unsigned char* szero = nullptr;  // order 2: per-cell "stored slopes are zero" flags
    unsigned* dep_ctr = nullptr;     // pass-overlap counters: kernels_per_step segments of dep_stride
    int dep_stride = 0;              // 0: the step's passes run as plain, fully ordered launches
    double* geo_buf = nullptr;
    Geo geo{};
    TimeRec* tm = nullptr;
    TimeRec* tm_host = nullptr;     // pinned mirror for reads
    int* gauge_cells = nullptr;     // lsh_get_gauge_eta: device copy of the last cell list
    double* gauge_out = nullptr;    // and its gathered values
    int gauge_cap = 0;
    std::vector<int> gauge_host;    // the cell list gauge_cells holds
    cudaGraphExec_t g_chunk = nullptr, g_one = nullptr;
    long long launches = 0;
    int kernels_per_step = 0;
    bool has_state = false;
};

namespace {

int fail_cuda(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    (void)cudaGetLastError();
    return (e == cudaErrorMemoryAllocation) ? LSH_ERR_GPU_OOM : LSH_ERR_CUDA;
}

#define LSH_CUDA(call)                                          \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return fail_cuda(e_, #call);     \
    } while (0)

int check_params(const lsh_params* p) {
    if (const char* why = lsh::params_problem(p)) {
        g_last_error = why;
        return LSH_ERR_INVALID;
    }
    return LSH_OK;
}

KArgs base_args(const lsh_ctx* ctx) {
    KArgs a;
    std::memset(&a, 0, sizeof(a));
    a.c = ctx->c;
    a.geo = ctx->geo;
    for (int k = 0; k < 7; ++k) {
        a.acc[k] = ctx->acc[k];
        a.sx[k] = ctx->sx[k]; a.sy[k] = ctx->sy[k];
        a.sxw[k] = ctx->sx[k]; a.syw[k] = ctx->sy[k];
    }
    a.eta_max = ctx->eta_max;
    a.eta_time = ctx->eta_time;
    a.szero = ctx->szero;
    a.tm = ctx->tm;
    return a;
}

dim3 grid_h(const lsh_ctx* ctx, int par) { return edge_grid_h(ctx->p.nx, ctx->p.ny, par); }
dim3 grid_v(const lsh_ctx* ctx, int par) { return edge_grid_v(ctx->p.nx, ctx->p.ny, par); }


template <int ORDER>
void enqueue_passes(const lsh_ctx* ctx, const KArgs& a, cudaStream_t s) {
    k_edges_h<true, ORDER><<<grid_h(ctx, 0), edge_block_h(), 0, s>>>(a, 0);
    k_edges_h<false, ORDER><<<grid_h(ctx, 1), edge_block_h(), 0, s>>>(a, 1);
    k_edges_v<ORDER><<<grid_v(ctx, 0), edge_block_v(), 0, s>>>(a, 0);
    k_edges_v<ORDER><<<grid_v(ctx, 1), edge_block_v(), 0, s>>>(a, 1);
}

// Enqueue one time step; returns the number of kernels launched.
int enqueue_step(const lsh_ctx* ctx, cudaStream_t s) {
    const dim3 nbc = cell_grid(ctx->p.nx, ctx->p.ny);
    if (ctx->dep_ctr) {
        KArgs a1 = base_args(ctx), a2 = base_args(ctx);
        for (int k = 0; k < 7; ++k) a1.W[k] = ctx->X[k];
        if (ctx->p.order == 1) {
            for (int k = 0; k < 6; ++k) a1.Wout[k] = ctx->X[k];
        } else {
            for (int k = 0; k < 6; ++k) a1.Wout[k] = ctx->Y[k];
            for (int k = 0; k < 6; ++k) a2.W[k] = ctx->Y[k];
            a2.W[6] = ctx->X[6];
            for (int k = 0; k < 6; ++k) { a2.Wout[k] = ctx->X[k]; a2.Xavg[k] = ctx->X[k]; }
        }
        return enqueue_step_overlap(ctx->p.nx, ctx->p.ny, ctx->p.order, a1, a2, ctx->dep_ctr, ctx->dep_stride, ctx->tm,
                                    2.0 * ctx->p.cfl, s);
    }
    if (ctx->p.order == 1) {
        KArgs a = base_args(ctx);
        for (int k = 0; k < 7; ++k) a.W[k] = ctx->X[k];
        for (int k = 0; k < 6; ++k) a.Wout[k] = ctx->X[k];
        enqueue_passes<1>(ctx, a, s);
        k_volume<0><<<nbc, cell_block(), 0, s>>>(a);
        k_advance<<<1, 1, 0, s>>>(ctx->tm, 2.0 * ctx->p.cfl);
        return 6;
    }
    KArgs a1 = base_args(ctx);
    for (int k = 0; k < 7; ++k) a1.W[k] = ctx->X[k];
    for (int k = 0; k < 6; ++k) a1.Wout[k] = ctx->Y[k];
    k_recon<<<nbc, cell_block(), 0, s>>>(a1);
    enqueue_passes<2>(ctx, a1, s);
    k_volume<1><<<nbc, cell_block(), 0, s>>>(a1);
    KArgs a2 = base_args(ctx);
    for (int k = 0; k < 6; ++k) a2.W[k] = ctx->Y[k];
    a2.W[6] = ctx->X[6];
    for (int k = 0; k < 6; ++k) { a2.Wout[k] = ctx->X[k]; a2.Xavg[k] = ctx->X[k]; }
    k_recon<<<nbc, cell_block(), 0, s>>>(a2);
    enqueue_passes<2>(ctx, a2, s);
    k_volume<2><<<nbc, cell_block(), 0, s>>>(a2);
    k_advance<<<1, 1, 0, s>>>(ctx->tm, 2.0 * ctx->p.cfl);
    return 13;
}

int build_graph(lsh_ctx* ctx, int nsteps, cudaGraphExec_t* out) {
    cudaGraph_t graph = nullptr;
    LSH_CUDA(cudaStreamBeginCapture(ctx->own, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < nsteps; ++i) enqueue_step(ctx, ctx->own);
    cudaError_t e = cudaStreamEndCapture(ctx->own, &graph);
    if (e != cudaSuccess) return fail_cuda(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail_cuda(e, "cudaGraphInstantiate");
    return LSH_OK;
}

int err_bits_to_status(int bits) {
    for (int s = 1; s < 31; ++s)
        if (bits & (1 << s)) return s;
    return LSH_OK;
}

int upload_state(lsh_ctx* ctx, const double* const src[LSH_NVARS], cudaMemcpyKind kind, double* dt0_out) {
    const size_t bytes = ctx->N * sizeof(double);
    for (int k = 0; k < 7; ++k) {
        if (!src[k]) { g_last_error = "null state pointer"; return LSH_ERR_INVALID; }
        LSH_CUDA(cudaMemcpyAsync(ctx->X[k], src[k], bytes, kind, ctx->stream));
    }
    KArgs a = base_args(ctx);
    for (int k = 0; k < 7; ++k) a.W[k] = ctx->X[k];
    const dim3 nbc = cell_grid(ctx->p.nx, ctx->p.ny);
    cudaStream_t s = ctx->stream;
    k_init_eta<<<nbc, cell_block(), 0, s>>>(a);
    TimeRec init{};
    init.rmax_bits = kRateInitBits;
    init.t_end = INFINITY;
    init.dt_min = ctx->p.dt_min;
    LSH_CUDA(cudaMemcpyAsync(ctx->tm, &init, sizeof(TimeRec), cudaMemcpyHostToDevice, s));
    launch_init_wave(a, ctx->p.nx, ctx->p.ny, s);
    k_cell_dt<<<nbc, cell_block(), 0, s>>>(a);
    k_init_finish<<<1, 1, 0, s>>>(ctx->tm, 2.0 * ctx->p.cfl);
    ctx->launches += 7;
    LSH_CUDA(cudaGetLastError());
    LSH_CUDA(cudaMemcpyAsync(ctx->tm_host, ctx->tm, sizeof(TimeRec), cudaMemcpyDeviceToHost, s));
    LSH_CUDA(cudaStreamSynchronize(s));
    ctx->has_state = true;
    if (dt0_out) *dt0_out = ctx->tm_host->dt;
    return LSH_OK;
}

int read_time(lsh_ctx* ctx) {
    LSH_CUDA(cudaMemcpyAsync(ctx->tm_host, ctx->tm, sizeof(TimeRec), cudaMemcpyDeviceToHost, ctx->stream));
    LSH_CUDA(cudaStreamSynchronize(ctx->stream));
    return LSH_OK;
}

int set_t_end(lsh_ctx* ctx, double t_end) {
    // update t_end and recompute `done` on the device stream (small H2D copy of two fields)
    if (int s = read_time(ctx)) return s;
    ctx->tm_host->t_end = t_end;
    ctx->tm_host->done = (ctx->tm_host->t >= t_end || ctx->tm_host->err) ? 1 : 0;
    LSH_CUDA(cudaMemcpyAsync(ctx->tm, ctx->tm_host, sizeof(TimeRec), cudaMemcpyHostToDevice, ctx->stream));
    return LSH_OK;
}

}  // namespace

extern "C" {

int lsh_params_default(lsh_params* p) {
    if (!p) return LSH_ERR_INVALID;
    std::memset(p, 0, sizeof(*p));
    p->nx = p->ny = 1;
    p->order = 1;
    p->coords = LSH_COORDS_CARTESIAN;
    p->friction_law = LSH_FRICTION_COULOMB;
    p->dx = p->dy = 1.0;
    p->radius = 6378136.6;
    p->borde_sup = p->borde_inf = p->borde_izq = p->borde_der = -1.0;
    p->cfl = 0.9;
    p->r = 0.5;
    p->gravity = 9.81;
    p->eps_h = 5e-3;
    p->L = p->H = 1.0;
    p->peso = p->beta = 1.0;
    return LSH_OK;
}

int lsh_check_device(void) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) { (void)cudaGetLastError(); return 1; }
    if (n == 0) return 1;
    for (int d = 0; d < n; ++d) {
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, d) == cudaSuccess && prop.major >= 1) return 0;
    }
    return 2;
}

const char* lsh_status_string(int s) {
    switch (s) {
        case LSH_OK: return "ok";
        case LSH_ERR_GPU_OOM: return "not enough GPU memory";
        case LSH_ERR_HOST_OOM: return "not enough CPU memory";
        case LSH_ERR_INVALID: return "invalid argument";
        case LSH_ERR_CUDA: return "CUDA error";
        case LSH_ERR_NUMERIC: return "NaN or Inf in the state";
        case LSH_ERR_IO: return "file missing or malformed";
        case LSH_ERR_NO_DEVICE: return "no CUDA device";
        case LSH_ERR_TIMEOUT: return "bounded device wait timed out";
        case LSH_ERR_STALL: return "time step below dt_min";
        default: return "unknown status";
    }
}

const char* lsh_last_error(void) { return g_last_error.c_str(); }

int lsh_create(const lsh_params* p, int device, lsh_ctx** out) {
    if (!out) return LSH_ERR_INVALID;
    *out = nullptr;
    if (int s = check_params(p)) return s;
    if (lsh_check_device() != 0) { g_last_error = "no CUDA device"; return LSH_ERR_NO_DEVICE; }
    lsh_ctx* ctx = new (std::nothrow) lsh_ctx();
    if (!ctx) return LSH_ERR_HOST_OOM;
    ctx->p = *p;
    ctx->c = lsh::make_consts(*p);
    ctx->N = size_t(p->nx) * p->ny;
    auto bail = [&](int s) { lsh_destroy(ctx); return s; };
    if (device >= 0) {
        cudaError_t e = cudaSetDevice(device);
        if (e != cudaSuccess) return bail(fail_cuda(e, "cudaSetDevice"));
    }
    {
        cudaError_t e = cudaGetDevice(&ctx->device);
        if (e != cudaSuccess) return bail(fail_cuda(e, "cudaGetDevice"));
        e = cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking);
        if (e != cudaSuccess) return bail(fail_cuda(e, "cudaStreamCreate"));
        ctx->stream = ctx->own;
    }
    // one slab: X(7) + Y(6) + acc(7) + eta(2) [+ sx, sy (14)] arrays of N, geometry, time record
    const size_t n_pad = (ctx->N + 31) & ~size_t(31);  // 256-byte aligned arrays
    const int n_arrays = 7 + 6 + 7 + 2 + ((p->order == 2) ? 14 : 0);
    const size_t geo_n = size_t(7) * (p->ny + 1);
    // pass-overlap counters: one per block row of each pass of a step (the
    // block rows of the edge and cell kernels), when the grids cover every
    // row in one launch
    const int dep_stride = dep_stride_for(p->nx, p->ny);
    const int kps = (p->order == 1) ? 6 : 13;
    const size_t dep_bytes = size_t(dep_stride) * kps * sizeof(unsigned);
    const size_t bytes = (size_t(n_arrays) * n_pad + ((geo_n + 31) & ~size_t(31))) * sizeof(double) + 256 +
                         ((p->order == 2) ? n_pad : 0) +  // + one byte per cell: slopes-are-zero flags
                         ((dep_bytes + 255) & ~size_t(255));
    {
        cudaError_t e = cudaMalloc(&ctx->slab, bytes);
        if (e != cudaSuccess) return bail(fail_cuda(e, "cudaMalloc"));
        e = cudaMallocHost((void**)&ctx->tm_host, sizeof(TimeRec));
        if (e != cudaSuccess) return bail(fail_cuda(e, "cudaMallocHost"));
    }
    double* cur = static_cast<double*>(ctx->slab);
    for (int k = 0; k < 7; ++k) { ctx->X[k] = cur; cur += n_pad; }
    for (int k = 0; k < 6; ++k) { ctx->Y[k] = cur; cur += n_pad; }
    for (int k = 0; k < 7; ++k) { ctx->acc[k] = cur; cur += n_pad; }
    ctx->eta_max = cur; cur += n_pad;
    ctx->eta_time = cur; cur += n_pad;
    if (p->order == 2) {
        for (int k = 0; k < 7; ++k) { ctx->sx[k] = cur; cur += n_pad; }
        for (int k = 0; k < 7; ++k) { ctx->sy[k] = cur; cur += n_pad; }
    }
    ctx->geo_buf = cur;
    cur += (geo_n + 31) & ~size_t(31);
    ctx->tm = reinterpret_cast<TimeRec*>(cur);
    unsigned char* tail = reinterpret_cast<unsigned char*>(cur) + 256;
    if (p->order == 2) {
        ctx->szero = tail;
        tail += n_pad;
        // no slope is known to be zero yet; wait before the legacy-stream copies below
        cudaError_t e = cudaMemsetAsync(ctx->szero, 0, n_pad, ctx->own);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->own);
        if (e != cudaSuccess) return bail(fail_cuda(e, "cudaMemset slope flags"));
    }
    if (dep_stride) {
        ctx->dep_ctr = reinterpret_cast<unsigned*>(tail);
        ctx->dep_stride = dep_stride;
        cudaError_t e = cudaMemsetAsync(ctx->dep_ctr, 0, dep_bytes, ctx->own);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->own);
        if (e != cudaSuccess) return bail(fail_cuda(e, "cudaMemset pass counters"));
    }

    const size_t st = size_t(p->ny + 1);
    std::vector<double> g(geo_n, 0.0);
    lsh::fill_geo(*p, g.data(), st);
    {
        cudaError_t e = cudaMemcpy(ctx->geo_buf, g.data(), geo_n * sizeof(double), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return bail(fail_cuda(e, "cudaMemcpy geometry"));
    }
    ctx->geo.area = ctx->geo_buf;
    ctx->geo.len_v = ctx->geo_buf + st;
    ctx->geo.len_h = ctx->geo_buf + 2 * st;
    ctx->geo.tanR = ctx->geo_buf + 3 * st;
    ctx->geo.wx = ctx->geo_buf + 4 * st;
    ctx->geo.wy = ctx->geo_buf + 5 * st;
    ctx->geo.inv_area = ctx->geo_buf + 6 * st;
    ctx->kernels_per_step = (p->order == 1) ? 6 : 13;
    *out = ctx;
    return LSH_OK;
}

int lsh_destroy(lsh_ctx* ctx) {
    if (!ctx) return LSH_OK;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->g_chunk) cudaGraphExecDestroy(ctx->g_chunk);
    if (ctx->g_one) cudaGraphExecDestroy(ctx->g_one);
    if (ctx->slab) cudaFree(ctx->slab);
    if (ctx->gauge_cells) cudaFree(ctx->gauge_cells);
    if (ctx->tm_host) cudaFreeHost(ctx->tm_host);
    if (ctx->own) cudaStreamDestroy(ctx->own);
    (void)cudaGetLastError();
    delete ctx;
    return LSH_OK;
}

int lsh_set_stream(lsh_ctx* ctx, void* s) {
    if (!ctx) return LSH_ERR_INVALID;
    ctx->stream = s ? static_cast<cudaStream_t>(s) : ctx->own;
    return LSH_OK;
}

int lsh_set_state(lsh_ctx* ctx, const double* const host_state[LSH_NVARS], double* dt0_out) {
    if (!ctx || !host_state) return LSH_ERR_INVALID;
    return upload_state(ctx, host_state, cudaMemcpyHostToDevice, dt0_out);
}

int lsh_set_state_device(lsh_ctx* ctx, const double* const dev_state[LSH_NVARS], double* dt0_out) {
    if (!ctx || !dev_state) return LSH_ERR_INVALID;
    return upload_state(ctx, dev_state, cudaMemcpyDeviceToDevice, dt0_out);
}

int lsh_step(lsh_ctx* ctx, int nsteps) {
    if (!ctx || nsteps < 0) return LSH_ERR_INVALID;
    if (!ctx->has_state) { g_last_error = "lsh_set_state has not been called"; return LSH_ERR_INVALID; }
    if (nsteps == 0) return LSH_OK;
    if (!ctx->g_chunk) { if (int s = build_graph(ctx, kGraphChunk, &ctx->g_chunk)) return s; }
    if (!ctx->g_one) { if (int s = build_graph(ctx, 1, &ctx->g_one)) return s; }
    const int full = nsteps / kGraphChunk, rest = nsteps % kGraphChunk;
    for (int i = 0; i < full; ++i) LSH_CUDA(cudaGraphLaunch(ctx->g_chunk, ctx->stream));
    for (int i = 0; i < rest; ++i) LSH_CUDA(cudaGraphLaunch(ctx->g_one, ctx->stream));
    ctx->launches += (long long)nsteps * ctx->kernels_per_step;
    return LSH_OK;
}

int lsh_synchronize(lsh_ctx* ctx) {
    if (!ctx) return LSH_ERR_INVALID;
    if (int s = read_time(ctx)) return s;
    return err_bits_to_status(ctx->tm_host->err);
}

int lsh_run_until(lsh_ctx* ctx, double t_end, long long max_steps, long long* steps_done) {
    if (!ctx) return LSH_ERR_INVALID;
    if (!ctx->has_state) { g_last_error = "lsh_set_state has not been called"; return LSH_ERR_INVALID; }
    if (int s = set_t_end(ctx, t_end)) return s;
    if (int s = read_time(ctx)) return s;
    const long long start = ctx->tm_host->steps;
    int status = LSH_OK;
    while (!ctx->tm_host->done) {
        long long left = (max_steps > 0) ? max_steps - (ctx->tm_host->steps - start) : (1LL << 40);
        if (left <= 0) break;
        const int batch = (int)std::min<long long>(left, 8 * kGraphChunk);
        if ((status = lsh_step(ctx, batch))) break;
        if ((status = read_time(ctx))) break;
    }
    if (status == LSH_OK) status = err_bits_to_status(ctx->tm_host->err);
    if (steps_done) *steps_done = ctx->tm_host->steps - start;
    // step-count mode again for later lsh_step calls
    int s2 = set_t_end(ctx, INFINITY);
    if (status == LSH_OK) status = s2;
    return status;
}

int lsh_get_state(lsh_ctx* ctx, double* const host_state[LSH_NVARS]) {
    if (!ctx || !host_state) return LSH_ERR_INVALID;
    const size_t bytes = ctx->N * sizeof(double);
    for (int k = 0; k < 7; ++k)
        if (host_state[k]) LSH_CUDA(cudaMemcpyAsync(host_state[k], ctx->X[k], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    LSH_CUDA(cudaStreamSynchronize(ctx->stream));
    return LSH_OK;
}

int lsh_get_state_device(lsh_ctx* ctx, double* const dev_state[LSH_NVARS]) {
    if (!ctx || !dev_state) return LSH_ERR_INVALID;
    const size_t bytes = ctx->N * sizeof(double);
    for (int k = 0; k < 7; ++k)
        if (dev_state[k]) LSH_CUDA(cudaMemcpyAsync(dev_state[k], ctx->X[k], bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    return LSH_OK;
}

int lsh_get_time(lsh_ctx* ctx, double* t, double* dt_next, long long* steps) {
    if (!ctx) return LSH_ERR_INVALID;
    if (int s = read_time(ctx)) return s;
    if (t) *t = ctx->tm_host->t;
    if (dt_next) *dt_next = ctx->tm_host->dt;
    if (steps) *steps = ctx->tm_host->steps;
    return LSH_OK;
}

int lsh_get_eta_max(lsh_ctx* ctx, double* eta_max, double* eta_time) {
    if (!ctx) return LSH_ERR_INVALID;
    const size_t bytes = ctx->N * sizeof(double);
    if (eta_max) LSH_CUDA(cudaMemcpyAsync(eta_max, ctx->eta_max, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    if (eta_time) LSH_CUDA(cudaMemcpyAsync(eta_time, ctx->eta_time, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    LSH_CUDA(cudaStreamSynchronize(ctx->stream));
    return LSH_OK;
}

int lsh_get_gauge_eta(lsh_ctx* ctx, int n, const int* cells, double* out) {
    if (!ctx || n < 0 || (n > 0 && (!cells || !out))) return LSH_ERR_INVALID;
    if (n == 0) return LSH_OK;
    if (n > ctx->gauge_cap) {
        // one buffer: n cell indices, then n values (256-byte aligned)
        if (ctx->gauge_cells) { cudaFree(ctx->gauge_cells); ctx->gauge_cells = nullptr; ctx->gauge_cap = 0; }
        const size_t idx_bytes = (size_t(n) * sizeof(int) + 255) & ~size_t(255);
        void* buf = nullptr;
        LSH_CUDA(cudaMalloc(&buf, idx_bytes + size_t(n) * sizeof(double)));
        ctx->gauge_cells = static_cast<int*>(buf);
        ctx->gauge_out = reinterpret_cast<double*>(static_cast<char*>(buf) + idx_bytes);
        ctx->gauge_cap = n;
        ctx->gauge_host.clear();
    }
    cudaStream_t s = ctx->stream;
    if (ctx->gauge_host.size() != size_t(n) || !std::equal(cells, cells + n, ctx->gauge_host.begin())) {
        ctx->gauge_host.assign(cells, cells + n);
        LSH_CUDA(cudaMemcpyAsync(ctx->gauge_cells, ctx->gauge_host.data(), size_t(n) * sizeof(int),
                                 cudaMemcpyHostToDevice, s));
    }
    k_gauge_eta<<<(n + 127) / 128, 128, 0, s>>>(ctx->X[0], ctx->X[6], ctx->gauge_cells, n, (long long)ctx->N,
                                                ctx->gauge_out);
    ctx->launches += 1;
    LSH_CUDA(cudaGetLastError());
    LSH_CUDA(cudaMemcpyAsync(out, ctx->gauge_out, size_t(n) * sizeof(double), cudaMemcpyDeviceToHost, s));
    LSH_CUDA(cudaStreamSynchronize(s));
    return LSH_OK;
}

int lsh_get_masks(lsh_ctx* ctx, uint8_t* mask) {
    if (!ctx || !mask) return LSH_ERR_INVALID;
    std::vector<double> h1(ctx->N), h2(ctx->N), qx(ctx->N), qy(ctx->N);
    double* dst[LSH_NVARS] = {h1.data(), nullptr, nullptr, h2.data(), qx.data(), qy.data(), nullptr};
    if (int s = lsh_get_state(ctx, dst)) return s;
    const double eps = ctx->p.eps_h;
    for (size_t i = 0; i < ctx->N; ++i) {
        uint8_t m = 0;
        if (h1[i] >= eps) m |= 1;
        if (h2[i] >= eps) { m |= 2; if (qx[i] == 0.0 && qy[i] == 0.0) m |= 4; }
        mask[i] = m;
    }
    return LSH_OK;
}

int lsh_profile_step(lsh_ctx* ctx, float* ms_out, int cap, int* n_kernels) {
    if (!ctx || !ms_out || cap < 1) return LSH_ERR_INVALID;
    if (!ctx->has_state) { g_last_error = "lsh_set_state has not been called"; return LSH_ERR_INVALID; }
    cudaStream_t s = ctx->stream;
    const int nk = ctx->kernels_per_step;
    std::vector<cudaEvent_t> ev(nk + 1);
    for (auto& e : ev) LSH_CUDA(cudaEventCreate(&e));
    const dim3 nbc = cell_grid(ctx->p.nx, ctx->p.ny);
    int i = 0;
    auto mark = [&]() { cudaEventRecord(ev[i++], s); };
    mark();
    if (ctx->p.order == 1) {
        KArgs a = base_args(ctx);
        for (int k = 0; k < 7; ++k) a.W[k] = ctx->X[k];
        for (int k = 0; k < 6; ++k) a.Wout[k] = ctx->X[k];
        k_edges_h<true, 1><<<grid_h(ctx, 0), edge_block_h(), 0, s>>>(a, 0); mark();
        k_edges_h<false, 1><<<grid_h(ctx, 1), edge_block_h(), 0, s>>>(a, 1); mark();
        k_edges_v<1><<<grid_v(ctx, 0), edge_block_v(), 0, s>>>(a, 0); mark();
        k_edges_v<1><<<grid_v(ctx, 1), edge_block_v(), 0, s>>>(a, 1); mark();
        k_volume<0><<<nbc, cell_block(), 0, s>>>(a); mark();
    } else {
        for (int stage = 0; stage < 2; ++stage) {
            KArgs a = base_args(ctx);
            if (stage == 0) {
                for (int k = 0; k < 7; ++k) a.W[k] = ctx->X[k];
                for (int k = 0; k < 6; ++k) a.Wout[k] = ctx->Y[k];
            } else {
                for (int k = 0; k < 6; ++k) a.W[k] = ctx->Y[k];
                a.W[6] = ctx->X[6];
                for (int k = 0; k < 6; ++k) { a.Wout[k] = ctx->X[k]; a.Xavg[k] = ctx->X[k]; }
            }
            k_recon<<<nbc, cell_block(), 0, s>>>(a); mark();
            k_edges_h<true, 2><<<grid_h(ctx, 0), edge_block_h(), 0, s>>>(a, 0); mark();
            k_edges_h<false, 2><<<grid_h(ctx, 1), edge_block_h(), 0, s>>>(a, 1); mark();
            k_edges_v<2><<<grid_v(ctx, 0), edge_block_v(), 0, s>>>(a, 0); mark();
            k_edges_v<2><<<grid_v(ctx, 1), edge_block_v(), 0, s>>>(a, 1); mark();
            if (stage == 0) k_volume<1><<<nbc, cell_block(), 0, s>>>(a);
            else k_volume<2><<<nbc, cell_block(), 0, s>>>(a);
            mark();
        }
    }
    k_advance<<<1, 1, 0, s>>>(ctx->tm, 2.0 * ctx->p.cfl); mark();
    ctx->launches += nk;
    int status = LSH_OK;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[nk]);
    if (e != cudaSuccess) status = fail_cuda(e, "lsh_profile_step");
    for (int k = 0; k < nk && k < cap && status == LSH_OK; ++k) cudaEventElapsedTime(&ms_out[k], ev[k], ev[k + 1]);
    for (auto& ee : ev) cudaEventDestroy(ee);
    if (n_kernels) *n_kernels = nk;
    return status;
}

int lsh_probe_fp64_peak(int device, double* gflops) {
    if (!gflops) return LSH_ERR_INVALID;
    if (lsh_check_device() != 0) return LSH_ERR_NO_DEVICE;
    if (device >= 0) LSH_CUDA(cudaSetDevice(device));
    int dev = 0, sms = 0;
    LSH_CUDA(cudaGetDevice(&dev));
    LSH_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* out = nullptr;
    LSH_CUDA(cudaMalloc(&out, sizeof(double)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int threads = 256, blocks = sms * 8, iters = 4096;
    k_fp64_probe<<<blocks, threads>>>(out, 64, 1.0000001, 1e-9);  // warm-up
    cudaEventRecord(e0);
    k_fp64_probe<<<blocks, threads>>>(out, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return fail_cuda(e, "lsh_probe_fp64_peak");
    const double flops = 2.0 * 8.0 * double(iters) * threads * blocks;
    *gflops = flops / (ms * 1e-3) / 1e9;
    return LSH_OK;
}

int lsh_get_launch_count(lsh_ctx* ctx, long long* launches) {
    if (!ctx || !launches) return LSH_ERR_INVALID;
    *launches = ctx->launches;
    return LSH_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ allocation-free stepping
//
// lsh_step_noalloc (include/lsh.h) runs the first-order step with all of its
// scratch in the file-scope array below instead of allocated memory.  Layout
// (doubles): 7 accumulators of LSH_NOALLOC_MAX_CELLS, then 6 per-row geometry
// arrays of LSH_NOALLOC_MAX_ROWS + 1, then the 64-byte time record.  Host code
// must not use the array's name as an address: the device address is looked
// up once per device with cudaGetSymbolAddress (with that device current) and
// passed to the kernels.

namespace {

constexpr size_t kNaAccStride = LSH_NOALLOC_MAX_CELLS;
constexpr size_t kNaGeoStride = LSH_NOALLOC_MAX_ROWS + 1;
constexpr size_t kNaGeoOffset = 7 * kNaAccStride;
constexpr size_t kNaTimeOffset = (kNaGeoOffset + 7 * kNaGeoStride + 31) & ~size_t(31);
constexpr size_t kNaDoubles = kNaTimeOffset + sizeof(TimeRec) / sizeof(double);

__device__ __align__(256) double g_noalloc_scratch[kNaDoubles];

constexpr int kNaMaxDevices = 64;
double* g_noalloc_base[kNaMaxDevices] = {};
std::mutex g_noalloc_mu;
// host-side geometry staging for the upload (no heap allocation per call)
double g_noalloc_geo_host[7 * kNaGeoStride];

// Move the running min of per-cell dt into dt (initial-dt pass of a no-alloc call).
__global__ void k_noalloc_take_dt(TimeRec* tm, double two_cfl) {
    tm->dt = dt_of(tm->rmax_bits, two_cfl);
    tm->rmax_bits = kRateInitBits;
}

}  // namespace

extern "C" int lsh_step_noalloc(const lsh_params* p, double* const dev_state[LSH_NVARS], int nsteps,
                                double* t_io, double* dt_io, void* cuda_stream) {
    if (int s = check_params(p)) return s;
    if (!dev_state || !t_io || !dt_io || nsteps < 0) { g_last_error = "lsh_step_noalloc: null pointer or nsteps < 0"; return LSH_ERR_INVALID; }
    for (int k = 0; k < LSH_NVARS; ++k)
        if (!dev_state[k]) { g_last_error = "lsh_step_noalloc: null state array"; return LSH_ERR_INVALID; }
    if (p->order != 1) { g_last_error = "lsh_step_noalloc: only the first-order step (order 1) runs without allocation"; return LSH_ERR_INVALID; }
    if ((long long)p->nx * p->ny > LSH_NOALLOC_MAX_CELLS || p->ny > LSH_NOALLOC_MAX_ROWS) {
        g_last_error = "lsh_step_noalloc: grid larger than LSH_NOALLOC_MAX_CELLS (65536) cells or LSH_NOALLOC_MAX_ROWS (4096) rows";
        return LSH_ERR_INVALID;
    }
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    int dev = 0;
    LSH_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNaMaxDevices) { g_last_error = "lsh_step_noalloc: device index out of range"; return LSH_ERR_INVALID; }
    if (!g_noalloc_base[dev]) {
        double* base = nullptr;
        cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&base), g_noalloc_scratch);
        if (e != cudaSuccess) return fail_cuda(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_base[dev] = base;
    }
    double* base = g_noalloc_base[dev];

    lsh::fill_geo(*p, g_noalloc_geo_host, kNaGeoStride);
    LSH_CUDA(cudaMemcpyAsync(base + kNaGeoOffset, g_noalloc_geo_host, 7 * kNaGeoStride * sizeof(double),
                             cudaMemcpyHostToDevice, s));
    TimeRec* tm = reinterpret_cast<TimeRec*>(base + kNaTimeOffset);
    TimeRec init{};
    init.t = *t_io;
    init.dt = *dt_io;
    init.t_end = INFINITY;
    init.dt_min = p->dt_min;
    init.rmax_bits = kRateInitBits;
    LSH_CUDA(cudaMemcpyAsync(tm, &init, sizeof(TimeRec), cudaMemcpyHostToDevice, s));

    KArgs a;
    std::memset(&a, 0, sizeof(a));
    a.c = lsh::make_consts(*p);
    a.c.track_eta = 0;
    const double* g = base + kNaGeoOffset;
    a.geo.area = g;
    a.geo.len_v = g + kNaGeoStride;
    a.geo.len_h = g + 2 * kNaGeoStride;
    a.geo.tanR = g + 3 * kNaGeoStride;
    a.geo.wx = g + 4 * kNaGeoStride;
    a.geo.wy = g + 5 * kNaGeoStride;
    a.geo.inv_area = g + 6 * kNaGeoStride;
    for (int k = 0; k < 7; ++k) { a.W[k] = dev_state[k]; a.acc[k] = base + k * kNaAccStride; }
    for (int k = 0; k < 6; ++k) a.Wout[k] = dev_state[k];
    a.tm = tm;

    const int nx = p->nx, ny = p->ny;
    const dim3 nbc = cell_grid(nx, ny);
    if (!(*dt_io > 0.0)) {
        // initial dt (ShallowWater.cu:236-257) into the time record
        launch_init_wave(a, nx, ny, s);
        k_cell_dt<<<nbc, cell_block(), 0, s>>>(a);
        k_noalloc_take_dt<<<1, 1, 0, s>>>(tm, 2.0 * p->cfl);
    }
    const dim3 gh0 = edge_grid_h(nx, ny, 0), gh1 = edge_grid_h(nx, ny, 1);
    const dim3 gv0 = edge_grid_v(nx, ny, 0), gv1 = edge_grid_v(nx, ny, 1);
    for (int i = 0; i < nsteps; ++i) {
        k_edges_h<true, 1><<<gh0, edge_block_h(), 0, s>>>(a, 0);
        k_edges_h<false, 1><<<gh1, edge_block_h(), 0, s>>>(a, 1);
        k_edges_v<1><<<gv0, edge_block_v(), 0, s>>>(a, 0);
        k_edges_v<1><<<gv1, edge_block_v(), 0, s>>>(a, 1);
        k_volume<0><<<nbc, cell_block(), 0, s>>>(a);
        k_advance<<<1, 1, 0, s>>>(tm, 2.0 * p->cfl);
    }
    LSH_CUDA(cudaGetLastError());
    TimeRec out{};
    LSH_CUDA(cudaMemcpyAsync(&out, tm, sizeof(TimeRec), cudaMemcpyDeviceToHost, s));
    LSH_CUDA(cudaStreamSynchronize(s));
    *t_io = out.t;
    *dt_io = out.dt;
    return err_bits_to_status(out.err);
}

namespace lsh {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace lsh
