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
#include "lsh_queue.cuh"
#include "lsh_setup.h"

using lsh::KArgs;
using lsh::kCellBlock;
using lsh::kEdgeBlock;
using lsh::kRateInitBits;

namespace {

constexpr int kBatchGraphSteps = 8;
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

// The step's passes: reconstruction (second order), the four colour edge
// passes and the Euler stage, per stage.
int build_plan(lsh_batch* b) {
    std::vector<int> nx(b->n), ny(b->n);
    for (int s = 0; s < b->n; ++s) { nx[s] = b->params[s].nx; ny[s] = b->params[s].ny; }
    std::vector<QPassSpec> passes;
    const int stages = (b->order == 2) ? 2 : 1;
    for (int st = 0; st < stages; ++st) {
        if (b->order == 2) passes.push_back({kOpRecon, kBCell, st});
        passes.push_back({kOpH0, kBH0, st});
        passes.push_back({kOpH1, kBH1, st});
        passes.push_back({kOpV0, kBV0, st});
        passes.push_back({kOpV1, kBV1, st});
        passes.push_back({(b->order == 1) ? kOpVol0 : (st == 0 ? kOpVol1 : kOpVol2), kBCell, st});
    }
    return build_queue_plan(nx, ny, passes, b->d_args, &b->d_plan_mem, b->plan, b->n_ctr);
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
    static const int ctas[] = {8, 12, 16, 20, 24, 32};
    static const int fetches[] = {1, 2, 4, 8};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    lsh_tune best = b->tune;
    best.ms_per_step = INFINITY;
    for (int c : ctas) {
        if (c > kBMaxCtas) continue;
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
