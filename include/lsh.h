/*
 * lsh.h -- C ABI of the GB300-native two-layer finite-volume time step
 * (shallow water over a Savage-Hutter granular layer, LandSlide-HySEA scheme).
 *
 * Everything here is plain C: opaque context, plain pointers and sizes, int
 * status codes.  No CUDA or torch types appear in any signature; streams are
 * passed as `void*` (a cudaStream_t).
 *
 * Reference interface this replaces:
 *   extern "C" int shallowWater(TDatoCluster*, float xmin, ..., int num_puntos_guardar)
 *     src/GPU/ShallowWater.cu:125-131 (definition), src/GPU/main.cxx:12-18 (declaration)
 *   extern "C" int comprobarSoporteCUDA()     src/GPU/ComprobarSoporteCUDA.cu:5
 * The one-call compatibility entry point with the reference's exact argument
 * list is declared in lsh_compat.h.  The functions below split that call into
 * create / set-state / step / read-back so a host (C, C++, ctypes) can drive the
 * time loop, keep the state resident in HBM and capture the loop in a CUDA graph.
 *
 * Grid convention (same as the reference): cell (i, j) has linear index
 * j*nx + i, i = column (x, east), j = row (y).  Horizontal edge row y lies
 * between rows y-1 and y; its normal points toward increasing j
 * (Arista_kernel.cu:754-834).  Row 0's outer edge is the "sup" boundary, row
 * ny-1's the "inf" boundary, column 0's the "izq" boundary, column nx-1's the
 * "der" boundary.  In spherical coordinates row j lies at latitude
 * lat0 + (j + 0.5)*dlat and column i at longitude lon0 + (i + 0.5)*dlon.
 *
 * State arrays are FP64, nx*ny each, in this order:
 *   h1 (water depth), q1x, q1y (water discharge), h2 (granular thickness),
 *   q2x, q2y (granular discharge), H (bottom depth below the reference level,
 *   positive downward).  Free surface eta1 = h1 + h2 - H.
 */
#ifndef LSH_H
#define LSH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  0/1/2 keep the reference's meaning (ShallowWater.cu:124,
 * 50-57, 212-216); the rest are new. */
#define LSH_OK              0
#define LSH_ERR_GPU_OOM     1  /* device allocation failed                       */
#define LSH_ERR_HOST_OOM    2  /* host allocation failed                         */
#define LSH_ERR_INVALID     3  /* bad argument / size / parameter                */
#define LSH_ERR_CUDA        4  /* a CUDA runtime call failed                     */
#define LSH_ERR_NUMERIC     5  /* NaN or negative depth detected in the state    */
#define LSH_ERR_IO          6  /* file missing / unreadable / malformed          */
#define LSH_ERR_NO_DEVICE   7  /* no CUDA device (comprobarSoporteCUDA == 1 / 2)  */
#define LSH_ERR_TIMEOUT     8  /* a bounded device wait gave up                   */
#define LSH_ERR_STALL       9  /* time step collapsed below dt_min                */

#define LSH_NVARS 7            /* h1 q1x q1y h2 q2x q2y H */

enum { LSH_COORDS_CARTESIAN = 0, LSH_COORDS_SPHERICAL = 1 };
enum { LSH_FRICTION_COULOMB = 0, LSH_FRICTION_POULIQUEN = 1 };

/*
 * Solver parameters.  Field meaning follows the reference's shallowWater()
 * arguments (ShallowWater.cu:125-131) and data.dat (main.cxx:24-60), in the
 * reference's normalised units when L/H normalisation is used
 * (Problema.cxx:262-285).  Angles are in radians (Problema.cxx:239-256).
 * Fields the reference hard-codes are exposed with its values as defaults
 * (lsh_params_default): peso = beta = 1 (main.cxx:161), eps_h = 5e-3/H
 * (Problema.cxx:287).
 */
typedef struct lsh_params {
    int32_t nx, ny;          /* cells in x (columns) and y (rows)                     */
    int32_t order;           /* 1: first order + forward Euler (the reference scheme) */
                             /* 2: MUSCL (minmod) reconstruction + TVD-RK2 (Heun)     */
    int32_t coords;          /* LSH_COORDS_*                                          */
    int32_t friction_law;    /* LSH_FRICTION_* (reference #define COULOMB)            */
    int32_t track_eta_max;   /* 1: update eta1 max / time every step (A18)            */
    int32_t eig_sort;        /* 0: the reference's compare-and-swap sequence for the  */
                             /*    eigenvalue bounds (Arista_kernel.cu:193-234, with  */
                             /*    its (2,1) compare: not a full sort); 1: a true     */
                             /*    ascending sort (conserves mass at wall edges)      */
    double dx, dy;           /* Cartesian cell width / height (ancho_vol, alto_vol)   */
    double lon0, lat0;       /* spherical: corner longitude / latitude, degrees       */
    double dlon, dlat;       /* spherical: cell size, degrees                         */
    double radius;           /* spherical: sphere radius, same length unit as dx      */
    double borde_sup, borde_inf, borde_izq, borde_der; /* 1 open, -1 wall, 0 no-flux   */
    double cfl;              /* CFL number                                            */
    double r;                /* density ratio rho1/rho2                               */
    double angle1, angle2, angle3, angle4; /* friction angles, radians (2..4: Pouliquen) */
    double mfc, mf0, mfs;    /* interlayer, water-bottom (Manning), sediment-bottom   */
    double vmax1, vmax2;     /* speed caps (<= 0: off)                                */
    double gravity;          /* 9.81, or 1 when normalised                           */
    double eps_h;            /* dry threshold                                         */
    double L, H;             /* normalisation scales (1, 1 when not normalised)       */
    double peso, beta;       /* reference constants, 1 and 1                          */
    double dt_min;           /* stall guard: dt below this sets LSH_ERR_STALL (0 off) */
} lsh_params;

typedef struct lsh_ctx lsh_ctx;  /* opaque solver context: owns all device memory */

/* Fill `p` with the reference defaults (Coulomb law, first order, Cartesian,
 * walls, CFL 0.9, r 0.5, g 9.81, eps_h 5e-3, peso = beta = 1, L = H = 1). */
int lsh_params_default(lsh_params* p);

/* comprobarSoporteCUDA (ComprobarSoporteCUDA.cu:5-25): 0 = a CUDA device is
 * present, 1 = no device, 2 = no CUDA-capable device. */
int lsh_check_device(void);

/* Create a context on `device` (-1: current device).  Allocates the FP64 SoA
 * state (ping-pong), accumulators and the device-resident time/dt record.
 * Replaces inicializarDatosCuda (ShallowWater.cu:14-110). */
int lsh_create(const lsh_params* p, int device, lsh_ctx** out);
int lsh_destroy(lsh_ctx* ctx);

/* Run subsequent work on this cudaStream_t (NULL: the context's own stream). */
int lsh_set_stream(lsh_ctx* ctx, void* cuda_stream);

/* Upload the state from HOST arrays (nx*ny doubles each, order above; pointers
 * may be pageable or pinned).  Resets t = 0, eta1 max = h1 + h2 - H with time
 * 0 (Problema.cxx:542-546) and runs the initial-dt edge pass
 * (ShallowWater.cu:236-263).  `dt0_out` (may be NULL) receives that dt. */
int lsh_set_state(lsh_ctx* ctx, const double* const host_state[LSH_NVARS], double* dt0_out);

/* Same, from DEVICE arrays already resident on the context's device. */
int lsh_set_state_device(lsh_ctx* ctx, const double* const dev_state[LSH_NVARS], double* dt0_out);

/* Advance `nsteps` time steps on the device.  Asynchronous: enqueues a CUDA
 * graph of the steps on the context stream and returns.  dt and t stay on the
 * device (no host sync per step, unlike ShallowWater.cu:439-442). */
int lsh_step(lsh_ctx* ctx, int nsteps);

/* Advance until t >= t_end (the reference's loop condition, ShallowWater.cu:269)
 * or `max_steps` steps (<= 0: no limit).  Synchronous.  `steps_done` may be NULL. */
int lsh_run_until(lsh_ctx* ctx, double t_end, long long max_steps, long long* steps_done);

/* Wait for queued work; returns the sticky device error word as a status. */
int lsh_synchronize(lsh_ctx* ctx);

/* Copy the state to HOST arrays (synchronous). */
int lsh_get_state(lsh_ctx* ctx, double* const host_state[LSH_NVARS]);

/* Copy the state into DEVICE arrays on the context stream (asynchronous). */
int lsh_get_state_device(lsh_ctx* ctx, double* const dev_state[LSH_NVARS]);

/* Current time, the dt the next step will use, and the number of steps taken. */
int lsh_get_time(lsh_ctx* ctx, double* t, double* dt_next, long long* steps);

/* eta1 maximum and its time, nx*ny each (either may be NULL). */
int lsh_get_eta_max(lsh_ctx* ctx, double* eta_max, double* eta_max_time);

/* Per-cell bit mask of the current state: bit0 h1 >= eps_h, bit1 h2 >= eps_h,
 * bit2 granular layer at rest (h2 >= eps_h and q2 == 0: Coulomb stop). */
int lsh_get_masks(lsh_ctx* ctx, uint8_t* host_mask);

/* The reference's gauge value at `n` cells, gathered on the device:
 * out[g] = h1 - H at cells[g] (eta1 without the granular layer and before
 * the Hmin shift, as ShallowWater.cu:318-331 prints it); a cell index
 * outside the grid gives NaN.  Synchronous; moves 8 bytes per gauge to the
 * host (the reference copies its whole layer-1 array back per gauge row,
 * ShallowWater.cu:320). */
int lsh_get_gauge_eta(lsh_ctx* ctx, int n, const int* cells, double* out);

/* Number of kernels this library launched since the context was created
 * (each graph replay counts its kernel nodes). */
int lsh_get_launch_count(lsh_ctx* ctx, long long* launches);

/* Allocation-free stepping.  No counterpart in the reference.
 * For hosts that cannot allocate device memory: a coupling framework or plugin
 * host that owns every byte of GPU memory through its own pool (a
 * cudaMalloc behind its back would break its accounting or fail against its
 * reservation), or a real-time loop that must not pay for an allocation.
 * The caller owns the state.  The call allocates nothing and calls no
 * allocating routine, but it is not launch-only: every call copies the
 * per-row geometry and the time record (t, dt) from host memory to the
 * device on `cuda_stream`, launches the step's kernels, copies the time
 * record back and synchronises `cuda_stream` to read it.
 * Advances the FIRST-ORDER step (order must be 1) `nsteps` times on the
 * caller's DEVICE arrays dev_state[7] (h1 q1x q1y h2 q2x q2y H, nx*ny each,
 * updated in place) on `cuda_stream` (NULL: the legacy default stream).
 * *dt_io: the dt of the first step; <= 0 means "run the initial-dt pass
 * first".  On return *t_io and *dt_io hold the time and the next step's dt.
 * eta1 max is not tracked.
 * Its accumulators, per-row geometry and time record live in one file-scope
 * __device__ array sized for LSH_NOALLOC_MAX_CELLS cells and
 * LSH_NOALLOC_MAX_ROWS rows (about 3.9 MB), which every GPU that loads the
 * library holds until the process exits.  Larger grids are rejected with
 * LSH_ERR_INVALID.  The first call on a device looks that array's device
 * address up (cudaGetSymbolAddress, with that device current); make that
 * first call before any stream capture.  The accumulators are written, not
 * added to, by the step's first edge pass, and the time record is rewritten
 * by every call, so nothing left by an earlier call is read.  All calls of
 * one process share the one array (each process has its own copy), so calls
 * that overlap on the GPU (on other streams, or from other host threads)
 * race: serialise them. */
#define LSH_NOALLOC_MAX_CELLS 65536
#define LSH_NOALLOC_MAX_ROWS  4096
int lsh_step_noalloc(const lsh_params* p, double* const dev_state[LSH_NVARS], int nsteps,
                     double* t_io, double* dt_io, void* cuda_stream);

/* Diagnostics (no counterpart in the reference).
 * lsh_profile_step: run ONE time step eagerly (not from a graph) with a CUDA
 * event between consecutive kernels on the context stream; ms_out[i] gets the
 * duration of the i-th kernel of the step (order 1: 6 kernels -- 4 edge
 * passes, volume, clock; order 2: 13 -- per stage reconstruction, 4 edge
 * passes, volume; then clock).  *n_kernels gets the count (<= cap written).
 * lsh_probe_fp64_peak: FP64 FMA throughput of this device, GFLOP/s
 * (2 flops per DFMA), from a dependent-chain microkernel timed with events. */
int lsh_profile_step(lsh_ctx* ctx, float* ms_out, int cap, int* n_kernels);
int lsh_probe_fp64_peak(int device, double* gflops);

/* Diagnostic: the bounded waits between passes give up instead of hanging.
 * One block runs the overlapped step's wait and the work queue's wait on
 * completion counters that nothing increments; each gives up after its bound
 * (about 2 s of device time) and records it.  *status_out = LSH_ERR_TIMEOUT
 * when both waits gave up and reported (the expected outcome), LSH_OK when
 * either did not; *ms_out (may be null) gets the kernel's duration.  The
 * device is used again afterwards, and the call returns LSH_OK if it
 * answers.  Takes about 4 s.  No reference counterpart. */
int lsh_probe_wait_bound(int device, int* status_out, double* ms_out);

/* ---------------------------------------------------------------------------
 * Batched ensemble (no counterpart in the reference): n scenarios with their
 * own parameters and uneven grids (all of one `order`) advanced together.
 * A time step of the whole ensemble is ONE persistent launch: its CTAs pull
 * work items -- (pass, scenario, 2-D tile of edges or cells) -- from a device
 * queue in pass order, and an item waits only for its own scenario's rows of
 * the pass before it (completion counters); a small kernel then advances
 * every scenario's clock.  A run of steps is a CUDA graph.  Every scenario
 * stays bit-identical to its single-grid run (lsh_create...). */
typedef struct lsh_batch lsh_batch;
typedef struct lsh_tune {
    int32_t ctas_per_sm;        /* persistent CTAs of 64 threads per SM (1-20)  */
    int32_t items_per_fetch;    /* work items a CTA takes from the queue at once */
    double ms_per_step;         /* measured by lsh_batch_autotune               */
} lsh_tune;
int lsh_batch_create(const lsh_params* params, int n, int device, lsh_batch** out);
int lsh_batch_destroy(lsh_batch* b);
/* upload scenario `s` from host arrays and run its initial-dt pass */
int lsh_batch_set_state(lsh_batch* b, int s, const double* const host_state[LSH_NVARS], double* dt0_out);
int lsh_batch_step(lsh_batch* b, int nsteps);              /* asynchronous */
int lsh_batch_synchronize(lsh_batch* b);
int lsh_batch_get_state(lsh_batch* b, int s, double* const host_state[LSH_NVARS]);
int lsh_batch_get_time(lsh_batch* b, int s, double* t, double* dt_next, long long* steps);
/* autotuner: time the candidate CTA counts and fetch sizes on live steps and
 * keep the fastest (the trial steps advance the simulation) */
int lsh_batch_autotune(lsh_batch* b, int trial_steps, lsh_tune* best);
int lsh_batch_set_tune(lsh_batch* b, const lsh_tune* tune);
int lsh_batch_get_tune(lsh_batch* b, lsh_tune* tune);
int lsh_batch_get_launch_count(lsh_batch* b, long long* launches);

/* ------------------------------------------------------------------------
 * Discrete adjoint (no counterpart in the reference, which has no
 * differentiation): the gradient of
 *   J = w * sum_{n=1..N} sum_g (eta1_n[g] - target[n-1][g])^2 + <bar_final, X_N>,
 * eta1 = h1 + h2 - H at gauge cells after each step, with respect to the
 * initial h1, q1x, q1y, h2, q2x, q2y of every cell and to (angle1, mf0, mfs, r).
 * dt is the CFL step of the previous state and is differentiated as such.
 * Checkpoints follow a binomial (revolve) schedule in as many state slots as
 * the memory budget holds (default 180 GB, capped by free device memory).
 * Coulomb friction law only.
 * ------------------------------------------------------------------------ */
typedef struct lsh_adjoint lsh_adjoint;

typedef struct lsh_adjoint_stats {
    int32_t slots;              /* checkpoint slots (states) held              */
    int32_t nsteps;             /* steps of the recorded forward run           */
    int64_t forward_steps;      /* steps run by lsh_adjoint_forward            */
    int64_t recompute_steps;    /* steps re-advanced by the schedule           */
    int64_t reversed_steps;     /* steps reversed (each recomputed once more)  */
    double ms_forward;          /* wall time of the last lsh_adjoint_forward   */
    double ms_gradient;         /* wall time of the last lsh_adjoint_gradient  */
    double slot_bytes;          /* device bytes per checkpoint slot            */
} lsh_adjoint_stats;

int lsh_adjoint_create(const lsh_params* params, int device, int n_gauges, const int* gauge_cells,
                       lsh_adjoint** out);
int lsh_adjoint_destroy(lsh_adjoint* a);
/* thin-layer projection (default 0: the exact discrete adjoint): after every
 * step, the adjoint of a layer thinner than h_adj (h, qx, qy of that layer)
 * is set to 0, i.e. the gradient of the linearisation in which such layers
 * are passive.  Over long runs with wet/dry fronts the exact adjoint grows
 * without bound through the 1/h and sqrt(h) derivatives of thin layers; a
 * few millimetres to centimetres keeps it finite. */
int lsh_adjoint_set_thin_layer(lsh_adjoint* a, double h_adj);
/* ordered != 0: run the forward, recomputed and adjoint passes each as a
 * full-grid launch after the one before, instead of overlapped (the default).
 * The results are the same bits either way; this checks that. */
int lsh_adjoint_set_ordered(lsh_adjoint* a, int ordered);
/* device bytes the checkpoint slots may take */
int lsh_adjoint_set_budget(lsh_adjoint* a, double bytes);
/* run nsteps from host_state (7 arrays); target: nsteps x n_gauges (NULL: no
 * misfit); misfit: J without the weight; gauge_series: nsteps x n_gauges (may be NULL) */
int lsh_adjoint_forward(lsh_adjoint* a, const double* const host_state[LSH_NVARS], int nsteps, const double* target,
                        double* misfit, double* gauge_series);
/* gradient of misfit_weight * J + <bar_final, X_N> (bar_final: 6 arrays or
 * NULL); grad_state: 6 host arrays (entries may be NULL); grad_params[4]:
 * d/d(angle1 [rad], mf0, mfs, r) */
int lsh_adjoint_gradient(lsh_adjoint* a, double misfit_weight, const double* const bar_final[6],
                         double* grad_state[6], double grad_params[4]);
int lsh_adjoint_get_stats(lsh_adjoint* a, lsh_adjoint_stats* out);
/* simulated time after each step of the recorded run (nsteps values): the
 * time axis of the gauge series */
int lsh_adjoint_get_times(lsh_adjoint* a, double* t_out);
/* the recorded run's final state X_N (6 host arrays, entries may be NULL);
 * valid after lsh_adjoint_forward, before lsh_adjoint_gradient */
int lsh_adjoint_get_state(lsh_adjoint* a, double* const host_state[6]);
/* ------------------------------------------------------------------------
 * Batched adjoint (no counterpart in the reference): n scenarios (uneven
 * grids, each with its own parameters and gauges) run forward and reversed
 * together, for one step count.  One
 * checkpoint schedule drives every member with the same slot count, taken
 * from a joint budget (default 180 GB, capped by free device memory) over
 * the members' summed slot bytes.  Every operation of the schedule
 * runs all members of an order at once, on one stream the members share: a
 * forward step is one persistent work-queue launch over every member's
 * tiles, and a reversed step is one queue launch of the recomputation plus
 * one persistent launch of the whole adjoint step.  Each member's misfit and
 * gradient are bit-identical to an lsh_adjoint of its own with that slot
 * count.
 * ------------------------------------------------------------------------ */
typedef struct lsh_adjoint_batch lsh_adjoint_batch;

/* params[n]; n_gauges[n] (NULL: none) and gauge_cells[n] (member i's cells) */
int lsh_adjoint_batch_create(int n, const lsh_params* params, const int* n_gauges, const int* const* gauge_cells,
                             int device, lsh_adjoint_batch** out);
int lsh_adjoint_batch_destroy(lsh_adjoint_batch* b);
int lsh_adjoint_batch_set_thin_layer(lsh_adjoint_batch* b, double h_adj);
/* device bytes all members' checkpoint slots may take together */
int lsh_adjoint_batch_set_budget(lsh_adjoint_batch* b, double bytes);
/* host_states: n x LSH_NVARS arrays (member i's variable k at [i LSH_NVARS + k]);
 * targets[n] (NULL, or entries NULL: no misfit), misfits[n] (may be NULL),
 * gauge_series[n] (may be NULL, entries may be NULL): as lsh_adjoint_forward */
int lsh_adjoint_batch_forward(lsh_adjoint_batch* b, const double* const* host_states, int nsteps,
                              const double* const* targets, double* misfits, double* const* gauge_series);
/* gradient of misfit_weights[i] * J_i (NULL: weights 1) for every member;
 * grad_states: n x 6 host arrays (may be NULL, entries may be NULL);
 * grad_params: n x 4 (may be NULL) */
int lsh_adjoint_batch_gradient(lsh_adjoint_batch* b, const double* misfit_weights, double* const* grad_states,
                               double* grad_params);
/* slots per member, steps, schedule counts per member; ms_* are the batch's
 * wall times; slot_bytes is the bytes of one slot of every member together */
int lsh_adjoint_batch_get_stats(lsh_adjoint_batch* b, lsh_adjoint_stats* out);
/* member i, owned by the batch (lsh_adjoint_destroy refuses it); after a
 * batch forward run it may be run on its own with the batch's slot count;
 * lsh_adjoint_batch_gradient then refuses the batch if the members' records
 * no longer stand at the same point of the schedule */
int lsh_adjoint_batch_member(lsh_adjoint_batch* b, int i, lsh_adjoint** out);

/* the checkpoint schedule alone (no device work): the forward steps it takes
 * to reverse nsteps with `slots` slots (its first descent included; the
 * forward run's remaining steps to X_N not) and the optimum
 * r n - beta(s + 1, r - 1); status 0 when every step is reversed once, in
 * order, from the right state */
int lsh_revolve_plan(int nsteps, int slots, long long* forward_steps, long long* optimal);

/* Human-readable text for a status code. */
const char* lsh_status_string(int status);

/* Last CUDA error text recorded by the library (thread-local). */
const char* lsh_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* LSH_H */
