#!/usr/bin/env python
"""Headline benchmark: FP64 cell-updates/s of the two-layer time step on the
2048 x 2048 second-order (MUSCL + TVD-RK2) spherical fjord (0.0002 degree
cells at 60 N, 2e7 m^3 slide), synthetic seeded input.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one full time step of the whole grid (both RK stages).  Timed on
the device with CUDA events around exactly K steps (one CUDA graph launch per
16 steps), barrier + synchronize on both sides, max over ranks.  Inputs are
larger than L2 (state + accumulators + slopes ~ 1 GB), so no flush is needed.
N > 1 runs independent replicas, one per GPU (the time step has no
cross-replica exchange; the reference's MPI row decomposition is out of scope),
so scaling is weak and `value` sums all ranks' cell-updates.

--impl reference times the reference scheme on the host cores instead: the
FP64 CPU restatement in oracle/ (the reference's own CPU-side code has no
time step -- its solver exists only as CUDA kernels), all host threads, the
same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FP64 cell-updates/s at 2048^2"
UNIT = "cell-updates/s"
MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
# FP64 operations per cell-update of the 2048^2 fjord step as the reference
# scheme performs them (no dry or single-layer shortcuts), counted by running
# the FP64 oracle on an operation-counting scalar (oracle/count.h); an FMA
# counts 2, a division, square root, exp or cube root 1.  Comparisons (171
# per cell-update) are not counted.  tests/test_oracle_opcount.py recomputes it.
FJORD2048_FLOPS_PER_CELL_STEP = 804.0

# Counters of the step kernels on the 2048^2 fjord, read from ncu captures
# (one step inside the timed range: the first step after the 20 warm-up steps):
#   ncu --clock-control none --metrics sm__thread_inst_executed_pipe_fp64_pred_on.sum,\
#       sm__pipe_fp64_cycles_active.sum,sm__cycles_elapsed.sum,\
#       dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum \
#       -k regex:"k_edges|k_volume|k_recon" -s 240 -c 12 \
#       python bench.py --steps 2 --warmup 20 --no-cpu-baseline --no-e2e
# They hold only for the kernel sources and the workload generator they were
# captured on.  Those files are hashed (COUNTER_SOURCES); when the hash is not
# COUNTERS_SOURCE_HASH the bench prints null for every figure derived from
# them until a new capture replaces the numbers and the hash.
COUNTER_SOURCES = ("landslidehysea_gb300/csrc/lsh_core.cu", "landslidehysea_gb300/csrc/lsh_kernels.cuh",
                   "landslidehysea_gb300/csrc/lsh_passes.cuh", "landslidehysea_gb300/csrc/lsh_scheme.cuh",
                   "landslidehysea_gb300/csrc/lsh_fpmath.h", "landslidehysea_gb300/csrc/lsh_setup.h",
                   "landslidehysea_gb300/build.py", "landslidehysea_gb300/scenarios.py")
COUNTERS_SOURCE_HASH = "032c79f00d393a67"
# FP64-pipe thread instructions per cell-update of one step (6.060e8 per step
# / 4,194,304 cells).  The FP64 pipe takes one such instruction per lane as
# the measured peak's DFMA does, so the peak instruction rate is the measured
# FP64 FLOP/s / 2.
FJORD2048_FP64_INSTR_PER_CELL_STEP = 144.49
# DRAM bytes (read + write) per launch of each step kernel; edge_h0 is the
# first (accumulator-writing) horizontal pass.  A second-order step launches
# recon and the four edge passes twice, each volume kernel once.
FJORD2048_DRAM_BYTES_PER_LAUNCH = {
    "recon": 139.65e6, "edge_h0": 356.35e6, "edge_h1": 170.95e6, "edge_v0": 170.5e6, "edge_v1": 167.4e6,
    "volume1": 651.1e6, "volume2": 699.1e6,
}
# Algorithmic HBM bytes per cell-step (FP64 state with perfect reuse): first
# order 13 x 8 = 104 B (read 6 state + H, write 6 state); TVD-RK2 104 B for
# stage 1 plus 152 B for stage 2 (read 6 + H + the step's initial 6, write 6).
ALGO_BYTES_PER_CELL_STEP = {1: 104, 2: 256}


def source_hash(paths=COUNTER_SOURCES):
    """Short SHA-256 of the files the ncu counters depend on."""
    import hashlib
    h = hashlib.sha256()
    for rel in paths:
        with open(os.path.join(ROOT, rel), "rb") as f:
            h.update(rel.encode() + b"\0" + f.read())
    return h.hexdigest()[:16]


def counters_current():
    return source_hash() == COUNTERS_SOURCE_HASH


def step_dram_bytes():
    """DRAM bytes of one second-order step from the per-launch counters."""
    d = FJORD2048_DRAM_BYTES_PER_LAUNCH
    return 2 * (d["recon"] + d["edge_h0"] + d["edge_h1"] + d["edge_v0"] + d["edge_v1"]) + d["volume1"] + d["volume2"]


def edge_dram_bytes():
    d = FJORD2048_DRAM_BYTES_PER_LAUNCH
    return 2 * (d["edge_h0"] + d["edge_h1"] + d["edge_v0"] + d["edge_v1"])


def flops_per_cell_step(ops):
    """FP64 flops from an operation count by kind (FMA = 2)."""
    return (ops["add"] + ops["mul"] + 2 * ops["fma"] + ops["div"] + ops["sqrt"] + ops["exp"] + ops["cbrt"]
            + ops["pow"])
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=48)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--ref-build", choices=("cpu", "cuda"), default="cpu",
                    help="--impl reference: the FP64 CPU restatement (cpu, the reference arm) or the reference's own "
                         "CUDA kernels compiled for this GPU (cuda: FP32, first order, Cartesian shelf of --n)")
    ap.add_argument("--n", type=int, default=2048, help="grid size (n x n); the headline is 2048")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", choices=("fjord", "shelf", "ensemble", "adjoint", "adjoint-batch", "adjoint-fd"),
                    default="fjord",
                    help="fjord: the 2048^2 headline; ensemble: the batched 256-scenario ensemble vs serial; "
                         "adjoint: gradient of the 16-gauge misfit on the 1024^2 fjord vs its forward")
    ap.add_argument("--adj-n", type=int, default=1024, help="adjoint workload grid size")
    ap.add_argument("--adj-steps", type=int, default=4000, help="adjoint workload steps")
    ap.add_argument("--adj-budget-gb", type=float, default=None, help="checkpoint budget (default 180 GB or free)")
    ap.add_argument("--adj-thin", type=float, default=0.1,
                    help="thin-layer projection of the adjoint, metres (0: the exact adjoint)")
    ap.add_argument("--fd-steps", type=int, default=500, help="adjoint-fd workload steps")
    ap.add_argument("--vmax", type=float, default=0.0,
                    help="adjoint and adjoint-fd workloads: speed caps vmax1 = vmax2 in m/s (0: off, as configured)")
    ap.add_argument("--fd-rels", default="1e-2,1e-3,1e-4,1e-5,1e-6",
                    help="adjoint-fd relative difference steps (the last is the reference)")
    ap.add_argument("--count", type=int, default=256, help="ensemble scenarios")
    ap.add_argument("--ens-sizes", default="128,256,512,768",
                    help="ensemble: grid sizes the scenarios are drawn from (one size: a uniform ensemble)")
    ap.add_argument("--ens-kind", choices=("shelf", "fjord"), default="shelf",
                    help="ensemble: the 200^2 shelf generator at each size (the 256-scenario ensemble) or the fjord generator")
    ap.add_argument("--cal-count", type=int, default=64, help="batched-adjoint scenarios")
    ap.add_argument("--cal-steps", type=int, default=300, help="batched-adjoint steps (the full calibration: 3000)")
    ap.add_argument("--cal-serial", type=int, default=1, help="also run the members one by one (1) or not (0)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, dist, device):
    """The largest of every rank's x (timings: the job ends with its slowest rank)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, units_per_rank, seconds):
    """Units per second of the whole job: every rank's units over the slowest rank's time."""
    return world * units_per_rank / seconds


def shard(count, rank, world):
    """Scenario ids of one rank when an ensemble is split over `world` GPUs:
    round-robin, so sizes drawn at random balance across ranks."""
    return list(range(rank, count, world))


def init_dist(world, local, backend):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def workload(n, kind="fjord"):
    """fjord: the headline second-order spherical fjord; shelf: the plain
    method's first-order Cartesian shelf (25 m cells, walls), at n x n."""
    from landslidehysea_gb300 import scenarios
    return scenarios.shelf(n=n) if kind == "shelf" else scenarios.fjord(n=n)


def config_dict(sc, n, extra=None):
    if sc.params.order == 1:
        d = {"workload": f"shelf{n}x{n}_order1_cartesian", "grid": [n, n], "cells": n * n, "order": 1,
             "coords": "cartesian", "dx_m": sc.params.dx, "seed": 0, "cfl": sc.params.cfl,
             "l2": "inputs larger than L2" if n * n * 8 * 21 > 129e6 else "inputs smaller than L2",
             "parallelism": "replicas"}
    else:
        d = {"workload": f"fjord{n}x{n}_order2_spherical", "grid": [n, n], "cells": n * n, "order": 2,
             "coords": "spherical", "cell_deg": 0.0002, "lat_c": 60.0, "slide_m3": 2e7, "seed": 0,
             "wet_fraction": round(sc.meta["wet_fraction"], 4), "cfl": sc.params.cfl,
             "l2": "inputs larger than L2 (state+accumulators+slopes ~1 GB)", "parallelism": "replicas"}
    if extra:
        d.update(extra)
    return d


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        exe = shutil.which("nvidia-smi")
        if exe:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen([exe, f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.idx), "-lms", "200", "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        with open(MEASURED_PEAKS) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def algorithmic_bytes_per_launch(kernel_index, order, cells):
    """Bytes one launch of kernel `kernel_index` of a step must move (8-byte
    doubles), from the kernel's dataflow: each edge pass touches every cell
    once, reading its state (7) and, at second order, the 7 slopes of the
    pass direction, plus a read-modify-write of its 7 accumulators (the first
    pass only writes them)."""
    d = 8
    if order == 2:
        names = ["recon", "edge_h0", "edge_h1", "edge_v0", "edge_v1", "volume1",
                 "recon", "edge_h0", "edge_h1", "edge_v0", "edge_v1", "volume2", "clock"]
        per = {"recon": 7 + 14, "edge_h0": 14 + 7, "edge_h1": 14 + 14, "edge_v0": 14 + 14, "edge_v1": 14 + 14,
               "volume1": 7 + 7 + 4 + 6, "volume2": 6 + 1 + 7 + 4 + 6 + 6, "clock": 0}
    else:
        names = ["edge_h0", "edge_h1", "edge_v0", "edge_v1", "volume", "clock"]
        per = {"edge_h0": 7 + 7, "edge_h1": 7 + 14, "edge_v0": 7 + 14, "edge_v1": 7 + 14, "volume": 7 + 7 + 6,
               "clock": 0}
    nm = names[kernel_index]
    return nm, per[nm] * d * cells


def _oracle(threads):
    """The FP64 CPU oracle with `threads` OpenMP threads (0: every host core)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    used = pyoracle.set_threads(threads if threads > 0 else (os.cpu_count() or 1))
    return pyoracle, used


def time_oracle(sc, steps, warmup, threads=0):
    """Cell-updates/s of the oracle on scenario `sc`: `warmup` untimed steps
    from t = 0, then `steps` timed ones."""
    pyoracle, used = _oracle(threads)
    arrs = pyoracle.state_arrays(sc.state)
    t, dt, _ = pyoracle.run(sc.params, arrs, warmup) if warmup else (0.0, pyoracle.initial_dt(sc.params, arrs), 0)
    t0 = time.perf_counter()
    pyoracle.run(sc.params, arrs, steps, t=t, dt=dt)
    el = time.perf_counter() - t0
    return sc.nx * sc.ny * steps / el, used, el


def cpu_baseline(sc, n):
    """The bounded CPU baseline of the default run (about 40 s on 16 cores):
    the bench workload itself for 100 steps after 2 warm-up steps on every
    host core; beside it the 200^2 first-order shelf of the plain method for
    its full 1000 steps on every core and on one core (the serial
    transcription)."""
    from landslidehysea_gb300 import scenarios
    v, used, el = time_oracle(sc, 100, 2)
    c0 = scenarios.shelf(n=200)
    v0, used0, el0 = time_oracle(c0, 1000, 0)
    v1, _, el1 = time_oracle(c0, 1000, 0, threads=1)
    _oracle(0)
    return {"value": v, "unit": UNIT, "cores": used, "kind": "port",
            "sample": f"100 steps of the {n}^2 workload after 2 warm-up steps ({el:.1f} s), FP64 oracle on "
                      f"{used} threads",
            "shelf200_order1_1000_steps": {"value": v0, "cores": used0, "seconds": round(el0, 2)},
            "shelf200_order1_serial_1000_steps": {"value": v1, "cores": 1, "seconds": round(el1, 2)}}


def run_reference_cuda(args):
    """The reference's own CUDA build on this GPU: its unmodified kernel
    sources compiled for sm_103a (oracle/build_ref.sh, through a shim for the
    removed texture API) and driven through one rank's shallowWater() step
    sequence (oracle/ref_cuda_driver.cpp), FP32, on the first-order Cartesian
    shelf of --n (its native scheme).  Timed by wall clock over --steps
    after --warmup steps, as the reference times its loop (MPI_Wtime).
    `check_one_step` compares one step from the initial state with the FP64
    oracle: the depths (relative to their scale) and dt agree to FP32
    rounding.  Over many steps the FP32 state departs from FP64 on these
    inputs (a slide at its Coulomb threshold, 1e-5 m dry threshold under
    100 m of water): the host build of the same sources does the same."""
    import numpy as np
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    if not pyoracle.ref_cuda_available():
        print(json.dumps({"impl": "reference", "unavailable": "the reference CUDA build (oracle/_ref) is absent: "
                                                              "its cubin is compiled where the reference sources are"}))
        return 0
    sc = workload(args.n, "shelf")
    steps, warm = max(1, args.steps), max(1, args.warmup)
    try:
        one, trace1, _, _ = pyoracle.ref_cuda_run(sc.params, sc.state, 0, 1, device=local)
        arrs, trace, t, ms = pyoracle.ref_cuda_run(sc.params, sc.state, warm, steps, device=local)
    except RuntimeError as e:
        print(json.dumps({"impl": "reference", "unavailable": str(e)}))
        return 0
    value = sc.nx * sc.ny * steps / (ms * 1e-3)
    pyoracle.set_threads(os.cpu_count() or 1)
    o = pyoracle.state_arrays(sc.state)
    dt0 = pyoracle.initial_dt(sc.params, o)
    _, dt1, _ = pyoracle.run(sc.params, o, 1, dt=dt0)
    depth = {}
    for i, v in ((0, "h1"), (3, "h2")):
        scale = max(float(np.abs(o[i]).max()), float(np.abs(sc.state[v]).max()), 1e-30)
        depth[v] = float(np.abs(one[i] - o[i]).max()) / scale
    check = {"depth_rel_of_scale": depth, "dt0_rel": abs(float(trace1[0]) - dt0) / dt0,
             "dt1_rel": abs(float(trace1[1]) - dt1) / dt1}
    line = {"impl": "reference", "build": "reference CUDA kernels (FP32) compiled for sm_103a",
            "metric": f"FP32 cell-updates/s at {args.n}^2, first order (reference CUDA build)", "value": value,
            "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": warm, "ms_per_step": ms / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_dict(sc, args.n, {"runner": "oracle/ref_cuda_driver.cpp + oracle/_ref/ref_kernels.cubin"}),
            "sim_time_s": t, "dt_last": float(trace[-1]), "check_one_step": check}
    print(json.dumps(line), flush=True)
    return 0


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    if args.ref_build == "cuda":
        return run_reference_cuda(args)
    sc = workload(args.n)
    steps, warm = max(1, args.steps), max(1, args.warmup)
    value, threads, el = time_oracle(sc, steps, warm)
    sample = f"{steps} full steps of the {args.n}^2 grid after {warm} warm-up steps ({el:.1f} s)"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
            "warmup": warm, "ms_per_step": 1e3 * el / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(sc, args.n, {"runner": "FP64 CPU restatement of the reference scheme (oracle/)"}),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    import torch

    rank, world, local = dist_env()
    dist = init_dist(world, local, "nccl")
    torch.cuda.set_device(local)
    from landslidehysea_gb300 import build as B
    if rank == 0 or world == 1:
        B.build()
    if dist:
        dist.barrier()
    from landslidehysea_gb300._abi import VARS
    from landslidehysea_gb300.solver import Solver, probe_fp64_peak

    sc = workload(args.n, args.workload)
    cells = sc.nx * sc.ny
    # a dedicated (non-legacy) stream shared by the library and the timing events
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    assert stream.cuda_stream != 0
    s = Solver(sc.params, device=local)
    s.set_stream(stream.cuda_stream)
    s.set_state(sc.state)
    s.step(args.warmup)
    s.synchronize()

    def barrier():
        if dist:
            dist.barrier()

    launches0 = s.launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        s.step(args.steps)
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
    ms = ev0.elapsed_time(ev1)
    launches = s.launch_count() - launches0
    s.synchronize()
    t_sim, dt_next, nsteps = s.time()
    ms = max_over_ranks(ms, dist, "cuda")
    value = whole_job_rate(world, cells * args.steps, ms * 1e-3)

    # per-kernel event timing of a few extra steps (the step's kernel families)
    prof = [s.profile_step() for _ in range(3)]
    nk = len(prof[0])
    mean = [statistics.mean(p[k] for p in prof) for k in range(nk)]
    order = sc.params.order
    names_ms = {}
    for k in range(nk):
        nm, _ = algorithmic_bytes_per_launch(k, order, cells)
        names_ms.setdefault(nm, []).append(mean[k])
    hbm, peak_kind = peaks()
    try:
        fp64_peak = probe_fp64_peak(local)
    except Exception:
        fp64_peak = None
    current = counters_current() and args.n == 2048 and args.workload == "fjord"
    ms_step = ms / args.steps
    rate = value / world
    fp64 = None
    if fp64_peak:
        peak_i = fp64_peak / 2.0
        ach = FJORD2048_FP64_INSTR_PER_CELL_STEP * rate / 1e9 if current else None
        fp64 = {"bound": "fp64", "achieved": round(ach, 1) if current else None, "peak": round(peak_i, 1),
                "unit": "G FP64 instr/s", "frac": round(ach / peak_i, 4) if current else None,
                "instr_per_cell_step": FJORD2048_FP64_INSTR_PER_CELL_STEP if current else None,
                "counters_source_hash": source_hash(), "counters_current": current,
                "what": "FP64-pipe thread instructions the step kernels execute per cell-update (ncu count on "
                        "this workload, valid for the hashed kernel sources only) x cell-updates/s, over the "
                        "measured FP64 instruction rate (lsh_probe_fp64_peak DFMA GFLOP/s / 2)",
                "scheme_gflops": round(FJORD2048_FLOPS_PER_CELL_STEP * rate / 1e9, 1)
                if args.n == 2048 and args.workload == "fjord" else None,
                "scheme_flops_per_cell_step": FJORD2048_FLOPS_PER_CELL_STEP,
                "scheme_note": "the reference scheme's FP64 operations (oracle count, FMA = 2) at this rate; "
                               "the kernels skip exact-zero work on dry cells and single-layer edges, so this "
                               "can exceed the FLOP peak"}
    # the HBM roofline of the step: the algorithmic bytes per cell-step (FP64
    # state with perfect reuse) over the step time, against the measured copy
    # bandwidth; traffic is what ncu measured the step's launches move
    algo = ALGO_BYTES_PER_CELL_STEP[order] * cells
    achieved = algo / (ms_step * 1e-3) / 1e9
    edge_ms = sum(sum(v) for k, v in names_ms.items() if k.startswith("edge"))
    all_ms = sum(mean)
    edge_traffic = edge_dram_bytes() if current else None
    roofline = {"bound": "hbm", "kernel": f"whole step ({nk} launches)", "achieved": round(achieved, 2),
                "peak": hbm, "unit": "GB/s", "frac": round(achieved / hbm, 5),
                "traffic": step_dram_bytes() if current else None,
                "algorithmic_bytes": algo, "algorithmic_bytes_per_cell_step": ALGO_BYTES_PER_CELL_STEP[order],
                "peak_kind": f"{peak_kind} hbm_gbs",
                "dominant_family": {
                    "kernels": "k_edges_h / k_edges_v (4 colour passes per stage)",
                    "launches_per_step": sum(1 for k in names_ms for _ in names_ms[k] if k.startswith("edge")),
                    "share_of_step": round(edge_ms / all_ms, 4), "ms_per_step": round(edge_ms, 4),
                    "dram_bytes_per_step": edge_traffic,
                    "dram_gbs": round(edge_traffic / (edge_ms * 1e-3) / 1e9, 1) if current else None,
                    "dram_frac": round(edge_traffic / (edge_ms * 1e-3) / 1e9 / hbm, 4) if current else None},
                "step_kernel_ms": {k: round(statistics.mean(v), 4) for k, v in names_ms.items()},
                "fp64_peak_gflops_measured": round(fp64_peak, 1) if fp64_peak else None,
                "counters_current": current,
                "note": "the step is bound by the FP64 pipe (fp64_roofline), not by HBM"}
    s.close()

    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(sc, local, args, torch, np, VARS, Solver, dist)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(sc, args.n)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config_dict(sc, args.n, {"sim_time_s": t_sim, "dt_s": dt_next}),
                "bound": "fp64", "roofline": roofline, "fp64_roofline": fp64, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": launches,
                "clocks": clk.summary()}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def measure_e2e(sc, local, args, torch, np, VARS, Solver, dist):
    """The same metric through the C ABI with HOST buffers: upload the state
    from pinned host memory (lsh_set_state), then per step one lsh_step and a
    blocking read of the step's result (t, dt: lsh_get_time, as the
    reference reads dt back every step), then download the state
    (lsh_get_state), all inside the timed region."""
    cells = sc.nx * sc.ny
    pinned = {}
    for v in VARS:
        t = torch.empty((sc.ny, sc.nx), dtype=torch.float64, pin_memory=True)
        t.numpy()[...] = sc.state[v]
        pinned[v] = t
    host_in = {v: pinned[v].numpy() for v in VARS}
    # the result lands in pinned buffers too, allocated once like the inputs
    host_out = {v: torch.empty((sc.ny, sc.nx), dtype=torch.float64, pin_memory=True).numpy() for v in VARS}
    s = Solver(sc.params, device=local)
    s.set_state(host_in)
    s.step(2)
    s.synchronize()
    if dist:
        dist.barrier()
    steps = args.steps
    t0 = time.perf_counter()
    s.set_state(host_in)
    for _ in range(steps):
        s.step(1)
        s.time()
    s.get_state(host_out)
    el = time.perf_counter() - t0
    s.close()
    el = max_over_ranks(el, dist, "cuda")
    world = dist.get_world_size() if dist else 1
    state_bytes = 7 * cells * 8
    return {"value": whole_job_rate(world, cells * steps, el), "unit": UNIT, "h2d_bytes_per_step": state_bytes / steps,
            "d2h_bytes_per_step": 64 + state_bytes / steps, "seconds": el,
            "what": "lsh_set_state(pinned host) + K x (lsh_step(1) + lsh_get_time) + lsh_get_state(pinned host)"}


def run_ensemble(args):
    """Batched ensemble: `count` second-order shelf scenarios on grids drawn
    from {128, 256, 512, 768}^2 (per-scenario seeds, Coulomb angle, r and
    slide volume), advanced together by the persistent work-queue kernels of
    lsh_batch (autotuned), against the same scenarios stepped one after the
    other with single-grid contexts (each its own CUDA graph).  Both arms run
    the same K steps per scenario from the same state.  With N GPUs the
    scenarios are split round-robin (no collective on the data path), the
    job's time is the slowest rank's and the work is fixed: strong scaling."""
    import torch
    rank, world, local = dist_env()
    dist = init_dist(world, local, "nccl")
    torch.cuda.set_device(local)
    from landslidehysea_gb300 import build as B
    if rank == 0 or world == 1:
        B.build()
    if dist:
        dist.barrier()
    from landslidehysea_gb300 import scenarios
    from landslidehysea_gb300.solver import Batch, Solver
    ids = shard(args.count, rank, world)
    sizes = tuple(int(x) for x in args.ens_sizes.split(","))

    def members(ks):
        if args.ens_kind == "fjord":
            return [scenarios.fjord(n=sizes[k % len(sizes)], seed=k) for k in ks]
        return scenarios.ensemble(args.count, sizes=sizes, ids=list(ks))

    scs = members(ids)
    all_cells = sum(s_.nx * s_.ny for s_ in members(range(args.count))) if world > 1 else \
        sum(s_.nx * s_.ny for s_ in scs)

    def barrier():
        if dist:
            dist.barrier()

    b = Batch([sc.params for sc in scs], device=local)
    for k, sc in enumerate(scs):
        b.set_state(k, sc.state)
    tune = b.autotune(trial_steps=4)
    b.step(args.warmup)
    b.synchronize()
    done_before = b.time(0)[2]
    launches0 = b.launch_count()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        barrier()
        t0 = time.perf_counter()
        b.step(args.steps)
        b.synchronize()
        el = time.perf_counter() - t0
        barrier()
    launches = b.launch_count() - launches0
    b.close()
    el = max_over_ranks(el, dist, "cuda")
    value = all_cells * args.steps / el

    # serial: the same scenarios, one context at a time, K steps each after
    # the same number of earlier steps; CUDA events on the solver's stream
    stream = torch.cuda.Stream()
    serial_ms = 0.0
    for sc in scs:
        with Solver(sc.params, device=local) as s:
            s.set_stream(stream.cuda_stream)
            s.set_state(sc.state)
            s.step(done_before)
            s.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.step(args.steps)
            e1.record(stream)
            e1.synchronize()
            serial_ms += e0.elapsed_time(e1)
    serial_ms = max_over_ranks(serial_ms, dist, "cuda")
    serial = all_cells * args.steps / (serial_ms * 1e-3)
    sizes = {}
    for sc in scs:
        sizes[sc.nx] = sizes.get(sc.nx, 0) + 1
    if rank == 0:
        line = {"metric": "FP64 cell-updates/s, batched ensemble", "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
                "higher_is_better": True, "scaling": "strong" if world > 1 else "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic",
                "config": {"workload": f"ensemble{args.count}_{args.ens_kind}_order2", "scenarios": args.count,
                           "sizes": list(sizes),
                           "grids_rank0": {str(k): v for k, v in sorted(sizes.items())}, "cells": all_cells,
                           "order": 2, "split": "round-robin over ranks" if world > 1 else None,
                           "l2": f"inputs larger than L2 (~{all_cells * 36 * 8 / 1e9 / world:.0f} GB per GPU)"},
                "serial": {"value": serial, "ms_per_step": serial_ms / args.steps,
                           "what": "each scenario alone through lsh_create/lsh_step (16-step CUDA graphs)"},
                "batched_vs_serial": value / serial, "tune": tune, "gpu_launches": launches,
                "clocks": clk.summary()}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def run_adjoint(args):
    """Adjoint workload: the 16-gauge misfit of an N-step run of the n^2
    second-order spherical fjord against a twin run whose Coulomb angle,
    Manning coefficients and density ratio are perturbed by seeded +-5%;
    gradient with respect to the initial h2 field and (angle1, mf0, mfs, r).
    `value` is the wall time of lsh_adjoint_gradient (the reverse sweep with
    all recomputation) over that of the same N steps through lsh_step (the
    product's forward, CUDA graphs); `total_ratio` adds lsh_adjoint_forward
    (the recorded forward run with its gauge series and checkpoints)."""
    import copy
    import numpy as np
    import torch
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    from landslidehysea_gb300 import build as B
    B.build()
    from landslidehysea_gb300 import scenarios
    from landslidehysea_gb300.solver import Adjoint, Solver
    sc = scenarios.fjord(n=args.adj_n)
    p = sc.params
    if args.vmax > 0:
        p.vmax1 = p.vmax2 = args.vmax
    ij = [(int(i), int(j)) for i, j in sc.gauges if i >= 0 and j >= 0]
    gauges = np.array([j * p.nx + i for i, j in ij], dtype=np.int32)
    nsteps = args.adj_steps
    rng = np.random.default_rng(2024)
    twin = copy.copy(p)
    f = 1.0 + 0.05 * rng.choice([-1.0, 1.0], 4)
    twin.angle1, twin.mf0, twin.mfs, twin.r = p.angle1 * f[0], p.mf0 * f[1], p.mfs * f[2], p.r * f[3]
    with Adjoint(twin, gauges) as T:
        T.set_budget(0.0 + 6 * 8 * (p.nx * p.ny + 32) + 1.0)
        _, target = T.forward(sc.state, nsteps)
    # the forward alone: N steps through lsh_step
    s = Solver(p, device=local)
    s.set_state(sc.state)
    s.synchronize()
    t0 = time.perf_counter()
    s.step(nsteps)
    s.synchronize()
    t_fwd = time.perf_counter() - t0
    s.close()
    with Adjoint(p, gauges, device=local) as A:
        if args.adj_budget_gb is not None:
            A.set_budget(args.adj_budget_gb * 1e9)
        A.set_thin_layer(args.adj_thin)
        with ClockSampler(local) as clk:
            t0 = time.perf_counter()
            J, _ = A.forward(sc.state, nsteps, target)
            t1 = time.perf_counter()
            g, gp = A.gradient()
            t2 = time.perf_counter()
        st = A.stats()
    ratio = (t2 - t1) / t_fwd
    line = {"metric": "adjoint/forward wall time, 16-gauge misfit gradient", "value": ratio, "unit": "x",
            "n_gpus": 1, "steps": nsteps, "warmup": 0, "ms_per_step": 1e3 * (t2 - t0) / nsteps,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"fjord{args.adj_n}x{args.adj_n}_order2_spherical_adjoint", "steps": nsteps,
                       "gauges": int(gauges.size), "twin_perturbation": [float(x) for x in f],
                       "thin_layer_m": args.adj_thin,
                       "gradient": ["h2 field", "angle1", "mf0", "mfs", "r"]},
            "value_is": "lsh_adjoint_gradient wall time (reverse sweep, checkpoint recomputation and the per-step "
                        "recomputation included) / N steps of lsh_step",
            "total_ratio": (t2 - t0) / t_fwd,
            "forward_s": t_fwd, "adjoint_forward_s": t1 - t0, "adjoint_gradient_s": t2 - t1, "misfit": J,
            "grad_params": gp, "grad_h2_l2": float(np.linalg.norm(g["h2"])), "stats": st,
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def twin_target(p, state, gauges, nsteps, seed=2024):
    """The adjoint workload's calibration target: the gauge series of a twin
    run whose (angle1, mf0, mfs, r) are scaled by seeded +-5%."""
    import copy
    import numpy as np
    from landslidehysea_gb300.solver import Adjoint
    rng = np.random.default_rng(seed)
    twin = copy.copy(p)
    f = 1.0 + 0.05 * rng.choice([-1.0, 1.0], 4)
    twin.angle1, twin.mf0, twin.mfs, twin.r = p.angle1 * f[0], p.mf0 * f[1], p.mfs * f[2], p.r * f[3]
    with Adjoint(twin, gauges) as T:
        T.set_budget(0.0 + 6 * 8 * (p.nx * p.ny + 32) + 1.0)
        _, target = T.forward(state, nsteps)
    return target, f


def run_adjoint_fd(args):
    """Finite-difference check of the adjoint workload's parameter gradient:
    the 16-gauge misfit J of an N-step run of the n^2 second-order fjord
    against its twin's gauge series (as --workload adjoint), differentiated
    with respect to (angle1, mf0, mfs, r) by lsh_adjoint_gradient -- the
    exact discrete adjoint (thin-layer projection 0) and the projected one
    (--adj-thin) -- and by FP64 central differences of J itself,
    (J(p + d e_k) - J(p - d e_k)) / 2d, at relative steps d / |p_k| of
    --fd-rels (default 1e-2 ... 1e-6).  Prints the gradients, the
    differences and their relative gaps; `value` is the projected gradient's
    largest relative gap to the difference at the last step.  `roughness`
    holds J and the simulated time after the N steps at angle1 (1 + k 1e-7),
    k = -3..3: a discrete branch switch (the CFL step's arg-max cell, a speed
    cap) shows there as a jump that no finite difference can resolve."""
    import copy
    import numpy as np
    import torch
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    from landslidehysea_gb300 import build as B
    B.build()
    from landslidehysea_gb300 import scenarios
    from landslidehysea_gb300.solver import Adjoint
    sc = scenarios.fjord(n=args.adj_n)
    p = sc.params
    if args.vmax > 0:
        p.vmax1 = p.vmax2 = args.vmax
    gauges = scenarios.gauge_cells(sc)
    n = args.fd_steps
    target, f = twin_target(p, sc.state, gauges, n)
    names = ("angle1", "mf0", "mfs", "r")
    slot = 6 * 8 * (p.nx * p.ny + 32)

    def misfit(q, with_time=False):
        with Adjoint(q, gauges, device=local) as A:
            A.set_budget(slot + 1.0)
            J, _ = A.forward(sc.state, n, target)
            t_end = float(A.times()[-1])
        return (J, t_end) if with_time else J

    t0 = time.perf_counter()
    grads = {}
    for label, thin in (("exact", 0.0), ("projected", args.adj_thin)):
        with Adjoint(p, gauges, device=local) as A:
            if thin:
                A.set_thin_layer(thin)
            J0, _ = A.forward(sc.state, n, target)
            _, gp = A.gradient()
        grads[label] = {k: gp[k] for k in names}
    rels = [float(x) for x in args.fd_rels.split(",")]
    fd = {}
    for k in names:
        base = getattr(p, k)
        fd[k] = {}
        for rel in rels:
            d = rel * abs(base)
            qp, qm = copy.copy(p), copy.copy(p)
            setattr(qp, k, base + d)
            setattr(qm, k, base - d)
            fd[k][f"{rel:g}"] = (misfit(qp) - misfit(qm)) / (2.0 * d)
    rough = []
    for k in range(-3, 4):
        q = copy.copy(p)
        q.angle1 = p.angle1 * (1.0 + k * 1e-7)
        J, t_end = misfit(q, with_time=True)
        rough.append({"k": k, "J": J, "t_end": t_end})
    el = time.perf_counter() - t0

    def gap(g, ref):
        return abs(g - ref) / abs(ref) if ref != 0.0 else None

    report = {}
    for k in names:
        ref = fd[k][f"{rels[-1]:g}"]
        report[k] = {"exact": grads["exact"][k], "projected": grads["projected"][k], "fd": fd[k],
                     "gap_exact": gap(grads["exact"][k], ref), "gap_projected": gap(grads["projected"][k], ref),
                     "fd_spread": max(gap(v, ref) or 0.0 for v in fd[k].values())}
    gaps = [report[k]["gap_projected"] for k in names if report[k]["gap_projected"] is not None]
    line = {"metric": "adjoint parameter gradient vs FP64 central differences (largest relative gap, projected)",
            "value": max(gaps) if gaps else None, "unit": "relative", "n_gpus": 1, "steps": n, "warmup": 0,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"fjord{args.adj_n}x{args.adj_n}_order2_spherical_adjoint_fd", "steps": n,
                       "gauges": int(gauges.size), "twin_perturbation": [float(x) for x in f],
                       "thin_layer_m": args.adj_thin, "fd_relative_steps": rels, "vmax_mps": args.vmax},
            "misfit": J0, "parameters": report, "roughness": rough, "seconds": el}
    print(json.dumps(line), flush=True)
    return 0


def run_adjoint_batch(args):
    """Batched adjoint calibration: `cal_count` fjord scenarios on grids drawn
    from 256^2 .. 1024^2 (seed = scenario id), each with the 16-gauge misfit
    against its twin run (Coulomb angle, Manning coefficients and density
    ratio scaled by seeded +-5%), run forward and reversed together under one
    checkpoint schedule with a joint budget (default 180 GB or free memory).
    `value` is cell-steps of all scenarios over the wall time of
    lsh_adjoint_batch_forward + lsh_adjoint_batch_gradient; `serial` runs the
    same members one after another through lsh_adjoint_forward / _gradient
    with the same slot count, and must give the same gradients bit for bit."""
    import numpy as np
    import torch
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    from landslidehysea_gb300 import build as B
    B.build()
    from landslidehysea_gb300 import scenarios
    from landslidehysea_gb300.solver import AdjointBatch
    nsteps = args.cal_steps
    mem = [scenarios.calibration_member(k) for k in range(args.cal_count)]
    scs = [m[0] for m in mem]
    gauges = [scenarios.gauge_cells(sc) for sc in scs]
    cells = [sc.params.nx * sc.params.ny for sc in scs]
    # the twins' gauge series (one checkpoint slot each: a plain forward run)
    with AdjointBatch([m[1] for m in mem], gauges, device=local) as T:
        T.set_budget(sum(6 * 8 * ((c + 31) // 32 * 32) for c in cells) + 1.0)
        _, targets = T.forward([sc.state for sc in scs], nsteps)
    line = {"metric": "batched adjoint: gradient cell-steps/s (forward + reverse sweep)", "unit": "cell-steps/s",
            "n_gpus": 1, "steps": nsteps, "warmup": 0, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"calibration{args.cal_count}_fjord_order2_spherical_adjoint",
                       "scenarios": args.cal_count, "steps": nsteps,
                       "sizes": {str(n): sum(1 for sc in scs if sc.params.nx == n) for n in scenarios.CALIBRATION_SIZES},
                       "cells": int(sum(cells)), "gauges_per_scenario": 16, "thin_layer_m": args.adj_thin,
                       "gradient": ["h2 field", "angle1", "mf0", "mfs", "r"]}}
    work = float(sum(cells)) * nsteps
    with AdjointBatch([sc.params for sc in scs], gauges, device=local) as A:
        if args.adj_budget_gb is not None:
            A.set_budget(args.adj_budget_gb * 1e9)
        A.set_thin_layer(args.adj_thin)
        with ClockSampler(local) as clk:
            t0 = time.perf_counter()
            J, _ = A.forward([sc.state for sc in scs], nsteps, targets)
            t1 = time.perf_counter()
            _, gp = A.gradient(want_state=True)
            t2 = time.perf_counter()
        st = A.stats()
        line.update({"value": work / (t2 - t0), "ms_per_step": 1e3 * (t2 - t0) / nsteps,
                     "forward_s": t1 - t0, "gradient_s": t2 - t1, "gradient_over_forward": (t2 - t1) / (t1 - t0),
                     "stats": st, "clocks": clk.summary(),
                     "misfit_sum": float(np.sum(J)),
                     "grad_params_first": gp[0]})
        if args.cal_serial:
            same = True
            ts = time.perf_counter()
            for i, sc in enumerate(scs):
                m = A.member(i)
                m.forward(sc.state, nsteps, targets[i])
                _, g1 = m.gradient()
                same = same and g1 == gp[i]
            t_serial = time.perf_counter() - ts
            line["serial"] = {"value": work / t_serial, "seconds": t_serial, "same_gradients": bool(same),
                              "what": "the same members one after another (lsh_adjoint_forward + lsh_adjoint_gradient, "
                                      "the batch's slot count)"}
            line["batched_over_serial"] = t_serial / (t2 - t0)
    line["gpu_launches"] = None
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "ours" and args.workload == "ensemble":
        return run_ensemble(args)
    if args.impl == "ours" and args.workload == "adjoint":
        return run_adjoint(args)
    if args.impl == "ours" and args.workload == "adjoint-batch":
        return run_adjoint_batch(args)
    if args.impl == "ours" and args.workload == "adjoint-fd":
        return run_adjoint_fd(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)  # fjord (the headline) or shelf


if __name__ == "__main__":
    sys.exit(main())
