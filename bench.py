"""Benchmark: SCIDDICA-T debris flow, 2048 x 2048 FP64 cells, von Neumann,
flat boundary, 4000 steps -- one "bench step" is one full 4000-step run from
the seeded initial state (the configuration the headline metric is quoted
on).  Metric: cell-updates per second (rows * cols * CA steps / time).

  value  device-resident: inputs already in HBM (restored from a device
         snapshot, not timed), the 4000 CA steps of each run timed with CUDA
         events on the model's stream; L2 is flushed (256 MiB write) before
         every run
  e2e    the same run through the C API with host buffers: z and h are
         copied from pinned host memory into the model
         (calCopySubstateFromHost2Dr), the program's init and the steps run,
         h is copied back (calCopySubstateToHost2Dr); host timer around each
         run
  roofline  the step (K1 + K2 of the split step): 24 algorithmic bytes per
         cell-update (z read + h read + h write, FP64) / the mean step time
         of the timed runs (CUDA events around each 4000-step run), i.e.
         value x 24 B; the two kernels are also timed one launch at a time
         over 400 steps from step 1000 (at_step_1000)
  cpu_baseline  the CPU port of the reference (oracle/, OpenMP build, all
         host cores) on a bounded sample of the same workload

--impl reference times that CPU port alone, on all host cores, on the same
workload (each bench step = 64 CA steps of the 2048^2 grid from the initial
state); it is the reference's algorithm restated (the reference sources are
not available on the benchmark machine).

With --gpus N > 1 (torchrun) every rank runs an independent replica of the
workload on its own GPU (the model has no cross-grid exchange): weak
scaling, value = all ranks' cell-updates / max time over ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ROWS = COLS = 2048
CA_STEPS = 4000
SEED = 2
P_R, P_EPS = 0.5, 0.001
BYTES_PER_CELL_UPDATE = 24  # z read + h read + h write (FP64)
# FP64 operations of one wet cell-update (5 + up to 5 minimisation
# iterations x (<= 5 adds + 1 division) + 8 of the update; an upper
# estimate of the reference's own operation count per wet cell)
FP64_OPS_PER_WET_CELL = 70
REF_SAMPLE_STEPS = 64
SERIAL_SAMPLE_STEPS = 8  # the 1-core serial comparator's sample (CA steps of the full grid)
# how the 4000 steps are issued: a launch sequence per step, a recorded step
# replayed as a CUDA graph, or one device-driven graph launch for the loop
# or every step in one cooperative launch of the persistent split-step kernel
LOOPS = {"eager": 0, "graph": 1, "device": 2, "persistent": 4}
# The plain step: the split step (K1 + K2 per step) unless
# OPENCAL_SDT_KERNEL selects the sparse fused step (one launch per step) or
# the dense single kernel.  Kernels of ours per CA step and per run: the device loop
# adds its step-count check per step, the persistent loop (split step only)
# is one kernel per run; every run starts with the priming kernel.
STEP_KERNEL = os.environ.get("OPENCAL_SDT_KERNEL", "split")


def launches_per_step(loop):
    if loop == "persistent":
        return 0
    base = 2 if STEP_KERNEL == "split" else 1
    return base + (1 if loop == "device" else 0)


LAUNCHES_PER_RUN = {"eager": 1, "graph": 1, "device": 1, "persistent": 2}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(n_gpus):
    """Rank, world size, local rank and the process group of a torchrun
    launch (one process per GPU, NCCL; gloo on a host without a GPU, which
    the multi-process tests use); (0, 1, 0, None) for a single process."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
        return rank, world, local, dist
    return 0, 1, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x: float) -> float:
    """The largest x of all ranks (the job's time is its slowest rank's)."""
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reference_arm(args):
    """The reference algorithm on the host cores (OpenMP build of the port)."""
    rank, world, _, dist = dist_setup(args.gpus)
    if rank != 0:
        return
    import oracle
    from opencal_gb300 import workloads as W
    oracle.build()
    z, h = W.sciddicaT_inputs(ROWS, COLS, seed=SEED)
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    for _ in range(args.warmup):
        oracle.sciddicaT(z, h, REF_SAMPLE_STEPS, toroidal=False, ac=False, kind="omp", want_cells=False)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.sciddicaT(z, h, REF_SAMPLE_STEPS, toroidal=False, ac=False, kind="omp", want_cells=False)
        times.append(time.perf_counter() - t0)
    units = ROWS * COLS * REF_SAMPLE_STEPS
    value = units * len(times) / sum(times)
    sample = f"{REF_SAMPLE_STEPS} CA steps of the {ROWS}x{COLS} grid from the seeded initial state per bench step"
    line = {
        "metric": "cell_updates_per_s", "value": value, "unit": "cell-updates/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded DEM + source)",
        "config": {"workload": f"SCIDDICA-T {ROWS}x{COLS} FP64, VN, flat, plain (no active cells)",
                   "sample": sample},
        "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_sample(z, h):
    """The oracle on the host: OpenMP build on every core (the reported
    baseline) and the serial build on one core (the serial reference's
    semantics, OpenCAL-OMP/source/cal2DRun.c:125-139 without OpenMP)."""
    import oracle
    oracle.build()
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    oracle.sciddicaT(z, h, REF_SAMPLE_STEPS, toroidal=False, ac=False, kind="omp", want_cells=False)
    dt = time.perf_counter() - t0
    t0 = time.perf_counter()
    oracle.sciddicaT(z, h, SERIAL_SAMPLE_STEPS, toroidal=False, ac=False, kind="serial", want_cells=False)
    ds = time.perf_counter() - t0
    return {"value": ROWS * COLS * REF_SAMPLE_STEPS / dt, "unit": "cell-updates/s", "cores": cores, "kind": "port",
            "sample": f"{REF_SAMPLE_STEPS} CA steps of the {ROWS}x{COLS} grid, OpenMP on all host cores",
            "serial": {"value": ROWS * COLS * SERIAL_SAMPLE_STEPS / ds, "unit": "cell-updates/s", "cores": 1,
                       "kind": "port",
                       "sample": f"{SERIAL_SAMPLE_STEPS} CA steps of the {ROWS}x{COLS} grid, serial build, one "
                                 "core"}}


def gpu_arm(args):
    rank, world, local, dist = dist_setup(args.gpus)
    import opencal_gb300 as cal
    from opencal_gb300 import workloads as W
    cal.build()
    m = cal.models()
    m.cal_sciddicaT_open.restype = C.c_void_p
    m.cal_sciddicaT_open.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                     C.c_void_p, C.c_void_p, C.c_int]
    for fn in ("cal_sciddicaT_reset", "cal_sciddicaT_close", "cal_sciddicaT_stream"):
        getattr(m, fn).argtypes = [C.c_void_p]
    m.cal_sciddicaT_stream.restype = C.c_void_p
    m.cal_sciddicaT_steps.argtypes = [C.c_void_p, C.c_int, C.c_int]
    m.cal_sciddicaT_kernel_times.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    m.cal_sciddicaT_wet_count.argtypes = [C.c_void_p]
    m.cal_sciddicaT_host_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    m.cal_sciddicaT_persist_failed.argtypes = [C.c_void_p]
    m.cal_sciddicaT_read.argtypes = [C.c_void_p, C.c_void_p]
    m.cal_sciddicaT_trace.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    m.cal_fp64_peak.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_float)]

    import torch  # device memory for the L2 flush buffer and events
    torch.cuda.set_device(local)
    z, h = W.sciddicaT_inputs(ROWS, COLS, seed=SEED)
    sess = m.cal_sciddicaT_open(ROWS, COLS, 0, 0, P_R, P_EPS, z.ctypes.data, h.ctypes.data, cal.MODE_FUSED)
    if not sess:
        raise cal.CALError("cal_sciddicaT_open failed: " + cal.core().calGetErrorString().decode())
    stream = torch.cuda.ExternalStream(m.cal_sciddicaT_stream(sess))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def one_run():
        m.cal_sciddicaT_reset(sess)
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            m.cal_sciddicaT_steps(sess, CA_STEPS, LOOPS[args.loop])
            e1.record(stream)
        return e0, e1

    for _ in range(args.warmup):
        e0, e1 = one_run()
        e1.synchronize()

    clocks = ClockSampler(local)
    barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    t_wall0 = time.perf_counter()
    events = [one_run() for _ in range(args.steps)]
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    barrier(dist)
    clk = clocks.stop()
    run_ms = [a.elapsed_time(b) for a, b in events]
    dev_s = max_over_ranks(dist, sum(run_ms) / 1e3)
    units = ROWS * COLS * CA_STEPS * args.steps * world
    value = units / dev_s

    # the step's two kernels timed with events around every launch, over 400
    # steps from the mid-run state (step 1000)
    m.cal_sciddicaT_reset(sess)
    m.cal_sciddicaT_steps(sess, 1000, 0)
    h1000 = np.empty_like(h)
    m.cal_sciddicaT_read(sess, h1000.ctypes.data)
    wet = int(np.count_nonzero(h1000 > P_EPS))
    nk = 400
    ka = (C.c_float * nk)()
    kb = (C.c_float * nk)()
    m.cal_sciddicaT_kernel_times(sess, nk, ka, kb)
    k1_ms, k2_ms = float(np.mean(list(ka))), float(np.mean(list(kb)))
    kavg_ms = k1_ms + k2_ms
    kernel_desc = "SCIDDICA-T step = sdt2::k1_outflows (wet cells) + sdt2::k2_update (flagged tiles)"
    if STEP_KERNEL == "sparse":
        kernel_desc = ("SCIDDICA-T sparse fused step sdt3::k_sparse_step (one launch per step over the flagged "
                       "32x16 tiles, h layers used alternately)")
    elif STEP_KERNEL == "single":
        kernel_desc = "SCIDDICA-T dense fused step sdt::fused_step (every tile every step)"
    if args.loop == "persistent":
        kernel_desc = ("SCIDDICA-T split step, all 4000 steps in one cooperative launch of sdt2::k_persist "
                       "(K1 and K2 phases separated by grid barriers)")
    peak, peak_kind = _peaks()
    # the metric's formula: cell-updates/s of the timed runs x 24 B; per step,
    # the runs' event time / 4000 (launch gaps included)
    step_ms = float(np.mean(run_ms)) / CA_STEPS
    achieved = ROWS * COLS * BYTES_PER_CELL_UPDATE / (step_ms * 1e-3) / 1e9
    achieved_1000 = ROWS * COLS * BYTES_PER_CELL_UPDATE / (kavg_ms * 1e-3) / 1e9

    # end to end through the C API with host buffers
    pin_z = torch.from_numpy(z).pin_memory()
    pin_h = torch.from_numpy(h).pin_memory()
    out = torch.empty_like(pin_h).pin_memory()
    e2e_times = []
    for it in range(max(1, min(args.steps, 3)) + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m.cal_sciddicaT_host_run(sess, pin_z.data_ptr(), pin_h.data_ptr(), CA_STEPS, LOOPS[args.loop],
                                 out.data_ptr())
        t1 = time.perf_counter()
        if it > 0:
            e2e_times.append(t1 - t0)
    e2e_value = ROWS * COLS * CA_STEPS * world / max_over_ranks(dist, float(np.mean(e2e_times)))

    # correctness guard on the timed path: a run in the timed mode is finite,
    # no grid barrier gave up, and it equals, bit for bit, the end-to-end run
    # and a run with one launch sequence per step
    m.cal_sciddicaT_reset(sess)
    m.cal_sciddicaT_steps(sess, CA_STEPS, LOOPS[args.loop])
    barrier_failed = m.cal_sciddicaT_persist_failed(sess) if args.loop == "persistent" else 0
    hh = np.empty_like(h)
    m.cal_sciddicaT_read(sess, hh.ctypes.data)
    m.cal_sciddicaT_reset(sess)
    m.cal_sciddicaT_steps(sess, CA_STEPS, 0)
    he = np.empty_like(h)
    m.cal_sciddicaT_read(sess, he.ctypes.data)
    # the boundary trace (not timed): one split step at a time with a trace
    # kernel after each -- the first step at which the two-cell edge band is
    # wet, the mass leaving through the flat boundary per step, the wet cells
    # of every step
    m.cal_sciddicaT_reset(sess)
    outflux = np.zeros(CA_STEPS)
    wet_steps = np.zeros(CA_STEPS, np.int32)
    edge = C.c_int(-1)
    trace_rc = m.cal_sciddicaT_trace(sess, CA_STEPS, outflux.ctypes.data, wet_steps.ctypes.data, C.byref(edge))
    ht = np.empty_like(h)
    m.cal_sciddicaT_read(sess, ht.ctypes.data)
    m.cal_sciddicaT_close(sess)
    consistent = (bool(hh.tobytes() == he.tobytes() == out.numpy().tobytes() == ht.tobytes()) and not barrier_failed
                  and trace_rc == 0)
    import math
    mass0 = math.fsum(h.ravel())
    mass_t = math.fsum(hh.ravel())
    out_total = math.fsum(outflux)
    boundary = {
        "edge_reached_step": int(edge.value),
        "mass0": mass0, "mass_final": mass_t, "mass_out_through_boundary": out_total,
        "mass_balance_rel": (mass0 - out_total - mass_t) / mass0,
        "how": "split step one launch pair at a time with a trace kernel after each (not timed): first step "
               "after which a cell of the two-cell edge band holds h != 0; the outflows of border cells towards "
               "absent neighbours summed per step; balance = (M0 - outflux - M_T) / M0 with exactly rounded sums",
    }
    wet_total = int(wet_steps.astype(np.int64).sum())
    parity = None
    gpath = os.path.join(ROOT, "tests", "golden", "sciddicaT_2048.json")
    if os.path.exists(gpath):
        import hashlib
        with open(gpath) as f:
            gold = json.load(f)
        parity = {"oracle_h_sha256_equal": hashlib.sha256(hh.tobytes()).hexdigest() == gold["plain"]["h_sha256"],
                  "oracle_edge_step_equal": int(edge.value) == gold["plain"]["edge_step"],
                  "fixture": "tests/golden/sciddicaT_2048.json (oracle, OpenMP build, same inputs)"}
    # measured FP64 throughput (DADD and DFMA instructions per second)
    fp64 = {}
    for name, op in (("dadd", 1), ("dfma", 0)):
        rate, tms = C.c_double(0.0), C.c_float(0.0)
        if m.cal_fp64_peak(op, C.byref(rate), C.byref(tms)) == 0:
            fp64[name] = rate.value

    if rank != 0:
        return
    # DRAM bytes of one step from the committed ncu capture of the timed form
    traffic = None
    tname = "persist" if args.loop == "persistent" else STEP_KERNEL
    tpath = os.path.join(ROOT, "profiles", f"sciddicaT_{tname}_step_2048.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get("dram_bytes_per_step")
    line = {
        "metric": "cell_updates_per_s", "value": value, "unit": "cell-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(np.mean(run_ms)), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded DEM + elliptical source)",
        "config": {"workload": f"SCIDDICA-T {ROWS}x{COLS} FP64, von Neumann, flat, plain (no active cells), "
                               f"{CA_STEPS} CA steps per bench step, {STEP_KERNEL} step, step loop: {args.loop}",
                   "l2": "flushed (256 MiB write) before every run", "seed": SEED, "p_r": P_R, "p_eps": P_EPS,
                   "parallelism": f"replicas x{world}"},
        "wall_s": t_wall,
        "gpu_launches": (launches_per_step(args.loop) * CA_STEPS + LAUNCHES_PER_RUN[args.loop]) * args.steps,
        "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": int(2 * z.nbytes),
                "d2h_bytes_per_step": int(h.nbytes)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "kernel": kernel_desc,
                     "basis": "achieved = 24 B x rows x cols per step (dense algorithmic bytes) / mean step "
                              "time of the timed runs (CUDA events on the model's stream around each 4000-step "
                              "run, / 4000), i.e. value x 24 B; traffic = ncu DRAM bytes per step of the timed "
                              "form around step 1000 (fields stay in L2)",
                     "step_avg_ms": step_ms,
                     "at_step_1000": {"k1_ms": k1_ms, "k2_ms": k2_ms, "achieved": achieved_1000,
                                      "frac": achieved_1000 / peak,
                                      "how": "events around each of the two kernels, 400 eager steps from "
                                             "step 1000"},
                     "wet_cells_at_step_1000": wet,
                     "bytes_per_step": ROWS * COLS * BYTES_PER_CELL_UPDATE},
        "finite": bool(np.isfinite(hh).all()),
        "consistent": consistent,
        "parity_vs_oracle": parity,
        "boundary": boundary,
        "wet_cell_updates_per_s": wet_total * args.steps * world / dev_s,
        "clocks": clk,
    }
    if fp64.get("dadd"):
        run_s = float(np.mean(run_ms)) * 1e-3
        ach = wet_total * FP64_OPS_PER_WET_CELL / run_s / 1e9
        line["roofline"]["fp64"] = {
            "achieved": ach, "peak": fp64["dadd"] / 1e9, "unit": "GFLOP/s", "frac": ach / (fp64["dadd"] / 1e9),
            "peak_dfma_gflops": 2 * fp64.get("dfma", 0.0) / 1e9,
            "basis": f"wet cell-updates of the run ({wet_total}, from the trace) x {FP64_OPS_PER_WET_CELL} FP64 "
                     "operations (adds, multiplies, divisions as one each) / mean run time; peak = DADD "
                     "instructions per second measured live (cal_fp64_peak: independent chains on every SM, CUDA "
                     "events; the kernel's FP64 work is adds and multiplies, no FMA)"}
    if not args.no_ac:
        line["active_cells_on"] = active_cells_section(m, cal, z, h, hh)
    if not args.no_processes:
        line["processes_plain"] = processes_plain_section(m, cal, z, h, hh)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(z, h)
    if not args.no_calibration:
        line["calibration"] = calibration_section(args)
    print(json.dumps(line), flush=True)


def processes_plain_section(m, cal, z, h, h_plain):
    """The same plain workload through the generic engine: the reference
    program's two elementary processes (device processes registered with
    calAddElementaryProcess2D) and its steering, run by calRunCAStep2D
    (eager: a launch sequence per step; graph: the recorded step replayed) or
    calRunDeviceSteps2D (one device-driven graph launch for the loop).  The
    engine updates and fills only the tiles a process changed (change
    tracking).  Three times: as the reference program stands; with both
    processes declared pure (calSetElementaryProcessPure2D), which lets the
    process kernels skip the tiles whose neighbourhood did not change since
    they last changed nothing there; and with their reads declared too
    (calSetElementaryProcessReads2D), which stages z, h and the outflows into
    shared memory by TMA tile by tile; and pure with the flows process's
    early return on dry cells declared (calSetElementaryProcessGuard2Dr),
    which runs it on each tile's wet cells packed into consecutive threads.
    Every form must give the split step's bits."""
    import torch
    m.cal_sciddicaT_set_pure.argtypes = [C.c_int]
    m.cal_sciddicaT_set_staged.argtypes = [C.c_int]
    m.cal_sciddicaT_set_guard.argtypes = [C.c_int]
    out = {}
    for label, pure, staged, guard in (("as_written", 0, 0, 0), ("declared_pure", 1, 0, 0),
                                       ("declared_pure_and_reads", 1, 1, 0), ("declared_pure_and_guard", 1, 0, 1)):
        m.cal_sciddicaT_set_pure(pure)
        m.cal_sciddicaT_set_staged(staged)
        m.cal_sciddicaT_set_guard(guard)
        sess = m.cal_sciddicaT_open(ROWS, COLS, 0, 0, P_R, P_EPS, z.ctypes.data, h.ctypes.data, cal.MODE_PROCESSES)
        m.cal_sciddicaT_set_pure(0)
        m.cal_sciddicaT_set_staged(0)
        m.cal_sciddicaT_set_guard(0)
        if not sess:
            return {"error": "cal_sciddicaT_open (processes) failed: " + cal.core().calGetErrorString().decode()}
        stream = torch.cuda.ExternalStream(m.cal_sciddicaT_stream(sess))
        forms, same = {}, True
        for name, loop in (("eager", 0), ("graph", 1), ("device", 2)):
            ms = []
            for it in range(3):
                m.cal_sciddicaT_reset(sess)
                with torch.cuda.stream(stream):
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    rc = m.cal_sciddicaT_steps(sess, CA_STEPS, loop)
                    e1.record(stream)
                e1.synchronize()
                if rc:
                    m.cal_sciddicaT_close(sess)
                    return {"error": f"cal_sciddicaT_steps (processes, {label}, {name}) failed: {rc}"}
                if it:
                    ms.append(e0.elapsed_time(e1))
            hp = np.empty_like(h)
            m.cal_sciddicaT_read(sess, hp.ctypes.data)
            same = same and hp.tobytes() == h_plain.tobytes()
            forms[name] = float(np.mean(ms))
        m.cal_sciddicaT_close(sess)
        best = min(forms, key=forms.get)
        out[label] = {"ms_per_run": forms, "best": best,
                      "value": ROWS * COLS * CA_STEPS / (forms[best] * 1e-3), "unit": "cell-updates/s",
                      "identical_to_split_step": bool(same)}
    out["workload"] = (f"SCIDDICA-T {ROWS}x{COLS} FP64, flat, plain, {CA_STEPS} CA steps, the reference program's "
                       "device processes + steering through the run loop")
    return out


def active_cells_section(m, cal, z, h, h_plain):
    """The same workload with active cells on, 4000 steps per run, eager and
    device-driven loops, in two forms: the reference program (its three
    device processes over the device-compacted active-cell list, an update
    after each, the steering resetting the active cells' outflows; model
    created with CAL_OPT_ACTIVE_CELLS) and the active-cells split step (two
    kernels per step, epoch marks for the active set; also every step in
    one cooperative launch).  The two must give identical bits; agreement with the plain run's final h (the modes differ
    by rounding where the reference keeps stale outflows at cells removed
    exactly at the threshold) and mass are reported."""
    import torch
    forms, outs = {}, {}
    for form, mode in (("processes", cal.MODE_PROCESSES), ("split", cal.MODE_FUSED)):
        sess = m.cal_sciddicaT_open(ROWS, COLS, 0, 1, P_R, P_EPS, z.ctypes.data, h.ctypes.data, mode)
        if not sess:
            return {"error": f"cal_sciddicaT_open ({form}) failed: " + cal.core().calGetErrorString().decode()}
        stream = torch.cuda.ExternalStream(m.cal_sciddicaT_stream(sess))
        loops = (("eager", 0), ("device", 2)) + ((("persistent", 4),) if form == "split" else ())
        for name, loop in loops:
            ms = []
            for it in range(3):
                m.cal_sciddicaT_reset(sess)
                with torch.cuda.stream(stream):
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    rc = m.cal_sciddicaT_steps(sess, CA_STEPS, loop)
                    e1.record(stream)
                e1.synchronize()
                if rc or (loop == 4 and m.cal_sciddicaT_persist_failed(sess)):
                    m.cal_sciddicaT_close(sess)
                    return {"error": f"cal_sciddicaT_steps ({form}, {name}) failed: {rc}"}
                if it:
                    ms.append(e0.elapsed_time(e1))
            forms[f"{form}_{name}"] = float(np.mean(ms))
        hac = np.empty_like(h)
        m.cal_sciddicaT_read(sess, hac.ctypes.data)
        outs[form] = hac
        m.cal_sciddicaT_close(sess)
    best = min(forms, key=forms.get)
    hac = outs["split"]
    scale = np.maximum(np.abs(h_plain), 1e-300)
    rel = np.abs(hac - h_plain) / scale
    wet = np.abs(h_plain) > P_EPS
    return {
        "workload": f"SCIDDICA-T {ROWS}x{COLS} FP64, flat, active cells on, {CA_STEPS} CA steps",
        "ms_per_run": forms, "best": best,
        "value": ROWS * COLS * CA_STEPS / (forms[best] * 1e-3), "unit": "cell-updates/s",
        "identical_forms": bool(outs["split"].tobytes() == outs["processes"].tobytes()),
        "wet_cells_at_end": int(np.count_nonzero(hac > P_EPS)),
        "max_rel_diff_vs_plain_wet_cells": float(rel[wet].max()) if wet.any() else 0.0,
        "max_abs_diff_vs_plain": float(np.abs(hac - h_plain).max()),
        "mass_rel_diff_vs_plain": float(abs(hac.sum() - h_plain.sum()) / max(abs(h_plain.sum()), 1e-300)),
    }


ENS_INSTANCES = 256
ENS_STEPS = 1000
ENS_SEED = 4
CALIB_TARGET = 0.9     # fraction of instances recovered (identifiable parameters within 1e-3)
CALIB_FD_SAMPLE = 8    # instances on which the drop-in arm's own trajectory is run


def calibration_section(args):
    """Batched calibration: 256 SCIDDICA-T instances, rows and cols uniform in
    128..1024, each with its own seeded DEM and source (seed 1000 + i) and its
    own p_r in [0.3, 0.7], p_eps in [5e-4, 5e-3]; 1000 steps each.  Targets
    are forward runs at the true parameters; the calibration starts from
    p_r * 1.08, p_eps * 0.92.

    batched: one calibration iteration = one ensemble forward + adjoint
      (all instances' losses and gradients), timed on the host around the
      synchronous call, after one untimed iteration;
    plain: the same iteration with the plain GPU drop-in per instance and
      central finite differences (five 1000-step runs per instance),
      timed over all 256 instances (one session open at a time; opening
      and closing the sessions is not timed)."""
    import torch

    from opencal_gb300 import ensemble as E
    from opencal_gb300 import workloads as W
    dims, ptrue = W.ensemble_spec(ENS_INSTANCES, seed=ENS_SEED)
    zs, hs = W.ensemble_inputs(dims)
    ens = E.Ensemble(dims, ptrue, zs, hs, ENS_STEPS)
    shape, tune_ms = ens.autotune(100)
    tgt = ens.forward()
    tg_host = ens.unpack(tgt)
    active = ens.active_tiles()
    p0 = [(p[0] * 1.08, p[1] * 0.92) for p in ptrue]
    ens.set_params(p0)
    ens.loss_grad(tgt)  # untimed
    t_b = []
    for _ in range(3):
        t0 = time.perf_counter()
        loss, grad = ens.loss_grad(tgt)
        t_b.append(time.perf_counter() - t0)
    batched_s = float(np.median(t_b))
    g_launches0, g_nodes = ens.graph_stats()
    tape = ens.tape_info()
    # the same evaluation launch by launch, once
    ens.set_graph(False)
    t0 = time.perf_counter()
    ens.loss_grad(tgt)
    batched_eager_s = time.perf_counter() - t0
    ens.set_graph(True)
    # and with the sqrt(T) segments recomputed from checkpoints (the mode
    # taken when the whole rollout's tape does not fit), once after a
    # recording call
    ens.set_tape("segments")
    ens.loss_grad(tgt)
    t0 = time.perf_counter()
    ens.loss_grad(tgt)
    batched_segments_s = time.perf_counter() - t0
    ens.set_tape("auto")

    # the plain drop-in per instance with central differences (five runs):
    # its run loop (the recorded step replayed), and the fastest single-grid
    # loop of this library (every step in one cooperative launch)
    fd_s, fdp_s = 0.0, 0.0
    rel = []
    for b in range(ENS_INSTANCES):
        for loop in (1, 4):
            sess = E.FDSession(zs[b], hs[b], p0[b][0], p0[b][1], ENS_STEPS, tg_host[b], loop=loop)
            t0 = time.perf_counter()
            f0, g = sess.fd_grad(*p0[b])
            dt = time.perf_counter() - t0
            sess.close()
            if loop == 1:
                fd_s += dt
                den = np.maximum(np.abs(grad[b]), 1e-300)
                rel.append(np.abs(g - grad[b]) / den)
            else:
                fdp_s += dt
    rel = np.asarray(rel)

    # recovery at 1e-3: only parameters that h_T determines to 1e-3 count
    # (identifiable: both 1e-3 perturbations change h_T), for both arms alike
    mask = E.identifiable(ens, tgt, ptrue, rel=1e-3)
    ens.set_params(p0)
    cal = E.calibrate(ens, tgt, p0, iters=args.calib_iters, p_true=ptrue, tol=1e-3, mask=mask,
                      stop_at=CALIB_TARGET)
    k_b = cal["converged_at"] or cal["iterations"]
    ttr_b = float(np.sum(cal["iter_s"][:k_b]))
    # the drop-in arm's own trajectory (same optimiser, central differences)
    # on a sample of instances, for the same number of iterations
    sample = list(range(0, ENS_INSTANCES, ENS_INSTANCES // CALIB_FD_SAMPLE))[:CALIB_FD_SAMPLE]
    fd_traj = E.calibrate_fd([(zs[b], hs[b], tg_host[b], p0[b], ptrue[b], mask[b]) for b in sample], ENS_STEPS,
                             iters=k_b)
    batched_on_sample = [float(np.mean(r[sample])) for r in cal["recovered_each"][:k_b]]
    ens.close()
    del tgt
    torch.cuda.empty_cache()
    return {
        "workload": f"{ENS_INSTANCES} SCIDDICA-T FP64 instances, rows/cols uniform 128..1024 "
                    f"({sum(r * c for r, c in dims)} cells), own DEM/source/p_r/p_eps, {ENS_STEPS} steps, "
                    "loss = sum (h_T - target)^2",
        "metric": "calibration_iters_per_s", "unit": "iterations/s",
        "batched_iter_s": batched_s, "batched_iters_per_s": 1.0 / batched_s,
        "plain_fd_iter_s": fd_s, "plain_fd_iters_per_s": 1.0 / fd_s,
        "speedup": fd_s / batched_s,
        "plain_fd_persistent_iter_s": fdp_s, "speedup_vs_persistent_fd": fdp_s / batched_s,
        "tile_shape": shape, "autotune_ms": tune_ms,
        "active_tiles_per_step_mean": float(active.mean()),
        "fd_vs_adjoint_rel_diff_median": [float(np.median(rel[:, 0])), float(np.median(rel[:, 1]))],
        "calibration": {"start": "p_r * 1.08, p_eps * 0.92", "iterations": cal["iterations"],
                        "identifiable_1e-3": {"p_r": float(mask[:, 0].mean()), "p_eps": float(mask[:, 1].mean()),
                                              "rule": "h_T at the true parameters with that parameter scaled "
                                                      "by 1 -/+ 1e-3 differs from the target in both cases"},
                        "recovered_1e-3_by_iteration": cal["recovered"],
                        "recovery_target": CALIB_TARGET,
                        "iterations_to_target": cal["converged_at"],
                        "p_r_within_1e-3": float(np.mean(cal["rel_err"][:, 0] < 1e-3)),
                        "p_eps_within_1e-3": float(np.mean(cal["rel_err"][:, 1] < 1e-3)),
                        "median_rel_err": [float(np.median(cal["rel_err"][:, 0])),
                                           float(np.median(cal["rel_err"][:, 1]))]},
        "time_to_recovery_s": {
            "batched": ttr_b,
            "plain_fd": k_b * fd_s,
            "plain_fd_persistent": k_b * fdp_s,
            "ratio": k_b * fd_s / ttr_b,
            "ratio_vs_persistent_fd": k_b * fdp_s / ttr_b,
            "how": f"batched: measured wall time of the iterations until {CALIB_TARGET:.0%} of the instances have "
                   "their identifiable parameters within 1e-3 (all 256 instances); plain drop-in: the same number "
                   "of iterations x its measured iteration time over all 256 instances; the drop-in's own "
                   f"trajectory (same optimiser, central differences) on {len(sample)} instances recovers as "
                   "the batched arm does on them (fd_sample_recovered vs batched_sample_recovered)",
            "fd_sample_recovered": fd_traj["recovered"],
            "batched_sample_recovered": batched_on_sample,
        },
        # one launch of the recorded evaluation; its nodes: forward (init +
        # one step kernel per step, each taping its tiles), loss; backward
        # per step: tape restore, coefficients, gather; the result copies
        "gpu_launches_per_batched_iter": 1,
        "graph_nodes_per_batched_iter": g_nodes,
        "batched_iter_s_launch_by_launch": batched_eager_s,
        "tape": {"whole_rollout": tape["full"], "bytes": tape["need_bytes"],
                 "batched_iter_s_sqrt_t_segments": batched_segments_s},
    }


SCIARA_BYTES_PER_CELL_UPDATE = 65  # Sz, Slt, St r/w (48) + Mb r (1) + Msl r/w (16)
SCIARA_CPU_SAMPLE_STEPS = 4


def sciara_arm(args):
    """SCIARA-fv2 hazard-mapping scenarios: --scenarios scenarios of --size^2
    cells at 10 m on 8 seeded volcanoes (cone 3000 m over 20.48 km at 4096^2,
    +-5 m fractal noise), each scenario with its own 1-3 vents near the summit
    and emission rates uniform in 10..50 m^3/s over 6 phases of 3600 s; 360
    steps of 60 s, all scenarios advanced together by the split step.  Then
    the adjoint of the final-thickness misfit with respect to every emission
    rate, against targets from the same scenarios run with rates * 0.9.
    Metric: cell-updates/s of the forward (scenarios x cells x steps / device
    time of the step loop).  One JSON line."""
    import opencal_gb300 as cal
    from opencal_gb300 import workloads as W
    cal.build()
    t0 = time.perf_counter()
    scs = W.sciara_scenarios(args.scenarios, args.size, args.size)
    gen_s = time.perf_counter() - t0
    with cal.SciaraBatch([(z, v, [[x * 0.9 for x in r] for r in rt], et) for z, v, rt, et in scs]) as sb:
        sb.run()
        target = np.concatenate([a.ravel() for a in sb.read("slt")])
    with cal.SciaraBatch(scs) as sb:
        for _ in range(args.warmup):
            sb.run()
        clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
        clocks.start()
        fw = []
        for _ in range(args.steps):
            steps, ms = sb.run()
            fw.append(ms)
        clk = clocks.stop()
        lava = sb.lava_cells()
        loss, grads, lg_ms = sb.loss_grad(target)
    del target
    cpu = None
    if not args.no_cpu_baseline:
        import oracle
        oracle.build()
        cores = os.cpu_count() or 1
        os.environ.setdefault("OMP_NUM_THREADS", str(cores))
        z, v, rt, et = scs[0]
        t0 = time.perf_counter()
        oracle.sciara(z, v, rt, et, SCIARA_CPU_SAMPLE_STEPS, kind="omp", want_cells=False)
        dt = time.perf_counter() - t0
        cpu = {"value": z.size * SCIARA_CPU_SAMPLE_STEPS / dt, "unit": "cell-updates/s", "cores": cores,
               "kind": "port", "sample": f"the first {SCIARA_CPU_SAMPLE_STEPS} steps of scenario 0 "
                                         f"({args.size}^2, every cell), OpenMP on all host cores"}
    fw_ms = float(np.median(fw))
    cells = sb.cells
    peak, peak_kind = _peaks()
    value = cells * steps / (fw_ms * 1e-3)
    achieved = value * SCIARA_BYTES_PER_CELL_UPDATE / 1e9  # dense-equivalent GB/s
    line = {
        "metric": "cell_updates_per_s", "value": value, "unit": "cell-updates/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": fw_ms / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded volcano cones, vents, emission rates)",
        "config": {"workload": f"SCIARA-fv2 {args.scenarios} scenarios x {args.size}^2 at 10 m on 8 volcanoes, "
                               f"Moore, flat + border mask, 6 emission phases x 3600 s, {steps} steps, split step "
                               "(vents, lava-cell flows, flagged-tile update) for all scenarios at once",
                   "input_generation_s": gen_s, "l2": "no flush: the step touches only the lava cells' tiles"},
        "forward_ms": fw_ms, "forward_runs_ms": fw, "loss_grad_ms": lg_ms,
        "adjoint": {"what": "dL/d(emission rate) of every vent and phase, L = sum (Slt_T - target)^2, "
                            "decisions frozen, undo tape; loss_grad_ms = forward with tape + adjoint",
                    "loss_median": float(np.median(loss)),
                    "grad_abs_max": float(max(np.abs(g).max() for g in grads))},
        "lava_cells_final": lava,
        "dense_equivalent": {"gbs": achieved, "hbm_peak_gbs": peak, "peak_source": peak_kind,
                             "basis": f"{SCIARA_BYTES_PER_CELL_UPDATE} B per cell-update of the dense grids; the "
                                      "split step touches only the lava cells and their tiles, so this exceeds "
                                      "the HBM peak by the work that sparsity skips"},
        "clocks": clk, "cpu_baseline": cpu, "gpu_launches_per_step": 3,
    }
    print(json.dumps(line), flush=True)


MBUSU_CELLS = 130 * 160 * 30
MBUSU_CPU_SAMPLE_STEPS = 20


def mbusu_arm(args):
    """mbusu, the reference's 3D subsurface-flow example (160 x 30 x 130
    cells, von Neumann 3D, toroidal, 8 real substates, float time step from
    a global minimum), through the 3D C API: one bench step = the whole run
    to its stop condition (10 days of simulated time, 8662 steps) as one
    device-driven loop.  Metric: cell-updates/s.  The CPU baseline is the
    OpenMP oracle on the first 20 steps.  One JSON line."""
    import opencal_gb300 as cal
    import oracle
    cal.build()
    cap = args.max_steps  # 0: until the stop condition
    mode = args.mbusu_mode
    for _ in range(args.warmup):
        cal.mbusu(cap, mode=mode)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    runs = [cal.mbusu(cap, mode=mode, timing=True) for _ in range(args.steps)]
    clk = clocks.stop()
    ms = float(np.median([r["ms"] for r in runs]))
    steps = runs[0]["steps"]
    value = MBUSU_CELLS * steps / (ms * 1e-3)
    cpu = None
    if not args.no_cpu_baseline:
        oracle.build()
        cores = os.cpu_count() or 1
        os.environ.setdefault("OMP_NUM_THREADS", str(cores))
        t0 = time.perf_counter()
        oracle.mbusu(MBUSU_CPU_SAMPLE_STEPS, kind="omp")
        dt = time.perf_counter() - t0
        cpu = {"value": MBUSU_CELLS * MBUSU_CPU_SAMPLE_STEPS / dt, "unit": "cell-updates/s", "cores": cores,
               "kind": "port", "sample": f"the first {MBUSU_CPU_SAMPLE_STEPS} steps (initialisation included), "
                                         "OpenMP on all host cores"}
    line = {
        "metric": "cell_updates_per_s", "value": value, "unit": "cell-updates/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "the program's own initial state",
        "config": {"workload": "mbusu 160x30x130 (3D von Neumann, toroidal), 8 real substates, "
                               + ("until 10 days" if not cap else f"first {cap} steps")
                               + f" ({steps} steps), "
                               + ("one device-driven loop" if mode == 2 else "a recorded step replayed" if mode == 1
                                  else "a launch sequence per step")
                               + " (EP, min-reduction steering, device stop)",
                   "l2": "no flush: the 40 MB of state is L2-resident by design"},
        "run_ms": [r["ms"] for r in runs], "steps_per_run": steps, "delta_t_cum": runs[0]["delta_t_cum"],
        "bound": "FP64 pipe: eight pow calls per cell-update",
        "clocks": clk, "cpu_baseline": cpu, "gpu_launches_per_step": 5,
    }
    print(json.dumps(line), flush=True)


ADJ_SIZE, ADJ_STEPS, ADJ_SEED = 1024, 2000, 3
ADJ_CPU_SAMPLE_STEPS = 100


def adjoint_arm(args):
    """SCIDDICA-T single-grid adjoint: 1024^2, T = 2000 steps, L = sum (h_T -
    h_target)^2 with the target from the run at p_r = 0.42, p_eps = 0.0015,
    gradient with respect to p_r, p_eps and h0 at p_r = 0.5, p_eps = 0.001 by
    the hand-written adjoint (forward with sqrt(T) checkpoints + reverse
    sweep, csrc/models/sciddicaT_adjoint.cu) through torch.autograd.  One
    bench step = one gradient evaluation; metric cell-updates/s of the
    forward (rows x cols x T per evaluation).  Compared with central finite
    differences for (p_r, p_eps) on the GPU (4 forward runs) and with the
    OpenMP oracle's forward, extrapolated to the same 4 runs."""
    import torch
    import opencal_gb300 as cal
    from opencal_gb300 import adjoint as A
    from opencal_gb300 import workloads as W
    cal.build()
    z, h0 = W.sciddicaT_inputs(ADJ_SIZE, ADJ_SIZE, seed=ADJ_SEED)
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    zt = torch.from_numpy(z).to(dev)
    ht = torch.from_numpy(h0).to(dev)
    with torch.no_grad():
        target = A.rollout(zt, ht, 0.42, 0.0015, ADJ_STEPS)

    def grad_eval():
        pr = torch.tensor(0.5, dtype=torch.float64, device=dev, requires_grad=True)
        pe = torch.tensor(0.001, dtype=torch.float64, device=dev, requires_grad=True)
        h = ht.clone().requires_grad_(True)
        loss = ((A.rollout(zt, h, pr, pe, ADJ_STEPS) - target) ** 2).sum()
        loss.backward()
        return float(loss.detach()), float(pr.grad), float(pe.grad)

    def loss_at(pr, pe):
        with torch.no_grad():
            return float(((A.rollout(zt, ht, pr, pe, ADJ_STEPS) - target) ** 2).sum())

    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        grad_eval()
    clocks = ClockSampler(dev.index)
    clocks.start()
    times = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        loss, gr, ge = grad_eval()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    adj_ms = float(np.median(times))
    # central finite differences for (p_r, p_eps): four forward runs
    d_r, d_e = 1e-6 * 0.5, 1e-6 * 0.001
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fd_r = (loss_at(0.5 + d_r, 0.001) - loss_at(0.5 - d_r, 0.001)) / (2 * d_r)
    fd_e = (loss_at(0.5, 0.001 + d_e) - loss_at(0.5, 0.001 - d_e)) / (2 * d_e)
    e1.record(stream)
    e1.synchronize()
    fd_ms = e0.elapsed_time(e1)
    # the same loss and gradients by the ensemble engine with one instance:
    # tile work-lists, so dry regions cost nothing (csrc/models/sciddicaT_batch.cu)
    from opencal_gb300.ensemble import Ensemble
    ens = Ensemble([(ADJ_SIZE, ADJ_SIZE)], [(0.5, 0.001)], [z], [h0], ADJ_STEPS, device=dev)
    tgt = ens.pack([target.cpu().numpy()])
    for _ in range(max(1, args.warmup)):
        ens.loss_grad(tgt, want_h0_grad=True)
    sparse = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        s_loss, s_grad, _ = ens.loss_grad(tgt, want_h0_grad=True)
        torch.cuda.synchronize(dev)
        sparse.append(1e3 * (time.perf_counter() - t0))
    ens.close()
    sparse_ms = float(np.median(sparse))
    cpu = None
    if not args.no_cpu_baseline:
        import oracle
        oracle.build()
        cores = os.cpu_count() or 1
        os.environ.setdefault("OMP_NUM_THREADS", str(cores))
        t0 = time.perf_counter()
        oracle.sciddicaT(z, h0, ADJ_CPU_SAMPLE_STEPS, toroidal=False, ac=False, p_r=0.5, p_eps=0.001, kind="omp",
                         want_cells=False)
        dt = time.perf_counter() - t0
        cpu = {"value": ADJ_SIZE * ADJ_SIZE * ADJ_CPU_SAMPLE_STEPS / dt, "unit": "cell-updates/s", "cores": cores,
               "kind": "port", "sample": f"{ADJ_CPU_SAMPLE_STEPS} forward steps of the {ADJ_SIZE}^2 grid, OpenMP on "
                                         "all host cores",
               "fd_gradient_s_extrapolated": 4 * dt * ADJ_STEPS / ADJ_CPU_SAMPLE_STEPS}
    cells = ADJ_SIZE * ADJ_SIZE * ADJ_STEPS
    line = {
        "metric": "cell_updates_per_s", "value": cells / (adj_ms * 1e-3), "unit": "cell-updates/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": adj_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded DEM + source, seed 3)",
        "config": {"workload": f"SCIDDICA-T adjoint {ADJ_SIZE}^2 FP64, VN, flat, plain, T = {ADJ_STEPS}: one "
                               "gradient evaluation (forward with sqrt(T) checkpoints + reverse sweep) w.r.t. "
                               "p_r, p_eps and h0",
                   "l2": "no flush: 8 MiB grids"},
        "gradient_ms": adj_ms, "gradient_runs_ms": times,
        "fd_gradient_ms": fd_ms, "adjoint_vs_fd_speedup": fd_ms / adj_ms,
        "sparse_engine": {"what": "the same loss and gradients (p_r, p_eps, h0) by the ensemble engine with one "
                                  "instance (tile work-lists; host-timed, synchronised)",
                          "gradient_ms": sparse_ms, "runs_ms": sparse, "loss": float(s_loss[0]),
                          "grad_rel_diff_vs_dense": [abs(s_grad[0, 0] - gr) / max(abs(gr), 1e-300),
                                                     abs(s_grad[0, 1] - ge) / max(abs(ge), 1e-300)]},
        "gradient": {"loss": loss, "dL_dpr": gr, "dL_dpeps": ge, "fd_dL_dpr": fd_r, "fd_dL_dpeps": fd_e,
                     "rel_diff": [abs(gr - fd_r) / max(abs(fd_r), 1e-300), abs(ge - fd_e) / max(abs(fd_e), 1e-300)]},
        "clocks": clk, "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


LIFE_SIZE, LIFE_STEPS, LIFE_CPU_SAMPLE_STEPS = 1024, 1000, 100


def life_arm(args):
    """Game of Life B3/S23, 1024^2 toroidal Moore, alive ~ Bernoulli(0.3)
    (seed 1), 1000 generations: the reference program (one device process
    per generation through the C API, byte substate), one fused launch per
    generation, and temporal blocking (k generations per launch in shared
    memory) for k = 4, 8, and the bit-sliced form (32 cells per word, a
    carry-save adder tree per word) for k = 8, 16, 32; all must give the
    same bits.  One bench step
    = one 1000-generation run of each; value = the fastest form's
    cell-updates/s; 2 B per cell-update by the metric's formula (the 1 MiB
    state is L2-resident, so this is not an HBM figure)."""
    import opencal_gb300 as cal
    from opencal_gb300 import workloads as W
    cal.build()
    s0 = W.life_state(LIFE_SIZE, LIFE_SIZE, p=0.3, seed=1)
    forms = [("processes", cal.MODE_PROCESSES, 1), ("processes_reads_declared", cal.MODE_PROCESSES, 1),
             ("processes_pure", cal.MODE_PROCESSES, 1), ("processes_pure_reads_declared", cal.MODE_PROCESSES, 1),
             ("fused", cal.MODE_FUSED, 1)] + \
            [(f"blocked{k}", cal.MODE_FUSED_BLOCKED, k) for k in (4, 8)] + \
            [(f"bits{k}", cal.MODE_BITS, k) for k in (8, 16, 32)]
    decl = {"processes_reads_declared": 2, "processes_pure": 1, "processes_pure_reads_declared": 3}
    m = cal.models()
    m.cal_life2d_set_declarations.argtypes = [C.c_int]
    results, outs = {}, {}
    for name, mode, k in forms:
        m.cal_life2d_set_declarations(decl.get(name, 0))
        for _ in range(args.warmup):
            cal.life2d(s0, LIFE_STEPS, mode=mode, block=k)
        ms = []
        for _ in range(args.steps):
            out, t = cal.life2d(s0, LIFE_STEPS, mode=mode, block=k, timing=True)
            ms.append(t)
        results[name] = float(np.median(ms))
        outs[name] = out
    m.cal_life2d_set_declarations(0)
    same = all(o.tobytes() == outs["processes"].tobytes() for o in outs.values())
    best = min(results, key=results.get)
    cells = LIFE_SIZE * LIFE_SIZE * LIFE_STEPS
    value = cells / (results[best] * 1e-3)
    cpu = None
    if not args.no_cpu_baseline:
        import oracle
        oracle.build()
        cores = os.cpu_count() or 1
        os.environ.setdefault("OMP_NUM_THREADS", str(cores))
        t0 = time.perf_counter()
        oracle.life2d(s0, LIFE_CPU_SAMPLE_STEPS, kind="omp")
        dt = time.perf_counter() - t0
        cpu = {"value": LIFE_SIZE * LIFE_SIZE * LIFE_CPU_SAMPLE_STEPS / dt, "unit": "cell-updates/s",
               "cores": cores, "kind": "port",
               "sample": f"{LIFE_CPU_SAMPLE_STEPS} generations, OpenMP on all host cores"}
    line = {
        "metric": "cell_updates_per_s", "value": value, "unit": "cell-updates/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": results[best], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic (Bernoulli(0.3), seed 1)",
        "config": {"workload": f"Life B3/S23 {LIFE_SIZE}^2 toroidal Moore, {LIFE_STEPS} generations",
                   "l2": "no flush: the 1 MiB state is L2-resident by design"},
        "forms_ms": results, "best": best, "identical_results": same,
        "dense_equivalent_gbs": 2 * value / 1e9, "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def ncu_case_ensemble(args):
    """A fixed, untimed ensemble sequence for ncu captures: the first 32
    instances of the calibration ensemble, one forward of --ncu-steps steps
    and one loss + gradient evaluation against it."""
    from opencal_gb300 import ensemble as E
    from opencal_gb300 import workloads as W
    dims, ptrue = W.ensemble_spec(ENS_INSTANCES, seed=ENS_SEED)
    dims, ptrue = dims[:32], ptrue[:32]
    zs, hs = W.ensemble_inputs(dims)
    ens = E.Ensemble(dims, ptrue, zs, hs, args.ncu_steps)
    ens.set_shape("32x16")
    tgt = ens.forward()
    ens.set_params([(p[0] * 1.08, p[1] * 0.92) for p in ptrue])
    loss, grad = ens.loss_grad(tgt)
    print(json.dumps({"cells": ens.cells, "active_tiles_mean": float(ens.active_tiles().mean()),
                      "loss_median": float(np.median(loss))}), flush=True)


def ncu_case_processes(args):
    """A fixed, untimed sequence for ncu captures of the generic engine: the
    2048^2 session in processes mode (the reference program's device
    processes; processes_ac: with active cells on), --ncu-warm steps, then
    --ncu-steps steps, launch by launch (--loop eager) or device-driven
    (--loop device); --declare: 1 pure, 2 reads staged, 3 both."""
    import opencal_gb300 as cal
    from opencal_gb300 import workloads as W
    cal.build()
    m = cal.models()
    m.cal_sciddicaT_open.restype = C.c_void_p
    m.cal_sciddicaT_open.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                     C.c_void_p, C.c_void_p, C.c_int]
    m.cal_sciddicaT_steps.argtypes = [C.c_void_p, C.c_int, C.c_int]
    m.cal_sciddicaT_close.argtypes = [C.c_void_p]
    m.cal_sciddicaT_set_pure.argtypes = [C.c_int]
    m.cal_sciddicaT_set_staged.argtypes = [C.c_int]
    m.cal_sciddicaT_set_guard.argtypes = [C.c_int]
    ac = 1 if args.ncu_case == "processes_ac" else 0
    z, h = W.sciddicaT_inputs(ROWS, COLS, seed=SEED)
    m.cal_sciddicaT_set_pure(args.declare & 1)
    m.cal_sciddicaT_set_staged((args.declare >> 1) & 1)
    m.cal_sciddicaT_set_guard((args.declare >> 2) & 1)
    sess = m.cal_sciddicaT_open(ROWS, COLS, 0, ac, P_R, P_EPS, z.ctypes.data, h.ctypes.data, cal.MODE_PROCESSES)
    m.cal_sciddicaT_set_pure(0)
    m.cal_sciddicaT_set_staged(0)
    m.cal_sciddicaT_set_guard(0)
    loop = {"eager": 0, "graph": 1, "device": 2}.get(args.loop, 0)
    t0 = time.perf_counter()
    rc = m.cal_sciddicaT_steps(sess, args.ncu_warm, loop)
    rc |= m.cal_sciddicaT_steps(sess, args.ncu_steps, loop)
    cal.core().calGetLastError()
    m.cal_sciddicaT_close(sess)
    print(json.dumps({"case": args.ncu_case, "declare": args.declare, "loop": args.loop, "rc": rc,
                      "steps": args.ncu_warm + args.ncu_steps, "wall_s": time.perf_counter() - t0}), flush=True)
    if rc:
        raise SystemExit(1)


def ncu_case(args):
    """A fixed, untimed sequence for ncu captures: open the 2048^2 session
    (activecells: with active cells on), run --ncu-steps fused steps from the
    initial state, report the wet fraction.  No torch, no extra
    allocations."""
    if args.ncu_case == "ensemble":
        return ncu_case_ensemble(args)
    if args.ncu_case in ("processes", "processes_ac"):
        return ncu_case_processes(args)
    ac = 1 if args.ncu_case == "activecells" else 0
    import opencal_gb300 as cal
    from opencal_gb300 import workloads as W
    cal.build()
    m = cal.models()
    m.cal_sciddicaT_open.restype = C.c_void_p
    m.cal_sciddicaT_open.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                     C.c_void_p, C.c_void_p, C.c_int]
    m.cal_sciddicaT_steps.argtypes = [C.c_void_p, C.c_int, C.c_int]
    m.cal_sciddicaT_read.argtypes = [C.c_void_p, C.c_void_p]
    m.cal_sciddicaT_close.argtypes = [C.c_void_p]
    z, h = W.sciddicaT_inputs(ROWS, COLS, seed=SEED)
    sess = m.cal_sciddicaT_open(ROWS, COLS, 0, ac, P_R, P_EPS, z.ctypes.data, h.ctypes.data, cal.MODE_FUSED)
    done = 0
    for target in sorted(set([args.ncu_steps] + [s for s in (500, 1000, 2000, 3000, 4000) if s < args.ncu_steps])):
        m.cal_sciddicaT_steps(sess, target - done, LOOPS[args.loop])
        done = target
        hh = np.empty_like(h)
        m.cal_sciddicaT_read(sess, hh.ctypes.data)
        print(json.dumps({"step": done, "wet_fraction": float(np.count_nonzero(hh > P_EPS)) / hh.size,
                          "mass": float(hh.sum())}), flush=True)
    m.cal_sciddicaT_close(sess)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="opencal", choices=["opencal", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--loop", default="persistent", choices=sorted(LOOPS))
    ap.add_argument("--no-ac", action="store_true", help="skip the active-cells-on run of the workload")
    ap.add_argument("--no-processes", action="store_true", help="skip the generic-engine (device processes) figure")
    ap.add_argument("--no-calibration", action="store_true", help="skip the batched-calibration section")
    ap.add_argument("--calib-iters", type=int, default=40)
    ap.add_argument("--ncu-case", nargs="?", const="split",
                    choices=["split", "ensemble", "activecells", "processes", "processes_ac"],
                    help="untimed fixed sequence for ncu captures")
    ap.add_argument("--ncu-steps", type=int, default=1002)
    ap.add_argument("--ncu-warm", type=int, default=400, help="processes cases: steps before the captured ones")
    ap.add_argument("--declare", type=int, default=0, choices=range(8),
                    help="processes cases, bits: 1 processes declared pure, 2 reads declared, 4 flows guard declared")
    ap.add_argument("--workload", default="sciddicaT", choices=["sciddicaT", "sciara", "mbusu", "adjoint", "life"],
                    help="sciddicaT: the headline line; sciara: the SCIARA-fv2 scenario measurement; "
                         "mbusu: the 3D subsurface-flow program; adjoint: the SCIDDICA-T gradient at 1024^2, T = 2000; "
                         "life: Game of Life 1024^2")
    ap.add_argument("--scenarios", type=int, default=64)
    ap.add_argument("--max-steps", type=int, default=0,
                    help="mbusu: stop after this many steps (0: at its stop condition); for short profiles")
    ap.add_argument("--mbusu-mode", type=int, default=2, choices=[0, 1, 2],
                    help="mbusu: 0 launches per step, 1 recorded step replayed, 2 device-driven loop "
                         "(ncu cannot profile the kernels of 2's conditional graph)")
    ap.add_argument("--size", type=int, default=4096)
    args = ap.parse_args()
    if args.workload == "sciara":
        sciara_arm(args)
    elif args.workload == "mbusu":
        mbusu_arm(args)
    elif args.workload == "adjoint":
        adjoint_arm(args)
    elif args.workload == "life":
        life_arm(args)
    elif args.ncu_case:
        ncu_case(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
