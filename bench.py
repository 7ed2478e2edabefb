"""Benchmark: scatterer-line projections per second of the COLE simulation on one
GB300 (the 3-D LUT volume workload: 2M fixed scatterers x 64x64 lines, 256x64x64
beam LUT, 3.5 MHz / bw 0.15 / 50 MHz, decimation 8, phase delay on), and the
same workload on the reference's CPU algorithm.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload volume_3d_lut|sector_2d_fixed|sector_spline]

One step = one simulate_lines over the whole scan (projection, pulse
convolution, demodulation, decimation).  Prints one JSON line on rank 0.

* value: projections/s with the phantom resident on the device, IQ left on the
  device, CUDA events around each step on the simulator's stream, L2 flushed
  (a 512 MiB memset) between steps outside the timed events.  The timed steps
  run without the per-stage instrumentation; the stage times (stage_ms) and the
  projection kernel's time come from a second loop of the same steps.
* e2e: the same metric through the C ABI with host buffers, host wall clock:
  every step (frame) uploads the scatterers from pinned host memory and reads
  the IQ back.  A fixed-scatterer phantom runs as a stream of frames through
  bcsim_simulate_fixed_frames, a spline phantom through
  bcsim_simulate_spline_frames (frame k+1's upload overlaps frame k), where a
  frame's data exceed L2; otherwise per step (bcsim_set_*_scatterers +
  bcsim_simulate_lines).  e2e.single_frame is the per-step form for every
  workload.
* roofline: the projection kernel against the FP32 pipe: the per-projection
  flop count (flops_per_projection) times the pairs the kernel visits (counted
  by one instrumented run outside the timed region; the exact slot masks skip
  pairs of weight 0), and its HBM traffic.
* cpu_baseline: the CPU port of the reference algorithm (oracle, reference float
  arithmetic, FFT convolution) on all host cores, on a subset of the lines.
* rel_rms: the timed step's IQ against the FP64 CPU oracle on a spread of lines.
* batch: the 64 uneven jobs of the batch workload as one Batch.run against one
  simulate_lines per job (IQ to the host in both), and the batched output's
  IQ error against the FP64 oracle on a sample of jobs and lines.
* serve: Poisson request streams at 200, 1000 and 3000 requests/s over 8
  resident phantoms, served by the continuous-batching server and, live, by
  serial plain execution: latency percentiles and throughput of both.

Lines are independent, so N GPUs run N independent replicas of the workload
(weak scaling, no collective).
"""
from __future__ import annotations

import argparse
import gc
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

METRIC = "scatterer-line projections/s"
# DRAM traffic of one projection launch of the default workloads (ncu, full size)
NCU_TRAFFIC_BYTES = {"volume_3d_lut": 380.37e6 + 359.62e6}
MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def flops_per_projection(lut: bool, phase_delay: bool, spline_degree=None) -> float:
    """Algorithmic FP32 flops of one scatterer-line projection (FMA = 2):
    offset (3) + three dot products (15) + distance (5) + bin index (3) +
    Gaussian exponent (5) + amplitude (1) + accumulation (2) = 34; a lookup-table
    beam replaces the Gaussian exponent by 3 normalisations and 7 trilinear
    lerps (27); the sub-sample phase adds 6; a spline scatterer adds its
    position, 3 FMAs per non-zero basis function (6 (p+1))."""
    f = 34.0
    if lut:
        f += 27.0 - 5.0
    if phase_delay:
        f += 6.0
    if spline_degree is not None:
        f += 6.0 * (spline_degree + 1)
    return f


def make_job(name: str, num_scatterers: int = 0, lines: str = ""):
    """The named workload, optionally with fewer scatterers / lines (for
    profiling captures on a small case); "batch_uneven:J" is job J of the
    64-job batch workload."""
    from openbcsim_gb300 import workloads as W

    if name.startswith("batch_uneven:"):
        return W.batch_uneven()[int(name.split(":", 1)[1])]

    kw = {}
    if num_scatterers:
        kw["num_scatterers"] = num_scatterers
    if lines:
        parts = [int(x) for x in lines.split(",")]
        if name == "volume_3d_lut":
            kw["n_az"], kw["n_el"] = parts[0], parts[-1]
        else:
            kw["num_lines"] = parts[0]
    return getattr(W, name)(**kw)


def run_simulate_only(args):
    """Configure and run warmup + steps simulations, nothing else (the command
    that profiling captures wrap)."""
    import openbcsim_gb300 as gb

    job = make_job(args.workload, args.num_scatterers, args.lines)
    sim = gb.RfSimulator("gpu")
    gb.configure_job(sim, job)
    apply_params(sim, args.param)
    out = None
    for _ in range(args.warmup + args.steps):
        out = sim.simulate_lines_line_major(out)
    print(f"simulated {args.warmup + args.steps} x {job.name}: {job.num_scatterers} scatterers x "
          f"{job.scan.num_lines} lines, |IQ|max {float(np.abs(out).max()):.4g}")


def apply_params(sim, params):
    """--param key=value pairs passed to set_parameter."""
    for kv in params or []:
        k, v = kv.split("=", 1)
        sim.set_parameter(k, v)


def rank_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(values, device):
    """Element-wise maximum of this rank's values over the process group (the
    slowest replica's times), or the values themselves on one rank."""
    import torch

    dist = torch.distributed
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while active."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
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
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


def sm_count():
    import torch

    return torch.cuda.get_device_properties(0).multi_processor_count


def run_gpu(args):
    import torch

    import openbcsim_gb300 as gb

    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    if world > 1 and not torch.distributed.is_initialized():
        torch.distributed.init_process_group("nccl")
    job = make_job(args.workload, args.num_scatterers, args.lines)
    sim = gb.RfSimulator("gpu")
    sim.set_parameter("gpu_device", str(local))
    gb.configure_job(sim, job)
    # every timed step redoes the whole pipeline, including the per-scatterer
    # distance/bin/phase pass and the sort (no reuse of records between steps)
    sim.set_parameter("record_cache", "off")
    apply_params(sim, args.param)
    # the timed steps run without the per-stage instrumentation; a second loop
    # of the same steps with it gives the stage times
    sim.set_parameter("store_kernel_details", "off")
    L, nd = sim.output_shape()
    dev_out = torch.empty((L, nd), dtype=torch.complex64, device="cuda")
    stream = torch.cuda.ExternalStream(sim.stream())
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def step():
        sim.simulate_lines_device(dev_out.data_ptr(), dev_out.numel())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # ---- device-resident timed region ----
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    proj_ms = []
    stage = {}
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            starts[i].record(stream)
        step()
        ends[i].record(stream)
        ends[i].synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    launches_per_step = int(sim.get_debug_data("kernel_launches")[0])
    # ---- the same steps with the per-stage CUDA events (outside the timed
    # region): stage times, and the projection kernel's time for the roofline ----
    sim.set_parameter("store_kernel_details", "on")
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        step()
        proj_ms.append(sim.get_debug_data("fixed_projection_kernel_ms")[-1] if job.fixed else
                       sim.get_debug_data("spline_projection_kernel_ms")[-1])
        for k in STAGE_KEYS:
            if _has(sim, k):
                stage.setdefault(k, []).append(sim.get_debug_data(k)[-1])
    sim.set_parameter("store_kernel_details", "off")
    total_s = max_over_ranks([sum(step_ms) / 1e3], "cuda")[0]
    projections = job.projections
    value = projections * args.steps * world / total_s


    # ---- e2e through the C ABI with pinned host buffers ----
    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True)
        t.numpy()[:] = a
        return t.numpy()

    host_in = [pinned(f.xyza) for f in job.fixed]
    host_sp = [(sp.degree, pinned(sp.knots), pinned(sp.control_points), pinned(sp.amplitudes)) for sp in job.splines]
    host_out = torch.empty((L, nd), dtype=torch.complex64, pin_memory=True)
    out_np = host_out.numpy()

    def e2e_step():
        # the phantom is uploaded every step (a fresh frame), the IQ read back
        sim.clear_fixed_scatterers()
        for h in host_in:
            sim.add_fixed_scatterers(h)
        if host_sp:
            sim.clear_spline_scatterers()
            for deg, kn, cp, am in host_sp:
                sim.add_spline_scatterers(deg, kn, cp, am)
        sim.simulate_lines_line_major(out_np)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    e2e_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_single = sum(e2e_ms) / 1e3
    # a stream of frames of a fixed-scatterer phantom through one C-ABI call
    # (bcsim_simulate_fixed_frames): every frame is uploaded and its IQ read back,
    # frame k+1's upload overlapping frame k's simulation.  No L2 flush fits
    # between the frames of one call, so this form is used only where one
    # frame's bins alone exceed L2 (0.55 GB on the 3-D volume; smaller
    # workloads keep the per-step form, flushed)
    bins_bytes = L * job.num_samples * (16 if job.phase_delay else 8)
    l2_bytes = getattr(torch.cuda.get_device_properties(0), "L2_cache_size", 0) or (129 << 20)
    frames_mode = len(host_in) == 1 and not host_sp and bins_bytes > 2 * l2_bytes
    # a stream of spline frames (bcsim_simulate_spline_frames): every frame
    # uploads fresh control points and amplitudes, which with its bins exceed
    # L2 (0.23 GB on the spline sector)
    sp_bytes = sum(kn.nbytes + cp.nbytes + am.nbytes for _, kn, cp, am in host_sp)
    spline_frames_mode = not host_in and len(host_sp) == 1 and sp_bytes + bins_bytes > 1.5 * l2_bytes
    e2e_total = e2e_single
    if frames_mode or spline_frames_mode:
        outs = [torch.empty((L, nd), dtype=torch.complex64, pin_memory=True).numpy() for _ in range(args.steps)]
        W = max(1, min(args.warmup, args.steps))

        def stream_of(count, o):
            if frames_mode:
                sim.simulate_fixed_frames([host_in[0]] * count, o)
            else:
                deg, kn, cp, am = host_sp[0]
                sim.simulate_spline_frames(deg, kn, [cp] * count, [am] * count, o)

        stream_of(W, outs[:W])
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        stream_of(args.steps, outs)
        e2e_total = time.perf_counter() - t0
    e2e_total, e2e_single = max_over_ranks([e2e_total, e2e_single], "cuda")
    h2d = sum(h.nbytes for h in host_in) + sum(kn.nbytes + cp.nbytes + am.nbytes for _, kn, cp, am in host_sp)
    d2h = L * nd * 8

    # ---- one instrumented run (outside every timed region): the (record, line)
    # pairs the shared-origin kernel visits and those with a non-zero weight, and
    # the (scatterer, line) pairs the per-pair kernel evaluates after its tile
    # culling ----
    shared_path = "prep_sort_ms" in stage
    visited = nonzero = idle_steps = per_pair = None
    sim.set_parameter("count_pairs", "on")
    sim.simulate_lines_device(dev_out.data_ptr(), dev_out.numel())
    torch.cuda.synchronize()
    if shared_path:
        visited = int(sim.get_debug_data("evaluated_pairs")[0])
        nonzero = int(sim.get_debug_data("weighted_pairs")[0])
        idle_steps = int(sim.get_debug_data("idle_walk_steps")[0])
    per_pair = int(sim.get_debug_data("per_pair_evaluated_pairs")[0])
    sim.set_parameter("count_pairs", "off")

    if rank != 0:
        return None
    lut = not hasattr(job.beam, "sigma_lateral")
    fpp = flops_per_projection(lut, job.phase_delay, job.splines[0].degree if job.splines and not job.fixed else None)
    proj_avg_ms = statistics.mean(proj_ms)
    # units one launch processes: the pairs the shared-origin kernel visits (the
    # others have weight exactly 0 and are skipped by the slot masks), or the
    # pairs the per-pair kernel evaluates (its tiles leave out scatterers none of
    # their lines can see)
    units = visited if shared_path else per_pair
    achieved_tflops = units * fpp / (proj_avg_ms / 1e3) / 1e12
    all_pairs_tflops = projections * fpp / (proj_avg_ms / 1e3) / 1e12
    sms = sm_count()
    clock_mhz = clk.get("sm_mhz") or 2070.0
    fp32_peak = sms * 128 * 2 * clock_mhz * 1e6 / 1e12
    peaks = {}
    if os.path.exists(MEASURED_PEAKS):
        with open(MEASURED_PEAKS) as f:
            peaks = json.load(f)
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    # phantom (16 B per fixed scatterer, 12 K + 4 B per spline scatterer) + table + IQ
    alg_bytes = (sum(f.xyza.nbytes for f in job.fixed) +
                 sum(sp.control_points.shape[0] * (12 * sp.control_points.shape[1] + 4) for sp in job.splines) +
                 (job.beam.samples.nbytes if lut else 0) + L * nd * 8)
    # DRAM bytes (read + write) of one projection launch, from an ncu capture of
    # that launch at full size (dram__bytes_read.sum + dram__bytes_write.sum);
    # --traffic-bytes overrides
    traffic = NCU_TRAFFIC_BYTES.get(args.workload) if not (args.num_scatterers or args.lines or args.param) else None
    if args.traffic_bytes:
        traffic = float(args.traffic_bytes)
    result = {
        "metric": METRIC, "value": value, "unit": "projections/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_s * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (time of flight f64)", "data": "synthetic (seeded)",
        "config": {"workload": f"{job.name}: {job.num_scatterers} {'fixed' if job.fixed else 'spline'} scatterers x {L} lines, "
                               f"{'256x64x64 LUT beam' if lut else 'Gaussian beam'}, ns={job.num_samples}, "
                               f"decimation {job.decimation}, phase delay {'on' if job.phase_delay else 'off'}",
                   "projections_per_step": projections, "l2": "flushed between steps (512 MiB memset)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": projections * args.steps * world / e2e_total, "unit": "projections/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_total * 1e3 / args.steps,
                "mode": ("frames: one bcsim_simulate_fixed_frames call of `steps` frames from pinned host memory, "
                         "frame k+1 uploaded while frame k is simulated; one frame's bins exceed L2") if frames_mode else
                        ("spline frames: one bcsim_simulate_spline_frames call of `steps` frames from pinned host "
                         "memory, frame k+1's control points uploaded while frame k is simulated; one frame's "
                         "upload and bins exceed L2") if spline_frames_mode else
                        "per step: clear + add scatterers (upload), simulate_lines (IQ to pinned host memory), L2 flushed",
                "single_frame": {"value": projections * args.steps * world / e2e_single,
                                 "ms_per_step": e2e_single * 1e3 / args.steps,
                                 "mode": "per step: clear + add scatterers (upload), simulate_lines, L2 flushed"}},
        "roofline": {"bound": "fp32", "kernel": "project_shared_kernel" if shared_path else "project_generic_kernel",
                     "achieved": achieved_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved_tflops / fp32_peak, "traffic": traffic,
                     "flops_per_unit": fpp, "units_per_launch": units,
                     "unit_counted": "visited (record, line) pairs" if shared_path
                                     else "evaluated (scatterer, line) pairs",
                     "pairs": {"all": projections, "visited": visited, "nonzero_weight": nonzero,
                               "per_pair_evaluated": per_pair,
                               "idle_warp_steps": idle_steps},
                     "all_pairs_convention": {"achieved": all_pairs_tflops, "frac": all_pairs_tflops / fp32_peak,
                                              "note": "flops_per_unit x N x L: counts the pairs that the exact "
                                                      "culling skips, so it can exceed the peak"},
                     "kernel_ms": proj_avg_ms,
                     "peak_source": f"nominal FP32 FMA rate: {sms} SMs x 128 lanes x 2 x {clock_mhz:.0f} MHz "
                                    "(median SM clock sampled during the timed steps)"},
        "roofline_hbm": {"achieved": alg_bytes / (proj_avg_ms / 1e3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                         "frac": alg_bytes / (proj_avg_ms / 1e3) / 1e9 / hbm_peak,
                         "algorithmic_bytes": alg_bytes, "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
        "clocks": clk,
        "gpu_launches": args.steps * launches_per_step,
        "gpu_launches_note": f"{launches_per_step} kernels of this library per step (the CUB radix sort of the "
                             "shared-origin path launches its own kernels in addition)",
        "stage_ms": {k: statistics.mean(v) for k, v in stage.items()},
        "wall_s": wall,
    }
    if world == 1 and not args.no_cpu_baseline:   # the host baseline at N = 1 only
        result["cpu_baseline"] = cpu_baseline(job, args.cpu_seconds)
    if world == 1 and not args.no_extras:
        # the metric's other figures, each outside every timed region above:
        # the timed output's IQ error against the FP64 oracle, the batched
        # uneven jobs against plain execution, and the served request stream
        # against serial plain execution
        result["rel_rms"] = headline_rel_rms(job, dev_out.cpu().numpy())
        del dev_out, flush, sim
        torch.cuda.empty_cache()
        result["batch"] = batch_section(args)
        result["serve"] = serve_section(args)
    return result


def headline_rel_rms(job, iq):
    """Relative RMS of the timed step's IQ (the last timed simulation's output)
    against the FP64 oracle over a spread of lines: 64 spread over the scan
    plus, for a square grid of lines, its corners, edge middles and centre."""
    from oracle import oracle as O

    L = job.scan.num_lines
    idx = [np.linspace(0, L - 1, 64).round().astype(int)]
    n = int(round(np.sqrt(L)))
    if n * n == L:
        idx.append(np.array([0, n - 1, L - n, L - 1, n // 2, L - n + n // 2, (n // 2) * n, (n // 2) * n + n - 1,
                             (n // 2) * n + n // 2]))
    idx = np.unique(np.concatenate(idx))
    t0 = time.perf_counter()
    ref = O.simulate(_subset_idx(job, idx), O.MODE_FP64)
    err = O.rel_rms(iq[idx], ref)
    return {"value": err, "tolerance": 1e-4, "lines": int(len(idx)), "of_lines": L,
            "reference": "FP64 CPU oracle (oracle/cole_oracle.c), same inputs",
            "oracle_s": time.perf_counter() - t0}


def _subset_idx(job, idx):
    import copy

    from openbcsim_gb300 import workloads as W

    sub = copy.copy(job)
    s = job.scan
    sub.scan = W.ScanSequence(s.origins[idx], s.directions[idx], s.lateral_dirs[idx], s.timestamps[idx],
                              s.line_length)
    return sub


STAGE_KEYS = ["kernel_memset_ms", "prep_sort_ms", "fixed_projection_kernel_ms", "spline_projection_kernel_ms",
              "kernel_convolve_demodulate_ms", "total_ms"]


def _has(sim, key):
    try:
        sim.get_debug_data(key)
        return True
    except RuntimeError:
        return False


def cpu_baseline(job, seconds: float, threads: int = 0):
    """The reference CPU algorithm on a contiguous subset of the lines, all
    host cores; `seconds` bounds the sample.  Uses the compiled reference
    (oracle/_ref) where it exists, else the oracle's port of it (REF32 float
    arithmetic, FFT convolution)."""
    from oracle import oracle as O

    cores = threads or os.cpu_count()
    kind = "reference" if O.ref_available() else "port"
    L = job.scan.num_lines
    n_lines = max(1, min(L, cores))
    sub = _subset(job, 0, n_lines)
    t0 = time.perf_counter()
    _cpu_run(sub, kind, cores)
    dt = time.perf_counter() - t0
    # grow the sample to about `seconds` of work
    target = int(min(L, max(n_lines, n_lines * seconds / max(dt, 1e-3))))
    target = max(cores, (target // cores) * cores) if target >= cores else target
    sub = _subset(job, 0, target)
    t0 = time.perf_counter()
    _cpu_run(sub, kind, cores)
    dt = time.perf_counter() - t0
    value = job.num_scatterers * target / dt
    return {"value": value, "unit": "projections/s", "cores": cores, "kind": kind,
            "sample": f"{target} of {L} lines of the same workload ({job.num_scatterers} scatterers), "
                      f"{dt:.1f} s", "seconds": dt}


def _subset(job, lo, hi):
    import copy

    from openbcsim_gb300 import workloads as W

    sub = copy.copy(job)
    s = job.scan
    sub.scan = W.ScanSequence(s.origins[lo:hi], s.directions[lo:hi], s.lateral_dirs[lo:hi], s.timestamps[lo:hi],
                              s.line_length)
    return sub


def _cpu_run(job, kind, cores):
    from oracle import oracle as O

    if kind == "reference":
        return O.ref_simulate(job, threads=cores)
    return O.simulate(job, O.MODE_REF32, threads=cores)


def run_reference(args):
    rank, world, _ = rank_info()
    if rank != 0:
        return None
    job = make_job(args.workload)
    from oracle import oracle as O

    cores = os.cpu_count()
    kind = "reference" if O.ref_available() else "port"
    # one step = a bounded sample of the workload's lines
    L = job.scan.num_lines
    n_lines = min(L, max(cores, args.ref_lines))
    sub = _subset(job, 0, n_lines)
    for _ in range(args.warmup):
        _cpu_run(_subset(job, 0, min(L, cores)), kind, cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _cpu_run(sub, kind, cores)
    dt = time.perf_counter() - t0
    value = job.num_scatterers * n_lines * args.steps / dt
    sample = f"{n_lines} of {L} lines per step ({job.num_scatterers} scatterers)"
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "projections/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": {"workload": job.name, "projections_per_step": job.num_scatterers * n_lines},
            "cpu_baseline": {"value": value, "unit": "projections/s", "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "projections/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def batch_section(args):
    """Config 4: 64 uneven jobs (fixed and spline, uneven N, L, depth, pulse,
    decimation), results on the host.  plain: one simulate_lines per job, in
    order (the one-simulation path); batched: one Batch.run.  Each form timed
    over `batch_steps` runs after warm-up, host wall clock."""
    import torch

    import openbcsim_gb300 as gb
    from openbcsim_gb300 import workloads as W

    torch.cuda.set_device(0)
    jobs = W.batch_uneven(num_jobs=args.jobs, scale=args.batch_scale)
    sims = []
    for j in jobs:
        s = gb.RfSimulator("gpu")
        gb.configure_job(s, j)
        apply_params(s, args.param)
        sims.append(s)
    # IQ into pinned host buffers (as the headline's e2e), so that the device-to-
    # host copies run asynchronously in both forms
    outs = [torch.empty(s.output_shape(), dtype=torch.complex64, pin_memory=True).numpy() for s in sims]
    total = sum(j.projections for j in jobs)

    def plain():
        for s, o in zip(sims, outs):
            s.simulate_lines_line_major(o)

    batch = gb.Batch(sims, use_graph=True)
    for _ in range(max(3, args.warmup)):
        plain()
        batch.run(outs)
    torch.cuda.synchronize()
    steps = args.batch_steps
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(steps):
        plain()
    t_plain = (time.perf_counter() - t0) / steps
    t0 = time.perf_counter()
    for _ in range(steps):
        batch.run(outs)
    t_batch = (time.perf_counter() - t0) / steps
    clk = clocks.stop()
    n_spline = sum(1 for j in jobs if j.splines)
    # the batched output against the FP64 oracle: the eight smallest jobs whole,
    # eight lines spread over each of four of the largest (outside the timing)
    from oracle import oracle as O

    order = sorted(range(len(jobs)), key=lambda k: jobs[k].projections)
    errs = []
    t0 = time.perf_counter()
    for k in order[:8]:
        errs.append(O.rel_rms(outs[k], O.simulate(jobs[k], O.MODE_FP64)))
    for k in order[-4:]:
        L = jobs[k].scan.num_lines
        idx = np.unique(np.linspace(0, L - 1, 8).round().astype(int))
        errs.append(O.rel_rms(outs[k][idx], O.simulate(_subset_idx(jobs[k], idx), O.MODE_FP64)))
    check = {"max": max(errs), "tolerance": 1e-4, "jobs_checked": len(errs), "oracle_s": time.perf_counter() - t0,
             "sample": "the 8 smallest jobs whole, 8 spread lines of each of the 4 largest"}
    return {"workload": f"batch_uneven: {len(jobs)} jobs ({n_spline} spline), {total:.4e} projections per step, "
                        f"scale {args.batch_scale}",
            "unit": "projections/s", "steps": steps,
            "batched": {"value": total / t_batch, "ms_per_step": t_batch * 1e3},
            "plain": {"value": total / t_plain, "ms_per_step": t_plain * 1e3,
                      "form": "one simulate_lines per job, in order, IQ to pinned host memory"},
            "batched_over_plain": t_plain / t_batch, "io": "IQ to pinned host memory every step (both forms)",
            "rel_rms": check, "clocks": clk}


def run_batch(args):
    res = batch_section(args)
    return {"metric": METRIC + " (batched uneven jobs)", "value": res["batched"]["value"], "unit": "projections/s",
            "n_gpus": 1, "steps": res["steps"], "warmup": args.warmup, "ms_per_step": res["batched"]["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (time of flight f64)",
            "data": "synthetic (seeded)", "config": {"workload": res["workload"], "l2": "jobs' data far exceed L2"},
            "plain": res["plain"], "batched_over_plain": res["batched_over_plain"], "clocks": res["clocks"]}


def _pct(v, q):
    v = sorted(v)
    return v[min(len(v) - 1, int(round(q * (len(v) - 1))))] if v else None


def serve_stream(args, phantoms, sims, rate, seconds):
    """One Poisson stream (config 5) served live by the continuous-batching
    server, then replayed live by serial plain execution (one simulate_lines
    at a time in arrival order, each starting when the request has arrived and
    the previous one is done).  Latency = arrival to result on the host."""
    import torch

    import openbcsim_gb300 as gb
    from openbcsim_gb300 import workloads as W

    reqs = W.request_stream(phantoms, rate_hz=rate, seconds=seconds)
    # objects of earlier sections that only the cyclic collector frees (their
    # device teardown synchronises) are freed here, not in the middle of the
    # stream; the collector stays off while both forms are timed
    gc.collect()
    torch.cuda.synchronize()
    gc.disable()
    try:
        return _serve_stream_timed(args, phantoms, sims, rate, seconds, reqs, gb)
    finally:
        gc.enable()


def _serve_stream_timed(args, phantoms, sims, rate, seconds, reqs, gb):
    import queue

    from openbcsim_gb300 import workloads as W

    server = gb.Server(hbm_budget_bytes=64 << 30, max_slots_per_phantom=4, max_in_flight=args.max_in_flight)
    pids = [server.add_phantom(s) for s in sims]
    # warm-up: per phantom, as many requests of the stream's largest shape (256
    # lines, decimation 4) as can be in flight at once, so that the slots the
    # stream uses have grown before it starts
    big = W.sector_scan(256, 35.0, 0.12)
    for k, s in enumerate(phantoms):
        sc = s.scan
        server.wait(server.submit(pids[k], sc.origins, sc.directions, sc.line_length, sc.lateral_dirs,
                                  sc.timestamps, 8))
        warm = [server.submit(pids[k], big.origins, big.directions, big.line_length, big.lateral_dirs,
                              np.full(256, float(sc.timestamps[0]), np.float32), 4)
                for _ in range(args.max_in_flight)]
        for rid in warm:
            server.wait(rid)
    # the client: this thread submits at the arrival times, a second one
    # collects the results in order as they complete
    ids = queue.Queue()
    lat = []

    def collect():
        for _ in range(len(reqs)):
            lat.append(server.wait(ids.get())[1])

    collector = threading.Thread(target=collect)
    collector.start()
    t_start = time.perf_counter()
    for r in reqs:
        now = time.perf_counter() - t_start
        if r.arrival > now:
            time.sleep(r.arrival - now)
        sc = r.scan
        ids.put(server.submit(pids[r.phantom], sc.origins, sc.directions, sc.line_length, sc.lateral_dirs,
                              sc.timestamps, r.decimation))
    collector.join()
    wall = time.perf_counter() - t_start
    st = server.stats()
    server.close()
    n_proj = sum(phantoms[r.phantom].num_scatterers * r.scan.num_lines for r in reqs)
    # serial plain execution of the same stream, live
    serial_lat, busy = [], 0.0
    t_start = time.perf_counter()
    for r in reqs:
        now = time.perf_counter() - t_start
        if r.arrival > now:
            time.sleep(r.arrival - now)
        s = sims[r.phantom]
        sc = r.scan
        t0 = time.perf_counter()
        s.set_parameter("radial_decimation", str(r.decimation))
        s.set_scan_sequence(sc.origins, sc.directions, sc.line_length, sc.lateral_dirs, sc.timestamps)
        s.simulate_lines_line_major()
        t1 = time.perf_counter()
        busy += t1 - t0
        serial_lat.append((t1 - t_start - r.arrival) * 1e3)
    serial_wall = time.perf_counter() - t_start
    return {"rate_hz": rate, "seconds": seconds, "requests": len(reqs),
            "server": {"value": n_proj / wall, "wall_s": wall,
                       "latency_ms": {"p50": _pct(lat, 0.5), "p99": _pct(lat, 0.99), "max": max(lat)},
                       "completed": st["completed"], "failed": st["failed"]},
            "serial_plain": {"value": n_proj / serial_wall, "wall_s": serial_wall, "busy_s": busy,
                             "latency_ms": {"p50": _pct(serial_lat, 0.5), "p99": _pct(serial_lat, 0.99),
                                            "max": max(serial_lat)}},
            "server_over_serial_throughput": serial_wall / wall}


def serve_section(args):
    """Config 5 at the configured rate (200 requests/s) and at rates that load
    the GPU, each stream `serve_seconds` long."""
    import torch

    import openbcsim_gb300 as gb
    from openbcsim_gb300 import workloads as W

    torch.cuda.set_device(0)
    phantoms = W.served_phantoms(scale=args.batch_scale)
    sims = []
    for j in phantoms:
        s = gb.RfSimulator("gpu")
        gb.configure_job(s, j)
        sims.append(s)
    clocks = ClockSampler(0)
    clocks.start()
    streams = [serve_stream(args, phantoms, sims, float(r), args.serve_seconds) for r in args.rates.split(",")]
    clk = clocks.stop()
    return {"workload": "served_stream: Poisson arrivals over 8 resident phantoms (fixed 100k-2M, spline 50k-500k "
                        "scatterers), 1-256 lines per request at random angles and times, decimation 4-16",
            "unit": "projections/s", "max_in_flight": args.max_in_flight, "streams": streams, "clocks": clk}


def run_serve(args):
    res = serve_section(args)
    top = res["streams"][-1]
    return {"metric": METRIC + " (served stream)", "value": top["server"]["value"], "unit": "projections/s",
            "n_gpus": 1, "steps": top["requests"], "warmup": 8, "ms_per_step": top["server"]["wall_s"] * 1e3 /
            max(1, top["requests"]), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (time of flight f64)", "data": "synthetic (seeded)",
            "config": {"workload": res["workload"], "max_in_flight": res["max_in_flight"]},
            "streams": res["streams"], "clocks": res["clocks"]}


def run_imaging(args):
    """Post-processing rows: B-mode (envelope, log compression, scan conversion)
    of config 1's frame (128 lines x 780 samples) into the image size the
    reference's GUI uses (70 degree sector, 12 cm, 6000 dots per metre), and the
    colour-Doppler estimate + image of a 16-frame packet of it.  GPU: frames/s
    through the C ABI with host IQ in and the image out (host clock), and
    simulate_bmode (simulation + image, the IQ staying on the device).  CPU: the
    oracle's restatement of the same steps, one host thread."""
    import openbcsim_gb300 as gb
    from oracle import imaging as OI
    from openbcsim_gb300 import workloads as W

    job = W.sector_2d_fixed()
    sim = gb.RfSimulator("gpu")
    gb.configure_job(sim, job)
    width = float(np.float32(np.deg2rad(70.0)))
    nx, ny = gb.ScanGeometry.image_size("sector", width, job.scan.line_length, 6000.0)
    geo = gb.ScanGeometry("sector", width, job.scan.line_length, nx, ny)
    iq = sim.simulate_lines_line_major().copy()
    P = 16
    rng = np.random.default_rng(5)
    packet = (iq[None] * np.exp(1j * rng.uniform(-0.3, 0.3, (P, 1, 1)) * np.arange(P)[:, None, None])).astype(
        np.complex64)

    def timed(fn, steps):
        for _ in range(args.warmup):
            fn()
        t0 = time.perf_counter()
        for _ in range(steps):
            fn()
        return (time.perf_counter() - t0) / steps

    clocks = ClockSampler(0)
    clocks.start()
    t_bmode = timed(lambda: sim.bmode_image(iq, 60.0, 1.0, 0.0, geo), args.steps * 10)
    t_sim_bmode = timed(lambda: sim.simulate_bmode(60.0, 1.0, 0.0, geo), args.steps)
    t_sim = timed(lambda: sim.simulate_lines_line_major(), args.steps)
    t_doppler = timed(lambda: sim.color_doppler(packet, geo), args.steps * 10)
    clk = clocks.stop()
    t_cpu_bmode = timed(lambda: OI.bmode(iq, 60.0, 1.0, 0.0, geo), 3)
    t_cpu_doppler = timed(lambda: OI.color_image(*OI.color_doppler(packet), geo), 3)
    return {"metric": "B-mode frames/s (post-processing of an IQ frame)", "value": 1.0 / t_bmode, "unit": "frames/s",
            "n_gpus": 1, "steps": args.steps * 10, "warmup": args.warmup, "ms_per_step": t_bmode * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": f"sector_2d_fixed IQ {iq.shape[0]} lines x {iq.shape[1]} samples -> "
                                   f"{nx} x {ny} sector image (70 deg, {job.scan.line_length} m, 6000 dots/m); "
                                   f"colour Doppler packet of {P} frames",
                       "io": "host IQ in, image out, per step"},
            "simulate_bmode": {"value": 1.0 / t_sim_bmode, "unit": "frames/s", "ms_per_step": t_sim_bmode * 1e3,
                               "simulate_lines_ms": t_sim * 1e3},
            "color_doppler": {"value": 1.0 / t_doppler, "unit": "packets/s", "ms_per_step": t_doppler * 1e3,
                              "packet_bytes": int(packet.nbytes)},
            "cpu_baseline": {"value": 1.0 / t_cpu_bmode, "unit": "frames/s", "cores": 1, "kind": "port",
                             "sample": "the same frame, oracle/imaging_oracle.c (envelope, log compression, "
                                       "Cartesianator restatement)",
                             "color_doppler": {"value": 1.0 / t_cpu_doppler, "unit": "packets/s"}},
            "clocks": clk}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="volume_3d_lut")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-lines", type=int, default=64)
    ap.add_argument("--num-scatterers", type=int, default=0, help="override the workload's scatterer count")
    ap.add_argument("--lines", default="", help="override the line count (volume: 'n_az,n_el')")
    ap.add_argument("--param", action="append", default=[], help="engine parameter key=value (repeatable)")
    ap.add_argument("--mode", default="single", choices=["single", "batch", "serve", "imaging"],
                    help="single: the headline workload; batch: 64 uneven jobs; serve: Poisson request stream; "
                         "imaging: B-mode and colour-Doppler post-processing")
    ap.add_argument("--jobs", type=int, default=64)
    ap.add_argument("--batch-scale", type=float, default=1.0, help="scale of N and L in batch/serve modes")
    ap.add_argument("--rates", default="200,1000,3000", help="serve: request rates (req/s) of the streams")
    ap.add_argument("--serve-seconds", type=float, default=6.0)
    ap.add_argument("--batch-steps", type=int, default=10)
    ap.add_argument("--no-extras", action="store_true",
                    help="single mode: leave out the rel_rms, batch and serve figures")
    ap.add_argument("--max-in-flight", type=int, default=3, help="serve mode: requests on the GPU at once")
    ap.add_argument("--simulate-only", action="store_true", help="only run warmup+steps simulations (profiling)")
    ap.add_argument("--traffic-bytes", type=float, default=None,
                    help="DRAM bytes per projection launch from an ncu capture (reported as roofline.traffic)")
    args = ap.parse_args()
    if args.simulate_only:
        run_simulate_only(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.mode == "batch":
        res = run_batch(args)
    elif args.mode == "serve":
        res = run_serve(args)
    elif args.mode == "imaging":
        res = run_imaging(args)
    else:
        res = run_reference(args) if args.impl == "reference" else run_gpu(args)
    if res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
