"""Benchmark: PIV vectors/s of the multipass drop-in on one GB300.

Workload ("config2"): one 2048x2048 uint16 (12-bit) particle-image pair, Oseen
vortex (rc 200 px, peak 8 px), three passes 64 -> 32 -> 16 px windows with
overlap 0.5, WorkFIX neighbour threshold 2, thin-plate-spline interpolation
between passes and at the end (subdomains of 200 vectors, smoothing 0.5).
One step = ``WorkPIV.calcul`` of one pair; the counted vectors are the final
field's (65025 per pair).

* ``value``: device-resident images, CUDA events around each step, L2 flushed
  (a 512 MiB write) between steps outside the timed events.
* ``e2e``: the public API from pinned host images to host ``MultipassPIVResults``
  (host<->device copies inside the timed region): ``WorkPIV.calcul_series`` over a
  series of pairs (two pairs in flight, each on its own host thread and CUDA
  stream: 3.8-4.1 ms per pair against 4.1-4.5 with three), and
  ``single_call``: ``WorkPIV.calcul``, one pair per call.
* ``roofline``: the dominant kernel (the TPS subdomain solve), timed with CUDA
  events inside the timed steps: its algorithmic bytes (one write and one read of
  each subdomain's FP64-sized system) per launch over the launch time, against the
  measured HBM copy bandwidth of MEASURED_PEAKS.json; ``traffic`` is the DRAM
  bytes ncu measured for that kernel.  ``passes`` gives the same for each
  correlation pass: FP32 FFT flops and unique image bytes over the pass time.
* ``accuracy_vs_fp64``: the timed result against the FP64 oracle (complex128
  FFTs, float64 fit): displacement and final-field errors in px.
* ``cpu_baseline``: the CPU oracle (numpy restatement of the reference path), one
  thread, on pairs of the same 2048x2048 workload.

``--impl reference`` times that CPU oracle on all host cores (one process per
core, one 2048x2048 pair of the workload per process and step) with the same
metric.

Multi-GPU: replicas only (pairs are independent; no collective on the data path).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "PIV vectors/s at <=0.005 px vs FP64; plain FP32 vs batched tensor-core form"
UNIT = "vectors/s"
WORKLOAD = "config2: 2048x2048 uint16 pair, Oseen vortex, 3 passes 64/32/16 px, overlap 0.5, fix thr 2, TPS subdom 200 smoothing 0.5"
SAMPLE_SHAPE = (2048, 2048)
#: FP32 FFT work per window of n x n (2 R2C + 1 C2R at 2.5 N log2 N, plus the
#: conjugate product and energies)
def fft_flops(n):
    import math

    return 3 * 2.5 * n * n * math.log2(n * n) + 5 * n * n

# ncu dram__bytes_read.sum + dram__bytes_write.sum of k_tps_solve_mp per subdomain:
# one CTA of 16 warps per subdomain (launches of at most one subdomain per SM; 72
# subdomains of the config-2 recipe at 1024^2) and two 8-warp CTAs per SM (the
# 342-subdomain launch of the 2048^2 workload)
TPS_DRAM_BYTES_PER_SUBDOMAIN_WIDE = (126.285056e6 + 80.334336e6) / 72
TPS_DRAM_BYTES_PER_SUBDOMAIN_NARROW = (837.309952e6 + 579.323136e6) / 342


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--size", type=int, default=2048,
                    help="image side (2048 = the config; smaller sizes for profiling)")
    ap.add_argument("--no-precision-sweep", action="store_true",
                    help="skip the tensor-core precision sweep (the 4096^2 single-pass workload)")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched heterogeneous workload (256 single-pass pairs)")
    ap.add_argument("--batched-only", action="store_true",
                    help="run only the batched heterogeneous workload (one JSON line)")
    ap.add_argument("--no-refinement", action="store_true",
                    help="skip the deform-and-correlate refinement workload (8 pairs 2048^2)")
    ap.add_argument("--refinement-only", action="store_true",
                    help="run only the refinement workload (one JSON line)")
    ap.add_argument("--sweep-only", action="store_true",
                    help="run only the precision sweep (one JSON line; for profiling)")
    ap.add_argument("--forms", default=",".join(TC_FORMS),
                    help="forms of the precision sweep (fp32_fft, bf16x1, bf16x3, fp16x3)")
    ap.add_argument("--sweep-size", type=int, default=4096,
                    help="image side of the precision sweep (4096 = the workload)")
    ap.add_argument("--window-sizes", default=None,
                    help="run only single passes of these window sizes (e.g. 16,24,32,48,64; "
                         "one JSON line)")
    ap.add_argument("--preproc", action="store_true",
                    help="time the preprocessing tools instead (second JSON line format)")
    return ap.parse_args()


# ------------------------------------------------------------------------------------
# CPU oracle (reference arm and cpu_baseline): runs in separate processes
# ------------------------------------------------------------------------------------
def _oracle_sample(pair):
    """Run the oracle multipass on one pair of the workload; returns (vectors, seconds)."""
    from fluidimage_gb300 import WorkPIV, workloads
    from oracle import piv as O

    (im0, im1), _ = workloads.config2_images(pair=pair, shape=SAMPLE_SHAPE)
    params = workloads.config2_params(WorkPIV.create_default_params())
    t0 = time.perf_counter()
    res = O.multipass(im0, im1, params)
    dt = time.perf_counter() - t0
    return int(res[-1].deltaxs.size), dt


def _oracle_samples(min_seconds):
    """Oracle multipass on successive pairs of the workload until ``min_seconds`` of
    work; returns (vectors, seconds, pairs)."""
    nvec, dt, n = 0, 0.0, 0
    while dt < min_seconds and n < 200:
        v, t = _oracle_sample(n)
        nvec, dt, n = nvec + v, dt + t, n + 1
    return nvec, dt, n


def cpu_baseline_single(min_seconds=10.0):
    env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1", MKL_NUM_THREADS="1")
    code = ("import sys, json; sys.path.insert(0, %r); import bench; "
            "print(json.dumps(bench._oracle_samples(%r)))" % (str(ROOT), float(min_seconds)))
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                         timeout=600)
    if out.returncode != 0:
        return None
    nvec, dt, n = json.loads(out.stdout.strip().splitlines()[-1])
    return {"value": nvec / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n} {SAMPLE_SHAPE[0]}x{SAMPLE_SHAPE[1]} pairs of the same workload "
                      f"({nvec} final vectors, 3 passes + fix + TPS each) in {dt:.1f} s, "
                      "numpy oracle, 1 thread"}


_PAIR_CACHE = {}


def _oracle_step(pair):
    """One reference-arm task: the oracle multipass on pair ``pair`` of the workload
    (images generated on the first call of the worker process and kept); returns
    (vectors, seconds)."""
    from fluidimage_gb300 import WorkPIV, workloads
    from oracle import piv as O

    if pair not in _PAIR_CACHE:
        (im0, im1), _ = workloads.config2_images(pair=pair, shape=SAMPLE_SHAPE)
        _PAIR_CACHE[pair] = (im0, im1)
    im0, im1 = _PAIR_CACHE[pair]
    params = workloads.config2_params(WorkPIV.create_default_params())
    t0 = time.perf_counter()
    res = O.multipass(im0, im1, params)
    return int(res[-1].deltaxs.size), time.perf_counter() - t0


def run_reference(args):
    """Reference arm: the CPU oracle on all host cores, one worker process per core,
    each processing one pair of the workload per step (the reference's own
    parallelism: one process per image pair)."""
    import multiprocessing as mp

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    os.environ.update(OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1", MKL_NUM_THREADS="1")
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    step_times, nvec_total = [], 0
    with ctx.Pool(cores) as pool:
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            res = pool.map(_oracle_step, range(cores), chunksize=1)
            dt = time.perf_counter() - t0
            if step >= args.warmup:
                step_times.append(dt)
                nvec_total = sum(r[0] for r in res)
    ms = 1e3 * statistics.mean(step_times)
    value = nvec_total / (ms / 1e3)
    sample = (f"{cores} worker processes x one {SAMPLE_SHAPE[0]}x{SAMPLE_SHAPE[1]} pair of "
              "the workload each per step (numpy oracle, 1 thread per process)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "device": f"host CPU, {cores} cores (no GPU used)",
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": WORKLOAD, "same_config": True,
                                        "sample": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        """Start sampling every 20 ms; returns once the first sample arrived (the
        timed region starts after it)."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        t_end = time.perf_counter() + 3.0
        while not self.lines and time.perf_counter() < t_end:
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def stop(self, t0=None, t1=None):
        """Summary of the samples read between host times t0 and t1 (all samples
        when none falls there)."""
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = [ln for t, ln in self.lines if t0 is None or t0 <= t <= t1]
        if not lines:
            lines = [ln for _, ln in self.lines]
        for line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[3:7]):
                if flag.lower() in ("active", "1"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def max_over_ranks(values, dist=None, device="cpu"):
    """Element-wise maximum over ranks of per-rank times (the slowest replica sets
    the job's time); ``values`` unchanged on one process."""
    if dist is None:
        return [float(v) for v in values]
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def replica_throughput(units_per_rank, world, ms):
    """Whole-job units/s of ``world`` replicas that each processed
    ``units_per_rank`` units in ``ms`` (the maximum over ranks)."""
    return world * units_per_rank / (ms / 1e3)


def run_gpu(args):
    import torch

    from fluidimage_gb300 import WorkPIV, _lib, engine, workloads

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist_

        dist_.init_process_group("nccl")
        dist = dist_
    lib = _lib.load()

    (im0, im1), _ = workloads.config2_images(pair=rank, shape=(args.size, args.size))
    params = workloads.config2_params(WorkPIV.create_default_params())
    work = WorkPIV(params, device=dev)
    t0 = torch.from_numpy(im0.view(np.int16)).to(dev)
    t1 = torch.from_numpy(im1.view(np.int16)).to(dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    for _ in range(args.warmup):
        outs = work.calcul_device(t0, t1)
    torch.cuda.synchronize()
    nvec_final = outs[-1].layout.nvec

    timer = engine.KernelTimer()
    clocks = ClockSampler(local)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = lib.fi_launch_count()
    clocks.start()
    t_timed0 = time.perf_counter()
    step_ms = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        engine.TIMER = timer
        ev0.record()
        outs = work.calcul_device(t0, t1)
        ev1.record()
        engine.TIMER = None
        torch.cuda.synchronize()
        step_ms.append(ev0.elapsed_time(ev1))
    torch.cuda.synchronize()
    clk = clocks.stop(t_timed0, time.perf_counter())
    launches = lib.fi_launch_count() - launches0
    if dist is not None:
        dist.barrier()
    ms = statistics.mean(step_ms)

    # ---- the same step writing every correlation plane to device memory, as
    # upstream's HeavyPIVResults.correls holds them (keep_correls=True)
    work_planes = WorkPIV(params, device=dev, keep_correls=True)
    for _ in range(2):
        outs_p = work_planes.calcul_device(t0, t1)
    planes_ms = []
    for _ in range(5):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record()
        outs_p = work_planes.calcul_device(t0, t1)
        ev1.record()
        torch.cuda.synchronize()
        planes_ms.append(ev0.elapsed_time(ev1))
    planes_bytes = int(sum(pd.planes.numel() * pd.planes.element_size() for pd in outs_p
                           if pd.planes is not None))
    del outs_p, work_planes

    # ---- end to end through the public API (pinned host images -> host results)
    h0 = torch.from_numpy(im0.view(np.int16)).pin_memory()
    h1 = torch.from_numpy(im1.view(np.int16)).pin_memory()
    res = work.calcul({"arrays": (h0, h1), "names": ("im0", "im1")})
    d2h = _result_bytes(res)
    # one call per pair (WorkPIV.calcul), L2 flushed before each
    single_ms = []
    for _ in range(args.e2e_steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t_start = time.perf_counter()
        res = work.calcul({"arrays": (h0, h1), "names": ("im0", "im1")})
        torch.cuda.synchronize()
        single_ms.append(1e3 * (time.perf_counter() - t_start))
    # a series of pairs (WorkPIV.calcul_series: two pairs in flight, each on its own
    # host thread and CUDA stream, so that one pair's kernels fill the GPU while the
    # other waits on the host); four distinct pinned pairs in rotation
    # (circular shifts of the pair), each step moving > 0.5 GB of TPS matrices
    # through L2
    series = [(h0, h1)] + [
        (torch.from_numpy(np.roll(im0, 97 * k, axis=1).view(np.int16)).pin_memory(),
         torch.from_numpy(np.roll(im1, 97 * k, axis=1).view(np.int16)).pin_memory())
        for k in (1, 2, 3)]

    def couples(count):
        for i in range(count):
            yield {"arrays": series[i % len(series)], "names": ("im0", "im1")}

    for _ in work.calcul_series(couples(len(series))):
        pass
    n_series = max(args.e2e_steps, 32)
    torch.cuda.synchronize()
    t_start = time.perf_counter()
    for _ in work.calcul_series(couples(n_series)):
        pass
    torch.cuda.synchronize()
    series_ms = 1e3 * (time.perf_counter() - t_start) / n_series
    if dist is not None:
        dist.barrier()
    ms, series_ms, single_mean = max_over_ranks(
        [ms, series_ms, statistics.mean(single_ms)], dist, dev)
    value = replica_throughput(nvec_final, world, ms)
    e2e_value = replica_throughput(nvec_final, world, series_ms)
    single_value = replica_throughput(nvec_final, world, single_mean)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    kern = timer.summary()
    peaks, peak_kind = _peaks()
    roof = roofline(kern, outs, work, peaks, peak_kind)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (FFT correlation); TPS to f64 accuracy (double-float projection, f32 + 3xTF32 Cholesky, double-float refinement)",
        "data": "synthetic",
        "config": {"workload": WORKLOAD if args.size == 2048 else
                   WORKLOAD.replace("2048x2048", f"{args.size}x{args.size}"),
                   "pairs_per_step_per_gpu": 1,
                   "final_vectors_per_pair": nvec_final,
                   "l2": "512 MiB flush write between timed steps (untimed)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(im0.nbytes + im1.nbytes),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": series_ms,
                "api": f"WorkPIV.calcul_series over {n_series} pairs, 2 pairs in flight "
                       "(own host thread and CUDA stream each)",
                "single_call": {"value": single_value, "unit": UNIT,
                                "ms_per_step": single_mean,
                                "api": "WorkPIV.calcul, one pair per call, L2 flushed before"}},
        "gpu_launches": int(launches),
        "tps_subdomains": int(sum(t.nb_subdom for pd in outs for t in (pd.tps_next, pd.tps_final)
                                  if t is not None and hasattr(t, "nb_subdom"))),
        "tps_lu_fallbacks": int(sum(int(t.mp_status.sum().item()) for pd in outs
                                    for t in (pd.tps_next, pd.tps_final) if t is not None)),
        "tps_outer_iterations": _iter_stats(outs),
        "kernels": {k: {kk: round(vv, 4) for kk, vv in v.items()} for k, v in kern.items()},
        "roofline": roof,
        "correlation": pass_lines(kern, outs, work),
        "planes_kept": {"ms_per_step": statistics.mean(planes_ms),
                        "plane_bytes_per_step": planes_bytes,
                        "note": "the timed step with every correlation plane written to "
                                "device memory (keep_correls=True; upstream keeps them in "
                                "HeavyPIVResults.correls); not part of value"},
        "clocks": clk,
    }
    if not args.no_precision_sweep:
        line["precision_sweep"] = precision_sweep(args, dev, flush, peaks, peak_kind)
    line["window_sizes"] = window_size_passes(args, dev)
    if not args.no_batched:
        line["batched"] = batched_workload(args, dev, flush)
    if not args.no_refinement:
        line["refinement"] = refinement_workload(args, dev)
    if not args.no_cpu_baseline:
        line["accuracy_vs_fp64"] = accuracy_vs_fp64(res, im0, im1, params)
        line["cpu_baseline"] = cpu_baseline_single()
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def _iter_stats(outs):
    """Outlier-replacement solves per subdomain and component (and refinement sweeps
    of the mixed-precision solver), per TPS call."""
    stats = []
    for pd in outs:
        for t in (pd.tps_next, pd.tps_final):
            if t is not None:
                it = t.iters.cpu().numpy()
                st = {"subdomains": t.nb_subdom, "mean": round(float(it.mean()), 2),
                      "max": int(it.max())}
                if t.mp_sweeps is not None:
                    sw = t.mp_sweeps.cpu().numpy()
                    st["refine_sweeps_mean"] = round(float(sw.mean()), 2)
                    st["refine_sweeps_max"] = int(sw.max())
                stats.append(st)
    return stats


def _result_bytes(res):
    total = 0
    for r in res.passes:
        for v in vars(r).values():
            if isinstance(v, np.ndarray):
                total += v.nbytes
    return total


def _tps_calls(outs):
    return [t for pd in outs for t in (pd.tps_next, pd.tps_final)
            if t is not None and hasattr(t, "nb_subdom")]


def roofline(kern, outs, work, peaks, peak_kind):
    """Roofline of the dominant library entry point (largest total time in the timed
    steps), from its algorithmic bytes per launch and its CUDA-event time per
    launch, against the measured HBM copy bandwidth."""
    name, stats = max(kern.items(), key=lambda kv: kv[1]["total_ms"])
    avg_s = stats["avg_ms"] / 1e3
    peak = float(peaks["hbm_gbs"])
    if name in ("fi_tps_solve", "fi_tps_solve_mp"):
        import torch

        calls = _tps_calls(outs)
        # algorithmic bytes: one write and one read of each subdomain's
        # (N+3) x (N+3) system at 8 bytes per entry (the reference's FP64 matrix)
        nbytes = sum(float((16.0 * (t.counts.astype(np.float64) + 3) ** 2).sum())
                     for t in calls)
        per_launch = nbytes / max(len(calls), 1)
        achieved = per_launch / avg_s / 1e9
        # DRAM bytes per subdomain from ncu captures of this kernel (one per launch
        # shape), times the subdomains of each launch, averaged over the launches
        nsm = torch.cuda.get_device_properties(0).multi_processor_count
        traffic = sum(
            t.nb_subdom * (TPS_DRAM_BYTES_PER_SUBDOMAIN_WIDE if t.nb_subdom <= nsm
                           else TPS_DRAM_BYTES_PER_SUBDOMAIN_NARROW)
            for t in calls) / max(len(calls), 1)
        # the reference's work for the same solves (FP64 LU, 2/3 (N+3)^3 flops per
        # solve and outlier iteration): a speed note, not a roofline
        lu = 0.0
        for t in calls:
            it = t.iters.cpu().numpy().reshape(-1, 2).sum(axis=1)
            lu += float((2.0 / 3.0 * (t.counts.astype(np.float64) + 3) ** 3 * it).sum())
        return {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "algorithmic_bytes_per_launch": per_launch,
                "work": "one write + one read of each subdomain's (N+3)^2 system at 8 B "
                        "per entry, per launch",
                "traffic_source": "ncu dram__bytes_read+write per subdomain (captures of "
                                  "both launch shapes) x subdomains, per launch",
                "peak_source": f"hbm_gbs of MEASURED_PEAKS.json ({peak_kind})",
                "note": "latency-bound kernel (block-synchronous 32-wide tile steps); "
                        "reference-equivalent FP64 LU rate "
                        f"{lu / max(len(calls), 1) / avg_s / 1e12:.2f} TFLOP/s",
                "avg_ms": stats["avg_ms"], "launches": stats["launches"]}
    H, W = work._pipelines[next(iter(work._pipelines))].imshape
    per_launch = 2.0 * H * W * 2
    achieved = per_launch / avg_s / 1e9
    return {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": None,
            "peak_source": f"hbm_gbs of MEASURED_PEAKS.json ({peak_kind})",
            "avg_ms": stats["avg_ms"], "launches": stats["launches"]}


def pass_lines(kern, outs, work):
    """Per correlation pass (one window size): windows, time, FP32 FFT work rate
    and unique image bytes rate (CUDA events around each launch)."""
    import torch

    H, W = work._pipelines[next(iter(work._pipelines))].imshape
    props = torch.cuda.get_device_properties(0)
    lines = []
    for pd in outs:
        n = pd.layout.n
        st = kern.get(f"fi_piv_pass[n={n}]")
        if st is None:
            continue
        s = st["avg_ms"] / 1e3
        nwin = pd.layout.nvec
        lines.append({
            "n": n, "windows": nwin, "ms": st["avg_ms"],
            "fp32_tflops": nwin * fft_flops(n) / s / 1e12,
            "image_gbs": 2.0 * H * W * 2 / s / 1e9,
            "vectors_per_s": nwin / s,
        })
    # nominal FP32 FMA rate of the SMs (128 lanes x 2 flops x max clock)
    clock = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("sm_max_mhz", 2070.0) \
        if (ROOT / "MEASURED_PEAKS.json").exists() else 2070.0
    fp32_peak = props.multi_processor_count * 128 * 2 * clock * 1e6 / 1e12
    for ln in lines:
        ln["fp32_frac_of_nominal"] = ln["fp32_tflops"] / fp32_peak
    return {"fp32_nominal_tflops": fp32_peak, "passes": lines}


TC_FORMS = ("fp32_fft", "bf16x1", "bf16x3", "fp16x3")


def precision_sweep(args, dev, flush, peaks, peak_kind, accuracy=True):
    """The plain FP32 FFT pass against the tensor-core DFT pass in its three forms on
    the precision-sweep workload: one 4096^2 uint16 pair, 32 px windows at overlap
    0.75 (259 081 vectors), sinusoidal displacement, WorkFIX and the final TPS.
    Per form: the correlation pass alone and the whole step (device-resident
    images, CUDA events, L2 flushed between steps), the tensor pipe's executed
    flops, and the error against the FP64 oracle on a 4096 x 768 band."""
    import torch

    from fluidimage_gb300 import WorkPIV, engine, workloads
    from oracle import accuracy as A

    shape = (args.sweep_size, args.sweep_size)
    (im0, im1), _ = workloads.config4_images(shape=shape)
    t0 = torch.from_numpy(im0.view(np.int16)).to(dev)
    t1 = torch.from_numpy(im1.view(np.int16)).to(dev)
    band = (slice(0, 768), slice(None))
    b0, b1 = np.ascontiguousarray(im0[band]), np.ascontiguousarray(im1[band])
    params_ref = workloads.config4_params(WorkPIV.create_default_params())
    ref = A.fp64_multipass(b0, b1, params_ref) if accuracy else None
    out = {"workload": f"{shape[0]}x{shape[1]} uint16 12-bit, density 0.06, diameter 2.5 px, noise 1 %, "
                       "d = 5 (sin 2 pi y/512, cos 2 pi x/512) px, 32 px windows overlap 0.75, "
                       "WorkFIX thr 2, final TPS subdom 256",
           "accuracy_band": "rows 0-767 (all columns)", "forms": {}}
    steps = max(1, min(args.steps, 10))
    forms = [f for f in args.forms.split(",") if f]
    for form in forms:
        params = workloads.config4_params(WorkPIV.create_default_params())
        params.piv0.method_correl = "gb300" if form == "fp32_fft" else f"gb300_tc_{form}"
        work = WorkPIV(params, device=dev)
        for _ in range(max(1, args.warmup)):
            outs = work.calcul_device(t0, t1)
        torch.cuda.synchronize()
        timer = engine.KernelTimer()
        step_ms = []
        for _ in range(steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            engine.TIMER = timer
            e0.record()
            outs = work.calcul_device(t0, t1)
            e1.record()
            engine.TIMER = None
            torch.cuda.synchronize()
            step_ms.append(e0.elapsed_time(e1))
        kern = timer.summary()
        name = "fi_piv_pass[n=32]" if form == "fp32_fft" else "fi_piv_pass_tc[n=32]"
        pass_ms = kern[name]["avg_ms"]
        nvec = outs[0].layout.nvec
        entry = {"pass_ms": pass_ms, "pass_vectors_per_s": nvec / (pass_ms / 1e3),
                 "step_ms": statistics.mean(step_ms),
                 "step_vectors_per_s": nvec / (statistics.mean(step_ms) / 1e3),
                 "vectors": nvec}
        if form == "fp32_fft":
            entry["fp32_tflops"] = nvec * fft_flops(32) / (pass_ms / 1e3) / 1e12
        else:
            terms = 1 if form == "bf16x1" else 3
            # executed dense MMA flops per window: 4 stages of M 128 tiles over 8
            # windows: 2 x (2 x 2 x 128 x 32 x 32) + 2 x 128 x 64 x 64 x 2 +
            # 2 x 128 x 64 x 64 + 2 x 2 x 128 x 32 x 32, per term
            flops = terms * (2 * 2 * 2 * 128 * 32 * 32 + 2 * 2 * 128 * 64 * 64
                             + 2 * 128 * 64 * 64 + 2 * 2 * 128 * 32 * 32) / 8
            achieved = nvec * flops / (pass_ms / 1e3) / 1e12
            entry.update({"tensor_tflops_executed": achieved,
                          "tensor_frac_of_bf16_peak": achieved / float(peaks["bf16_tflops"]),
                          "peak_source": f"bf16_tflops of MEASURED_PEAKS.json ({peak_kind})",
                          "mma_flops_per_window": flops})
        if accuracy:
            wb = WorkPIV(params, device=dev)
            resb = wb.calcul({"arrays": (b0, b1), "names": ("im0", "im1")})
            acc = A.summary(resb.passes, ref)
            acc.pop("passes", None)
            entry["accuracy_vs_fp64"] = acc
        out["forms"][form] = entry
    base = out["forms"].get("fp32_fft")
    for form in forms:
        if form == "fp32_fft" or base is None:
            continue
        f = out["forms"][form]
        f["pass_speedup_vs_fp32_fft"] = base["pass_ms"] / f["pass_ms"]
        f["step_speedup_vs_fp32_fft"] = base["step_ms"] / f["step_ms"]
    return out


def batched_workload(args, dev, flush):
    """The batched heterogeneous workload: 256 single-pass jobs, image sizes drawn from
    512^2, 1024x768, 2048^2, 4096x2160 (4 distinct uint16 pairs each), windows from
    16-64 px, overlap 0.5 or 0.75, WorkFIX.  One pair at a time
    (WorkPIV.calcul_device per pair, the schedule of the multipass workload) against
    PIVBatch (one persistent launch per window size, batched minima and WorkFIX)
    launched directly, after its autotuner, and replayed as a CUDA graph.
    Device-resident images, CUDA events, L2 flushed between steps."""
    import torch

    from fluidimage_gb300 import PIVBatch, WorkPIV, _lib, workloads

    t_gen = time.perf_counter()
    jobs, draws = workloads.config3_jobs(WorkPIV.create_default_params)
    gen_s = time.perf_counter() - t_gen
    dev_pairs, djobs = {}, []
    for im0, im1, params in jobs:
        if id(im0) not in dev_pairs:
            dev_pairs[id(im0)] = (torch.from_numpy(im0.view(np.int16)).to(dev),
                                  torch.from_numpy(im1.view(np.int16)).to(dev))
        djobs.append((*dev_pairs[id(im0)], params))
    works = [WorkPIV(p, device=dev, interp_last=False) for _, _, p in djobs]
    steps = max(3, min(args.steps, 10))

    def timed(fn):
        for _ in range(max(1, args.warmup)):
            fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return statistics.mean(ms)

    def one_at_a_time():
        for w, (t0, t1, _) in zip(works, djobs):
            w.calcul_device(t0, t1)

    ms_single = timed(one_at_a_time)
    batch = PIVBatch(djobs, device=dev)
    ms_launch = timed(batch.run)
    tuning = batch.autotune()
    ms_tuned = timed(batch.run)
    batch.capture()
    ms_graph = timed(batch.run)
    nvec = batch.total_vectors
    lib = _lib.load()
    launches0 = lib.fi_launch_count()
    batch.launches()
    torch.cuda.synchronize()
    per_run = lib.fi_launch_count() - launches0
    return {
        "workload": "256 single-pass jobs over 16 distinct uint16 12-bit pairs (4 per size "
                    "512^2, 1024x768, 2048^2, 4096x2160), windows 16/24/32/48/64, overlap "
                    "0.5/0.75, WorkFIX; uniform shifts or 4-Oseen superpositions (<= 6 px)",
        "jobs_per_window_size": {str(n): sum(1 for d in draws if d[1] == n)
                                 for n in sorted({d[1] for d in draws})},
        "vectors": nvec, "image_generation_s": round(gen_s, 1),
        "one_at_a_time": {"ms": ms_single, "vectors_per_s": nvec / (ms_single / 1e3),
                          "api": "WorkPIV.calcul_device per pair"},
        "batched": {"ms": ms_launch, "vectors_per_s": nvec / (ms_launch / 1e3)},
        "batched_autotuned": {"ms": ms_tuned, "vectors_per_s": nvec / (ms_tuned / 1e3),
                              "choices": {str(k): v for k, v in tuning.items()}},
        "batched_graph": {"ms": ms_graph, "vectors_per_s": nvec / (ms_graph / 1e3),
                          "kernel_launches_per_run": int(per_run)},
        "speedup_graph_vs_one_at_a_time": ms_single / ms_graph,
    }


def refinement_workload(args, dev, pairs=8, steps=20):
    """Deform-and-correlate refinement: 8 pairs 2048^2 (float32 images, Oseen plus
    sinusoid field of peak 7 px); the plain 3-pass PIV (the multipass workload's
    parameters) gives the node field (64 x 64 x 2 per pair, the final field at the
    32 px node grid), then 20 Adam steps (lr 0.05 px) on the mean squared soft-argmax
    residual of the 32 x 32 windows (temperature 0.1), all pairs in one batch.  RMS
    error against the imposed field at the inner nodes, and the device time of each
    stage (CUDA events)."""
    import torch

    from fluidimage_gb300 import WorkPIV, deform, workloads

    shape = (2048, 2048)
    xn, yn = deform.node_grid(*shape)
    ims0, ims1, truth = [], [], []
    for k in range(pairs):
        (a, b), field = workloads.config5_images(pair=k, shape=shape)
        ims0.append(a)
        ims1.append(b)
        gx, gy = np.meshgrid(xn.astype(np.float64), yn.astype(np.float64))
        truth.append(np.stack(field(gx, gy)))
    t0 = torch.as_tensor(np.array(ims0), device=dev)
    t1 = torch.as_tensor(np.array(ims1), device=dev)
    truth = torch.as_tensor(np.array(truth, dtype=np.float32), device=dev)
    txn, tyn = torch.as_tensor(xn, device=dev), torch.as_tensor(yn, device=dev)
    params = workloads.config2_params(WorkPIV.create_default_params())
    work = WorkPIV(params, device=dev)
    work_deform = WorkPIV(params, device=dev, deform=True)

    def plain(w=work):
        nodes = []
        for k in range(pairs):
            outs = w.calcul_device(t0[k], t1[k])
            fin = outs[-1].tps_final
            lay = outs[-1].layout
            fx = fin.out_x.view(lay.iyvecs.size, lay.ixvecs.size)[1::4, 1::4]
            fy = fin.out_y.view(lay.iyvecs.size, lay.ixvecs.size)[1::4, 1::4]
            nodes.append(torch.stack([fx, fy]).float())
        return torch.stack(nodes).contiguous()

    for _ in range(max(1, args.warmup)):
        nodes0 = plain()
        plain(work_deform)
        deform.refine(nodes0, t0, t1, txn, tyn, steps=2)
    torch.cuda.synchronize()

    def timed(f):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = f()
        e1.record()
        torch.cuda.synchronize()
        return out, e0.elapsed_time(e1)

    inner = (slice(None), slice(None), slice(2, -2), slice(2, -2))

    def rms(n):
        return float(((n - truth)[inner] ** 2).sum(dim=1).mean().sqrt())

    nodes0, ms_plain = timed(plain)
    nodes_d, ms_deform = timed(lambda: plain(work_deform))
    frontier = [{"form": "3-pass window shift", "ms": ms_plain, "rms_px": rms(nodes0)},
                {"form": "3-pass deformation (central)", "ms": ms_deform, "rms_px": rms(nodes_d)}]
    refined = {}
    for k in sorted({5, 10, steps}):
        nodes_k, ms_k = timed(lambda: deform.refine(nodes0, t0, t1, txn, tyn, steps=k, lr=0.05))
        refined[k] = (nodes_k, ms_k)
        frontier.append({"form": f"3-pass window shift + {k} Adam steps", "ms": ms_plain + ms_k,
                         "rms_px": rms(nodes_k)})
    return {
        "workload": f"{pairs} pairs 2048x2048 float32 (uint16 12-bit particles), Oseen + "
                    "sinusoid field of peak 7 px; nodes 64x64x2 per pair at the 32 px window "
                    "centres; loss mean |soft-argmax residual|^2 of the 32 px windows, T 0.1",
        "plain_3pass_ms": ms_plain,
        "refine_ms": refined[steps][1], "adam_steps": steps,
        "rms_error_px": {"plain_3pass": rms(nodes0), "refined": rms(refined[steps][0])},
        "time_vs_error": frontier,
        "error_note": "vector error |d - truth| at the inner nodes (2-node margin); times are "
                      "device times of all 8 pairs (CUDA events)",
    }


def run_refinement_only(args):
    import torch

    print(json.dumps(refinement_workload(args, torch.device("cuda"))), flush=True)


def run_batched_only(args):
    """The batched heterogeneous workload alone, one JSON line."""
    import torch

    dev = torch.device("cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    print(json.dumps(batched_workload(args, dev, flush)), flush=True)


def accuracy_vs_fp64(res, im0, im1, params):
    """The timed result against the FP64 oracle (the checker)."""
    from oracle import accuracy as A

    t0 = time.perf_counter()
    ref = A.fp64_multipass(im0, im1, params)
    acc = A.summary(res.passes, ref)
    acc.pop("passes", None)
    acc["oracle_seconds"] = round(time.perf_counter() - t0, 1)
    return acc


def run_preproc(args):
    """Preprocessing tools on 2048^2 uint16 frames of the config-2 images: device
    throughput (CUDA events, L2 flushed between steps) next to the scipy oracle on
    a 512^2 crop (one thread)."""
    import torch

    from fluidimage_gb300 import preproc as P, workloads

    (im0, im1), _ = workloads.config2_images(shape=(args.size, args.size))
    frames = np.array([im0, im1] * 4)  # 8 frames for the temporal tool
    dev = torch.device("cuda")
    t_img = P.to_device(im0, dev)
    t_stack = P.to_device(frames, dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    cases = [
        ("sliding_minima", dict(window_size=30), t_img, im0),
        ("sliding_median", dict(window_size=30), t_img, im0),
        ("temporal_minima", dict(), t_stack, frames),
        ("sharpen", dict(), t_img, im0),
        ("equalize_hist_adapt", dict(), t_img, im0),
        ("equalize_hist_local", dict(radius=10), t_img, im0),
    ]
    out = {"metric": "preprocessing Mpixel/s", "unit": "Mpixel/s", "workload":
           f"{args.size}x{args.size} uint16 frames of the config-2 pair", "tools": {}}
    for name, kw, t, host in cases:
        fn = getattr(P, name)
        for _ in range(max(args.warmup, 1)):
            fn(t, **kw)
        torch.cuda.synchronize()
        ms = []
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn(t, **kw)
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        npx = t.numel()
        gpu = npx / (statistics.median(ms) / 1e3) / 1e6
        code = ("import sys, time, json, numpy as np; sys.path.insert(0, %r); "
                "from oracle import preproc as O; a = np.load(sys.argv[1]); "
                "t0 = time.perf_counter(); getattr(O, %r)(a, **json.loads(sys.argv[2])); "
                "print(a.size / (time.perf_counter() - t0) / 1e6)" % (str(ROOT), name))
        crop = host[..., :512, :512]
        path = Path(tempfile.gettempdir()) / f"_preproc_{name}_{os.getpid()}.npy"
        np.save(path, np.ascontiguousarray(crop))
        env = dict(os.environ, OMP_NUM_THREADS="1")
        cpu = float(subprocess.run([sys.executable, "-c", code, str(path), json.dumps(kw)],
                                   capture_output=True, text=True, env=env,
                                   check=True).stdout.strip())
        path.unlink()
        out["tools"][name] = {"gpu_mpixel_s": gpu, "ms_per_call": statistics.median(ms),
                              "cpu_baseline_mpixel_s": cpu, "cpu_cores": 1,
                              "cpu_sample": "512x512 crop, scipy oracle"}
    print(json.dumps(out), flush=True)


def window_size_passes(args, dev, sizes=(8, 12, 16, 24, 32, 48, 64), reps=10):
    """One FP32 pass (with WorkFIX) per window size on the 2048^2 pair of the
    multipass workload, overlap 0.5, no interpolation: the window count, the best of
    ``reps`` CUDA-event timings and the time per window."""
    import torch

    from fluidimage_gb300 import WorkPIV, workloads

    (im0, im1), _ = workloads.config2_images(pair=0, shape=(args.size, args.size))
    d0 = torch.as_tensor(im0.view(np.int16), device=dev)
    d1 = torch.as_tensor(im1.view(np.int16), device=dev)
    out = {}
    for n in sizes:
        params = WorkPIV.create_default_params()
        params.piv0.shape_crop_im0 = n
        params.multipass.number = 1
        params.multipass.use_tps = False
        params.fix.threshold_diff_neighbour = None
        work = WorkPIV(params, device=dev, interp_last=False)
        for _ in range(3):
            work.calcul_device(d0, d1)
        torch.cuda.synchronize()
        nvec = work._pipelines[next(iter(work._pipelines))].layouts[0].nvec
        times = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            work.calcul_device(d0, d1)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        ms = min(times)
        out[str(n)] = {"windows": nvec, "ms": ms, "ns_per_window": ms * 1e6 / nvec}
    return {"workload": f"one {args.size}x{args.size} uint16 pair, single FP32 pass + WorkFIX "
                        "per window size, overlap 0.5", "passes": out}


def run_window_sizes_only(args):
    import torch

    sizes = tuple(int(v) for v in args.window_sizes.split(","))
    print(json.dumps(window_size_passes(args, torch.device("cuda"), sizes)), flush=True)


def run_sweep_only(args):
    """The precision sweep alone (no accuracy check), one JSON line."""
    import torch

    dev = torch.device("cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    peaks, peak_kind = _peaks()
    out = precision_sweep(args, dev, flush, peaks, peak_kind, accuracy=False)
    print(json.dumps(out), flush=True)


def main():
    args = parse_args()
    if args.preproc:
        run_preproc(args)
    elif args.sweep_only:
        run_sweep_only(args)
    elif args.batched_only:
        run_batched_only(args)
    elif args.refinement_only:
        run_refinement_only(args)
    elif args.window_sizes:
        run_window_sizes_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
