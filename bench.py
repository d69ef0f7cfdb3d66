#!/usr/bin/env python3
"""Benchmark of the GB300 strip-PET list-mode TOF MLEM iteration.

One step = one MLEM iteration over every event of the workload (default: the
full-size plain case, 500 x 450 pixels at 2 mm, 2e7 events from a seeded
10-ellipse phantom).  Prints one JSON line.

  value   event-iterations/s with the events already prepared in HBM (device
          time of K iterations, CUDA events on the library's stream)
  e2e     the same metric through the C ABI with host buffers: each e2e step
          uploads the events from pinned host memory, prepares them, runs the
          workload's iteration count from a uniform image and reads the image
          back (jpet_strip_run's work), timed on the host
  roofline  kernel-pixel evaluations/s against the measured ex2 (SFU) rate:
          the iteration evaluates one exp per in-ellipse pixel
  cpu_baseline  the CPU restatement of the reference's OpenMP path on this
          host's cores, on a bounded sample of the same events

--impl reference times that CPU path alone (the reference GPU backend does not
compile with CUDA >= 12, so the reference's CPU float path is the reference).
Multi-GPU (torchrun): every rank runs an independent replica (the path has no
exchange step); value is the sum over ranks / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "j-pet-mlem_gb300")
sys.path.insert(0, os.path.join(PKG, "python"))

METRIC = ("event·iterations/sec and kernel-pixel evals/sec at stated L2 tol vs FP64; "
          "% SFU/atomic roofline")
UNIT = "event·iterations/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="plain-2mm-20M")
    p.add_argument("--events", type=int, default=0, help="override the event count")
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-peaks", action="store_true", help="skip the peak microbenchmarks")
    p.add_argument("--no-batch", action="store_true",
                   help="skip the batched form (64 reconstructions per graph launch)")
    p.add_argument("--batch-instances", type=int, default=64)
    p.add_argument("--no-adjoint", action="store_true",
                   help="skip the differentiable form (adjoint throughput and calibration)")
    p.add_argument("--sample-events", type=int, default=1_000_000,
                   help="events of the FP64-oracle prefix in the precision report")
    p.add_argument("--no-accuracy", action="store_true",
                   help="skip the accuracy entry (stated configurations vs the oracles)")
    p.add_argument("--no-precision", action="store_true",
                   help="skip the precision entry (every accumulation mode vs FP64)")
    p.add_argument("--accuracy-events", type=int, default=2_000_000,
                   help="events of the prefix iterated against the reference float path")
    p.add_argument("--accuracy-report", action="store_true",
                   help="every iteration of the full workload against the FP64 GPU iteration")
    p.add_argument("--calibration-report", action="store_true",
                   help="blind width recalibration on the differentiable configuration")
    p.add_argument("--adjoint-report", action="store_true",
                   help="the adjoint entry alone (loss + gradient timing, no calibration)")
    p.add_argument("--adjoint-events", type=int, default=5_000_000)
    p.add_argument("--no-hybrid", action="store_true",
                   help="skip the 3D hybrid entry (384-detector ring, 200x200x125 voxels)")
    p.add_argument("--hybrid-events", type=int, default=10_000_000)
    p.add_argument("--hybrid-report", action="store_true",
                   help="the 3D hybrid entry alone")
    p.add_argument("--precision-report", action="store_true",
                   help="print the precision-stress comparison instead of the headline line")
    p.add_argument("--fp64-iterations", type=int, default=0,
                   help="precision report: compare the full-scale images with the FP64 GPU "
                        "iteration after this many iterations (default: all of them)")
    p.add_argument("--variant", type=int, default=0,
                   help="0 fast row-owned kernel, 1 exact kernel, 2 fast warp-per-event kernel")
    p.add_argument("--block-threads", type=int, default=0,
                   help="threads per CTA of the iteration kernel (0 = default)")
    p.add_argument("--raster-shape", type=int, default=0,
                   help="register shape of the fast kernel (0 auto, 1..6 = 8x1x1 .. 4x2x4)")
    p.add_argument("--precision", type=int, default=0,
                   help="0 FP32 tile sums, 1 compensated tile sums, 2 plus FP64 denominators, "
                        "3 fixed-point tile sums")
    return p.parse_args()


def config_of(wl, n_events, world):
    """The workload description both arms print."""
    return {"workload": wl.name, "events": n_events, "grid": f"{wl.n_z}x{wl.n_y}",
            "pixel_mm": wl.pixel, "sigma_z": wl.sigma_z, "sigma_dl": wl.sigma_dl,
            "phantom": wl.phantom, "seed": wl.seed,
            "l2": "inputs larger than L2 (prepared events and row tables, ~160 B each)",
            "parallelism": f"replicas{world}"}


def replica_value(local_ms, n_events, steps, world, device="cpu"):
    """Whole-job throughput of N independent replicas: every rank processed
    n_events per step; the job takes as long as the slowest rank (max over
    ranks of the timed region).  Returns (max_ms, event-iterations/s)."""
    import torch

    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    max_ms = float(t.item())
    return max_ms, world * n_events * steps / (max_ms * 1e-3)


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(device), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(smax),
                "power_w_max": max(power), "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks(device: int):
    lib = C.CDLL(os.path.join(PKG, "lib", "libjpet_peaks.so"))
    out = (C.c_double * 12)()
    rc = lib.jpet_peaks_measure(device, out)
    if rc != 0:
        raise RuntimeError(f"peak microbenchmark failed: {rc}")
    return {"ex2_per_s": out[0], "ffma_per_s": out[1], "shared_atomic_per_s": out[2],
            "global_atomic_per_s": out[3], "sms": int(out[4]), "sm_clock_khz": int(out[5]),
            "shared_atomic_u32_per_s": out[6], "shared_atomic_u64_per_s": out[7],
            "shared_rmw_per_s": out[8], "global_atomic_v4_floats_per_s": out[9],
            "global_atomic_v2_floats_per_s": out[10], "shared_ld64_floats_per_s": out[11]}


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_sample_rate(wl, events, budget_s: float, threads: int):
    """Times the CPU restatement of the reference's OpenMP path (one iteration
    from a uniform image) on a prefix of the events sized to ~budget_s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    og = oracle.Geometry(*wl.geometry_args())
    probe = min(len(events), 20000)
    t = time.perf_counter()
    oracle.mlem_f(og, events[:probe], 1, threads=threads, release=True)
    dt = max(time.perf_counter() - t, 1e-3)
    n = int(min(len(events), max(probe, probe * budget_s / dt)))
    t = time.perf_counter()
    _, st = oracle.mlem_f(og, events[:n], 1, threads=threads, release=True)
    dt = time.perf_counter() - t
    return n, dt, st


def reference_arm(args, wl, world, rank):
    if rank != 0:
        return
    import numpy as np

    threads = os.cpu_count() or 1
    n_all = args.events or wl.n_events
    # the events the GPU arm iterates (the same generator, seed and count; the
    # seeded CPU generator where no GPU is present), then a prefix sized so
    # that each step is a few seconds of the CPU path
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    try:
        import torch

        gpu = torch.cuda.is_available()
    except ImportError:
        gpu = False
    all_ev = wl.events(n_all, device=0 if gpu else None)
    og = oracle.Geometry(*wl.geometry_args())
    probe_ev = all_ev[:min(n_all, 20000)]
    t = time.perf_counter()
    oracle.mlem_f(og, probe_ev, 1, threads=threads, release=True)
    rate = len(probe_ev) / max(time.perf_counter() - t, 1e-3)
    budget = max(2.0, 120.0 / max(1, args.steps + args.warmup))
    n = int(min(n_all, max(len(probe_ev), rate * budget)))
    ev = np.ascontiguousarray(all_ev[:n])
    del all_ev
    rho = None
    for _ in range(args.warmup):
        rho, _ = oracle.mlem_f(og, ev, 1, rho, threads=threads, release=True)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        rho, st = oracle.mlem_f(og, ev, 1, rho, threads=threads, release=True)
        times.append(time.perf_counter() - t)
    total = sum(times)
    value = n * args.steps / total
    evals = st["n_kernel_calls"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_of(wl, n_all, world),
        "kernel_pixel_evals_per_s": evals * args.steps / total,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "build": "oracle/liboracle_strip_release.so (-O3, OpenMP, FMA contraction)",
                         "sample": f"first {n} of the {n_all} events the GPU arm iterates "
                                   f"({'GPU' if gpu else 'CPU'} generator, seed {wl.seed}), "
                                   f"one iteration per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def gb300_arm(args, wl, world, rank, local):
    import numpy as np
    import torch

    from jpet_strip import capi

    torch.cuda.set_device(local)
    if world > 1 and not torch.distributed.is_initialized():
        torch.distributed.init_process_group("nccl")
    n_events = args.events or wl.n_events
    events = wl.events(n_events, device=local)
    geom = capi.Geometry(*wl.geometry_args())
    peaks = None if args.no_peaks else measured_peaks(local)
    stream = torch.cuda.Stream()
    rec = capi.StripReconstruction(geom, device=local, variant=args.variant,
                                   precision=args.precision, raster_shape=args.raster_shape,
                                   block_threads=args.block_threads)
    rec.set_stream(stream.cuda_stream)
    rec.set_events(events)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            rec.iterate(1)
    rec.synchronize()
    counters = rec.counters()
    evals_per_iter = counters["n_kernel_calls"]
    launches_per_iter = 1 + (1 if counters["n_oversize"] > 0 else 0)

    clocks = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    for k in range(args.steps):
        starts[k].record(stream)
        rec.iterate(1)
        ends[k].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    per_step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms, value = replica_value(starts[0].elapsed_time(ends[-1]), n_events, args.steps,
                                    world, device="cuda")
    kernel_ms = statistics.mean(per_step_ms)
    evals_per_s = evals_per_iter / (kernel_ms * 1e-3)

    # accuracy at the stated configurations, and the CPU baseline
    accuracy = None
    cpu = None
    precision = None
    kopts = dict(variant=args.variant, precision=args.precision, raster_shape=args.raster_shape,
                 block_threads=args.block_threads)
    if rank == 0:
        if not args.no_accuracy:
            accuracy = accuracy_report(args, wl, geom, events, local, kopts)
        if not args.no_precision:
            precision = precision_modes(wl, geom, events, local)
        if not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            n, dt, st = cpu_sample_rate(wl, events, args.cpu_seconds, threads)
            cpu = {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
                   "build": "oracle/liboracle_strip_release.so (-O3, OpenMP, FMA contraction)",
                   "sample": f"first {n} of the {n_events} events the GPU arm iterates, "
                             f"one iteration from a uniform image",
                   "kernel_pixel_evals_per_s": st["n_kernel_calls"] / dt}

    # end to end through the C ABI with host buffers (pinned)
    pinned = torch.empty((n_events, 3), dtype=torch.float32, pin_memory=True)
    pinned.numpy()[:] = events
    ones = np.ones((wl.n_y, wl.n_z), np.float32)
    e2e_times = []
    host_img = None
    for k in range(args.e2e_steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rec.set_events(pinned.numpy())
        rec.rho = ones
        rec.iterate(wl.iterations)
        host_img = rec.rho
        t1 = time.perf_counter()
        if k > 0:
            e2e_times.append(t1 - t0)
    e2e_s = max(e2e_times) if world == 1 else max(e2e_times)
    e2e_value = world * n_events * wl.iterations / (sum(e2e_times) / len(e2e_times))
    rec.close()

    if rank != 0:
        return
    batched = None
    if not args.no_batch:
        try:
            batched = batch_summary(local, k=args.batch_instances)
        except Exception as exc:  # reported, the headline line still prints
            batched = {"error": f"{type(exc).__name__}: {exc}"}
    adjoint = None
    if not args.no_adjoint:
        try:
            adjoint = adjoint_summary(local, ex2_peak=(peaks or {}).get("ex2_per_s"))
        except Exception as exc:  # reported, the headline line still prints
            adjoint = {"error": f"{type(exc).__name__}: {exc}"}
    hybrid = None
    if not args.no_hybrid:
        try:
            hybrid = hybrid_summary(local, args.hybrid_events,
                                    sm_mhz=(clk or {}).get("sm_mhz"))
        except Exception as exc:  # reported, the headline line still prints
            hybrid = {"error": f"{type(exc).__name__}: {exc}"}
    hbm, hbm_kind = hbm_peak()
    roofline = None
    if peaks:
        ex2_peak = peaks["ex2_per_s"]
        atom_peak = peaks["shared_atomic_per_s"]
        if args.variant in (0, 3):
            # batch-union and row-owned kernels: one exp per kernel-pixel
            # evaluation and no shared-memory atomics (plain read-modify-write
            # of owned pixels)
            bound_sfu = True
        else:
            # one exp and one shared-memory float atomic per evaluation: the
            # lower of the two peaks binds
            bound_sfu = ex2_peak <= atom_peak
        peak = ex2_peak if bound_sfu else atom_peak
        roofline = {"bound": "sfu" if bound_sfu else "shared_atomic",
                    "achieved": evals_per_s / 1e9, "peak": peak / 1e9,
                    "unit": "Gex2/s" if bound_sfu else "Gatomic/s",
                    "frac": evals_per_s / peak,
                    "peak_source": "measured on this GPU by libjpet_peaks (ex2.approx and "
                                   "shared float atomicAdd throughput)",
                    "traffic": profile_traffic(n_events, variant=args.variant),
                    "sfu_frac": evals_per_s / ex2_peak,
                    "shared_atomic_frac": evals_per_s / atom_peak,
                    "hbm_peak_gbs": hbm, "hbm_peak_source": hbm_kind}
        if args.variant in (0, 3):
            traffic = profile_traffic(n_events, variant=args.variant)
            insts = profile_traffic(n_events, "warp_instructions_per_launch", args.variant)
            if traffic:
                roofline["hbm_achieved_gbs"] = traffic / (kernel_ms * 1e-3) / 1e9
                roofline["hbm_frac"] = roofline["hbm_achieved_gbs"] / hbm
            sm_mhz = (clk or {}).get("sm_mhz") or (clk or {}).get("sm_max_mhz")
            if insts and sm_mhz:
                # 4 warp schedulers per SM issue one warp instruction per clock each
                n_sm = torch.cuda.get_device_properties(local).multi_processor_count
                issue_peak = 4 * n_sm * sm_mhz * 1e6
                roofline["issue_frac"] = insts / (kernel_ms * 1e-3) / issue_peak
                roofline["issue_note"] = ("warp instructions per launch (ncu count of the "
                                          "committed profile, scaled by events) / kernel time / "
                                          "(4 schedulers x SMs x median SM clock): the roof "
                                          "that binds this instruction-bound kernel")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "kernel": {"variant": ["fast", "exact", "warp", "rows"][args.variant],
                   "raster_shape": args.raster_shape, "block_threads": args.block_threads,
                   "precision": ["fp32", "compensated", "fp64_den", "fixed"][args.precision]},
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_of(wl, n_events, world),
        "kernel_pixel_evals_per_s": world * evals_per_s,
        "evals_per_event": evals_per_iter / n_events,
        "roofline": roofline,
        "accuracy": accuracy,
        "precision": precision,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": int(12 * n_events + 4 * wl.n_y * wl.n_z),
                "d2h_bytes_per_step": int(4 * wl.n_y * wl.n_z),
                "iterations_per_step": wl.iterations, "seconds_per_step": e2e_s},
        "gpu_launches": launches_per_iter * args.steps,
        "clocks": clk,
        "peaks": peaks,
        "counters": counters,
        "kernel_ms_per_iteration": kernel_ms,
        "batched": batched,
        "adjoint": adjoint,
        "hybrid": hybrid,
    }
    print(json.dumps(line), flush=True)


def _rel(a, b):
    import numpy as np

    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def accuracy_report(args, wl, geom, events, local, kopts):
    """Accuracy at the stated configurations (tolerance 1e-5 relative L2 per
    iteration against the reference float path, 1e-4 after 20 iterations):
      prefix   the first accuracy-events (2e6) of this workload's events, every
               iteration of the workload (20): each GPU iteration started from
               the reference float path's previous image (single-step error),
               the free-running GPU iterations against the free-running
               reference float path, and both against the reference iteration
               at double (jpet_strip_reference_fp64, free-running; rel L2 and
               max-abs per iteration);
      full     every event, one iteration against that FP64 iteration (the
               20-iteration full-size comparison is bench.py --accuracy-report:
               at 2e7 events the FP64 iteration takes ~9 s);
      config1  the CPU-runnable case exactly: 200 x 180 at 5 mm, 1e6 events of
               the 3-ellipse phantom, 10 free-running iterations against the
               reference float path (and the FP64 oracle at the end)."""
    import concurrent.futures as cf

    import numpy as np
    import torch

    from jpet_strip import capi
    from jpet_strip.workloads import WORKLOADS

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    threads = os.cpu_count() or 1
    og = oracle.Geometry(*wl.geometry_args())
    iters = wl.iterations
    m = min(len(events), args.accuracy_events)
    pre = np.ascontiguousarray(events[:m])

    def oracle_chain(geom_o, ev, n_iter):
        out, rho = [], None
        for _ in range(n_iter):
            rho, _ = oracle.mlem_f(geom_o, ev, 1, rho, threads=threads)
            out.append(rho)
        return out

    pool = cf.ThreadPoolExecutor(max_workers=1)  # the CPU chain overlaps the GPU work
    fut = pool.submit(oracle_chain, og, pre, iters)
    pre_d = torch.from_numpy(pre).cuda(local)
    free_imgs, f64_imgs, f64 = [], [], None
    with capi.StripReconstruction(geom, device=local, **kopts) as r:
        r.set_events(pre)
        for _ in range(iters):
            r.iterate(1)
            free_imgs.append(r.rho)
    for _ in range(iters):
        f64, _ = capi.reference_fp64(geom, pre_d, 1, rho=f64, device=local)
        f64_imgs.append(f64)
    ref = fut.result()
    single = []
    with capi.StripReconstruction(geom, device=local, **kopts) as r:
        r.set_events(pre)
        for it in range(iters):
            if it > 0:
                r.rho = ref[it - 1]
            r.iterate(1)
            single.append(_rel(r.rho, ref[it]))
    prefix = {
        "events": m, "iterations": iters,
        "single_step_rel_l2_vs_reference_float": single,
        "free_rel_l2_vs_reference_float": [_rel(a, b) for a, b in zip(free_imgs, ref)],
        "free_rel_l2_vs_fp64": [_rel(a, b) for a, b in zip(free_imgs, f64_imgs)],
        "free_max_abs_vs_fp64": [float(np.abs(a - b).max()) for a, b in zip(free_imgs, f64_imgs)],
        "reference_float_rel_l2_vs_fp64": [_rel(a, b) for a, b in zip(ref, f64_imgs)],
        "reference_float_max_abs_vs_fp64": [float(np.abs(a - b).max())
                                            for a, b in zip(ref, f64_imgs)],
    }
    prefix["within_tolerance"] = bool(max(single) <= 1e-5 and
                                      prefix["free_rel_l2_vs_reference_float"][-1] <= 1e-4)
    # full size, one iteration against FP64
    ev_d = torch.from_numpy(np.ascontiguousarray(events)).cuda(local)
    t0 = time.perf_counter()
    f64_full, _ = capi.reference_fp64(geom, ev_d, 1, device=local)
    fp64_s = time.perf_counter() - t0
    with capi.StripReconstruction(geom, device=local, **kopts) as r:
        r.set_events(events)
        r.iterate(1)
        got = r.rho
    del ev_d
    full = {"events": len(events), "iterations": 1, "rel_l2_vs_fp64": _rel(got, f64_full),
            "max_abs_vs_fp64": float(np.abs(got - f64_full).max()),
            "fp64_seconds_per_iteration": fp64_s}
    # config 1 exactly as stated
    w1 = WORKLOADS["plain-5mm-1M"]
    g1 = capi.Geometry(*w1.geometry_args())
    o1 = oracle.Geometry(*w1.geometry_args())
    ev1 = w1.events(w1.n_events, device=local)
    ref1 = oracle_chain(o1, ev1, w1.iterations)
    d1 = oracle.mlem_d(o1, ev1, w1.iterations, threads=threads)
    imgs1 = []
    with capi.StripReconstruction(g1, device=local, **kopts) as r:
        r.set_events(ev1)
        for _ in range(w1.iterations):
            r.iterate(1)
            imgs1.append(r.rho)
    config1 = {"workload": w1.name, "events": len(ev1), "iterations": w1.iterations,
               "free_rel_l2_vs_reference_float": [_rel(a, b) for a, b in zip(imgs1, ref1)],
               "final_rel_l2_vs_fp64": _rel(imgs1[-1], d1),
               "reference_float_final_rel_l2_vs_fp64": _rel(ref1[-1], d1)}
    pool.shutdown()
    return {"tolerance_per_iteration": 1e-5, "tolerance_20_iterations": 1e-4,
            "config2_prefix": prefix, "config2_full": full, "config1": config1}


def precision_modes(wl, geom, events, local):
    """Every accumulation mode on this workload: ms per iteration (CUDA events,
    3 iterations after a warm-up) and, after one iteration from a uniform image,
    rel L2 and max-abs against the reference iteration at double on the GPU."""
    import numpy as np
    import torch

    from jpet_strip import capi

    ev_d = torch.from_numpy(np.ascontiguousarray(events)).cuda(local)
    f64, _ = capi.reference_fp64(geom, ev_d, 1, device=local)
    del ev_d
    out = {"events": len(events), "reference": "jpet_strip_reference_fp64, one iteration"}
    modes = [("fp32", capi.PRECISION_FP32), ("compensated", capi.PRECISION_COMPENSATED),
             ("compensated_fp64_den", capi.PRECISION_FP64_DEN), ("fixed", capi.PRECISION_FIXED)]
    stream = torch.cuda.Stream(device=local)
    for name, prec in modes:
        with capi.StripReconstruction(geom, device=local, precision=prec) as r:
            r.set_stream(stream.cuda_stream)
            r.set_events(events)
            r.iterate(1)
            img = r.rho
            r.iterate(1)  # warm-up
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            r.synchronize()
            a.record(stream)
            r.iterate(3)
            b.record(stream)
            b.synchronize()
            out[name] = {"ms_per_iteration": a.elapsed_time(b) / 3,
                         "rel_l2_vs_fp64": _rel(img, f64),
                         "max_abs_vs_fp64": float(np.abs(img - f64).max())}
    return out


def accuracy_full_report(args, wl, local):
    """bench.py --accuracy-report: every iteration of the full workload, the
    default FP32 kernel against the reference iteration at double on the GPU
    (both free-running from a uniform image): rel L2 and max-abs per iteration."""
    import numpy as np
    import torch

    from jpet_strip import capi

    n = args.events or wl.n_events
    events = wl.events(n, device=local)
    geom = capi.Geometry(*wl.geometry_args())
    ev_d = torch.from_numpy(np.ascontiguousarray(events)).cuda(local)
    rel, mx = [], []
    f64 = None
    with capi.StripReconstruction(geom, device=local) as r:
        r.set_events(events)
        for _ in range(wl.iterations):
            r.iterate(1)
            f64, _ = capi.reference_fp64(geom, ev_d, 1, rho=f64, device=local)
            got = r.rho
            rel.append(_rel(got, f64))
            mx.append(float(np.abs(got - f64).max()))
    print(json.dumps({"metric": "per-iteration accuracy of the FP32 iteration vs FP64",
                      "config": {"workload": wl.name, "events": n, "iterations": wl.iterations},
                      "rel_l2_vs_fp64": rel, "max_abs_vs_fp64": mx}), flush=True)



def calibration_report(local):
    """bench.py --calibration-report: the differentiable configuration as stated
    (500 x 450 at 2 mm, 5e6 events of the seeded 10-ellipse phantom simulated
    with sigma (10, 42)), widths fitted blind -- MLEM image at the current
    widths from half the events, widths fitted to the other half -- from the
    mis-specified (14, 55) and, as a control, from the true (10, 42).  Prints
    the trajectories; with the activity image unknown the widths are not
    identifiable (a blurred image under narrower widths predicts the same
    events), which these runs measure."""
    from jpet_strip import capi, phantom
    from jpet_strip.autograd import recalibrate_sigma

    ev = capi.generate(phantom.random_ellipse_phantom(seed=3), 5_000_000, 450.0, 1000.0,
                       10.0, 42.0, seed=3, device=local)
    out = {"config": {"grid": "500x450", "pixel_mm": 2.0, "events": len(ev),
                      "true_sigma": [10.0, 42.0], "phantom": "random10, seed 3"}}
    for label, start in (("from_14_55", (14.0, 55.0)), ("from_true_10_42", (10.0, 42.0))):
        geom = capi.Geometry(450.0, 1000.0, 450, 500, 2.0, *start)
        t0 = time.perf_counter()
        sigma, hist = recalibrate_sigma(geom, ev, start, outer=12, device=local)
        out[label] = {"start": list(start), "final": [float(sigma[0]), float(sigma[1])],
                      "seconds": time.perf_counter() - t0,
                      "trajectory": [h["sigma"] for h in hist]}
    print(json.dumps(out), flush=True)


def profile_traffic(n_events, key="dram_bytes_per_launch", variant=0):
    """DRAM bytes (or warp instructions, key "warp_instructions_per_launch") per
    iteration-kernel launch from the committed ncu capture of the kernel the
    variant runs (dram__bytes_read.sum + dram__bytes_write.sum,
    smsp__inst_executed.sum of one launch), scaled from the captured event count
    to n_events."""
    name = {0: "iterate_union_traffic.json", 3: "iterate_rows_traffic.json",
            "hybrid": "hybrid_iterate_traffic.json"}.get(variant)
    if name is None:
        return None
    path = os.path.join(ROOT, "profiles", name)
    try:
        with open(path) as f:
            d = json.load(f)
        return d[key] * n_events / d.get("units", d.get("events"))
    except (OSError, KeyError, ValueError, ZeroDivisionError):
        return None


def _soa_device(ev):
    """Device AoS float32[n, 3] -> contiguous SoA rows (z_u, z_d, dl)."""
    t = ev.t().contiguous()
    return t, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr()


def batch_summary(local, iterations=10, k=64):
    """Batched form: k reconstructions of uneven sizes, one graph launch per
    call, untuned and autotuned, against the same instances run one handle
    at a time (each with its own launches).  Device-resident events; times are
    host wall-clock around complete calls.  Images are compared after one
    iteration (float summation order only) and after `iterations` (where MLEM
    amplifies those differences, as between two runs of one handle)."""
    import numpy as np
    import torch

    from jpet_strip import capi, workloads

    inst = workloads.batch_instances(k)
    geoms = [capi.Geometry(*wl.geometry_args()) for wl, _ in inst]
    events = [capi.generate_device(ell, wl.n_events, wl.radius, wl.length, wl.sigma_z,
                                   wl.sigma_dl, seed=wl.seed, device=local) for wl, ell in inst]
    n_total = int(sum(e.shape[0] for e in events))
    ones = [np.ones((g.n_y, g.n_z), np.float32) for g in geoms]
    # one handle at a time
    single_s = 0.0
    single_imgs = []
    single_one = []
    evals = 0
    for g, ev, one in zip(geoms, events, ones):
        t, zu, zd, dl = _soa_device(ev)
        with capi.StripReconstruction(g, device=local) as r:
            r.set_events_device(zu, zd, dl, ev.shape[0])
            r.iterate(1)
            single_one.append(r.rho)
            r.rho = one
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r.iterate(iterations)
            r.synchronize()
            single_s += time.perf_counter() - t0
            single_imgs.append(r.rho)
            evals += r.counters()["n_kernel_calls"]
        del t
    out = {"instances": k, "events": n_total, "iterations": iterations,
           "kernel_pixel_evals_per_iteration": int(evals),
           "single_handles": {"seconds": single_s,
                              "value": n_total * iterations / single_s}}
    with capi.StripBatch(geoms, device=local) as b:
        for i, ev in enumerate(events):
            b.set_events(i, ev)
        b.iterate(1)  # one batched iteration from the uniform image
        batch_one = [b.instance(i).rho.astype(np.float64) for i in range(k)]
        out["max_rel_l2_vs_single_handles_1_iteration"] = max(
            float(np.linalg.norm(batch_one[i] - single_one[i])
                  / max(np.linalg.norm(single_one[i]), 1e-30)) for i in range(k))
        # accuracy against FP64 after one iteration (the reference iteration at
        # double on the GPU), batched and single-handle, on every instance
        e_b, e_s = [], []
        for i in range(k):
            f64, _ = capi.reference_fp64(geoms[i], events[i], 1, device=local)
            nrm = max(np.linalg.norm(f64), 1e-30)
            e_b.append(float(np.linalg.norm(batch_one[i] - f64) / nrm))
            e_s.append(float(np.linalg.norm(single_one[i] - f64) / nrm))
        out["max_rel_l2_vs_fp64_1_iteration"] = {"batched": max(e_b), "single_handles": max(e_s)}
        for label in ("batched", "batched_tuned"):
            if label == "batched_tuned":
                t0 = time.perf_counter()
                b.tune()
                out["tune_seconds"] = time.perf_counter() - t0
            b.iterate(iterations)  # builds the work list and captures the graph
            for i in range(k):
                b.instance(i).rho = ones[i]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b.iterate(iterations)
            dt = time.perf_counter() - t0
            err = max(float(np.linalg.norm(b.instance(i).rho.astype(np.float64) - single_imgs[i])
                            / max(np.linalg.norm(single_imgs[i]), 1e-30)) for i in range(k))
            out[label] = {"seconds": dt, "value": n_total * iterations / dt,
                          "graph_launches": 1,
                          "kernels_per_iteration": b.launches_per_iteration(),
                          "max_rel_l2_vs_single_handles": err}
        plans = {}
        for i in range(k):
            p = b.plan(i)
            key = f"shape{p['raster_shape']}x{p['block_threads']}t{p['tile']}"
            plans[key] = plans.get(key, 0) + 1
        out["tuned_plans"] = plans
    out["speedup_tuned_vs_single"] = out["single_handles"]["seconds"] / out["batched_tuned"]["seconds"]
    return out


def adjoint_summary(local, n_events=5_000_000, ex2_peak=None, calibrate=True):
    """Differentiable form: 5e6 events of a centred point source simulated with
    sigma (10, 42) on the 2 mm grid.  Times one loss + gradient evaluation
    (dL/drho image and dL/dsigma) at the mis-specified widths (14, 55), then
    recalibrates the widths from (14, 55) by gradient descent with the source
    image known."""
    import numpy as np
    import torch

    from jpet_strip import capi, phantom
    from jpet_strip.autograd import calibrate_sigma

    geom = capi.Geometry(450.0, 1000.0, 450, 500, 2.0, 14.0, 55.0)
    ev = capi.generate(phantom.point_source(), n_events, 450.0, 1000.0, 10.0, 42.0, seed=3,
                       device=local)
    img = phantom.point_image(450, 500, 2.0, [(-1.0, -1.0)]) * np.float32(n_events)
    rho = torch.from_numpy(img).cuda(local)
    grad = torch.empty_like(rho)
    with capi.StripReconstruction(geom, device=local) as rec:
        rec.set_events(ev)
        rec.iterate(1)  # counts the kernel evaluations of the supports at (14, 55)
        evals = rec.counters()["n_kernel_calls"]
        rec.nll_grad(14.0, 55.0, rho.data_ptr(), None, grad.data_ptr())  # warm-up
        torch.cuda.synchronize()
        reps = 5
        t0 = time.perf_counter()
        for _ in range(reps):
            loss, gs, skipped = rec.nll_grad(14.0, 55.0, rho.data_ptr(), None, grad.data_ptr())
        dt = (time.perf_counter() - t0) / reps
    out = {"events": n_events, "grid": "500x450", "pixel_mm": 2.0,
           "true_sigma": [10.0, 42.0], "start_sigma": [14.0, 55.0],
           "loss_and_gradient_ms": 1e3 * dt, "events_per_s": n_events / dt,
           "kernel_evaluations": int(evals), "evals_per_s": evals / dt}
    if ex2_peak:
        # each evaluation needs one exp of K and its sigma derivatives
        out["roofline"] = {"bound": "sfu", "achieved": evals / dt / 1e9, "peak": ex2_peak / 1e9,
                           "unit": "Gex2/s", "frac": evals / dt / ex2_peak,
                           "note": "FP64 row terms and sigma derivatives per evaluation; the "
                                   "kernel is bound by FP64 and FP32 issue, not the SFU"}
    if calibrate:
        t0 = time.perf_counter()
        sigma, hist = calibrate_sigma(geom, ev, img, (14.0, 55.0), device=local)
        cal_s = time.perf_counter() - t0
        out.update({"recovered_sigma": [float(sigma[0]), float(sigma[1])],
                    "calibration_steps": len(hist), "calibration_seconds": cal_s,
                    "within_0p5_mm": bool(abs(sigma[0] - 10.0) < 0.5 and
                                          abs(sigma[1] - 42.0) < 0.5)})
    return out


def hybrid_summary(local, n_events=10_000_000, steps=5, warmup=2, cpu_seconds=10.0,
                   iterations=10, sm_mhz=None):
    """The 3D hybrid reconstruction (include/jpet_hybrid.h) on the "hybrid-384"
    configuration: a 384-detector ring of radius 430 mm, 200 x 200 pixels of
    4 mm and 125 planes, sigma_z / sigma_dl 15 / 60 mm (3d_hybrid_reconstruction's
    defaults), n_events responses of a seeded 3D ellipsoid phantom.
      value   event-iterations/s with the frame events resident on the device
              (CUDA events around `steps` iterations on the handle's stream)
      e2e     host responses -> set_responses (frame events and the filter on
              the device) -> uniform image -> `iterations` iterations -> image
              back to the host, through the C ABI
      cpu_baseline  the CPU restatement (release build, all host threads) on
              a prefix of the same frame events, one iteration
      parity  one iteration of that prefix on the GPU against the restatement"""
    import numpy as np
    import torch

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from jpet_strip import hybrid as HY
    from jpet_strip import hybrid_workloads as H

    t0 = time.perf_counter()
    g, _, _ = H.workload("hybrid-384")
    resp = H.responses(g, n_events, seed=3)
    gen_s = time.perf_counter() - t0
    stream = torch.cuda.Stream(device=local)
    with HY.HybridReconstruction(g, device=local) as r:
        r.set_stream(stream.cuda_stream)
        t0 = time.perf_counter()
        r << resp
        r.synchronize()
        set_s = time.perf_counter() - t0
        st = r.statistics()
        for _ in range(warmup):
            r(1)
        r.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        r(steps)
        b.record(stream)
        b.synchronize()
        ms = a.elapsed_time(b) / steps
        kept = r.n_events
        frames = r.frame_events()
        # end to end through the C ABI: host responses in, image out
        pinned = np.empty_like(resp)
        pinned[:] = resp
        ones = np.ones(g.n_voxels, np.float32)
        e2e = []
        for k in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r << pinned
            r.rho = ones
            r(iterations)
            img = r.rho
            if k:
                e2e.append(time.perf_counter() - t0)
        del img
    voxels = st["used_voxels"]
    out = {"workload": "hybrid-384", "detectors": g.n_detectors, "grid": "200x200x125",
           "voxel_mm": 4.0, "sigma_z_mm": 15.0, "sigma_dl_mm": 60.0,
           "pixel_infos": g.n_pixel_infos, "responses": n_events, "events_kept": kept,
           "voxels_per_iteration": voxels, "voxels_per_event": voxels / max(kept, 1),
           "ms_per_iteration": ms, "value": kept / (ms * 1e-3),
           "unit": "event-iterations/s", "voxel_evals_per_s": voxels / (ms * 1e-3),
           "generate_seconds": gen_s, "set_responses_seconds": set_s,
           "e2e": {"value": kept * iterations / e2e[0], "unit": "event-iterations/s",
                   "iterations_per_step": iterations, "seconds_per_step": e2e[0],
                   "h2d_bytes_per_step": int(resp.nbytes + 4 * g.n_voxels),
                   "d2h_bytes_per_step": int(4 * g.n_voxels)}}
    prof = profile_traffic(voxels, "warp_instructions_per_launch", variant="hybrid")
    if prof:
        # instruction-issue bound: 4 schedulers per SM issue one warp instruction
        # per clock each; the count is the committed capture's, scaled by voxels
        n_sm = torch.cuda.get_device_properties(local).multi_processor_count
        out["roofline"] = {"bound": "issue", "unit": "warp instructions/s",
                           "warp_instructions_per_launch": prof,
                           "achieved": prof / (ms * 1e-3),
                           "traffic": profile_traffic(voxels, variant="hybrid")}
        if sm_mhz:
            peak = 4 * n_sm * sm_mhz * 1e6
            out["roofline"].update({"peak": peak, "frac": prof / (ms * 1e-3) / peak,
                                    "sm_mhz": sm_mhz})
    # CPU baseline and parity on a prefix of the same frame events
    w, s = O.hybrid_setup(g)
    threads = os.cpu_count() or 1
    n = 2000
    dt = 0.0
    while True:
        t0 = time.perf_counter()
        want, cnt = O.hybrid_mlem(g, w, s, frames[:n], 1, threads=threads, release=True)
        dt = time.perf_counter() - t0
        if dt > cpu_seconds / 4 or n >= kept:
            break
        n = min(kept, int(n * max(2.0, cpu_seconds / 4 / max(dt, 1e-3))))
    cpu_rate = n / dt
    out["cpu_baseline"] = {"value": cpu_rate, "unit": "event-iterations/s", "cores": threads,
                           "kind": "port",
                           "build": "oracle/liboracle_strip_release.so (-O3, OpenMP, FMA "
                                    "contraction)",
                           "sample": f"first {n} of the {kept} frame events, one iteration "
                                     f"from a uniform image",
                           "voxel_evals_per_s": float(cnt[2]) / dt}
    with HY.HybridReconstruction(g, device=local) as r:
        r.set_frame_events(frames[:n])
        r(1)
        got = r.rho
    out["parity"] = {"events": n, "rel_l2_vs_oracle_1_iteration": _rel(got, want)}
    out["speedup_vs_cpu_baseline"] = out["value"] / cpu_rate
    return out


def precision_report(args, local):
    """Precision stress: the 1 mm lesion workload in every accumulation mode.
    Full scale: time per iteration and each image against the reference
    iteration at double on the GPU (jpet_strip_reference_fp64); a fixed
    1e6-event prefix: each mode, and that GPU FP64 iteration, against the CPU
    FP64 oracle (the reference's algorithm in double)."""
    import numpy as np
    import torch

    from jpet_strip import capi
    from jpet_strip.workloads import WORKLOADS

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    wl = WORKLOADS["stress-1mm-100M"]
    n = args.events or wl.n_events
    iters = wl.iterations
    geom = capi.Geometry(*wl.geometry_args())
    modes = [("fp32", capi.PRECISION_FP32), ("compensated", capi.PRECISION_COMPENSATED),
             ("compensated_fp64_den", capi.PRECISION_FP64_DEN), ("fixed", capi.PRECISION_FIXED)]
    ev = capi.generate_device(wl.ellipses(), n, wl.radius, wl.length, wl.sigma_z, wl.sigma_dl,
                              seed=wl.seed, device=local)
    t, zu, zd, dl = _soa_device(ev)
    # iterations after which the full-scale images meet the FP64 GPU iteration
    # (that iteration costs ~40 s at 1e8 events and 1 mm, so a report may stop
    # the comparison early; every mode is still timed over all iterations)
    k64 = min(iters, args.fp64_iterations) if args.fp64_iterations > 0 else iters
    full = {}
    imgs = {}
    for name, prec in modes:
        with capi.StripReconstruction(geom, device=local, precision=prec) as r:
            r.set_events_device(zu, zd, dl, n)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r.iterate(k64)
            r.synchronize()
            dt = time.perf_counter() - t0
            imgs[name] = r.rho.astype(np.float64)
            if iters > k64:
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                r.iterate(iters - k64)
                r.synchronize()
                dt += time.perf_counter() - t0
            full[name] = {"ms_per_iteration": 1e3 * dt / iters,
                          "value": n * iters / dt}
    # the FP64 yardstick at full scale: the reference iteration at double on the GPU
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ref64, _ = capi.reference_fp64(geom, ev, k64, device=local)
    fp64_s = time.perf_counter() - t0
    for name in imgs:
        d = imgs[name] - ref64
        full[name]["rel_l2_vs_fp64"] = float(np.linalg.norm(d) / np.linalg.norm(ref64))
        full[name]["max_abs_vs_fp64"] = float(np.abs(d).max())
    full["fp64_reference"] = {"ms_per_iteration": 1e3 * fp64_s / k64,
                              "value": n * k64 / fp64_s}
    full["fp64_comparison_after_iterations"] = k64
    del t
    m = min(n, args.sample_events)
    sample = ev[:m].cpu().numpy()
    og = oracle.Geometry(*wl.geometry_args())
    threads = os.cpu_count() or 1
    f64 = oracle.mlem_d(og, sample, iters, threads=threads)
    f32, _ = oracle.mlem_f(og, sample, iters, threads=threads)
    sub = {"reference_float": {"rel_l2_vs_fp64": float(np.linalg.norm(f32 - f64) / np.linalg.norm(f64)),
                               "max_abs_vs_fp64": float(np.abs(f32 - f64).max())}}
    for name, prec in modes:
        with capi.StripReconstruction(geom, device=local, precision=prec) as r:
            r.set_events(sample)
            r.iterate(iters)
            g = r.rho.astype(np.float64)
        sub[name] = {"rel_l2_vs_fp64": float(np.linalg.norm(g - f64) / np.linalg.norm(f64)),
                     "max_abs_vs_fp64": float(np.abs(g - f64).max())}
    g64, _ = capi.reference_fp64(geom, sample, iters, device=local)
    sub["fp64_reference_gpu"] = {"rel_l2_vs_fp64": float(np.linalg.norm(g64 - f64) / np.linalg.norm(f64)),
                                 "max_abs_vs_fp64": float(np.abs(g64 - f64).max())}
    line = {"metric": "precision stress: rel L2 / max-abs vs FP64 per accumulation mode",
            "config": {"workload": wl.name, "events": n, "grid": f"{wl.n_z}x{wl.n_y}",
                       "pixel_mm": wl.pixel, "sigma_z": wl.sigma_z, "sigma_dl": wl.sigma_dl,
                       "phantom": "10 random ellipses + 6 lesions of 5 mm at 8x",
                       "iterations": iters},
            "full_scale": full,
            "fp64_oracle_sample": {"events": m, "iterations": iters, "modes": sub}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    from jpet_strip.workloads import WORKLOADS

    wl = WORKLOADS[args.workload]
    world, rank, local = dist_env()
    if args.impl == "reference":
        reference_arm(args, wl, world, rank)
    elif args.precision_report:
        precision_report(args, local)
    elif args.accuracy_report:
        accuracy_full_report(args, wl, local)
    elif args.calibration_report:
        calibration_report(local)
    elif args.hybrid_report:
        print(json.dumps({"hybrid": hybrid_summary(local, args.hybrid_events)}), flush=True)
    elif args.adjoint_report:
        print(json.dumps({"adjoint": adjoint_summary(local, args.adjoint_events,
                                                     calibrate=False)}), flush=True)
    else:
        gb300_arm(args, wl, world, rank, local)


if __name__ == "__main__":
    main()
