"""Benchmark: particle-steps/s of the plain GPU WCSPH step on the 720k-particle
mDBC dam break (tank 1.61 x 0.8 m, column 0.6 x 0.3 m, dp = 0.0005 m, c0 = 35,
delta = 0.1, FP32 pair math with FP64 positions) on one GB300.

One bench step = one SPH time step (one body of the reference's RUN loop:
mDBC, predictor, rebuild, forces + corrector, rebuild, forces), replayed from
a CUDA graph through the C ABI.  Prints one JSON line (see README of the
driver contract): value (state resident in HBM), e2e (host buffers through
the C ABI: upload, re-bin, step, download per step), roofline of the pair
kernel, cpu_baseline (the CPU oracle on the host cores) and clocks.

``--impl reference`` times the reference's CPU algorithm on the same workload
instead (the oracle restatement, all host cores; the reference sources are
not present on the GPU host).

``--workload surrogate`` measures the learned surrogate: one step = one
window of 8 SPH steps (network, checked update, plain fallback), next to the
plain step on the same case.

``--workload ale`` measures the Riemann / ALE-SPH step instead: the BT-wall
dam break of cases/ALESPH_dambreakLong at dp = 0.0004 m (1,125,000 fluid
particles), FP32 fluxes with FP64 leap-frog integration.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PAIR_BYTES_PER_PARTICLE = 80.0   # mean algorithmic bytes of the two pair launches / particle
STEP_BYTES_PER_PARTICLE = 344.0  # algorithmic bytes per particle-step (byte model)
METRIC = "particle-steps/s, 720k dam break, 1 GB300: surrogate/batched vs plain, <=1% front err"
# ALE-SPH byte model per fluid particle: flux pass reads loc, key, v, rho - rho0,
# omega (32 B) and writes the three rates (16 B); whole step with a sort every
# step (leap-frog one 124 B, fluxes 48 B, leap-frog two + binning 164 B,
# placement 36 B, rank + scatter 188 B, scan 15 B); on kept cells (fluxes
# 48 B, leap-frog two in place with the skin check and the next step's
# leap-frog one 192 B) plus, per sort, histogram 28 B, scan 15 B, placement
# 36 B, rank + scatter of every field 270 B, copy back 256 B
ALE_FLUX_BYTES_PER_PARTICLE = 48.0
ALE_KEPT_STEP_BYTES = 240.0
ALE_SORT_BYTES = 605.0
INFER_KERNELS = 5  # one network forward: node kernel, then edge + node kernel for each of 2 layers
ALE_STEP_BYTES_PER_PARTICLE = 575.0
ALE_METRIC = "particle-steps/s, ALE-SPH dam break dp=0.0004 (1.1M fluid), 1 GB300"


def max_over_ranks(x, dist, device):
    """The largest of each rank's value (the timed region's length: the job
    is as slow as its slowest rank); `dist` None for one process."""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, units_per_rank, steps, ms):
    """Units all ranks processed per second over the slowest rank's time
    (weak scaling: every rank runs the same work)."""
    return world * units_per_rank * steps / (ms / 1000.0)


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


SM_COUNT = 152
# the pair kernel of each variant (tsph_set_tile_shape) and its ncu summary
PAIR_KERNELS = {0: "k_pairs_tiled (wide: 608 staged, 36 list entries)",
                1: "k_pairs_tiled (deep: 512 staged, 44 list entries)",
                2: "k_pairs_rec (pair records, window staging by cp.async.bulk)"}
PAIR_PROFILES = {"k_pairs_tiled": "k_pairs_tiled_dam_break_720k.md",
                 "k_pairs_rec": "k_pairs_rec_dam_break_720k.md"}


def profile_figures(kernel):
    """Figures of the kernel's committed ncu summary (lines "key: value"):
    dram_bytes_per_launch_fullsize, warp_inst_per_particle, smem_frac."""
    name = kernel.split()[0]
    p = os.path.join(ROOT, "profiles", PAIR_PROFILES.get(name, name + ".md"))
    out = {}
    if not os.path.exists(p):
        return out
    out["file"] = os.path.relpath(p, ROOT)
    keys = {"dram_bytes_per_launch_fullsize": "dram_bytes_per_launch",
            "warp_inst_per_particle": "warp_inst_per_particle", "smem_frac": "smem_frac"}
    for line in open(p):
        k = line.split(":", 1)[0].strip()
        if k in keys:
            try:
                out[keys[k]] = float(line.split(":", 1)[1].split()[0])
            except (ValueError, IndexError):
                pass
    return out


def graph_kernel_split(s, model, dt, flush, stream, steps=20):
    """Per-kernel time of `steps` replayed graph steps from CUPTI kernel
    records (tinysph_old_gb300.timeline), or None without CUPTI."""
    import torch

    from tinysph_old_gb300 import timeline

    try:
        tl = timeline.Timeline()
    except (FileNotFoundError, OSError):
        return None
    torch.cuda.synchronize()
    try:
        tl.start()
    except RuntimeError:  # CUPTI taken (e.g. under a profiler)
        return None
    with torch.cuda.stream(stream):
        for _ in range(steps):
            flush.zero_()
            s.step(model, dt, 1)
    stream.synchronize()
    torch.cuda.synchronize()
    tl.stop()
    out = timeline.split(tl.records(), steps)
    if not out["by_kernel"]:
        return None
    out["source"] = (f"CUPTI kernel records of {steps} graph steps (L2 flushed between "
                     "steps); exclusive_us partitions the busy time of a step")
    return out


def graph_timeline(s, model, dt, stream, steps):
    """Start, duration and idle time before each kernel of `steps`
    back-to-back replayed graph steps (CUPTI kernel records, microseconds
    from the first kernel), or None without CUPTI."""
    import torch

    from tinysph_old_gb300 import timeline

    try:
        tl = timeline.Timeline()
    except (FileNotFoundError, OSError):
        return None
    torch.cuda.synchronize()
    try:
        tl.start()
    except RuntimeError:
        return None
    with torch.cuda.stream(stream):
        s.step(model, dt, steps)
    stream.synchronize()
    torch.cuda.synchronize()
    tl.stop()
    recs = [r for r in tl.records() if r[1] != 0]
    if not recs:
        return None
    t0, last = recs[0][1], None
    out = []
    for name, st, en, _ in recs:
        idle = 0.0 if last is None else max(0.0, (st - last) * 1e-3)
        out.append([name, round((st - t0) * 1e-3, 2), round((en - st) * 1e-3, 2), round(idle, 2)])
        last = en if last is None else max(last, en)
    return out


def eager_split(run_step, stream, steps, flush):
    """Per-kernel time per step of `steps` eager steps (`run_step(k)` launches
    step k on `stream`, the L2 flushed before each, as in the timed region):
    CUPTI kernel records, or None without CUPTI.  Each kernel's launches per
    step and its time, gated kernels that exit at once included."""
    import torch

    from tinysph_old_gb300 import timeline

    try:
        tl = timeline.Timeline()
    except (FileNotFoundError, OSError):
        return None
    torch.cuda.synchronize()
    try:
        tl.start()
    except RuntimeError:
        return None
    with torch.cuda.stream(stream):
        for k in range(steps):
            flush.zero_()
            run_step(k)
    stream.synchronize()
    torch.cuda.synchronize()
    tl.stop()
    out = timeline.split(tl.records(), steps)
    out["source"] = (f"CUPTI kernel records of {steps} eager steps (L2 flushed between steps); "
                     "exclusive_us partitions the busy time of a step")
    return out


def measure_forms(plain_value):
    """The batched and surrogate forms of the metric, each run as its own
    bench process (shorter runs than their own workloads' defaults), against
    this run's plain step: {"batched": {...}, "surrogate": {...}}."""
    runs = {
        "batched": ["--workload", "batch", "--steps", "30", "--warmup", "3", "--no-cpu",
                    "--loop-steps", "0", "--e2e-steps", "2"],
        "surrogate": ["--workload", "surrogate", "--steps", "50", "--warmup", "2", "--no-cpu",
                      "--e2e-steps", "2"],
    }
    out = {}
    for name, extra in runs.items():
        try:
            res = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *extra],
                                 capture_output=True, text=True, timeout=600, cwd=ROOT)
            lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
            if res.returncode != 0 or not lines:
                out[name] = {"error": (res.stderr or "no result line").strip()[-300:]}
                continue
            d = json.loads(lines[-1])
        except (subprocess.TimeoutExpired, OSError, ValueError) as e:
            out[name] = {"error": str(e)[:300]}
            continue
        f = {"value": d.get("value"), "unit": d.get("unit"), "ms_per_step": d.get("ms_per_step"),
             "over_plain": d["value"] / plain_value if d.get("value") else None,
             "workload": d.get("config", {}).get("workload")}
        if name == "batched":
            f["launches_per_step"] = d.get("launches_per_step")
            f["grouped"] = (d.get("grouped") or {}).get("value")
            f["front_error"] = ("per case against the oracle and against separate plain runs to "
                                "FP32 rounding (tests/test_batch.py)")
        else:
            f["fallback_rate"] = d.get("fallback_rate")
            f["plain_same_loop"] = (d.get("plain") or {}).get("value")
            f["front_error_end"] = d.get("front_error_end")
        out[name] = f
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                                  "sw_power_cap"), parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_rate(case, steps, threads):
    """Particle-steps/s of the CPU oracle (the reference's algorithm in C,
    OpenMP, FP64) over `steps` full time steps of `case`."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    P = oracle.PortSystem.from_case(case)
    P.set_threads(threads)
    P.step(case.wall_model, case.dt, 1)  # warm-up
    t0 = time.perf_counter()
    P.step(case.wall_model, case.dt, steps)
    dt = time.perf_counter() - t0
    return P.np() * steps / dt, dt


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference_ale(args):
    """Reference arm of the ALE workload: the oracle's restatement of the
    reference's MUSCL.h RUN loop on all host cores."""
    from tinysph_old_gb300 import cases

    case = cases.dam_break_ale(dp=args.dp)
    threads = host_threads()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    P = oracle.PortAle.from_case(case)
    P.set_threads(threads)
    for k in range(args.warmup):
        P.ale_step(case.dt, k, 1)
    times = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        P.ale_step(case.dt, args.warmup + k, 1)
        times.append(time.perf_counter() - t0)
        if sum(times) > 150.0:
            break
    total = sum(times)
    n = P.np()
    value = n * len(times) / total
    print(json.dumps({
        "metric": ALE_METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": 1,
        "steps": len(times), "warmup": args.warmup, "ms_per_step": 1000 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (BT-wall dam break built like the reference's generators)",
        "impl": "reference",
        "config": {"workload": f"ALE-SPH dam break dp={args.dp}, {n} particles", "particles": n,
                   "dp": args.dp, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads,
                         "kind": "port", "sample": f"{len(times)} time steps of the {n}-particle case"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }), flush=True)


def run_ale(args, rank, world, local):
    """Our arm of the ALE workload (N = 1; replicas for N > 1)."""
    import numpy as np
    import torch

    from tinysph_old_gb300 import cases, sph

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    case = cases.dam_break_ale(dp=args.dp)
    stream = torch.cuda.Stream()
    s = sph.AleSystem(case.h, case.kap, case.cs, case.rho0, case.visco, case.delta, case.dp,
                      case.domain, stream=stream.cuda_stream)
    a = case.particles.arrays()
    nrm = np.zeros((case.np, 2))
    nn = np.asarray(case.particles.normals).reshape(-1, 2)
    nrm[:len(nn)] = nn
    s.add_particles(a["type"], a["r"], a["v"], a["rho"], a["p"], nrm)
    s.set_scheme(sph.ALE_MUSCL if args.scheme == "muscl" else sph.ALE_AS_WRITTEN)
    kept = not args.ale_sort_every_step
    s.set_keep_cells(kept)
    s.divide_to_cells()
    s.particle_to_cell()
    n = s.np
    nfluid = int(np.sum(a["type"] == 0))
    dt = case.dt
    step = 0
    for _ in range(args.warmup):
        s.step(dt, step, 1)
        step += 1
    s.sync()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sorts0 = s.sort_count()
    with ClockSampler(local) as clocks:
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                starts[k].record(stream)
                s.step(dt, step, 1)
                step += 1
                ends[k].record(stream)
        stream.synchronize()
    torch.cuda.synchronize()
    sorts_per_step = (s.sort_count() - sorts0) / args.steps if kept else 1.0
    split_state = {"step": step}

    def one_step(_k):
        s.step(dt, split_state["step"], 1)
        split_state["step"] += 1

    kernel_split = eager_split(one_step, stream, 20, flush)
    step = split_state["step"]
    step_bytes = (ALE_KEPT_STEP_BYTES + ALE_SORT_BYTES * sorts_per_step if kept
                  else ALE_STEP_BYTES_PER_PARTICLE)
    ms = sum(starts[k].elapsed_time(ends[k]) for k in range(args.steps))
    ms = max_over_ranks(ms, dist, "cuda")
    value = whole_job_rate(world, n, args.steps, ms)
    # flux kernel alone (one launch per call), events on the system's stream
    fl_us = []
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
            e0.record(stream)
            s.forces(dt)
            e1.record(stream)
        stream.synchronize()
        fl_us.append(1000.0 * e0.elapsed_time(e1))
    flux_us = statistics.median(fl_us)
    peak, peak_kind = measured_peaks()
    achieved = ALE_FLUX_BYTES_PER_PARTICLE * nfluid / (flux_us * 1e-6) / 1e9
    # e2e: host state in and out through the C ABI every step, pinned
    # buffers; the next step's input is staged while this step computes
    # (tsph_ale_upload_async, applied by tsph_ale_particle_to_cell) and this
    # step's result is read back while the next one computes
    # (tsph_ale_download_async / tsph_ale_download_wait)
    hr = torch.empty((n, 2), dtype=torch.float64, pin_memory=True)
    hv = torch.empty((n, 2), dtype=torch.float64, pin_memory=True)
    hrho = torch.empty((n,), dtype=torch.float64, pin_memory=True)
    mask = sph.ALE_F_R | sph.ALE_F_V | sph.ALE_F_RHO
    ptrs = dict(r=hr.data_ptr(), v=hv.data_ptr(), rho=hrho.data_ptr())
    outs = [tuple(torch.empty_like(t, pin_memory=True) for t in (hr, hv, hrho))
            for _ in range(2)]
    s.download_ptrs(mask, **ptrs)
    e2e_state = {"step": step}

    def e2e_step(k):
        o = outs[k % 2]
        s.particle_to_cell()  # applies this step's staged input
        s.step(dt, e2e_state["step"], 1)
        e2e_state["step"] += 1
        s.upload_async(mask, **ptrs)  # the next step's input, beside this step's kernels
        s.download_async(mask, r=o[0].data_ptr(), v=o[1].data_ptr(), rho=o[2].data_ptr())

    s.upload_async(mask, **ptrs)
    for k in range(2):  # warm
        e2e_step(k)
    s.download_wait()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.e2e_steps):
        e2e_step(k)
    s.download_wait()
    e2e_value = world * n * args.e2e_steps / (time.perf_counter() - t0)
    s.particle_to_cell()  # the last staged input
    step = e2e_state["step"]
    xfer = n * 40
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        threads = host_threads()
        P = oracle.PortAle.from_case(case)
        P.set_threads(threads)
        P.ale_step(dt, 0, 1)
        t0 = time.perf_counter()
        nst = 3
        P.ale_step(dt, 1, nst)
        tt = time.perf_counter() - t0
        cpu = {"value": P.np() * nst / tt, "unit": "particle-steps/s", "cores": threads,
               "kind": "port", "sample": f"{nst} time steps of the same {n}-particle case "
                                         f"({tt:.1f} s, FP64 C restatement, OpenMP)"}
    if rank == 0:
        line = {
            "metric": ALE_METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 fluxes, f64 integration",
            "data": "synthetic (BT-wall dam break built like the reference's generators)",
            "config": {"workload": f"ALE-SPH dam break dp={args.dp}, {n} particles "
                                   f"({nfluid} fluid), scheme {args.scheme}",
                       "particles": n, "fluid": nfluid, "dp": args.dp,
                       "cells": ("kept: sorted when a particle moved 0.95 (kh - 2h) / 2 since "
                                 "its binning or left the domain" if kept
                                 else "sorted every step (the reference's cell order)"),
                       "l2": "flushed (256 MB write) between timed steps",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": xfer,
                    "d2h_bytes_per_step": xfer,
                    "path": "tsph_ale_upload_async(r,v,rho) (staged during the previous step) + "
                            "tsph_ale_particle_to_cell + tsph_ale_step(1) + "
                            "tsph_ale_download_async(r,v,rho) (waited one step later), pinned "
                            "host buffers"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "kernel": "k_ale_flux",
                         "bytes_per_unit": ALE_FLUX_BYTES_PER_PARTICLE, "unit_count": nfluid,
                         "avg_launch_us": flux_us, "peak_kind": peak_kind},
            "step_roofline": {"bytes_per_particle_step": step_bytes,
                              "achieved_gbs": step_bytes * value / world / 1e9,
                              "frac": step_bytes * value / world / 1e9 / peak},
            "sorts_per_step": sorts_per_step,
            "kernel_us_per_step": kernel_split,
            # kept cells: the fluxes with part two and the next part one in
            # one launch (MUSCL: the gradient, the fluxes, part two), and
            # the six sort kernels (launched every step, gated on the
            # device); otherwise part one, fluxes, part two and four sort
            # kernels
            "gpu_launches": args.steps * ((7 if args.scheme != "muscl" else 9) if kept
                                          else (8 if args.scheme == "muscl" else 7)),
            "clocks": clocks.summary(),
            "health": s.health(),
        }
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


BATCH_METRIC = "particle-steps/s, 512 seeded dam-break/still-water cases (2k-100k particles), 1 GB300"


def run_batch(args, rank, world, local):
    """Batched workload: 512 seeded cases packed into ONE particle system
    (each case scaled to the system's spacing, gravity and removal box per
    case from the system's case table), one step = one time step of every
    case with one launch per kernel for the whole batch; next to it the same
    cases stepped one system at a time (the plain path looped per case)."""
    import numpy as np
    import torch

    from tinysph_old_gb300 import batch as B
    from tinysph_old_gb300 import sph

    torch.cuda.set_device(local)
    specs = B.sample_specs(args.cases, seed=args.seed)
    stream = torch.cuda.Stream()
    bt = B.Batch(specs, stream=stream.cuda_stream)
    s = bt.system
    n = bt.np
    for _ in range(args.warmup):
        bt.step(1)
    bt.sync()
    torch.cuda.synchronize()
    t0e, t1e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.kernel_launches(reset=True)
    with ClockSampler(local) as clocks:
        with torch.cuda.stream(stream):
            t0e.record(stream)
            bt.step(args.steps)
            t1e.record(stream)
        stream.synchronize()
    torch.cuda.synchronize()
    ms = t0e.elapsed_time(t1e)
    timed_launches = s.kernel_launches()
    value = n * args.steps / (ms / 1000.0)
    # every case to 0.5 s of its own time: the system steps until the case
    # with the smallest dt gets there (the coarser cases run further)
    t_half = round(0.5 / bt.dt) * ms / args.steps / 1000.0
    # the graph step split by kernel (CUPTI), as for the single case
    flush = torch.empty(1, dtype=torch.float32, device="cuda")
    split = graph_kernel_split(s, bt.wall_model, bt.dt, flush, stream, steps=10)
    # pair-kernel roofline (eager launches with events)
    s.set_profiling(True)
    s.profile(reset=True)
    s.step(bt.wall_model, bt.dt, 3)
    prof = s.profile(reset=True)
    s.set_profiling(False)
    pair_us = prof["pair_us"] / max(prof["pair_launches"], 1)
    nfl = sum(int(np.sum(c.type == 0)) for c in bt.cases)
    peak, peak_kind = measured_peaks()
    achieved = PAIR_BYTES_PER_PARTICLE * nfl / (pair_us * 1e-6) / 1e9
    # e2e: the whole batch's state in from pinned host memory and out again
    # per step through the C ABI; the next step's input is staged while this
    # step computes (tsph_upload_async, applied by tsph_particle_to_cell) and
    # this step's result is read back while the next one computes
    # (tsph_download_async / tsph_download_wait)
    hr = torch.empty((n, 2), dtype=torch.float64, pin_memory=True)
    hv = torch.empty((n, 2), dtype=torch.float64, pin_memory=True)
    hrho = torch.empty((n,), dtype=torch.float64, pin_memory=True)
    outs = [tuple(torch.empty_like(t, pin_memory=True) for t in (hr, hv, hrho))
            for _ in range(2)]
    mask = sph.F_R | sph.F_V | sph.F_RHO
    inp = dict(r=hr.data_ptr(), v=hv.data_ptr(), rho=hrho.data_ptr())
    s.download_ptrs(mask, **inp)

    def e2e_step(k):
        o = outs[k % 2]
        s.particle_to_cell()  # applies this step's staged input
        s.step(bt.wall_model, bt.dt, 1)
        s.upload_async(mask, **inp)  # the next step's input, beside this step's kernels
        s.download_async(mask, r=o[0].data_ptr(), v=o[1].data_ptr(), rho=o[2].data_ptr())

    s.upload_async(mask, **inp)
    for k in range(2):  # warm
        e2e_step(k)
    s.download_wait()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.e2e_steps):
        e2e_step(k)
    s.download_wait()
    e2e_value = n * args.e2e_steps / (time.perf_counter() - t0)
    s.particle_to_cell()  # the last staged input
    health = s.health()
    shape_used = s.tile_shape
    bt_cases, bt_dp = bt.cases, bt.dp
    s.close()
    del bt
    torch.cuda.empty_cache()
    # the earlier packing, for comparison: one system per group of equal
    # constants, groups on their own streams (one launch per kernel per group)
    gb = B.GroupedBatch(specs)
    for _ in range(args.warmup):
        gb.step(1)
    gb.sync()
    torch.cuda.synchronize()
    main = torch.cuda.current_stream()
    g0 = torch.cuda.Event(enable_timing=True)
    gends = [torch.cuda.Event(enable_timing=True) for _ in gb._streams]
    g0.record(main)
    for stq in gb._streams:
        stq.wait_event(g0)
    gb.step(args.steps)
    for stq, e in zip(gb._streams, gends):
        e.record(stq)
    torch.cuda.synchronize()
    gms = max(g0.elapsed_time(e) for e in gends)
    grouped = {"value": gb.np * args.steps / (gms / 1000.0), "unit": "particle-steps/s",
               "ms_per_step": gms / args.steps, "groups": len(gb.groups),
               "how": "one system per (kind, dp) group, each on its own stream"}
    for g in gb.groups:
        g.system.close()
    del gb
    torch.cuda.empty_cache()
    # the plain path looped over the cases: each case alone, one system at a
    # time (--loop-steps 0 leaves it out)
    loop_ms = 0.0
    loop_half = 0.0
    st0 = torch.cuda.Stream()
    for spec in (specs if args.loop_steps > 0 else []):
        a = B.case_arrays(spec)
        c = sph.ParticleSystem(a.h, a.kap, a.cs, 1000.0, 0.02, 0.1, spec.dp, a.domain, "fp32",
                               stream=st0.cuda_stream)
        c.add_particles(a.type, a.r, None, a.rho, a.p, a.gnr)
        c.divide_to_cells()
        c.particle_to_cell()
        c.step(a.wall_model, a.dt, 3)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st0)
        c.step(a.wall_model, a.dt, args.loop_steps)
        e1.record(st0)
        st0.synchronize()
        case_ms = e0.elapsed_time(e1) / args.loop_steps
        loop_ms += case_ms
        loop_half += round(0.5 / a.dt) * case_ms / 1000.0
        c.close()
    looped_value = n / (loop_ms / 1000.0) if loop_ms > 0 else None
    cpu = None
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        threads = host_threads()
        tot, tt = 0, 0.0
        for spec in specs[:4]:
            a = B.case_arrays(spec)
            P = oracle.PortSystem(a.h, a.kap, a.cs, 1000.0, 0.02, 0.1, spec.dp, a.domain)
            for i in range(a.np):
                P.L.orc_add_particle(P.s, int(a.type[i]), float(a.p[i]), float(a.rho[i]),
                                     float(a.r[i, 0]), float(a.r[i, 1]), 0.0, 0.0, 0.0, 0.0)
            for i in np.nonzero(a.type == 1)[0]:  # ghost nodes of the walls (walls come first)
                P.L.orc_add_gnr(P.s, float(a.gnr[i, 0]), float(a.gnr[i, 1]))
            P.set_threads(threads)
            P.divide_to_cells()
            P.particle_to_cell()
            t0 = time.perf_counter()
            P.step(a.wall_model, a.dt, 3)
            tt += time.perf_counter() - t0
            tot += a.np * 3
        cpu = {"value": tot / tt, "unit": "particle-steps/s", "cores": threads, "kind": "port",
               "sample": f"3 time steps of each of the first 4 cases ({tot // 3} particles, "
                         f"{tt:.1f} s, FP64 C restatement, OpenMP)"}
    by_dp = {}
    for c in bt_cases:
        k = f"{c.spec.kind} dp={c.spec.dp:g}"
        by_dp.setdefault(k, [0, 0])
        by_dp[k][0] += 1
        by_dp[k][1] += c.np
    line = {
        "metric": BATCH_METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 pair math, f64 positions",
        "data": "synthetic (seeded tanks built like the reference's generators)",
        "config": {"workload": f"{len(specs)} cases (seed {args.seed}) in one particle system "
                               f"(case table: per-case scale, gravity and removal box), {n} "
                               "particles; one step = one time step of every case",
                   "particles": n, "cases": by_dp, "system_dp": bt_dp,
                   "l2": "inputs larger than L2 (no flush)", "parallelism": "single GPU"},
        "launches_per_step": timed_launches / args.steps,
        "grouped": grouped,
        "looped": {"value": looped_value, "unit": "particle-steps/s",
                   "ms_per_step": loop_ms,
                   "speedup_batched": value / looped_value if looped_value else None,
                   "how": "each case alone in its own system, CUDA-graph steps, one after another"},
        "projected_s_to_0.5s_physical": {"batched": t_half, "looped": loop_half,
                                         "note": "batched: until the finest cases reach 0.5 s "
                                                 "(coarser cases run further)"},
        "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": n * 40,
                "d2h_bytes_per_step": n * 40,
                "path": "tsph_upload_async(r,v,rho) (staged during the previous step) + "
                        "tsph_particle_to_cell + tsph_step(1) + tsph_download_async(r,v,rho) "
                        "(waited one step later) of the whole batch, pinned host buffers"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": PAIR_KERNELS.get(shape_used, "k_pairs_rec"),
                     "bytes_per_unit": PAIR_BYTES_PER_PARTICLE, "unit_count": nfl,
                     "avg_launch_us": pair_us, "peak_kind": peak_kind},
        "kernel_us_per_step": split,
        "gpu_launches": int(timed_launches),
        "clocks": clocks.summary(),
        "health": health,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)


SURROGATE_MODEL = os.path.join(ROOT, "tinysph_old_gb300", "data", "surrogate_dam_break.npz")  # surrogate.MODEL_PATH


def run_surrogate(args, rank, world, local):
    """The learned surrogate on the 720k benchmark dam break: one bench step =
    one window of k = 8 SPH steps (graph export, BF16 network, update, forces
    pass, window check, plain fallback when the check fails), next to 8 plain
    steps from the same state; the water-front error against plain SPH at the
    end of the timed region."""
    import numpy as np
    import torch

    from tinysph_old_gb300 import cases, sph
    from tinysph_old_gb300 import surrogate as S

    torch.cuda.set_device(local)
    if not os.path.exists(SURROGATE_MODEL):
        raise SystemExit(f"missing trained model {SURROGATE_MODEL}")
    m = S.Model.load(SURROGATE_MODEL)
    case = cases.dam_break_benchmark(args.dp)
    k = m.k

    def make():
        s = sph.ParticleSystem.from_case(case)
        s.step(case.wall_model, case.dt, args.warmup * k)
        s.sync()
        return s

    def timed(s, body, nsteps):
        st = torch.cuda.ExternalStream(s.stream_ptr())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(nsteps):
            body()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    plain = make()
    n = plain.np
    with ClockSampler(local) as clocks:
        ms_plain = timed(plain, lambda: plain.step(case.wall_model, case.dt, k), args.steps)
        sur = make()
        ro = S.Rollout(sur, m, case.dt, case.wall_model, case.h, use_net=True)
        ro.run(3)  # warm-up windows (the network's first launches)
        ro.windows = ro.fallbacks = 0
        ro.checks.clear()
        plain.step(case.wall_model, case.dt, 3 * k)  # same physical time as the surrogate
        sur.kernel_launches(reset=True)
        ms_sur = timed(sur, ro.window, args.steps)
        # the engine's kernels (graph steps per kernel) + the network's forward
        # (one node kernel, then an edge and a node kernel per layer) per window
        sur_launches = sur.kernel_launches() + args.steps * INFER_KERNELS
    value = n * k * args.steps / (ms_sur / 1000.0)
    plain_value = n * k * args.steps / (ms_plain / 1000.0)
    fa, fb = plain.water_front(0.02), sur.water_front(0.02)
    # time of the network's forward alone
    gb = ro.gb.export(sur)
    g = gb.struct(case.h, m.u_in, m.s_in)
    inf_ms = timed(sur, lambda: ro.net.infer(g, ro.y.data_ptr()), 10) / 10
    # e2e: state in from pinned host memory, one window, state out
    hr = torch.empty((n, 2), dtype=torch.float64, pin_memory=True)
    hv = torch.empty((n, 2), dtype=torch.float64, pin_memory=True)
    hrho = torch.empty((n,), dtype=torch.float64, pin_memory=True)
    mask = sph.F_R | sph.F_V | sph.F_RHO
    sur.download_ptrs(mask, r=hr.data_ptr(), v=hv.data_ptr(), rho=hrho.data_ptr())
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        sur.upload_ptrs(mask, r=hr.data_ptr(), v=hv.data_ptr(), rho=hrho.data_ptr())
        sur.particle_to_cell()
        sur.mdbc_density()
        sur.density_to_pressure()
        sur.compute_forces(case.wall_model)
        ro.window()
        sur.download_ptrs(mask, r=hr.data_ptr(), v=hv.data_ptr(), rho=hrho.data_ptr())
    e2e_value = n * k * args.e2e_steps / (time.perf_counter() - t0)
    checks = np.array([c[:3] for c in ro.checks]) if ro.checks else np.zeros((1, 3))
    peak, peak_kind = measured_peaks()
    line = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_sur / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 network (tensor cores, f32 accumulate); f32 pair math, f64 positions",
        "data": "synthetic (dam-break lattice built like the reference's generators)",
        "config": {"workload": f"learned surrogate, mDBC dam break dp={args.dp}, {n} particles; "
                               f"one step = one window of {k} SPH steps",
                   "particles": n, "model": os.path.relpath(SURROGATE_MODEL, ROOT),
                   "l2": "inputs larger than L2 (no flush)", "parallelism": "single GPU"},
        "plain": {"value": plain_value, "ms_per_window": ms_plain / args.steps,
                  "surrogate_over_plain": value / plain_value},
        "fallback_rate": ro.fallback_rate,
        "check_median": {"density": float(np.median(checks[:, 0])),
                         "momentum": float(np.median(checks[:, 2]))},
        "front_error_end": abs(fb - fa) / fa,
        "infer_ms": inf_ms,
        "e2e": {"value": e2e_value, "unit": "particle-steps/s",
                "h2d_bytes_per_step": n * 40, "d2h_bytes_per_step": n * 40,
                "path": "tsph_upload(r,v,rho) + binning + forces pass + one surrogate window + "
                        "tsph_download(r,v,rho), pinned host buffers"},
        "roofline": {"bound": "hbm", "achieved": None, "peak": peak, "unit": "GB/s",
                     "frac": None, "traffic": None, "peak_kind": peak_kind,
                     "note": "the window mixes the network (tensor cores, SFU-bound edge sums) "
                             "and the plain step; the plain step's pair-kernel roofline is in "
                             "the dam_break workload's line"},
        "gpu_launches": int(sur_launches),
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)


def run_reference(args, rank, world):
    """The reference arm: the CPU restatement of the reference's step on all
    host cores, on the same workload.  Rank 0 only."""
    if rank != 0:
        return
    if args.workload == "ale":
        run_reference_ale(args)
        return
    from tinysph_old_gb300 import cases

    case = cases.dam_break_benchmark(args.dp)
    threads = host_threads()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    P = oracle.PortSystem.from_case(case)
    P.set_threads(threads)
    for _ in range(args.warmup):
        P.step(case.wall_model, case.dt, 1)
    # bounded: at most ~150 s of timed CPU work
    times = []
    budget = 150.0
    for k in range(args.steps):
        t0 = time.perf_counter()
        P.step(case.wall_model, case.dt, 1)
        times.append(time.perf_counter() - t0)
        if sum(times) > budget:
            break
    total = sum(times)
    n = P.np()
    value = n * len(times) / total
    line = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": len(times), "warmup": args.warmup, "ms_per_step": 1000 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (dam-break lattice built by the reference's generators)",
        "impl": "reference",
        "config": {"workload": f"mDBC dam break dp={args.dp}, {n} particles (plain WCSPH step)",
                   "particles": n, "dp": args.dp, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads,
                         "kind": "port",
                         "sample": f"{len(times)} full time steps of the {n}-particle case"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dam_break",
                    choices=["dam_break", "ale", "batch", "surrogate"])
    ap.add_argument("--cases", type=int, default=512, help="batch workload: number of cases")
    ap.add_argument("--seed", type=int, default=0, help="batch workload: case seed")
    ap.add_argument("--loop-steps", type=int, default=10,
                    help="batch workload: timed steps per case of the looped comparison")
    ap.add_argument("--scheme", default="as_written", choices=["as_written", "muscl"],
                    help="ALE interface states (ALE workload only)")
    ap.add_argument("--ale-sort-every-step", action="store_true",
                    help="ALE workload: sort every step (the reference's cell order) instead of "
                         "keeping the cells while every particle is within the skin")
    ap.add_argument("--dp", type=float, default=None,
                    help="particle spacing (default 0.0005 dam break, 0.0004 ALE)")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--e2e-steps", type=int, default=30)
    ap.add_argument("--cpu-steps", type=int, default=0,
                    help="CPU baseline sample (0 = auto, ~10-30 s)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="leave out the batched and surrogate forms measured beside the plain step")
    ap.add_argument("--timeline", type=int, default=0,
                    help="add the kernel timeline of this many back-to-back graph steps")
    ap.add_argument("--tile-shape", default="auto", choices=["auto", "wide", "deep", "rec"],
                    help="pair-kernel variant: timed on the particles (auto) or fixed, "
                         "e.g. to profile one variant")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.dp is None:
        args.dp = 0.0004 if args.workload == "ale" else 0.0005

    rank = _env_int("RANK", 0)
    world = _env_int("WORLD_SIZE", 1)
    local = _env_int("LOCAL_RANK", 0)

    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "ale":
        run_ale(args, rank, world, local)
        return
    if args.workload == "batch":
        if rank == 0:
            run_batch(args, rank, world, local)
        return
    if args.workload == "surrogate":
        if rank == 0:
            run_surrogate(args, rank, world, local)
        return

    import numpy as np
    import torch

    from tinysph_old_gb300 import cases, sph

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    case = cases.dam_break_benchmark(args.dp)
    stream = torch.cuda.Stream()
    s = sph.ParticleSystem(case.h, case.kap, case.cs, case.rho0, case.visco, case.delta,
                           case.dp, case.domain, args.precision, stream=stream.cuda_stream)
    a = case.particles.arrays()
    gnr = np.zeros((case.np, 2))
    gnr[:len(a["gnr"])] = a["gnr"]
    s.add_particles(a["type"], a["r"], a["v"], a["rho"], a["p"], gnr)
    s.divide_to_cells()
    s.particle_to_cell()
    tune = None
    if args.tile_shape != "auto":
        s.set_tile_shape(sph.TILE_SHAPES[args.tile_shape])
        shape = sph.TILE_SHAPES[args.tile_shape]
    else:
        # the autotuner's choice (median of 20 forces passes per variant)
        shape, tune_us = s.autotune()
        names = {v: k for k, v in sph.TILE_SHAPES.items()}
        tune = {"chosen": names.get(shape, str(shape)),
                "median_us": {names.get(k, str(k)): float(u) for k, u in enumerate(tune_us)}}
    n = s.np
    model = case.wall_model
    dt = case.dt

    # ---- warm-up (also captures the CUDA graph)
    for _ in range(args.warmup):
        s.step(model, dt, 1)
    s.sync()

    # ---- timed: one step per event pair, L2 flushed (256 MB write) in between
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    s.kernel_launches(reset=True)
    with ClockSampler(local) as clocks:
        t_wall0 = time.perf_counter()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                starts[k].record(stream)
                s.step(model, dt, 1)
                ends[k].record(stream)
        stream.synchronize()
        t_wall = time.perf_counter() - t_wall0
    torch.cuda.synchronize()
    # the library's kernels in the timed region (graph steps per kernel, the
    # conditional re-binning only when it ran; the L2 flush is torch's)
    timed_launches = s.kernel_launches()
    ms = sum(starts[k].elapsed_time(ends[k]) for k in range(args.steps))
    ms = max_over_ranks(ms, dist, "cuda")
    if dist:
        dist.barrier()
    value = whole_job_rate(world, n, args.steps, ms)
    health = s.health()

    # ---- the graph step split by kernel (CUPTI kernel records of replayed
    # graph steps, L2 flushed in between as in the timed loop)
    graph_split = graph_kernel_split(s, model, dt, flush, stream, steps=20)
    timeline_recs = graph_timeline(s, model, dt, stream, args.timeline) if args.timeline else None

    # ---- per-kernel timing for the roofline: eager launches of the same
    # kernels, each bracketed by CUDA events on the system's stream
    s.set_profiling(True)
    s.profile(reset=True)
    prof_steps = 5
    s.step(model, dt, prof_steps)
    prof = s.profile(reset=True)
    s.set_profiling(False)
    pair_avg_us = prof["pair_us"] / max(prof["pair_launches"], 1)
    nfluid = int(np.sum(a["type"] == 0))
    peak, peak_kind = measured_peaks()
    achieved = PAIR_BYTES_PER_PARTICLE * nfluid / (pair_avg_us * 1e-6) / 1e9
    pair_kernel = PAIR_KERNELS.get(shape, "k_pairs_tiled")
    pk = profile_figures(pair_kernel)
    sm_mhz = (clocks.summary() or {}).get("sm_mhz") or 2070.0
    graph_pair_us = None
    if graph_split and pair_kernel.split()[0] in graph_split["by_kernel"]:
        graph_pair_us = graph_split["by_kernel"][pair_kernel.split()[0]]["us"] / max(
            graph_split["by_kernel"][pair_kernel.split()[0]]["launches"], 1e-9)
    issue = None
    if pk.get("warp_inst_per_particle"):
        # issue rate against the SMs' peak: 4 schedulers per SM, one warp
        # instruction per scheduler per clock
        inst = pk["warp_inst_per_particle"] * nfluid
        issue = inst / (pair_avg_us * 1e-6) / (SM_COUNT * 4 * sm_mhz * 1e6)

    # ---- e2e through the C ABI with pinned host buffers: each step takes its
    # input state (r, v, rho) from pinned host memory, re-bins, steps and
    # reads its result back into pinned host memory.  The copies run on copy
    # streams beside the kernels: the next step's input is staged while this
    # step computes (tsph_upload_async, applied by tsph_particle_to_cell) and
    # this step's result is read back while the next one computes
    # (tsph_download_async / tsph_download_wait)
    hr = torch.empty((n, 2), dtype=torch.float64, pin_memory=True)
    hv = torch.empty((n, 2), dtype=torch.float64, pin_memory=True)
    hrho = torch.empty((n,), dtype=torch.float64, pin_memory=True)
    ha = torch.empty((n, 2), dtype=torch.float64, pin_memory=True)
    hdrho = torch.empty((n,), dtype=torch.float64, pin_memory=True)
    outs = [tuple(torch.empty_like(t, pin_memory=True) for t in (hr, hv, hrho))
            for _ in range(2)]
    # a step's whole input: r, v, rho and the last forces pass's a, drho (the
    # predictor's rates); its result read back: r, v, rho
    mask_in = sph.F_R | sph.F_V | sph.F_A | sph.F_RHO | sph.F_DRHO
    mask = sph.F_R | sph.F_V | sph.F_RHO
    inp = dict(r=hr.data_ptr(), v=hv.data_ptr(), rho=hrho.data_ptr(), a=ha.data_ptr(),
               drho=hdrho.data_ptr())
    s.download_ptrs(mask_in, **inp)

    def stage():
        s.upload_async(mask_in, **inp)

    def e2e_step(k):
        o = outs[k % 2]
        s.particle_to_cell()  # applies this step's staged input
        s.step(model, dt, 1)
        stage()  # the next step's input, beside this step's kernels
        s.download_async(mask, r=o[0].data_ptr(), v=o[1].data_ptr(), rho=o[2].data_ptr())

    stage()
    for k in range(2):  # warm
        e2e_step(k)
    s.download_wait()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.e2e_steps):
        e2e_step(k)
    s.download_wait()
    e2e_s = time.perf_counter() - t0
    # the input staged by the last step, stepped once more synchronously: the
    # results read back equal it (every e2e step starts from the same input)
    s.particle_to_cell()
    s.step(model, dt, 1)
    e2e_value = world * n * args.e2e_steps / e2e_s
    xfer_in = n * (16 + 16 + 16 + 8 + 8)
    xfer = n * (16 + 16 + 8)
    ref_after = s.download()
    e2e_ok = bool(np.array_equal(outs[(args.e2e_steps - 1) % 2][0].numpy(), ref_after["r"]))

    # ---- CPU baseline (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = host_threads()
        steps = args.cpu_steps
        if steps <= 0:
            r1, t1 = cpu_rate(case, 1, threads)
            steps = max(1, min(30, int(15.0 / max(t1, 1e-3))))
            rate, tt = cpu_rate(case, steps, threads)
        else:
            rate, tt = cpu_rate(case, steps, threads)
        cpu = {"value": rate, "unit": "particle-steps/s", "cores": threads, "kind": "port",
               "sample": f"{steps} full time steps of the same {n}-particle case "
                         f"({tt:.1f} s, FP64 C restatement of the reference, OpenMP)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 pair math, f64 positions" if args.precision == "fp32" else "f64",
            "data": "synthetic (dam-break lattice built like the reference's generators)",
            "config": {"workload": f"mDBC dam break dp={args.dp}, {n} particles "
                                   f"({nfluid} fluid), plain WCSPH step",
                       "particles": n, "fluid": nfluid, "dp": args.dp,
                       "l2": "flushed (256 MB write) between timed steps",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "e2e": {"value": e2e_value, "unit": "particle-steps/s",
                    "h2d_bytes_per_step": xfer_in, "d2h_bytes_per_step": xfer,
                    "path": "tsph_upload_async(r,v,a,rho,drho) (staged during the previous "
                            "step) + tsph_particle_to_cell + tsph_step(1) + "
                            "tsph_download_async(r,v,rho) (waited one step later), pinned host "
                            "buffers",
                    "result_matches_device_state": e2e_ok},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": pk.get("dram_bytes_per_launch"),
                         "kernel": pair_kernel,
                         "bytes_per_unit": PAIR_BYTES_PER_PARTICLE, "unit_count": nfluid,
                         "avg_launch_us": pair_avg_us,
                         "avg_launch_source": "eager launches bracketed by CUDA events",
                         "graph_avg_launch_us": graph_pair_us, "peak_kind": peak_kind,
                         # the kernel is issue-bound, not HBM-bound: its issue rate
                         # and shared-memory throughput against their peaks
                         "issue_frac": issue,
                         "warp_inst_per_particle": pk.get("warp_inst_per_particle"),
                         "smem_frac": pk.get("smem_frac"),
                         "profile": pk.get("file")},
            "step_roofline": {"bytes_per_particle_step": STEP_BYTES_PER_PARTICLE,
                              "achieved_gbs": STEP_BYTES_PER_PARTICLE * value / world / 1e9,
                              "frac": STEP_BYTES_PER_PARTICLE * value / world / 1e9 / peak},
            "kernel_us_per_step": graph_split or {
                "source": "unavailable (no CUPTI): see eager_kernel_us_per_step"},
            "eager_kernel_us_per_step": {
                "source": "5 steps launched eagerly, every kernel bracketed by CUDA events "
                          "(no graph, no programmatic dependent launch overlap): an upper "
                          "bound per category, not the graph step's split",
                **{k: prof[k] / prof_steps for k in ("pair_us", "sort_us", "mdbc_us",
                                                     "other_us")}},
            "autotune": tune,
            **({"timeline": {"steps": args.timeline, "columns": ["kernel", "start_us",
                                                                 "duration_us", "idle_before_us"],
                             "records": timeline_recs}} if args.timeline else {}),
            "gpu_launches": int(timed_launches),
            "clocks": clocks.summary(),
            "health": health,
            "wall_s_timed": t_wall,
        }
        if cpu:
            line["cpu_baseline"] = cpu
        if not args.no_forms and world == 1:
            line["forms"] = measure_forms(value)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
