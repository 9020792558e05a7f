#!/usr/bin/env python3
"""Benchmark: cell-updates/s of the plate-tectonics step on GB300, batched and served against the
plain one-world-at-a-time path, with p50/p99 world latency.

One step = advection + sort-based collision + Gaussian uplift + 20 hydraulic + 10 thermal
sub-iterations + CCL every 10 steps (amortised), the benchmark physics.  A cell-update is one
cell through one step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference] [--quick]

Headline (`value`): the mixed-size batch - 256 worlds, sides log-uniform on 128..1024 (half
square, half 2:1), plates uniform on 4..32, per-world seeds - advanced together, one launch per
phase over all worlds, each step one CUDA-graph replay; world state resident in HBM; tile shape
and sort digit width picked by the autotuner.  Beside it:
  plain        the same 256 worlds stepped one at a time through the plain path;
  served       a Poisson trace of world-generation requests (70% 256^2, 25% 1024^2, 5% 4096^2;
               steps 50..500; plates 8..48; 150 GB budget) at 80% of the plain path's capacity,
               served with continuous batching and one request at a time: p50/p99 latency,
               cell-updates/s, and a saturated trace (all requests at t=0) for capacity;
  plain_2048   one 2048^2 world, 32 plates (plain path; its k_hydro roofline);
  plain_8192   one 8192^2 world, 64 plates, velocities in [-2, 2], 8-connected CCL every step.
`issue_roofline` sets the same k_hydro launches against the SMs' instruction-issue limit, its actual bound.
`e2e` repeats the headline through the C ABI with host buffers (packed: one buffer per field for all
worlds; copies on a second stream overlap the previous or next step's compute): every step uploads each world's
state from pinned host memory, steps the batch, downloads heights and plate ids, and waits for them.
Reference arm: the reference path's CPU implementation (the oracle's C restatement, all host
threads) on a bounded sample of the same mixed-size workload.  With N > 1 (torchrun) every rank
runs its own batch (replicas; worlds never exchange data).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_WORLDS = 256
SHAPE_SEED = 2026
# Algorithmic bytes of one hydraulic sub-iteration per cell, as the roofline is defined for this
# path: read height, water, sediment (12) and flux (16); write the same 28 and the velocity (8).
HYDRO_BYTES_PER_CELL = 64
# The engine's own compulsory traffic: its fused sub-iteration never writes the velocity.
HYDRO_ENGINE_BYTES_PER_CELL = 56
# Algorithmic bytes of one whole step per cell, as defined for this path (u32 plate ids, the
# velocity write): advect 12, sort 16, resolve 28, uplift and blur 12, hydraulic 20 x 64, thermal
# 10 x 8, CCL 8 every 10 steps; 1436 with the CCL on every step.
STEP_BYTES_PER_CELL = 1428.8
STEP_BYTES_PER_CELL_CCL_EVERY_STEP = 1436.0
# The engine's own: advect + sort 25, words 13, resolve + uplift 14, thermal 80, hydraulic 20 x 56,
# CCL 5 every 10 steps.
STEP_ENGINE_BYTES_PER_CELL = 1252.5
BUDGET_BYTES = 150 * 10**9


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (copy, burst)"
        except Exception:
            pass
    return 6800.0, "fallback 6.8 TB/s"


MARCH_VARIANT = 9  # hydraulic variant of k_hydro_march


def _profile_number(name, key):
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    m = re.search(key + r":\s*([0-9.eE+]+)", p.read_text())
    return float(m.group(1)) if m else None


def profiled_traffic_per_cell(variant=MARCH_VARIANT):
    """DRAM bytes per cell of one hydraulic launch from the committed ncu summaries: for the
    marching kernel, captured on the mixed batch itself; for the tile kernels, a 2048^2 launch."""
    if variant == MARCH_VARIANT:
        return _profile_number("k_hydro_march_traffic.md", "traffic_bytes_per_cell_batch")
    v = _profile_number("k_hydro_2048.md", "traffic_bytes_per_launch_2048")
    return None if v is None else v / (2048 * 2048)


def profiled_instructions_per_cell(variant=MARCH_VARIANT):
    """Warp-instructions per cell of one hydraulic launch at 2048^2, from the committed ncu summary
    of the kernel that variant runs."""
    name = "k_hydro_march_2048.md" if variant == MARCH_VARIANT else "k_hydro_2048.md"
    v = _profile_number(name, "warp_instructions_per_launch_2048")
    return None if v is None else v / (2048 * 2048)


def issue_roofline(ipc, cells, ms, sm_mhz, sms, kernel="k_hydro"):
    """The hydraulic kernel against the issue limit: every SM issues at most one warp-instruction
    per cycle on each of its four schedulers."""
    if ipc is None or not sm_mhz or not sms:
        return None
    achieved = ipc * cells / (ms / 1e3) / 1e9
    peak = sms * 4 * sm_mhz * 1e6 / 1e9
    return {"bound": "issue", "kernel": kernel, "achieved": achieved, "peak": peak,
            "unit": "G warp-instructions/s", "frac": achieved / peak,
            "note": "warp-instructions per cell from one ncu capture of a 2048^2 launch (narrow strips, "
                    "edge tiles and short worlds issue more, so the batch figure is a lower bound); "
                    "peak = SMs x 4 schedulers x the SM clock sampled during the timed region"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)  # first sample before the timed region
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload_config():
    """The `config` both arms print for the headline workload (identical in both lines); what each
    arm ran it on goes in the arm's own keys."""
    cells = sum(W * H for W, H, *_ in mixed_worlds())
    return {"workload": f"batched mixed-size worlds: {N_WORLDS} worlds, sides log-uniform 128..1024 (half square, "
                        "half 2:1), plates 4..32, per-world seeds, benchmark physics, one step = every world advanced "
                        "one step",
            "worlds": N_WORLDS, "cells": cells}


def mixed_worlds(n=N_WORLDS, seed=SHAPE_SEED):
    """(W, H, plates, gen_seed, world_seed) of the mixed-size batch: side s log-uniform on
    [128, 1024]; even entries s x s, odd entries s x s/2; plates uniform on 4..32."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        s = int(round(math.exp(rng.uniform(math.log(128), math.log(1024)))))
        W, H = (s, s) if i % 2 == 0 else (s, max(1, s // 2))
        out.append((W, H, int(rng.integers(4, 33)), 10_000 + i, 20_000 + i))
    return out


def serve_trace(n, mean_service_s, load, seed=7, saturated=False):
    """Poisson arrivals at `load` x the plain path's capacity (1 / mean service time).  Sizes are
    stratified (70 % 256^2, 25 % 1024^2, 5 % 4096^2 of the n requests, in random order) so that a
    short trace carries the size mix it is meant to."""
    import master_thesis_gb300 as T

    rng = np.random.default_rng(seed)
    lam = load / mean_service_s
    n_big = max(1, round(0.05 * n))
    n_mid = round(0.25 * n)
    sides = np.array([4096] * n_big + [1024] * n_mid + [256] * (n - n_big - n_mid))
    rng.shuffle(sides)
    t = 0.0
    reqs = []
    for i in range(n):
        side = int(sides[i])
        steps = int(rng.integers(50, 501))
        plates = int(rng.integers(8, 49))
        t += rng.exponential(1.0 / lam)
        reqs.append(T.Request(width=side, height=side, plates=plates, steps=steps, velRange=1.0,
                              genSeed=30_000 + i, worldSeed=40_000 + i, arrival_s=0.0 if saturated else t))
    return reqs, lam


def timed_oracle(specs, seconds_cap, settings, start=0):
    """cell-updates/s of the oracle's step alone (world generation excluded).  Only the oracle is
    loaded: its own settings and generator stand in for the engine's."""
    import oracle as O

    cells, done, step_s, wall0 = 0, 0, 0.0, time.perf_counter()
    i = start
    while time.perf_counter() - wall0 < seconds_cap:
        W, H, P, gs, wsd = specs[i % len(specs)]
        h, ids, pl = O.generate_world(W, H, P, 1.0, gs)
        ow = O.OracleWorld(settings, h, ids, pl, wsd)
        t1 = time.perf_counter()
        ow.step(1)
        step_s += time.perf_counter() - t1
        cells += W * H
        done += 1
        i += 1
    return cells / step_s, done, step_s, cells


def run_reference(args, ws, rank):
    import oracle as O

    if rank != 0:
        return
    s = O.baseline_settings()
    specs = mixed_worlds()
    cores = os.cpu_count() or 1
    # each "step" is a bounded sample of the workload: consecutive worlds of the batch, one step
    # each, about 1.5 s of CPU work; warm-up samples first
    timed_oracle(specs, 1.5 * max(1, min(args.warmup, 3)), s)
    rates, worlds, secs, cells = [], 0, 0.0, 0
    start = 0
    for _ in range(args.steps):
        r, d, st, c = timed_oracle(specs, 1.5, s, start)
        start += d
        worlds += d
        secs += st
        cells += c
        rates.append(r)
    rate = cells / secs
    ref_gpu = reference_gpu_lines(s)
    line = {
        "metric": "cell_updates_per_s", "value": rate, "unit": "cell-updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Voronoi worlds, benchmark physics)", "impl": "reference",
        "config": workload_config(),
        "arm": {"parallelism": "host threads", "implementation": "the oracle's C restatement of the reference step"},
        "cpu_baseline": {"value": rate, "unit": "cell-updates/s", "cores": cores, "kind": "port",
                         "sample": f"{worlds} world-steps of the mixed-size batch ({cells} cell-updates, "
                                   f"{secs:.1f} s of stepping) on {cores} OpenMP threads"},
        "e2e": {"value": rate, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_gpu": ref_gpu,
    }
    print(json.dumps(line), flush=True)


# steps timed per reference-kernel case; the engine's plain_2048 / plain_8192 rows time as many
REF_GPU_STEPS = {"2048": 20, "8192": 5}
REF_GPU_OMITS = ("processCollisions is not launched (applyInelasticCollision reads past a local array; a "
                 "height and id copy stands in for it), and neither is the reference uplift chain "
                 "(moveContinentalCollisions, combinePropagatedCollisions, JFA*, applyUplift); the engine's "
                 "step runs its resolve and uplift, so the speed-up is a lower bound")


def reference_gpu_lines(s):
    """The reference's own CUDA kernels on this GPU (oracle/refgpu/ref_gpu_harness.cpp), one world
    at a time, at 2048^2 (32 plates) and 8192^2 (64 plates, velocities in [-2, 2], 8-connected CCL
    every step), over REF_GPU_STEPS steps after 2 warm-up steps."""
    try:
        import torch

        if not torch.cuda.is_available():
            return {"unavailable": "no CUDA GPU"}
        import oracle as O
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"{type(e).__name__}: {e}"}
    out = {"kernels": "getPixelMovements, registerPlateCollisions, determineCollisionType, "
                      "createCollisionTypeMatrix, thermalErosionKernel x thermal iterations, rain/flux/flow/"
                      "sediment/transport/evaporate + 2 copies x hydraulic iterations, copies back, "
                      "applyAccretion, CCL when due",
           "omitted": REF_GPU_OMITS,
           "launch": "256 threads per block, one thread per cell, one stream, no per-launch synchronisation"}
    # the reference's kernels print diagnostics from the device; keep them off stdout, which
    # carries the JSON line
    sys.stdout.flush()
    saved = os.dup(1)
    os.dup2(2, 1)
    try:
        for name, W, P, vel, ccl_every in (("2048", 2048, 32, 1.0, 10), ("8192", 8192, 64, 2.0, 1)):
            try:
                h, ids, pl = O.generate_world(W, W, P, vel, 1)
                st = O.baseline_settings()
                st.sim.iterationsForCCL = ccl_every
                ms = O.ref_gpu_time(W, W, h, ids, pl, st, steps=REF_GPU_STEPS[name], warmup=2)
                out[name] = {"value": W * W / (ms / 1e3), "unit": "cell-updates/s", "ms_per_step": ms,
                             "steps": REF_GPU_STEPS[name]}
            except Exception as e:  # noqa: BLE001
                out[name] = {"unavailable": f"{type(e).__name__}: {e}"}
        torch.cuda.synchronize()
    finally:
        os.dup2(saved, 1)
        os.close(saved)
    return out


def event_ms(torch, stream, fn):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def plain_world_rate(T, torch, stream, W, H, plates, vel, steps, settings):
    """cell-updates/s and ms/step of one world on the plain path (graph replay, resident state)."""
    w = T.World(settings, W, H, seed=1000)
    w.init_synthetic_device(plates, vel, 1)
    w.step(3, stream)
    stream.synchronize()
    ms = event_ms(torch, stream, lambda: w.step(steps, stream))
    w.check(stream)
    w.close()
    return W * H * steps / (ms / 1e3), ms / steps


def rank_worlds(rank):
    """The worlds one rank steps: replicas run their own mixed batch (a different shape seed per
    rank); no data crosses ranks."""
    return mixed_worlds(seed=SHAPE_SEED + rank)


def reduce_max(x, dist, device):
    """x maximised over the ranks (the slowest rank's time), or x alone without a process group."""
    import torch

    t = torch.tensor([x], device=device, dtype=torch.float64)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(x, dist, device):
    """x summed over the ranks (every replica's cells), or x alone without a process group."""
    import torch

    t = torch.tensor([x], device=device, dtype=torch.float64)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class EventClock:
    """Device time on the launching stream: CUDA events recorded before and after the steps."""

    def __init__(self, torch, stream):
        self.stream = stream
        self.e0 = torch.cuda.Event(enable_timing=True)
        self.e1 = torch.cuda.Event(enable_timing=True)

    def start(self):
        self.e0.record(self.stream)

    def stop(self):
        self.e1.record(self.stream)

    def ms(self):
        return self.e0.elapsed_time(self.e1)


def timed_region(step, steps, clock, sync, barrier, max_over_ranks):
    """The timed region every rank runs on its own replica: a barrier and a synchronize, `steps`
    steps between the clock's marks, a synchronize and a barrier.  Returns (this rank's ms, the
    slowest rank's ms)."""
    barrier()
    sync()
    clock.start()
    step(steps)
    clock.stop()
    sync()
    barrier()
    mine = clock.ms()
    return mine, max_over_ranks(mine)


def job_rate(cells_all_ranks, steps, ms_max):
    """Whole-job cell-updates/s: the cells of every rank's replica (summed over the ranks) times the
    steps, over the slowest rank's time."""
    return cells_all_ranks * steps / (ms_max / 1e3)


def run_engine(args, ws, rank, local):
    import torch

    import master_thesis_gb300 as T

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        return reduce_max(x, dist, "cuda")

    stream = torch.cuda.Stream()
    s = T.baseline_settings()  # hydraulicTile = sortRadixBits = 0: the autotuner's choice
    specs = rank_worlds(rank)
    total = sum(W * H for W, H, *_ in specs)
    tuning = T.autotune(s, [(W, H) for W, H, *_ in specs], stream)

    worlds = []
    batch = T.Batch()
    for W, H, P, gs, wsd in specs:
        w = T.World(s, W, H, seed=wsd)
        w.init_synthetic_device(P, 1.0, gs)
        batch.add(w, stream)
        worlds.append(w)
    batch.step(args.warmup, stream)
    stream.synchronize()
    batch.check(stream)

    launches0 = batch.launches
    with ClockSampler(local) as clk:
        _, ms = timed_region(lambda n: batch.step(n, stream), args.steps, EventClock(torch, stream),
                             torch.cuda.synchronize, barrier, max_over_ranks)
    launches = batch.launches - launches0
    batch.check(stream)
    total_all = reduce_sum(total, dist, "cuda")  # replicas hold different worlds
    value = job_rate(total_all, args.steps, ms)

    # dominant kernel: the fused hydraulic sub-iteration over the whole batch, on the same stream
    reps = 20
    batch.hydraulic(2, s.step.hydraulicDt, stream)
    hydro_ms = event_ms(torch, stream, lambda: batch.hydraulic(reps, s.step.hydraulicDt, stream)) / reps
    peak, peak_src = measured_peak_hbm()
    achieved = HYDRO_BYTES_PER_CELL * total / (hydro_ms / 1e3) / 1e9
    hv = tuning.hydraulicTile
    tpc = profiled_traffic_per_cell(hv)
    ipc = profiled_instructions_per_cell(hv)
    hkernel = "k_hydro_march" if hv == MARCH_VARIANT else "k_hydro"
    n_sms = torch.cuda.get_device_properties(local).multi_processor_count

    # e2e through the C ABI with host buffers: upload every world's state, step, download
    # heights and plate ids
    L = T.lib()
    sp = stream.cuda_stream
    up_fields = (T.FIELD_HEIGHT, T.FIELD_WATER, T.FIELD_SEDIMENT, T.FIELD_FLUX, T.FIELD_PLATE_ID)
    down_fields = (T.FIELD_HEIGHT, T.FIELD_PLATE_ID)
    # one packed pinned host buffer per field, the worlds in batch order
    hosts = [{f: torch.from_numpy(np.concatenate([w.download(f).ravel() for w in worlds])).pin_memory()
              for f in up_fields}]
    outs = [{f: torch.empty_like(hosts[0][f]).pin_memory() for f in down_fields}]

    up_copy, down_copy = torch.cuda.Stream(), torch.cuda.Stream()  # separate copy engines
    us, ds = up_copy.cuda_stream, down_copy.cuda_stream

    def e2e_run(nsteps):
        # every step: its inputs copied up (one packed buffer per field, staged on the upload stream
        # two steps ahead into the batch's double staging buffers, then scattered into the worlds),
        # the step, its results gathered and copied down on the download stream while the next step
        # computes
        def stage():
            for f, t in hosts[0].items():
                T.check(L.tecto_batch_stage_upload_async(batch.ptr, f, t.data_ptr(), t.numel() * t.element_size(),
                                                         us), "stage")
        stage()
        if nsteps > 1:
            stage()
        for k in range(nsteps):
            for f in hosts[0]:
                T.check(L.tecto_batch_commit_upload(batch.ptr, f, sp), "commit")
            if k + 2 < nsteps:
                stage()
            batch.step(1, stream)
            for f, t in outs[0].items():
                T.check(L.tecto_batch_gather_download(batch.ptr, f, sp), "gather")
                T.check(L.tecto_batch_fetch_download_async(batch.ptr, f, t.data_ptr(), t.numel() * t.element_size(),
                                                           ds), "fetch")
        stream.synchronize()
        up_copy.synchronize()
        down_copy.synchronize()

    e2e_run(2)
    e2e_steps = max(10, args.steps)  # the headline's step count: the pipeline's fill and drain amortise alike
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_run(e2e_steps)
    wall_ms = (time.perf_counter() - t0) * 1e3
    e2e_ms = max_over_ranks(wall_ms)
    e2e_value = job_rate(total_all, e2e_steps, e2e_ms)
    h2d = sum(t.numel() * t.element_size() for hs in hosts for t in hs.values())
    d2h = sum(t.numel() * t.element_size() for os_ in outs for t in os_.values())
    batch.check(stream)
    del hosts, outs
    batch.close()
    for w in worlds:
        w.close()
    torch.cuda.empty_cache()

    extras = {}
    if rank == 0 and not args.quick:
        extras = engine_extras(args, T, torch, stream, s, specs, total, value)
    barrier()

    if rank == 0:
        cores = os.cpu_count() or 1
        cpu_value, cpu_worlds, cpu_secs, cpu_cells = timed_oracle(specs, 12.0, s)
        line = {
            "metric": "cell_updates_per_s", "value": value, "unit": "cell-updates/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Voronoi worlds, benchmark physics)",
            "config": workload_config(),
            "arm": {"parallelism": f"replicas x{ws}",
                    "execution": "one launch per phase over all worlds, one CUDA-graph replay per step",
                    "cells_per_rank": total, "tuning": tuning.as_dict(),
                    "l2": f"no flush: the batch state (~{total * 107 / 1e9:.1f} GB) exceeds the 126 MB L2 "
                          "many times over every step"},
            "gpu_launches": int(launches),
            "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": {"bound": "hbm", "kernel": f"{hkernel} (hydraulic variant {hv}: one fused sub-iteration, "
                                                  "all worlds)",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None if tpc is None else tpc * total,
                         "traffic_note": ("ncu dram bytes of one launch over this batch (profiles/k_hydro_march_traffic.md)"
                                          if hv == MARCH_VARIANT else
                                          "ncu dram bytes of a 2048^2 launch, scaled per cell"),
                         "peak_source": peak_src, "ms_per_launch": hydro_ms,
                         "alg_bytes_per_launch": HYDRO_BYTES_PER_CELL * total,
                         "engine_alg_bytes_per_launch": HYDRO_ENGINE_BYTES_PER_CELL * total,
                         "engine_frac": HYDRO_ENGINE_BYTES_PER_CELL * total / (hydro_ms / 1e3) / 1e9 / peak,
                         "bytes_note": "64 B/cell: read h, w, s, flux, write them and the velocity; the fused kernel "
                                       "writes no velocity, so its own compulsory traffic is 56 B/cell (engine_*)"},
            "issue_roofline": issue_roofline(ipc, total, hydro_ms, clk.summary().get("sm_mhz"), n_sms, hkernel),
            "step_roofline": {"alg_bytes_per_cell": STEP_BYTES_PER_CELL,
                              "achieved_gbs": STEP_BYTES_PER_CELL * value / ws / 1e9,
                              "frac": STEP_BYTES_PER_CELL * value / ws / 1e9 / peak,
                              "engine_alg_bytes_per_cell": STEP_ENGINE_BYTES_PER_CELL,
                              "engine_frac": STEP_ENGINE_BYTES_PER_CELL * value / ws / 1e9 / peak},
            "cpu_baseline": {"value": cpu_value, "unit": "cell-updates/s", "cores": cores, "kind": "port",
                             "sample": f"{cpu_worlds} world-steps of the mixed-size batch ({cpu_cells} "
                                       f"cell-updates, {cpu_secs:.1f} s of stepping)"},
            "clocks": clk.summary(),
            **extras,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def engine_extras(args, T, torch, stream, s, specs, total, batched_value):
    peak, _ = measured_peak_hbm()
    out = {}

    # the same worlds, one at a time through the plain path, each with the autotuner's choice for
    # a single world of its size class (one representative shape tuned per class)
    classes = {}
    for W, H, *_ in specs:
        key = (round(2 * math.log2(W * H)),)
        classes.setdefault(key, (W, H))
    for W, H in classes.values():
        T.autotune(s, [(W, H)], stream)
    k = 4
    plain_ms = 0.0
    for W, H, P, gs, wsd in specs:
        w = T.World(s, W, H, seed=wsd)
        w.init_synthetic_device(P, 1.0, gs)
        w.step(1, stream)  # captures the world's step graphs
        stream.synchronize()
        t0 = time.perf_counter()
        ev = event_ms(torch, stream, lambda: w.step(k, stream))
        plain_ms += max(ev, (time.perf_counter() - t0) * 1e3)
        w.check(stream)
        w.close()
    plain_value = total * k / (plain_ms / 1e3)
    out["plain"] = {"value": plain_value, "unit": "cell-updates/s",
                    "workload": f"the same {N_WORLDS} worlds stepped one at a time on the plain path "
                                f"({k} steps each, graph replay, autotuned per size class: "
                                f"{len(classes)} classes)",
                    "batched_vs_plain": batched_value / plain_value}

    # plain one-world references
    v2048, ms2048 = plain_world_rate(T, torch, stream, 2048, 2048, 32, 1.0, REF_GPU_STEPS["2048"], s)
    w = T.World(s, 2048, 2048, seed=1000)
    w.init_synthetic_device(32, 1.0, 1)
    w.step(1, stream)
    w.hydraulic(2, s.step.hydraulicDt, stream)
    hms = event_ms(torch, stream, lambda: w.hydraulic(20, s.step.hydraulicDt, stream)) / 20
    w.close()
    ach = HYDRO_BYTES_PER_CELL * 2048 * 2048 / (hms / 1e3) / 1e9
    out["plain_2048"] = {"value": v2048, "unit": "cell-updates/s", "ms_per_step": ms2048,
                         "workload": "one 2048x2048 world, 32 plates",
                         "step_roofline_frac": STEP_BYTES_PER_CELL * v2048 / 1e9 / peak,
                         "k_hydro": {"ms_per_launch": hms, "achieved_gbs": ach, "frac": ach / peak}}
    s2 = T.baseline_settings()
    s2.sim.iterationsForCCL = 1
    s2.step.cclConnectivity = T.CCL_8
    v8192, ms8192 = plain_world_rate(T, torch, stream, 8192, 8192, 64, 2.0, REF_GPU_STEPS["8192"], s2)
    out["plain_8192"] = {"value": v8192, "unit": "cell-updates/s", "ms_per_step": ms8192,
                         "workload": "one 8192x8192 world, 64 plates, velocities in [-2, 2], 8-connected CCL "
                                     "every step",
                         "step_roofline_frac": STEP_BYTES_PER_CELL_CCL_EVERY_STEP * v8192 / 1e9 / peak,
                         "engine_step_roofline_frac": (STEP_ENGINE_BYTES_PER_CELL + 4.5) * v8192 / 1e9 / peak}
    torch.cuda.empty_cache()

    # the reference's own CUDA kernels on this GPU, the same worlds, as many steps as plain_2048 / 8192
    ref = reference_gpu_lines(s)
    vs = {"omitted_from_reference": REF_GPU_OMITS}
    for name, v, ms in (("2048", v2048, ms2048), ("8192", v8192, ms8192)):
        r = ref.get(name, {})
        if "ms_per_step" in r:
            vs[name] = {"engine_ms_per_step": ms, "reference_ms_per_step": r["ms_per_step"],
                        "engine_value": v, "reference_value": r["value"], "unit": "cell-updates/s",
                        "speedup": r["ms_per_step"] / ms, "steps": r["steps"]}
        else:
            vs[name] = r
    out["vs_reference_gpu"] = vs
    torch.cuda.empty_cache()

    # the widened rows: plate dynamics' cost per step, the reference's initialisation, the exports
    sd = T.baseline_settings()
    sd.step.plateDynamics = T.PLATE_DYNAMICS_REFERENCE
    _, msd = plain_world_rate(T, torch, stream, 2048, 2048, 32, 1.0, 20, sd)
    out["plate_dynamics_2048"] = {"ms_per_step": msd, "ms_per_step_without": ms2048,
                                  "overhead_frac": msd / ms2048 - 1.0,
                                  "workload": "one 2048x2048 world, 32 plates, plate dynamics on"}
    sp = T.baseline_settings()
    sp.step.plateDynamics = T.PLATE_DYNAMICS_REFERENCE
    sp.step.platePolicy = T.PLATE_RELABEL | T.PLATE_MERGE
    sp.sim.iterationsForCCL = 1
    _, msp = plain_world_rate(T, torch, stream, 2048, 2048, 32, 1.0, 20, sp)
    sc = T.baseline_settings()
    sc.sim.iterationsForCCL = 1
    _, msc = plain_world_rate(T, torch, stream, 2048, 2048, 32, 1.0, 20, sc)
    out["plate_policy_2048"] = {"ms_per_step": msp, "ms_per_step_ccl_every_step": msc,
                                "overhead_frac": msp / msc - 1.0,
                                "workload": "one 2048x2048 world, 32 plates, plate dynamics, relabel after a CCL "
                                            "on every step, merges; compared with the same CCL cadence alone"}
    si = T.default_settings()  # the reference's defaults: 16 plates, Voronoi generations of 200 and 500 seeds
    w = T.World(si, 2048, 2048, seed=1000)
    w.init_reference(stream)
    init_ms = []
    for _ in range(3):
        t0 = time.perf_counter()
        w.init_reference(stream)
        stream.synchronize()
        init_ms.append((time.perf_counter() - t0) * 1e3)
    import tempfile
    exp_ms = {}
    with tempfile.TemporaryDirectory() as d:
        for name, kind in (("height_gray16", T.EXPORT_HEIGHT_GRAY16), ("plates_rgb", T.EXPORT_PLATES_RGB)):
            t0 = time.perf_counter()
            w.export_png(kind, os.path.join(d, name + ".png"), si.kernel.minUpliftClamp, si.kernel.maxUpliftClamp,
                         stream)
            exp_ms[name] = (time.perf_counter() - t0) * 1e3
        t0 = time.perf_counter()
        w.save_snapshot(os.path.join(d, "w.snap"), stream)
        exp_ms["snapshot_save"] = (time.perf_counter() - t0) * 1e3
        t0 = time.perf_counter()
        w.load_snapshot(os.path.join(d, "w.snap"), stream)
        exp_ms["snapshot_load"] = (time.perf_counter() - t0) * 1e3
    w.close()
    # the reference's own configuration end to end: its initialisation, its default KernelSettings and
    # step constants (10 hydraulic sub-iterations at dt 1, one thermal pass), its uplift
    sr = T.default_settings()
    sr.step.upliftMode = T.UPLIFT_REFERENCE
    wr = T.World(sr, 2048, 2048, seed=1000)
    wr.init_reference(stream)
    wr.step(3, stream)
    stream.synchronize()
    msr = event_ms(torch, stream, lambda: wr.step(10, stream)) / 10
    wr.check(stream)
    wr.close()
    out["reference_physics_2048"] = {"ms_per_step": msr, "value": 2048 * 2048 / (msr / 1e3),
                                     "unit": "cell-updates/s",
                                     "workload": "one 2048x2048 world initialised as the reference does, its default "
                                                 "settings (split hydraulic path at dt 1), the reference uplift"}
    out["init_reference_2048"] = {"ms": min(init_ms), "workload": "2048x2048, the reference's default settings "
                                  "(16 plates, Voronoi generations of 200 and 500 seeds), wall time incl. host draws"}
    out["output_2048_ms"] = exp_ms

    # serving: plain-path service time per request size sets the arrival rate
    svc = {}
    for side in (256, 1024, 4096):
        v, msps = plain_world_rate(T, torch, stream, side, side, 24, 1.0, 10 if side < 4096 else 4, s)
        svc[side] = msps / 1e3
    mean_steps = 275.0
    mean_service = mean_steps * (0.70 * svc[256] + 0.25 * svc[1024] + 0.05 * svc[4096])
    n_req = args.serve_requests
    served = {"plain_step_ms": {str(k): round(v * 1e3, 4) for k, v in svc.items()},
              "mean_plain_service_s": mean_service, "budget_bytes": BUDGET_BYTES, "requests": n_req}
    for name, saturated in (("poisson", False), ("saturated", True)):
        reqs, lam = serve_trace(n_req, mean_service, 0.8, saturated=saturated)
        sv = T.Server(s, BUDGET_BYTES)
        res_c, st_c = sv.run_trace(reqs, stream)
        res_s, st_s = sv.run_trace_sequential(reqs, stream)
        sv.close()
        same = all(a.status == b.status == 0 and a.height_checksum == b.height_checksum
                   for a, b in zip(res_c, res_s))
        served[name] = {
            "arrival_rate_per_s": None if saturated else lam,
            "continuous": {"cell_updates_per_s": st_c.cell_updates_per_s, "p50_s": st_c.latency_p50_s,
                           "p99_s": st_c.latency_p99_s, "wall_s": st_c.wall_s, "max_active": st_c.max_active,
                           "peak_bytes": st_c.peak_bytes, "completed": st_c.completed},
            "one_at_a_time": {"cell_updates_per_s": st_s.cell_updates_per_s, "p50_s": st_s.latency_p50_s,
                              "p99_s": st_s.latency_p99_s, "wall_s": st_s.wall_s, "completed": st_s.completed},
            "throughput_ratio": st_c.cell_updates_per_s / max(st_s.cell_updates_per_s, 1e-9),
            "results_identical": bool(same),
        }
    out["served"] = served
    return out


def run_case(args):
    """Small fixed workloads for ncu captures (no timing, no JSON line):
    erosion2048  one 5-iteration thermal launch and one fused hydraulic launch (variant --hydro-tile,
                 default 4) on a 2048^2 world;
    erosion4096  the same on a 4096^2 world (each field 67 MB: a launch's working set is about
                 eight times the L2), one thermal launch of the default variant, two hydraulic
                 sub-iterations of the variant --hydro-tile (default 4);
    collide4096  three collide phases of one 4096^2 world (16 777 216 keys: the sort passes in their
                 form for large sorts), 8-bit sort digits;
    plain2048    4 steps of one 2048^2 world, 32 plates;
    policy2048   the same with plate dynamics, relabel after a CCL on every step, and merges;
    collide2048  three collide phases (advection fused into the sort, winner pick, collision types)
                 of one 2048^2 world, 32 plates, 8-bit sort digits;
    batch        the mixed-size batch, 4 steps, with the variants --hydro-tile, --thermal-tile and
                 --radix-bits (the autotuner's choices of a bench line: `--tuned-from LINE.json`)."""
    import torch

    import master_thesis_gb300 as T

    stream = torch.cuda.Stream()
    s = T.baseline_settings()
    s.step.thermalTile = args.thermal_tile
    if args.case == "erosion2048":
        s.step.hydraulicTile = args.hydro_tile
        w = T.World(s, 2048, 2048, seed=1000)
        w.init_synthetic_device(32, 1.0, 1)
        rng = np.random.default_rng(1)
        w.upload(T.FIELD_WATER, np.abs(rng.normal(0, 0.05, (2048, 2048))).astype(np.float32))
        w.upload(T.FIELD_SEDIMENT, np.abs(rng.normal(0, 0.01, (2048, 2048))).astype(np.float32))
        w.thermal(5, stream)
        w.hydraulic(1, s.step.hydraulicDt, stream)
        w.check(stream)
    elif args.case == "erosion4096":
        s.step.hydraulicTile = args.hydro_tile
        w = T.World(s, 4096, 4096, seed=1000)
        w.init_synthetic_device(32, 1.0, 1)
        w.step(1, stream)
        w.thermal(2, stream)
        w.hydraulic(2, s.step.hydraulicDt, stream)
        w.check(stream)
    elif args.case == "collide4096":
        s.step.sortRadixBits = 8
        w = T.World(s, 4096, 4096, seed=1000)
        w.init_synthetic_device(32, 1.0, 1)
        for _ in range(3):
            w.collide(stream)
        w.check(stream)
    elif args.case == "policy2048":
        s.step.plateDynamics = T.PLATE_DYNAMICS_REFERENCE
        s.step.platePolicy = T.PLATE_RELABEL | T.PLATE_MERGE
        s.sim.iterationsForCCL = 1
        w = T.World(s, 2048, 2048, seed=1000)
        w.init_synthetic_device(32, 1.0, 1)
        w.step(4, stream)
        w.check(stream)
    elif args.case == "collide2048":
        s.step.sortRadixBits = 8
        w = T.World(s, 2048, 2048, seed=1000)
        w.init_synthetic_device(32, 1.0, 1)
        for _ in range(3):
            w.collide(stream)
        w.check(stream)
    elif args.case == "plain2048":
        w = T.World(s, 2048, 2048, seed=1000)
        w.init_synthetic_device(32, 1.0, 1)
        w.step(4, stream)
        w.check(stream)
    else:
        s.step.hydraulicTile = args.hydro_tile
        s.step.sortRadixBits = args.radix_bits
        b = T.Batch()
        worlds = []
        for W, H, P, gs, wsd in mixed_worlds():
            w = T.World(s, W, H, seed=wsd)
            w.init_synthetic_device(P, 1.0, gs)
            b.add(w, stream)
            worlds.append(w)
        b.step(4, stream)
        b.check(stream)
    stream.synchronize()
    print("case", args.case, "ok")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--serve-requests", type=int, default=64)
    ap.add_argument("--quick", action="store_true", help="headline only (no plain/served/large-world lines)")
    ap.add_argument("--hydro-tile", type=int, default=4, help="hydraulic variant of the --case captures")
    ap.add_argument("--thermal-tile", type=int, default=0, help="thermal variant of the --case captures (0: the default)")
    ap.add_argument("--radix-bits", type=int, default=9, help="sort digit width of --case batch")
    ap.add_argument("--case", choices=["erosion2048", "erosion4096", "plain2048", "policy2048", "collide2048",
                                       "collide4096", "batch"],
                    help="a small fixed workload for profilers")
    ap.add_argument("--tuned-from", default=None,
                    help="take --hydro-tile / --thermal-tile / --radix-bits from the tuning of a bench JSON line")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.tuned_from:
        t = json.loads(open(args.tuned_from).read().strip().splitlines()[-1])["arm"]["tuning"]
        args.hydro_tile, args.thermal_tile, args.radix_bits = t["hydraulicTile"], t["thermalTile"], t["sortRadixBits"]
    ws, rank, local = dist_setup()
    if args.case:
        run_case(args)
    elif args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_engine(args, ws, rank, local)


if __name__ == "__main__":
    main()
