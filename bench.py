"""Benchmark of the GB300 landscape-evolution step (prints one JSON line).

Workload: the single-large-grid configuration -- a 4096x4096 fp32 spectral DEM
(Hurst 0.7, relief 0-1500 m, 30 m cells, 2% nodata border, 5000 pits, 300
plateaus) driven by a per-step climate series (rain lognormal mean 900 cv 0.3,
temperature N(9, 2)).  A "step" is one model timestep of the hot path: flow
direction with plateau routing and sink flooding, runoff and flow
accumulation, erosion, sediment routing and the surface/soil/vegetation update.

* value: cell-timesteps/s (masked-in cells x steps / s) with the state resident
  on the device, timed with CUDA events on the library's stream;
* e2e: the same metric through the public C ABI with the host side of the
  reference driver: each step uploads its climate and reads back the budget
  row, and every 50th/100th step downloads the grids lem.cpp writes then
  (writegrids, MEM_kernels/io.cpp:201-230);
* roofline: the dominant kernel's algorithmic bytes / its event-timed duration
  against the measured HBM copy bandwidth;
* cpu_baseline: the FP64 oracle on the host cores on a bounded sample.

Multi-GPU (torchrun): every rank runs an independent replica (the path does
not shard a single grid); value is the sum over ranks / the slowest rank.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic bytes per cell-timestep of each stage: the minimum traffic of the
# stage with fp32 fields and u8 codes, each field read or written once.
STAGE_BYTES = {
    "flow_direction": 38, "routing": 12, "runoff": 20, "accumulation": 11,
    "erosion": 72, "sediment": 37, "surface": 84,
}
# Per launch and per cell, the fields a kernel must read or write at least once
# (its share of its stage).  Routing (plateaus, flooding) and the coarse waves
# touch a data-dependent subset of cells and have no per-cell figure.
KERNEL_BYTES = {
    "k_flowdirs": 19,                 # FlowDirs, two launches per step: 38 / 2
    "k_fa_prep": 20,                  # runoff
    "k_fa_walk": 11, "k_fat_final": 9, "k_fat_local": 5,  # accumulation: R code, w (+ W fa)
    "k_erosion": 72,
    "k_sed_walk": 37, "k_sedt_final": 37, "k_sedt_local": 21,  # sediment: R code, ero/inci/geli, stone, soilT (+ W)
    "k_final": 84,
}
B_ALG = sum(STAGE_BYTES.values())


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock and throttle samples during the timed region."""

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                    rows.append(parts)
        except Exception:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world, local):
    if world <= 1:
        return None
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    return dist


def reduce_max(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def cpu_sample(scenario_mod, seconds=12.0, n=1024, max_steps=8):
    """The FP64 oracle on a bounded sample: one 1024x1024 window of the workload
    (same generator, Hurst, relief and border) stepped until `seconds` pass."""
    from oracle import oracle
    oracle.build()
    threads = oracle.num_threads()
    sc = scenario_mod.config_large(2, n=n, steps=max_steps)
    st = scenario_mod.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    m = oracle.OracleModel(sc.dem, 30.0, st, sc.init_rain, sc.init_temp, diagnostics=False)
    cells = int((st["mask"] == 1).sum())
    t0 = time.perf_counter()
    steps = 0
    while steps < max_steps:
        m.step(sc.rain[steps], sc.temp[steps], True)
        steps += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": cells * steps / dt, "unit": "cell-timesteps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} timesteps of a {n}x{n} grid from the same generator ({cells} active cells), "
                      f"FP64 oracle, {threads} OpenMP threads, {dt:.1f} s"}


def run_reference(args):
    """The reference's algorithm on the host cores (the oracle port: the reference
    itself is CUDA and has no CPU implementation; its kernels compile on the CPU
    only where its sources are present)."""
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    from parallem_gb300 import scenario as S
    n = args.ref_grid
    from oracle import oracle
    oracle.build()
    threads = oracle.num_threads()
    sc = S.config_large(2, n=n, steps=args.warmup + args.steps)
    st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    m = oracle.OracleModel(sc.dem, 30.0, st, sc.init_rain, sc.init_temp, diagnostics=False)
    cells = int((st["mask"] == 1).sum())
    for i in range(args.warmup):
        m.step(sc.rain[i], sc.temp[i], True)
    t0 = time.perf_counter()
    for i in range(args.warmup, args.warmup + args.steps):
        m.step(sc.rain[i], sc.temp[i], True)
    dt = time.perf_counter() - t0
    value = cells * args.steps / dt
    line = {
        "impl": "reference", "metric": "cell-timesteps/s", "value": value, "unit": "cell-timesteps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"single large grid, sampled at {n}x{n} on the host", "grid": n,
                   "cellsize_m": 30, "climate": "per-step series"},
        "cpu_baseline": {"value": value, "unit": "cell-timesteps/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} timesteps of a {n}x{n} grid ({cells} active cells)"},
        "e2e": {"value": value, "unit": "cell-timesteps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--grid", type=int, default=4096)
    ap.add_argument("--ref-grid", type=int, default=512)
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline sample")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

    rank, world, local = dist_env()
    dist = init_dist(world, local)
    from parallem_gb300 import build, lem
    from parallem_gb300 import scenario as S
    if rank == 0 or world == 1:
        build.build()
    barrier(dist)
    lem.select_device(local)
    total_steps = args.warmup + 2 * args.steps
    sc = S.config_large(2 + rank, n=args.grid, steps=total_steps)
    st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    cells = int((st["mask"] == 1).sum())
    g = lem.Model(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    g.set_state(st)

    # warm-up steps (untimed)
    for i in range(args.warmup):
        g.step(sc.rain[i], sc.temp[i], True)
    g.synchronize()
    barrier(dist)

    # timed region 1: resident state, device events on the library's stream
    launches0 = g.launches
    g.profiling(True)
    with ClockSampler(local) as clk:
        g.record(0)
        for i in range(args.warmup, args.warmup + args.steps):
            g.step(sc.rain[i], sc.temp[i], True)
        g.record(1)
        ms = g.elapsed_ms(0, 1)
    prof = g.profile()
    g.profiling(False)
    g.synchronize()
    launches = g.launches - launches0
    ms_max = reduce_max(dist, ms)
    cells_all = reduce_sum(dist, cells)
    value = cells_all * args.steps / (ms_max / 1e3)

    # timed region 2: end to end through the C ABI with host buffers
    barrier(dist)
    h2d = d2h = 0
    import ctypes as C
    tot = lem.Totals()
    L = lem.load()
    t0 = time.perf_counter()
    for j, i in enumerate(range(args.warmup + args.steps, args.warmup + 2 * args.steps)):
        clim = lem.Climate(float(sc.rain[i]), float(sc.temp[i]), 1)
        lem._check(L.lem_step(g.h, C.byref(clim), 0), "lem_step")
        h2d += C.sizeof(clim)
        lem._check(L.lem_get_totals(g.h, C.byref(tot)), "lem_get_totals")  # the budget row of the step
        d2h += C.sizeof(tot)
        if j % 50 == 0:  # writegrids: fd, fa, dem every 50 steps; erosion grids every 100
            for f in ("fd", "fa", "dem"):
                d2h += g.get(f).nbytes
        if j % 100 == 0:
            for f in ("ero", "inci", "geli", "depo"):
                d2h += g.get(f).nbytes
    g.synchronize()
    e2e_s = reduce_max(dist, time.perf_counter() - t0)
    e2e = cells_all * args.steps / e2e_s

    if rank != 0:
        g.close()
        if dist is not None:
            dist.destroy_process_group()
        return 0

    # roofline of the dominant kernel
    hbm, peak_kind = peaks()
    dom = max(prof.items(), key=lambda kv: kv[1][1]) if prof else ("none", (1, 1.0))
    kname, (klaunches, kms) = dom
    kbytes_per_launch = KERNEL_BYTES.get(kname, 0) * cells
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic_per_launch.json")
    if os.path.exists(tfile):
        try:
            traffic = json.load(open(tfile)).get(kname)
        except Exception:
            traffic = None
    bytes_source = "algorithmic"
    if kbytes_per_launch == 0 and traffic:
        # data-dependent kernel: its measured DRAM bytes per launch stand in
        kbytes_per_launch = traffic
        bytes_source = "ncu dram bytes per launch (data-dependent kernel)"
    achieved = kbytes_per_launch / (kms / klaunches / 1e3) / 1e9 if kms > 0 else 0.0
    cpu = None if args.no_cpu else cpu_sample(S)
    step_ms = ms_max / args.steps
    line = {
        "metric": "cell-timesteps/s", "value": value, "unit": "cell-timesteps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded spectral DEM and climate series)",
        "config": {"workload": f"single large grid {args.grid}x{args.grid}, per-step climate series",
                   "grid": args.grid, "active_cells": cells, "cellsize_m": 30, "hurst": 0.7, "relief_m": 1500,
                   "nodata": 0.02, "pits": 5000 if args.grid == 4096 else "scaled", "plateaus": 300,
                   "parallelism": f"replicas x{world}",
                   "l2": "resident state ~1.6 GB per replica, larger than L2 (no flush needed)"},
        "e2e": {"value": e2e, "unit": "cell-timesteps/s", "h2d_bytes_per_step": h2d / args.steps,
                "d2h_bytes_per_step": d2h / args.steps},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_kind": f"{peak_kind} hbm_gbs",
                     "algorithmic_bytes_per_launch": kbytes_per_launch, "bytes_source": bytes_source,
                     "traffic": traffic,
                     "step_level": {"bytes_per_cell_timestep": B_ALG,
                                    "achieved": B_ALG * cells / (step_ms / 1e3) / 1e9,
                                    "frac": B_ALG * cells / (step_ms / 1e3) / 1e9 / hbm}},
        "kernels": {k: {"launches": v[0], "ms_per_step": v[1] / args.steps} for k, v in
                    sorted(prof.items(), key=lambda kv: -kv[1][1])},
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    g.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
