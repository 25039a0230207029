"""Benchmark of the GB300 landscape-evolution step (prints one JSON line).

Workloads (--workload):
* ensemble (default): the batched ensemble -- 64 square fp32 spectral DEMs with
  sides log-uniform in [256, 2048] (Hurst U(0.6, 0.9), relief U(200, 2000) m,
  30 m cells, 1-5 % nodata border, pits and plateaus at the density of the
  4096x4096 grid), each with its own climate series, packed into one canvas
  and stepped together (lem_step_batch: one launch per kernel for all DEMs).
  The plain path on the same DEMs (one grid at a time) is timed beside it on
  a sample of the DEMs and reported as `plain`;
* grid: the single large grid -- 4096x4096 (Hurst 0.7, relief 0-1500 m, 2 %
  nodata, 5000 pits, 300 plateaus), one DEM per handle.
A "step" is one model timestep of the hot path for every DEM: flow direction
with plateau routing and sink flooding, runoff and flow accumulation, erosion,
sediment routing and the surface/soil/vegetation update.

* value: cell-timesteps/s (masked-in cells x steps / s) with the state resident
  on the device, timed with CUDA events on the library's stream;
* e2e: the same metric through the public C ABI with the host side of the
  reference driver: each step uploads every DEM's climate and reads back its
  budget row, and every 50th/100th step downloads the grids lem.cpp writes
  then (writegrids, MEM_kernels/io.cpp:201-230);
* roofline: the dominant kernel's algorithmic bytes / its event-timed duration
  against the measured HBM copy bandwidth, and the step-level figure;
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
    "k_flowdirs": 23,                 # FlowDirs, two launches per step: 38 / 2, + W plateau distance (routing)
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


def init_dist(world, local, backend=None):
    """One process group over the ranks (NCCL on the GPU machine; gloo where no GPU
    is visible, as in the CPU tests)."""
    if world <= 1:
        return None
    import torch
    import torch.distributed as dist
    if backend is None:
        backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return dist


def _dist_device(dist):
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def reduce_max(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=_dist_device(dist))
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=_dist_device(dist))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def whole_job(dist, cells, steps, ms):
    """The whole job's throughput: the cells all replicas stepped over the
    slowest replica's time (weak scaling: every rank steps its own DEMs).
    Returns (cell-timesteps/s, max ms, cells of all ranks)."""
    ms_max = reduce_max(dist, ms)
    cells_all = reduce_sum(dist, cells)
    return cells_all * steps / (ms_max / 1e3), ms_max, cells_all


def cpu_sample(sc, seconds=12.0, max_steps=8, label=""):
    """The FP64 oracle on a bounded sample of the workload: one DEM of it stepped
    until `seconds` pass."""
    from parallem_gb300 import scenario as S
    from oracle import oracle
    oracle.build()
    threads = oracle.num_threads()
    st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
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
    n = sc.dem.shape[0]
    return {"value": cells * steps / dt, "unit": "cell-timesteps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} timesteps of {label}a {n}x{n} DEM of the workload ({cells} active cells), "
                      f"FP64 oracle, {threads} OpenMP threads, {dt:.1f} s"}


def sample_scenario(args):
    """The DEM the host-core samples run on: for the ensemble its largest DEM
    below 1024x1024, for the single grid a 1024x1024 grid of the same generator."""
    from parallem_gb300 import scenario as S
    if args.workload == "ensemble":
        ens = S.config_ensemble(count=args.dems, steps=8)
        small = [x for x in ens if x.dem.shape[0] <= 1024]
        return max(small or ens, key=lambda x: x.dem.size)
    return S.config_large(2, n=1024, steps=8)


def run_reference(args):
    """The reference's algorithm on the host cores (the oracle port: the reference
    itself is CUDA and has no CPU implementation; its kernels compile on the CPU
    only where its sources are present), on a bounded sample of the workload."""
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    from parallem_gb300 import scenario as S
    from oracle import oracle
    oracle.build()
    threads = oracle.num_threads()
    sc = sample_scenario(args)
    st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    m = oracle.OracleModel(sc.dem, 30.0, st, sc.init_rain, sc.init_temp, diagnostics=False)
    cells = int((st["mask"] == 1).sum())
    n = sc.dem.shape[0]
    rain = list(sc.rain) * (1 + (args.warmup + args.steps) // len(sc.rain))
    temp = list(sc.temp) * (1 + (args.warmup + args.steps) // len(sc.temp))
    for i in range(args.warmup):
        m.step(rain[i], temp[i], True)
    t0 = time.perf_counter()
    for i in range(args.warmup, args.warmup + args.steps):
        m.step(rain[i], temp[i], True)
    dt = time.perf_counter() - t0
    value = cells * args.steps / dt
    line = {
        "impl": "reference", "metric": "cell-timesteps/s", "value": value, "unit": "cell-timesteps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(args) + f", sampled on the host as one {n}x{n} DEM",
                   "sample_dem": n, "cellsize_m": 30, "climate": "per-step series"},
        "cpu_baseline": {"value": value, "unit": "cell-timesteps/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} timesteps of one {n}x{n} DEM of the workload ({cells} active cells)"},
        "e2e": {"value": value, "unit": "cell-timesteps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def workload_name(args):
    if args.workload == "serve":
        return "serving: Poisson arrivals, sides log-uniform in [128, 4096], 10-500 steps, own climate series"
    if args.workload == "ensemble":
        return f"batched ensemble of {args.dems} DEMs, sides log-uniform in [256, 2048], per-DEM climate series"
    return f"single large grid {args.grid}x{args.grid}, per-step climate series"


class GridWork:
    """One large grid on one handle (the plain path)."""

    def __init__(self, lem, S, args, rank, total_steps):
        self.sc = S.config_large(2 + rank, n=args.grid, steps=max(total_steps, 100))  # the 100-step series
        st = S.initial_state(self.sc.dem, 30.0, self.sc.init_rain, self.sc.init_temp)
        self.cells = int((st["mask"] == 1).sum())
        self.g = lem.Model(self.sc.dem, 30.0, self.sc.init_rain, self.sc.init_temp)
        self.g.set_state(st)
        self.g.graphs(not args.no_graphs)
        self.lem = lem

    def step(self, i):
        self.g.step(self.sc.rain[i], self.sc.temp[i], True)

    def e2e_step(self, i, j):
        import ctypes as C
        lem = self.lem
        L = lem.load()
        clim = lem.Climate(float(self.sc.rain[i]), float(self.sc.temp[i]), 1)
        lem._check(L.lem_step(self.g.h, C.byref(clim), 0), "lem_step")
        tot = lem.Totals()
        lem._check(L.lem_get_totals(self.g.h, C.byref(tot)), "lem_get_totals")  # the budget row of the step
        h2d, d2h = C.sizeof(clim), C.sizeof(tot)
        if j % 50 == 0:  # writegrids: fd, fa, dem every 50 steps; erosion grids every 100
            for f in ("fd", "fa", "dem"):
                d2h += self.g.get(f).nbytes
        if j % 100 == 0:
            for f in ("ero", "inci", "geli", "depo"):
                d2h += self.g.get(f).nbytes
        return h2d, d2h

    def config(self, args):
        return {"workload": workload_name(args), "grid": args.grid, "active_cells": self.cells, "cellsize_m": 30,
                "hurst": 0.7, "relief_m": 1500, "nodata": 0.02, "pits": 5000 if args.grid == 4096 else "scaled",
                "plateaus": 300, "l2": "resident state ~5 GB, larger than L2 (no flush needed)"}

    def close(self):
        self.g.close()


class EnsembleWork:
    """The batched ensemble: every DEM in one canvas, one lem_step_batch per step."""

    def __init__(self, lem, S, args, rank, total_steps):
        from parallem_gb300.packing import TilePacker
        self.lem = lem
        # 200-step climate series per DEM, repeated beyond 200 steps (the DEMs
        # do not depend on the steps run)
        self.ens = S.config_ensemble(4 + rank, count=args.dems, steps=200)
        order = sorted(range(len(self.ens)), key=lambda i: -self.ens[i].dem.size)
        W = args.canvas
        H = 1024
        while True:  # the smallest canvas height that holds every DEM (largest first)
            p = TilePacker(W, H)
            if all(p.alloc(self.ens[i].dem.shape[1], self.ens[i].dem.shape[0]) is not None for i in order):
                break
            H += 512
        self.canvas = (W, H)
        self.b = lem.Batch(W, H, 30.0, max_dems=len(self.ens))
        self.ids = [None] * len(self.ens)
        self.cells = 0
        for i in order:
            sc = self.ens[i]
            st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
            k = self.b.add(sc.dem, sc.init_rain, sc.init_temp)
            self.b.set_state(k, st)
            self.ids[i] = k
            self.cells += int((st["mask"] == 1).sum())
        self.g = self.b  # timing, profiling and launch counts of the batch handle
        self.b.graphs(not args.no_graphs)

    def step(self, i):
        for sc, k in zip(self.ens, self.ids):
            self.b.set_climate(k, float(sc.rain[i % len(sc.rain)]), float(sc.temp[i % len(sc.temp)]), True)
        self.b.step()

    def e2e_step(self, i, j):
        import ctypes as C
        lem = self.lem
        L = lem.load()
        h2d = d2h = 0
        for sc, k in zip(self.ens, self.ids):
            clim = lem.Climate(float(sc.rain[i % len(sc.rain)]), float(sc.temp[i % len(sc.temp)]), 1)
            lem._check(L.lem_dem_set_climate(self.b.h, k, C.byref(clim)), "lem_dem_set_climate")
            h2d += C.sizeof(clim)
        lem._check(L.lem_step_batch(self.b.h, 0), "lem_step_batch")
        # writegrids: fd, fa, dem every 50 steps, erosion grids every 100.  The
        # grids leave through the asynchronous export (a snapshot on the step
        # stream, the copy to the host on the second stream); while a step runs
        # the host receives a share of the grids exported earlier, so the copies
        # and conversions overlap the steps, and all of them complete inside the
        # timed region.
        exports = getattr(self, "exports", [])
        if exports:
            take = -(-len(exports) // max(1, 50 - j % 50))
            for e in exports[:take]:
                d2h += sum(a.nbytes for a in e.wait().values())
            self.exports = exports[take:]
        n = len(self.ids)
        tot = (lem.Totals * n)()
        lem._check(L.lem_dem_get_totals_n(self.b.h, (C.c_int32 * n)(*self.ids), n, tot), "lem_dem_get_totals_n")
        d2h += C.sizeof(tot)  # every DEM's budget row of the step
        if j % 50 == 0:
            d2h += self.e2e_finish()
            names = ("fd", "fa", "dem") + (("ero", "inci", "geli", "depo") if j % 100 == 0 else ())
            self.exports = [self.b.export(k, names) for k in self.ids]
        return h2d, d2h

    def e2e_warm(self):
        """One untimed export of the largest field set of every DEM: the pinned
        host buffers the timed exports reuse."""
        self.exports = [self.b.export(k, ("fd", "fa", "dem", "ero", "inci", "geli", "depo")) for k in self.ids]
        self.e2e_finish()

    def e2e_finish(self):
        """Waits for the grids still on their way; returns the bytes the host received."""
        d2h = 0
        for e in getattr(self, "exports", []):
            d2h += sum(a.nbytes for a in e.wait().values())
        self.exports = []
        return d2h

    def plain_sample(self, args, steps=5, budget_s=25.0):
        """The plain path on the same DEMs, one handle and one grid at a time:
        every fourth DEM by size (all sizes covered), each with the batched arm's
        launch schedule -- CUDA-graph steps and the autotuner (lem_autotune(1):
        5 tuning steps) -- then 2 warm-up and `steps` device-timed steps."""
        lem = self.lem
        from parallem_gb300 import scenario as S
        order = sorted(range(len(self.ens)), key=lambda i: self.ens[i].dem.size)
        pick = order[::4]
        cells = 0
        secs = 0.0
        t_start = time.perf_counter()
        done = 0
        for i in pick:
            sc = self.ens[i]
            st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
            m = lem.Model(sc.dem, 30.0, sc.init_rain, sc.init_temp)
            m.set_state(st)
            m.graphs(not args.no_graphs)
            m.autotune(1)
            k = 0
            for _ in range(5 + 2):  # tuning, then warm-up steps
                m.step(sc.rain[k % len(sc.rain)], sc.temp[k % len(sc.temp)], True)
                k += 1
            m.synchronize()
            m.record(0)
            for _ in range(steps):
                m.step(sc.rain[k % len(sc.rain)], sc.temp[k % len(sc.temp)], True)
                k += 1
            m.record(1)
            secs += m.elapsed_ms(0, 1) / 1e3
            cells += int((st["mask"] == 1).sum()) * steps
            m.close()
            done += 1
            if time.perf_counter() - t_start > budget_s:
                break
        return {"value": cells / secs, "unit": "cell-timesteps/s",
                "sample": f"{done} of the {len(self.ens)} DEMs (every fourth by size), each on its own handle with "
                          f"graph steps and its own autotuned schedule, {steps} device-timed steps each"}

    def rounds(self):
        """Rounds of the step's device loops (canvas-wide, the last step)."""
        t = self.b.totals(self.ids[0])
        return {k: t[k] for k in ("plateau_sweeps", "merge_rounds", "label_rounds", "spill_rounds", "flood_edges")}

    def config(self, args):
        sides = sorted(x.dem.shape[0] for x in self.ens)
        return {"workload": workload_name(args), "dems": len(self.ens), "active_cells": self.cells,
                "canvas": f"{self.canvas[0]}x{self.canvas[1]}", "sides": [sides[0], sides[len(sides) // 2], sides[-1]],
                "cellsize_m": 30, "l2": "resident state ~20 GB, larger than L2 (no flush needed)"}

    def close(self):
        self.b.close()


def grid_sample(args, steps=5):
    """The plain path on the single large grid (4096x4096, per-step climate):
    graph steps, the autotuner's 13 steps, 3 warm-up steps, `steps` timed."""
    from parallem_gb300 import lem
    from parallem_gb300 import scenario as S
    sc = S.config_large(2, n=4096, steps=100)
    st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    cells = int((st["mask"] == 1).sum())
    g = lem.Model(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    g.set_state(st)
    g.graphs(True)
    g.autotune(3)
    k = 0
    for _ in range(13 + 3):
        g.step(sc.rain[k], sc.temp[k], True)
        k += 1
    g.synchronize()
    g.record(0)
    for _ in range(steps):
        g.step(sc.rain[k], sc.temp[k], True)
        k += 1
    g.record(1)
    ms = g.elapsed_ms(0, 1) / steps
    g.close()
    return {"workload": "single large grid 4096x4096, per-step climate series (the plain path)",
            "value": cells / (ms / 1e3), "unit": "cell-timesteps/s", "ms_per_step": ms, "active_cells": cells,
            "steps": steps}


def routing_sample():
    """The routing stress configuration in isolation: one 8192x8192 DEM with
    10 % of its cells in 1 m-quantised flats and 50k nested depressions; the
    flow-direction stage (with plateau routing and sink flooding) and the
    accumulation, SFD on the tiled path, SFD with the int32 contributing-cell
    counts (the global wave) and MFD with slope-proportional shares, each timed
    with events on the library's stream after one untimed run."""
    from parallem_gb300 import lem
    from parallem_gb300 import scenario as S
    sc = S.config_routing(3, n=8192)
    st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    cells = int((st["mask"] == 1).sum())
    out = {"workload": "routing stress 8192x8192: 10 % of cells in 1 m flats, 50k nested depressions, one step of "
                       "flow direction and accumulation", "active_cells": cells}

    def timed(g, fn):
        fn()  # untimed: first use
        g.set_state({"soilM": st["soilM"]})
        g.synchronize()
        g.record(0)
        fn()
        g.record(1)
        return g.elapsed_ms(0, 1)

    g = lem.Model(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    g.set_state(st)
    out["flow_direction_ms"] = timed(g, g.flow_direction)
    t = g.totals()
    out.update({k: t[k] for k in ("plateau_sweeps", "merge_rounds", "label_rounds", "spill_rounds", "flood_edges",
                                  "sinkcount", "initial_sinks", "initial_flats")})
    out["sfd_accumulation_ms"] = timed(g, lambda: g.flow_accumulation(0))
    out["sfd_contributing_counts_ms"] = timed(g, lambda: g.flow_accumulation(lem.STEP_CONTRIB))
    g.close()
    m = lem.Model(sc.dem, 30.0, sc.init_rain, sc.init_temp,
                  params=lem.make_params(flow_direction_type=1, mfd_proportions=1))
    m.set_state(st)
    m.flow_direction()
    out["mfd_accumulation_ms"] = timed(m, lambda: m.flow_accumulation(0))
    m.close()
    for k in ("flow_direction", "sfd_accumulation", "sfd_contributing_counts", "mfd_accumulation"):
        out[k + "_cells_per_s"] = cells / (out[k + "_ms"] / 1e3)
    return out


def serve_sample(rate=20.0, requests=24, canvas=(16384, 12288), budget_gb=150.0):
    """The serving workload at one arrival rate: Poisson arrivals, sides
    log-uniform in [128, 4096], 10-500 steps, own climate series, continuously
    batched under the HBM budget; p50/p99 latency from arrival to the result
    grids on the host."""
    from parallem_gb300 import serve as SV
    rng = np.random.default_rng(11)
    t = 0.0
    reqs = []
    for i in range(requests):
        t += float(rng.exponential(1.0 / rate))
        reqs.append(SV.make_request(i, rng, t))
    srv = SV.Server(canvas[0], canvas[1], budget_bytes=budget_gb * 1e9, max_dems=max(64, requests))
    warm = SV.make_request(-1, np.random.default_rng(1), 0.0, side_lo=128, side_hi=256, steps_lo=3, steps_hi=3)
    srv.run([warm])
    srv.steps_run = 0
    stats = srv.run(reqs)
    srv.close()
    return {"workload": "serving: Poisson arrivals, sides log-uniform in [128, 4096], 10-500 steps",
            "rate_per_s": rate, "requests": stats["requests"], "refused": stats["refused"],
            "p50_latency_s": stats["p50_latency_s"], "p99_latency_s": stats["p99_latency_s"],
            "value": stats["cell_timesteps_per_s"], "unit": "cell-timesteps/s", "wall_s": stats["wall_s"],
            "batch_steps": stats["batch_steps"], "hbm_budget_gb": budget_gb,
            "bytes_per_canvas_cell": stats["bytes_per_cell"]}


def run_serve(args):
    """The serving workload: Poisson arrivals of landscape-scenario requests
    (sides log-uniform in [128, 4096], 10-500 steps, own climate series)
    admitted by canvas room and the HBM budget, continuously batched; one JSON
    line with throughput and p50/p99 latency."""
    rank, world, local = dist_env()
    from parallem_gb300 import build, lem
    from parallem_gb300 import serve as SV
    build.build()
    lem.select_device(local)
    rng = np.random.default_rng(11 + rank)
    t = 0.0
    reqs = []
    for i in range(args.requests):
        t += float(rng.exponential(1.0 / args.rate))
        reqs.append(SV.make_request(i, rng, t))
    W, H = args.canvas_serve
    srv = SV.Server(W, H, budget_bytes=args.budget_gb * 1e9, max_dems=max(64, args.requests))
    # warm-up: one small request through the whole path
    warm = SV.make_request(-1, np.random.default_rng(1), 0.0, side_lo=128, side_hi=256, steps_lo=3, steps_hi=3)
    srv.run([warm])
    srv.steps_run = 0
    srv.b.synchronize()
    with ClockSampler(local) as clk:
        stats = srv.run(reqs)
    srv.close()
    if rank != 0:
        return 0
    line = {
        "metric": "cell-timesteps/s", "value": stats["cell_timesteps_per_s"], "unit": "cell-timesteps/s",
        "n_gpus": world, "steps": stats["batch_steps"], "warmup": 1, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded spectral DEMs and climate series)",
        "config": {"workload": "serving: Poisson arrivals, sides log-uniform in [128, 4096], 10-500 steps",
                   "rate_per_s": args.rate, "requests": args.requests, "canvas": f"{W}x{H}",
                   "hbm_budget_gb": args.budget_gb, "parallelism": f"replicas x{world}"},
        "latency": {"p50_s": stats["p50_latency_s"], "p99_s": stats["p99_latency_s"]},
        "wall_s": stats["wall_s"], "requests_done": stats["requests"],
        "e2e": {"value": stats["cell_timesteps_per_s"], "unit": "cell-timesteps/s",
                "note": "arrival to result on the host, grids streamed back"},
        "clocks": clk.summary(),
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="ensemble", choices=["ensemble", "grid", "serve"])
    ap.add_argument("--rate", type=float, default=20.0, help="serving: arrivals per second")
    ap.add_argument("--requests", type=int, default=24, help="serving: requests")
    ap.add_argument("--canvas-serve", type=int, nargs=2, default=[16384, 12288], help="serving: canvas W H")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="serving: HBM budget")
    ap.add_argument("--grid", type=int, default=4096, help="side of the single grid")
    ap.add_argument("--dems", type=int, default=64, help="DEMs of the ensemble")
    ap.add_argument("--canvas", type=int, default=8192, help="width of the ensemble's canvas")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline sample")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-path sample of the ensemble")
    ap.add_argument("--no-graphs", action="store_true", help="step eagerly instead of one CUDA graph per step")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch schedule (no autotuning steps)")
    ap.add_argument("--no-extras", action="store_true",
                    help="ensemble: skip the 4096x4096, 8192x8192 routing and serving samples")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "serve":
        return run_serve(args)

    rank, world, local = dist_env()
    dist = init_dist(world, local)
    from parallem_gb300 import build, lem
    from parallem_gb300 import scenario as S
    if rank == 0 or world == 1:
        build.build()
    barrier(dist)
    lem.select_device(local)
    tune_steps = 0 if args.no_tune else 13  # lem_autotune(3): one unmeasured step, then 3 x 4 candidate steps
    # the end-to-end region runs 100 steps: the reference writes its grids every
    # 50th and 100th step, so fewer steps would overweight those downloads
    e2e_steps = 100
    total_steps = tune_steps + args.warmup + 2 * args.steps + e2e_steps
    work = (EnsembleWork if args.workload == "ensemble" else GridWork)(lem, S, args, rank, total_steps)
    g = work.g
    cells = work.cells

    # autotuning steps, then warm-up steps (untimed)
    if tune_steps:
        g.autotune(3)
        for i in range(tune_steps):
            work.step(i)
    for i in range(tune_steps, tune_steps + args.warmup):
        work.step(i)
    g.synchronize()
    tuning = g.tuning()
    barrier(dist)
    i0 = tune_steps + args.warmup  # step index of the first timed step

    # timed region 1: resident state, device events on the library's stream
    # (each step one CUDA graph launch unless --no-graphs)
    launches0 = g.launches
    with ClockSampler(local) as clk:
        g.record(0)
        for i in range(i0, i0 + args.steps):
            work.step(i)
        g.record(1)
        ms = g.elapsed_ms(0, 1)
    g.synchronize()
    launches = g.launches - launches0
    value, ms_max, cells_all = whole_job(dist, cells, args.steps, ms)

    # timed region 2: the same steps launched eagerly with a pair of events
    # around every kernel (the per-kernel times and the roofline's duration)
    barrier(dist)
    g.profiling(True)
    g.record(2)
    for i in range(i0 + args.steps, i0 + 2 * args.steps):
        work.step(i)
    g.record(3)
    eager_ms = g.elapsed_ms(2, 3)
    prof = g.profile()
    g.profiling(False)
    g.synchronize()

    # timed region 3: end to end through the C ABI with host buffers
    if hasattr(work, "e2e_warm"):
        work.e2e_warm()
        g.synchronize()
    barrier(dist)
    h2d = d2h = 0
    t0 = time.perf_counter()
    for j, i in enumerate(range(i0 + 2 * args.steps, i0 + 2 * args.steps + e2e_steps)):
        a, b = work.e2e_step(i, j)
        h2d += a
        d2h += b
    if hasattr(work, "e2e_finish"):
        d2h += work.e2e_finish()
    g.synchronize()
    e2e_s = reduce_max(dist, time.perf_counter() - t0)
    e2e = cells_all * e2e_steps / e2e_s

    if rank != 0:
        work.close()
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
            traffic = json.load(open(tfile)).get(args.workload, {}).get(kname)
        except Exception:
            traffic = None
    bytes_source = "algorithmic"
    if kbytes_per_launch == 0 and traffic:
        # data-dependent kernel: its measured DRAM bytes per launch stand in
        kbytes_per_launch = traffic
        bytes_source = "ncu dram bytes per launch (data-dependent kernel)"
    achieved = kbytes_per_launch / (kms / klaunches / 1e3) / 1e9 if kms > 0 else 0.0
    plain = None
    if args.workload == "ensemble" and not args.no_plain:
        plain = work.plain_sample(args)
    cpu = None if args.no_cpu else cpu_sample(sample_scenario(args))
    step_ms = ms_max / args.steps
    config = work.config(args)
    config["parallelism"] = f"replicas x{world}"
    line = {
        "metric": "cell-timesteps/s", "value": value, "unit": "cell-timesteps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded spectral DEMs and climate series)",
        "config": config,
        "e2e": {"value": e2e, "unit": "cell-timesteps/s", "h2d_bytes_per_step": h2d / e2e_steps,
                "d2h_bytes_per_step": d2h / e2e_steps, "steps": e2e_steps},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_kind": f"{peak_kind} hbm_gbs",
                     "algorithmic_bytes_per_launch": kbytes_per_launch, "bytes_source": bytes_source,
                     "traffic": traffic,
                     "step_level": {"bytes_per_cell_timestep": B_ALG,
                                    "achieved": B_ALG * cells / (step_ms / 1e3) / 1e9,
                                    "frac": B_ALG * cells / (step_ms / 1e3) / 1e9 / hbm}},
        "graphs": not args.no_graphs,
        "tuning": tuning,
        "kernels": {k: {"launches": v[0], "ms_per_step": v[1] / args.steps} for k, v in
                    sorted(prof.items(), key=lambda kv: -kv[1][1])},
        "kernel_timing": {"source": f"{args.steps} eagerly launched steps after the timed region, "
                                    "CUDA events around every kernel on the library's stream",
                          "eager_ms_per_step": eager_ms / args.steps},
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    if plain is not None:
        line["plain"] = plain
        line["batched_over_plain"] = value / plain["value"]
    if hasattr(work, "rounds"):
        line["loop_rounds"] = work.rounds()
    work.close()
    if args.workload == "ensemble" and not args.no_extras and world == 1:
        # the other workloads, measured in the same run: the single large grid
        # on the plain path, the routing stress grid and serving at 20 requests/s
        line["grid_4096"] = grid_sample(args)
        line["routing_8192"] = routing_sample()
        line["serving"] = serve_sample()
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
