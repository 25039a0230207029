"""Serving: a continuous-batching request loop over one batch handle.

Landscape-scenario requests (a DEM, its initial state, a climate series and a
step count) arrive over time.  Each loop iteration

* drops requests cancelled while waiting, and removes cancelled ones from the
  batch at the step boundary;
* refuses, at once, a request that can never run: its DEM does not fit the
  canvas, or its reservation alone exceeds the HBM budget;
* admits, first come first served, every arrived request that fits: a free
  canvas region for its DEM, and its reservation within what the budget has
  left;
* advances every admitted request by one timestep with one lem_step_batch, so
  requests that arrive while others run join at the next step and their work
  overlaps on the device;
* starts, for every request that has run its steps, the asynchronous export
  of its result grids (lem_dem_export: a snapshot on the batch stream, the copy
  to the host on a second stream) and frees its region, so the next step does
  not wait for the download;
* completes the exports whose copies have finished.

A request's reservation is the device memory it holds: its region's 32x32
tiles at the batch handle's measured bytes per canvas cell (lem_device_bytes
over the canvas), plus its export snapshot while that is in flight.  Latency
is result-on-the-host minus arrival; throughput is the cell-timesteps of all
completed requests over the wall time.

No counterpart in the reference, which runs one scenario per process.
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import lem as L
from . import scenario as S

TILE = 32
# bytes per cell of each exported field's device copy (lem_dem_export's snapshot)
EXPORT_BYTES = {"dem": 8, "fa": 8, "slopes": 32, "fd": 1, "sfd": 1, "sfd_pass1": 1, "mask": 1, "contrib": 4,
                "watershed": 4}


@dataclass
class Request:
    rid: int
    dem: np.ndarray
    state: dict
    rain: np.ndarray
    temp: np.ndarray
    steps: int
    arrival: float                    # seconds from the start of the run
    outputs: tuple = ("dem", "fa", "soilT", "stone", "depo")
    cancel_at: float | None = None    # seconds from the start of the run (None: never)
    # filled in by the server
    status: str = "pending"           # pending, active, streaming, done, refused, cancelled
    reason: str = ""
    admitted: float = -1.0
    done: float = -1.0
    cells: int = 0
    reserved: int = 0                 # bytes held against the budget
    result: dict = field(default_factory=dict)
    totals: list = field(default_factory=list)


def make_request(rid: int, rng: np.random.Generator, arrival: float, side_lo: int = 128, side_hi: int = 4096,
                 steps_lo: int = 10, steps_hi: int = 500) -> Request:
    """A scenario of the serving workload: a square DEM with side log-uniform in
    [side_lo, side_hi], a step count uniform in [steps_lo, steps_hi] and its own
    climate series."""
    n = int(round(np.exp(rng.uniform(np.log(side_lo), np.log(side_hi)))))
    steps = int(rng.integers(steps_lo, steps_hi + 1))
    scale = (n / 4096.0) ** 2
    dem = S.make_dem(n, float(rng.uniform(0.6, 0.9)), float(rng.uniform(200.0, 2000.0)),
                     float(rng.uniform(0.01, 0.05)), max(1, int(5000 * scale)), max(1, int(300 * scale)),
                     int(rng.integers(1 << 30)))
    st = S.initial_state(dem, 30.0, 900.0, 9.0)
    sigma = np.sqrt(np.log(1.09))
    rain = rng.lognormal(np.log(900.0) - 0.5 * sigma * sigma, sigma, size=steps)
    temp = rng.normal(9.0, 2.0, size=steps)
    return Request(rid, dem, st, rain, temp, steps, arrival)


def _tiles(n: int) -> int:
    return (n + TILE - 1) // TILE * TILE


class Server:
    def __init__(self, canvas_w: int, canvas_h: int, budget_bytes: float = 150e9, max_dems: int = 1024,
                 params=None, graphs: bool = True, batch=None):
        self.b = batch if batch is not None else L.Batch(canvas_w, canvas_h, 30.0, max_dems=max_dems, params=params)
        self.b.graphs(graphs)  # each step one graph launch, captured again when requests join or leave
        self.W, self.H = canvas_w, canvas_h
        self.budget = float(budget_bytes)
        self.canvas_bytes = int(self.b.device_bytes())
        self.bytes_per_cell = self.canvas_bytes / float(canvas_w * canvas_h)
        self.active = {}      # batch id -> [request, steps done]
        self.streaming = []   # (request, export) whose grids are on their way to the host
        self.reserved = 0     # bytes held by active and streaming requests
        self.steps_run = 0
        self._cancel = set()
        self._lock = threading.Lock()

    def close(self):
        for r, ex in self.streaming:
            ex.wait()
        self.streaming = []
        self.b.close()

    def cancel(self, rid: int):
        """Cancels request `rid` (safe from another thread): a waiting request is
        dropped, a running one leaves the batch at the next step boundary."""
        with self._lock:
            self._cancel.add(rid)

    def reservation(self, r: Request) -> int:
        """Device bytes request r holds: its region's tiles, and its export snapshot."""
        hgt, wid = r.dem.shape
        tiles = _tiles(wid) * _tiles(hgt) * self.bytes_per_cell
        snap = wid * hgt * (sum(EXPORT_BYTES.get(f, 4) for f in r.outputs) + 1) + 4096
        return int(tiles + snap)

    def _cancelled(self, r: Request, now: float) -> bool:
        with self._lock:
            flagged = r.rid in self._cancel
        return flagged or (r.cancel_at is not None and now >= r.cancel_at)

    def _refusal(self, r: Request) -> str:
        hgt, wid = r.dem.shape
        if wid > self.W or hgt > self.H:
            return f"DEM {wid}x{hgt} does not fit the {self.W}x{self.H} canvas"
        need = self.reservation(r)
        if need > self.budget:
            return f"needs {need} bytes of device memory, the budget is {int(self.budget)}"
        return ""

    def _admit(self, r: Request, now: float) -> bool:
        need = self.reservation(r)
        if self.reserved + need > self.budget:
            return False
        i = self.b.add(r.dem, 900.0, 9.0)
        if i is None:
            return False
        self.b.set_state(i, r.state)
        self.b.set_step_flags(i, L.STEP_SET_OUTLET_FROM_FA)  # its first step, as lem.cpp's first iteration
        r.admitted = now
        r.status = "active"
        r.cells = int((r.state["mask"] == 1).sum())
        r.reserved = need
        self.reserved += need
        self.active[i] = [r, 0]
        return True

    def _release(self, r: Request):
        self.reserved -= r.reserved
        r.reserved = 0

    def run(self, requests: list, clock=time.perf_counter, keep_totals: bool = False) -> dict:
        """Serves `requests` (sorted by arrival) to completion; returns the statistics."""
        pending = list(requests)
        t0 = clock()
        done, refused, cancelled = [], [], []
        while pending or self.active or self.streaming:
            now = clock() - t0
            # cancellations: waiting requests are dropped, running ones leave the batch
            for r in [r for r in pending if r.arrival <= now and self._cancelled(r, now)]:
                pending.remove(r)
                r.status, r.done = "cancelled", now
                cancelled.append(r)
            for i in [i for i, (r, _) in self.active.items() if self._cancelled(r, now)]:
                r = self.active.pop(i)[0]
                self.b.remove(i)
                self._release(r)
                r.status, r.done = "cancelled", now
                cancelled.append(r)
            # refusals and admissions, first come first served
            while pending and pending[0].arrival <= now:
                why = self._refusal(pending[0])
                if why:
                    r = pending.pop(0)
                    r.status, r.reason, r.done = "refused", why, now
                    refused.append(r)
                    continue
                if not self._admit(pending[0], now):
                    break  # wait for room
                pending.pop(0)
            # exports whose copies have finished
            still = []
            for r, ex in self.streaming:
                if ex.ready():
                    r.result = ex.wait()
                    r.done = clock() - t0
                    r.status = "done"
                    self._release(r)
                    done.append(r)
                else:
                    still.append((r, ex))
            self.streaming = still
            if not self.active:
                if pending or self.streaming:  # idle until the next arrival or copy
                    nxt = pending[0].arrival - now if pending else 0.001
                    time.sleep(max(0.0, min(nxt, 0.01)))
                continue
            for i, (r, k) in self.active.items():
                self.b.set_climate(i, float(r.rain[k]), float(r.temp[k]), True)
            self.b.step()
            self.steps_run += 1
            finished = []
            for i, rk in self.active.items():
                rk[1] += 1
                if keep_totals:
                    rk[0].totals.append(self.b.totals(i))
                if rk[1] == rk[0].steps:
                    finished.append(i)
            for i in finished:
                r = self.active.pop(i)[0]
                # the snapshot is taken on the batch stream after this step; the
                # copy to the host overlaps the next steps
                self.streaming.append((r, self.b.export(i, r.outputs)))
                r.status = "streaming"
                self.b.remove(i)
        wall = clock() - t0
        lat = np.array([r.done - r.arrival for r in done])
        work = float(sum(r.cells * r.steps for r in done))
        return {"requests": len(done), "refused": len(refused), "cancelled": len(cancelled), "wall_s": wall,
                "batch_steps": self.steps_run,
                "p50_latency_s": float(np.percentile(lat, 50)) if lat.size else None,
                "p99_latency_s": float(np.percentile(lat, 99)) if lat.size else None,
                "cell_timesteps_per_s": work / wall if wall > 0 else 0.0,
                "bytes_per_cell": self.bytes_per_cell, "canvas_bytes": self.canvas_bytes}


def run_alone(r: Request, params=None) -> dict:
    """The same request on its own single-grid handle (the reference for the mix)."""
    m = L.Model(r.dem, 30.0, 900.0, 9.0, params=params)
    m.set_state(r.state)
    for k in range(r.steps):
        m.step(float(r.rain[k]), float(r.temp[k]), True, L.STEP_SET_OUTLET_FROM_FA if k == 0 else 0)
    out = {f: m.get(f) for f in r.outputs}
    m.close()
    return out
