"""Serving: a continuous-batching request loop over one batch handle.

Landscape-scenario requests (a DEM, its initial state, a climate series and a
step count) arrive over time.  Each loop iteration admits, first come first
served, every arrived request that fits -- a free canvas region for its DEM
and room under the HBM budget -- then advances every admitted request by one
timestep with one lem_step_batch, so requests that arrive while others run
join at the next step and their work overlaps on the device.  A request that
has run its steps streams its result grids back and leaves, freeing its region
for the next.  Latency is completion minus arrival; throughput is the
cell-timesteps of all requests over the wall time.

No counterpart in the reference, which runs one scenario per process.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import lem as L
from . import scenario as S

# device bytes per canvas cell of a batch handle (fields, tiles, flood tables)
BYTES_PER_CELL = 390


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
    # filled in by the server
    admitted: float = -1.0
    done: float = -1.0
    cells: int = 0
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


class Server:
    def __init__(self, canvas_w: int, canvas_h: int, budget_bytes: float = 150e9, max_dems: int = 1024,
                 params=None, graphs: bool = True):
        self.b = L.Batch(canvas_w, canvas_h, 30.0, max_dems=max_dems, params=params)
        self.b.graphs(graphs)  # each step one graph launch, captured again when requests join or leave
        self.budget = budget_bytes
        self.canvas_bytes = canvas_w * canvas_h * BYTES_PER_CELL
        self.active = {}      # batch id -> [request, steps done]
        self.steps_run = 0

    def close(self):
        self.b.close()

    def _admit(self, r: Request, now: float) -> bool:
        if self.canvas_bytes > self.budget:
            return False
        i = self.b.add(r.dem, 900.0, 9.0)
        if i is None:
            return False
        self.b.set_state(i, r.state)
        self.b.set_step_flags(i, L.STEP_SET_OUTLET_FROM_FA)  # its first step, as lem.cpp's first iteration
        r.admitted = now
        r.cells = int((r.state["mask"] == 1).sum())
        self.active[i] = [r, 0]
        return True

    def run(self, requests: list, clock=time.perf_counter, keep_totals: bool = False) -> dict:
        """Serves `requests` (sorted by arrival) to completion; returns the statistics."""
        pending = list(requests)
        t0 = clock()
        done = []
        while pending or self.active:
            now = clock() - t0
            while pending and pending[0].arrival <= now:
                if not self._admit(pending[0], now):
                    break  # first come first served: wait for room
                pending.pop(0)
            if not self.active:
                if pending:  # idle until the next arrival
                    time.sleep(max(0.0, min(pending[0].arrival - now, 0.01)))
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
                r.result = {f: self.b.get(i, f) for f in r.outputs}  # stream the result back
                r.done = clock() - t0
                self.b.remove(i)
                done.append(r)
        wall = clock() - t0
        lat = np.array([r.done - r.arrival for r in done])
        work = float(sum(r.cells * r.steps for r in done))
        return {"requests": len(done), "wall_s": wall, "batch_steps": self.steps_run,
                "p50_latency_s": float(np.percentile(lat, 50)) if lat.size else None,
                "p99_latency_s": float(np.percentile(lat, 99)) if lat.size else None,
                "cell_timesteps_per_s": work / wall if wall > 0 else 0.0}


def run_alone(r: Request, params=None) -> dict:
    """The same request on its own single-grid handle (the reference for the mix)."""
    m = L.Model(r.dem, 30.0, 900.0, 9.0, params=params)
    m.set_state(r.state)
    for k in range(r.steps):
        m.step(float(r.rain[k]), float(r.temp[k]), True, L.STEP_SET_OUTLET_FROM_FA if k == 0 else 0)
    out = {f: m.get(f) for f in r.outputs}
    m.close()
    return out
