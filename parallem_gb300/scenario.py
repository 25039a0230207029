"""Seeded synthetic landscape scenarios and initial model state.

The reference runs on an ESRI ASCII DEM (``30mfam.asc``) and a climate table
that are not part of its tree.  These generators stand in for them with
inputs of the stated shapes and value ranges:

* ``spectral_dem``: fractional-Brownian surface by spectral synthesis (random
  phases, amplitude ~ |k|^-(H+1)), rescaled to [0, relief] and stored as fp32;
* a nodata border (value -9999) whose inner edge is perturbed, at least two
  cells wide, covering the requested fraction of the grid;
* single-cell pits and clamped-elevation plateaus;
* ``initial_state``: the fields that setProcessMatrices and
  createSoilTfromformula give a new run (MEM_kernels/Data.cpp:115-209,
  MEM_kernels/memory.cu:197-214), with the par-file coefficients of
  default.par.

Everything here is host-side set-up; the per-step path runs on the GPU.
"""
from __future__ import annotations

import dataclasses
import numpy as np

NODATA = -9999.0

# default.par lines 11, 16-35 as parsed by readinpar (MEM_kernels/io.cpp:469-568)
DEFAULT_PAR = dict(
    flow_direction_type=0,
    mfd_proportions=0,
    soil_struct=2,
    profile_permeability=3,
    q_threshold=6.0,
    g_slope=1.0,
    kappa=0.00001,
    g_flowlim=600.0,
    flow_a=0.00001,
    flow_b=1.3,
    max_incision=0.001,
    ddk=0.9,
    dck=0.4,
    dgk=0.9,
    temp_inflex=6.0,
    temp_sens=6.0,
)
# initial soil values, default.par lines 14-21
DEFAULT_SOIL = dict(stone=20.0, fines=80.0, soilT=1.0, soilM=0.5, soilB=0.0, nut=10.0)


def spectral_dem(n_rows: int, n_cols: int, hurst: float, relief: float, rng: np.random.Generator) -> np.ndarray:
    """fBm surface by spectral synthesis, rescaled to [0, relief], fp32."""
    ky = np.fft.fftfreq(n_rows)[:, None]
    kx = np.fft.rfftfreq(n_cols)[None, :]
    k = np.sqrt(kx * kx + ky * ky)
    k[0, 0] = 1.0
    amp = k ** (-(hurst + 1.0))
    amp[0, 0] = 0.0
    phase = rng.uniform(0.0, 2.0 * np.pi, size=amp.shape)
    mag = rng.normal(size=amp.shape)
    spec = amp * mag * np.exp(1j * phase)
    z = np.fft.irfft2(spec, s=(n_rows, n_cols))
    z = (z - z.min()) / max(z.max() - z.min(), 1e-30) * relief
    return z.astype(np.float32)


def nodata_border(shape: tuple[int, int], fraction: float, rng: np.random.Generator) -> np.ndarray:
    """Boolean mask of a nodata border covering about `fraction` of the grid."""
    h, w = shape
    base = max(2, int(round(fraction * min(h, w) / 4.0)))
    yy, xx = np.mgrid[0:h, 0:w]
    dist = np.minimum(np.minimum(yy, h - 1 - yy), np.minimum(xx, w - 1 - xx))
    # perturb the inner edge with a smooth random field (wavelength ~ w/8)
    pert = spectral_dem(h, w, 0.9, 1.0, rng).astype(np.float64)
    width = 2 + np.floor((base - 2 + 0.5) * 2.0 * pert).astype(np.int64)
    return dist < np.maximum(width, 2)


def add_pits(z: np.ndarray, valid: np.ndarray, count: int, rng: np.random.Generator,
             depth=(0.5, 5.0)) -> None:
    h, w = z.shape
    ys = rng.integers(1, h - 1, size=count * 2)
    xs = rng.integers(1, w - 1, size=count * 2)
    placed = 0
    for y, x in zip(ys, xs):
        if placed == count:
            break
        if not valid[y - 1:y + 2, x - 1:x + 2].all():
            continue
        z[y, x] = np.float32(z[y, x] - rng.uniform(*depth))
        placed += 1


def add_plateaus(z: np.ndarray, valid: np.ndarray, count: int, rng: np.random.Generator,
                 across=(8, 40)) -> None:
    h, w = z.shape
    for _ in range(count):
        d = int(rng.integers(across[0], across[1] + 1))
        r = d / 2.0
        cy = int(rng.integers(int(r) + 2, max(int(r) + 3, h - int(r) - 2)))
        cx = int(rng.integers(int(r) + 2, max(int(r) + 3, w - int(r) - 2)))
        y0, y1 = max(1, int(cy - r)), min(h - 1, int(cy + r) + 1)
        x0, x1 = max(1, int(cx - r)), min(w - 1, int(cx + r) + 1)
        yy, xx = np.mgrid[y0:y1, x0:x1]
        disk = ((yy - cy) ** 2 + (xx - cx) ** 2 <= r * r) & valid[y0:y1, x0:x1]
        z[y0:y1, x0:x1][disk] = z[cy, cx]


def add_nested_depressions(z: np.ndarray, valid: np.ndarray, count: int, rng: np.random.Generator) -> None:
    """Bowl-shaped depressions, some inside others (depth 1-20 m, radius 2-30 cells)."""
    h, w = z.shape
    for _ in range(count):
        r = float(rng.uniform(2.0, 30.0))
        cy = int(rng.integers(2, h - 2))
        cx = int(rng.integers(2, w - 2))
        y0, y1 = max(1, int(cy - r)), min(h - 1, int(cy + r) + 1)
        x0, x1 = max(1, int(cx - r)), min(w - 1, int(cx + r) + 1)
        yy, xx = np.mgrid[y0:y1, x0:x1]
        d2 = ((yy - cy) ** 2 + (xx - cx) ** 2) / (r * r)
        bowl = np.clip(1.0 - d2, 0.0, None) * rng.uniform(1.0, 20.0)
        sub = z[y0:y1, x0:x1]
        sub -= (bowl * valid[y0:y1, x0:x1]).astype(np.float32)


@dataclasses.dataclass
class Scenario:
    dem: np.ndarray          # float64 (fp32-representable), nodata = -9999
    cellsize: float
    rain: np.ndarray         # per-step rainfall scalars (mm/yr)
    temp: np.ndarray         # per-step temperature scalars (C)
    init_rain: float
    init_temp: float
    recompute: bool          # True: SetClimateMatrices every step; False: run-in

    @property
    def shape(self):
        return self.dem.shape


def make_dem(n: int, hurst: float, relief: float, nodata_frac: float, pits: int, plateaus: int,
             seed: int, flats_frac: float = 0.0, depressions: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    z = spectral_dem(n, n, hurst, relief, rng)
    border = nodata_border(z.shape, nodata_frac, rng)
    valid = ~border
    if flats_frac > 0.0:
        # large flats: quantise elevations to 1 m in the lowest flats_frac of cells
        thr = np.quantile(z[valid], flats_frac)
        sel = valid & (z <= thr)
        z[sel] = np.floor(z[sel])
    if depressions:
        add_nested_depressions(z, valid, depressions, rng)
    add_pits(z, valid, pits, rng)
    add_plateaus(z, valid, plateaus, rng)
    z = z.astype(np.float64)
    z[border] = NODATA
    return z


def config_small(seed: int = 1) -> Scenario:
    """512x512, H=0.8, 0-400 m, 5% nodata border, 200 pits, 20 plateaus, 10 steps
    of constant 800 mm/yr and 10 C (the run-in climate of lem.cpp)."""
    dem = make_dem(512, 0.8, 400.0, 0.05, 200, 20, seed)
    steps = 10
    return Scenario(dem, 30.0, np.full(steps, 800.0), np.full(steps, 10.0), 800.0, 10.0, False)


def config_large(seed: int = 2, n: int = 4096, steps: int = 100) -> Scenario:
    """4096x4096, H=0.7, 0-1500 m, 2% nodata, 5000 pits, 300 plateaus; a per-step
    climate series: rain lognormal(mean 900, cv 0.3), temperature N(9, 2)."""
    scale = (n / 4096.0) ** 2
    dem = make_dem(n, 0.7, 1500.0, 0.02, max(1, int(5000 * scale)), max(1, int(300 * scale)), seed)
    rng = np.random.default_rng(seed + 1000)
    cv = 0.3
    sigma = np.sqrt(np.log(1.0 + cv * cv))
    mu = np.log(900.0) - 0.5 * sigma * sigma
    rain = rng.lognormal(mu, sigma, size=steps)
    temp = rng.normal(9.0, 2.0, size=steps)
    return Scenario(dem, 30.0, rain, temp, 900.0, 9.0, True)


def config_ensemble(seed: int = 4, count: int = 64, steps: int = 200, lo: int = 256, hi: int = 2048,
                    only=None) -> list:
    """The batched ensemble: `count` square DEMs with sides log-uniform in
    [lo, hi], Hurst U(0.6, 0.9), relief U(200, 2000) m, 1-5 % nodata border,
    pits and plateaus at the density of the 4096x4096 grid, each with its own
    climate series (rain lognormal mean 900 cv 0.3, temperature N(9, 2)).
    only: indices of the DEMs to build (the others are None); the random
    stream is the same, so a DEM is identical with or without it."""
    rng = np.random.default_rng(seed)
    out = []
    cv = 0.3
    sigma = np.sqrt(np.log(1.0 + cv * cv))
    mu = np.log(900.0) - 0.5 * sigma * sigma
    keep = None if only is None else set(only)
    for i in range(count):
        n = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        scale = (n / 4096.0) ** 2
        hurst, relief, nodata = float(rng.uniform(0.6, 0.9)), float(rng.uniform(200.0, 2000.0)), \
            float(rng.uniform(0.01, 0.05))
        dem = None
        if keep is None or i in keep:
            dem = make_dem(n, hurst, relief, nodata, max(1, int(5000 * scale)), max(1, int(300 * scale)),
                           seed * 1000 + i)
        rain = rng.lognormal(mu, sigma, size=steps)
        temp = rng.normal(9.0, 2.0, size=steps)
        out.append(Scenario(dem, 30.0, rain, temp, 900.0, 9.0, True) if dem is not None else None)
    return out


def ensemble_sides(seed: int = 4, count: int = 64, steps: int = 200, lo: int = 256, hi: int = 2048) -> list:
    """The side lengths config_ensemble draws for the same arguments, without
    building the DEMs."""
    rng = np.random.default_rng(seed)
    sides = []
    for _ in range(count):
        sides.append(int(round(np.exp(rng.uniform(np.log(lo), np.log(hi))))))
        rng.uniform(0.6, 0.9)
        rng.uniform(200.0, 2000.0)
        rng.uniform(0.01, 0.05)
        rng.lognormal(0.0, 1.0, size=steps)
        rng.normal(9.0, 2.0, size=steps)
    return sides


def config_routing(seed: int = 3, n: int = 8192) -> Scenario:
    """8192x8192 routing stress: 10% of cells in 1 m-quantised flats and 50k
    nested depressions; one step."""
    scale = (n / 8192.0) ** 2
    dem = make_dem(n, 0.7, 1500.0, 0.02, 0, 0, seed, flats_frac=0.10,
                   depressions=max(1, int(50000 * scale)))
    return Scenario(dem, 30.0, np.array([900.0]), np.array([9.0]), 900.0, 9.0, False)


def initial_state(dem: np.ndarray, cellsize: float, init_rain: float, init_temp: float,
                  soil: dict | None = None, soil_from_formula: bool = False) -> dict:
    """Initial fields of a run: createmask, init_setoutletcell, setProcessMatrices
    and the initial climate grids (MEM_kernels/memory.cu:217-242,
    MEM_kernels/Data.cpp:38-66,115-303).

    soilT: default.par line 18 gives the thickness used when no raster is read;
    soil_from_formula=True applies createSoilTfromformula instead
    ((z-400)/1400*5), which is negative below 400 m.
    """
    soil = dict(DEFAULT_SOIL, **(soil or {}))
    h, w = dem.shape
    mask = (dem != NODATA).astype(np.int32)
    flat = dem.ravel()
    m = mask.ravel() == 1
    cand = np.where(m & (flat < 1000.0))[0]
    outlet = int(cand[np.argmin(flat[cand])]) if cand.size else 0
    rescale = 10000.0 / (cellsize * cellsize)
    inc = (init_rain * 2 - init_rain) / h
    rainmat = (init_rain + np.arange(h, dtype=np.float64)[:, None] * inc) * np.ones((1, w))
    tempmat = init_temp - ((dem - 467.228) * 0.0065)
    tempeffect = 100 + (100 / (tempmat + 15))
    st = {}
    st["mask"] = mask
    st["outlet"] = outlet
    mk = mask == 1
    st["stone"] = np.where(mk, soil["stone"], 0.0)
    st["fines"] = np.where(mk, soil["fines"], 0.0)
    st["soilM"] = np.where(mk, soil["soilM"], 0.0)
    st["nut"] = np.where(mk, soil["nut"], 0.0)
    st["soilB"] = np.where(mk, soil["soilB"], 0.0)
    st["totB"] = np.where(mk, (3000.0 + (5.0 * (rainmat - tempeffect))) / rescale, 0.0)
    if soil_from_formula:
        st["soilT"] = np.where(dem > 0, ((dem - 400) / 1400) * 5, 0.0)
        st["soilT"] = np.where(mk, st["soilT"], 0.0)
    else:
        st["soilT"] = np.where(mk, soil["soilT"], 0.0)
    return st
