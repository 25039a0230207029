"""Writes the golden vectors of tests/golden/*.npz from the reference's own kernels.

The kernels are the reference's CUDA kernel bodies compiled for the CPU by
oracle/ref_build.py (a sequential schedule of the reference's grids of
threads, with the host loops of cuFlowDirection, correctmfdflow and erosionGPU
restated in oracle/ref_harness.cpp).  This needs the reference sources, so it
runs only where they are present:

    python tests/golden/make_golden.py

Each case is one timestep on a small seeded grid.  The file holds the inputs
(DEM, mask, outlet, soil fields, parameters, climate) and, stage by stage, what
the reference computes: direction codes, plateau distances, basin labels,
the raised DEM and the DEM after testoutletislowest; runoff, accumulation and
proportions; every process grid, the new DEM and the budget totals.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from parallem_gb300 import scenario as S  # noqa: E402

# name: (dem builder, flow_direction_type, mfd_proportions, climate of the step or None for the run-in)
CASES = {
    "sfd_noflat48": (lambda: S.make_dem(48, 0.8, 400.0, 0.06, 8, 0, 21), 0, 0, None),
    "sfd_plateaus48": (lambda: S.make_dem(48, 0.8, 400.0, 0.06, 8, 2, 22), 0, 0, None),
    "sfd_climate48": (lambda: S.make_dem(48, 0.7, 1500.0, 0.06, 6, 0, 23), 0, 0, (1100.0, 7.0)),
    "mfd_props48": (lambda: S.make_dem(48, 0.8, 400.0, 0.06, 8, 0, 24), 1, 1, None),
}
INIT_RAIN, INIT_TEMP = 900.0, 9.0
SCALARS = ("outlet", "sinkcount", "init_sinks", "init_flats", "FA_max", "fa_uncomputed", "sed_uncomputed",
           "totE", "totI", "totG", "totD", "totWC", "totWP", "totbio")


def run_case(name):
    from oracle import oracle
    make, flow, props, clim = CASES[name]
    dem = make()
    st = S.initial_state(dem, 30.0, INIT_RAIN, INIT_TEMP)
    params = oracle.make_params(flow_direction_type=flow, mfd_proportions=props)
    r = oracle.RefModel(dem, 30.0, st, INIT_RAIN, INIT_TEMP, params=params)
    out = {"in_dem": dem.astype(np.float64), "in_mask": st["mask"].astype(np.int32),
           "in_outlet": np.int64(st["outlet"]), "flow_direction_type": np.int64(flow),
           "mfd_proportions": np.int64(props), "init_rain": np.float64(INIT_RAIN),
           "init_temp": np.float64(INIT_TEMP)}
    for f in ("stone", "fines", "soilT", "soilM", "soilB", "nut", "totB"):
        out["in_" + f] = np.asarray(st[f], np.float64)
    if clim is not None:
        out["rain"], out["temp"] = np.float64(clim[0]), np.float64(clim[1])
        r.s.last_rain, r.s.last_temp = r.s.rain, r.s.temp
        r.s.rain, r.s.temp = clim
        oracle.lib().oracle_set_climate(oracle.C.byref(r.s), 0)
    r.flow_direction()
    for f in ("fd", "sfd", "slopes", "shortest_paths", "watershed", "dem_routed", "dem"):
        out["fd_" + f] = np.array(r[f])
    for k in ("outlet", "sinkcount", "init_sinks", "init_flats"):
        out["fd_" + k] = np.array(getattr(r.s, k))
    r.flow_accumulation()
    for f in ("runoff", "soilM", "fa", "prop"):
        out["fa_" + f] = np.array(r[f])
    for k in ("outlet", "FA_max", "fa_uncomputed"):
        out["fa_" + k] = np.array(getattr(r.s, k))
    r.erosion()
    for f in ("slopeptr", "ero", "inci", "geli", "depo", "dz", "wC", "wP", "stone", "fines", "soilT", "soilM",
              "soilB", "nut", "totB", "dem"):
        out["mod_" + f] = np.array(r[f])
    for k in SCALARS:
        out["mod_" + k] = np.array(getattr(r.s, k))
    return out


def main():
    from oracle import oracle
    oracle.build()
    if oracle.ref_lib() is None:
        raise SystemExit("the reference sources are needed to write the golden vectors")
    for name in sorted(CASES):
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **run_case(name))
        print("wrote", name)


if __name__ == "__main__":
    main()
