"""Multi-step drift: the GPU path and the FP64 oracle step the same scenario
side by side, each from its own previous state (no resynchronisation), over the
10 timesteps of the small plain-method configuration (512 x 512, constant
climate).  Per step the test reports how far the two runs have drifted apart:
the share of cells whose direction code differs, the largest and mean
elevation difference, the largest relative difference of the accumulation and
of the soil fields (against each field's largest magnitude).  Elevations are
fp64 in both, updated by fp32 increments on the GPU, so they drift by about
the fp32 rounding of the increments per step; the bounds below are a few
orders of magnitude above what is measured and catch a real divergence.
Set LEM_DRIFT_OUT to a file name to keep the statistics as JSON.
"""
import json
import os

import numpy as np
import pytest

from parallem_gb300 import scenario as S

pytestmark = pytest.mark.gpu

SOIL = ("stone", "fines", "soilT", "soilM", "soilB", "nut", "totB")


def test_ten_step_drift_against_the_oracle():
    from oracle import oracle
    from parallem_gb300 import build, lem
    oracle.build()
    build.build()
    sc = S.config_small(1)
    st = S.initial_state(sc.dem, 30.0, float(sc.rain[0]), float(sc.temp[0]))
    o = oracle.OracleModel(sc.dem, 30.0, st, float(sc.rain[0]), float(sc.temp[0]))
    g = lem.Model(sc.dem, 30.0, float(sc.rain[0]), float(sc.temp[0]))
    g.set_state(st)
    mask = st["mask"] == 1
    stats = []
    for i in range(len(sc.rain)):
        r, t = float(sc.rain[i]), float(sc.temp[i])
        flags = lem.STEP_SET_OUTLET_FROM_FA if i == 0 else 0
        g.step(r, t, bool(sc.recompute), flags)
        o.step(r, t, bool(sc.recompute), flags)
        g.synchronize()
        dz = np.abs(g.get("dem") - o["dem"])[mask]
        fa_g, fa_o = g.get("fa")[mask], o["fa"][mask]
        row = {
            "step": i + 1,
            "fd_differ": float(np.mean(g.get("fd")[mask] != o["fd"][mask])),
            "dem_max_abs_m": float(np.nanmax(dz)),
            "dem_mean_abs_m": float(np.nanmean(dz)),
            "fa_max_rel": float(np.nanmax(np.abs(fa_g - fa_o) / np.maximum(np.abs(fa_o), 1e-30))),
        }
        for f in SOIL:
            gv, ov = g.get(f)[mask], o[f][mask]
            scale = max(float(np.nanmax(np.abs(ov))), 1e-30)
            row[f + "_max_rel_scale"] = float(np.nanmax(np.abs(gv - ov)) / scale)
        stats.append(row)
    g.close()
    out = os.environ.get("LEM_DRIFT_OUT")
    if out:
        with open(out, "w") as fh:
            json.dump(stats, fh, indent=1)
    print(json.dumps(stats[-1]))
    last = stats[-1]
    assert last["fd_differ"] < 0.01
    assert last["dem_max_abs_m"] < 1e-2
    assert all(last[f + "_max_rel_scale"] < 1e-2 for f in SOIL)
