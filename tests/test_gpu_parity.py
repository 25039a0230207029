"""Parity of the CUDA path (through the C ABI) with the FP64 oracle.

Every comparison starts both sides from the same state and runs one stage or
one step.  Tolerances (stated per check):
* direction codes, sink counts, contributing-cell counts: bit-exact;
* slopes: 2e-6 relative + 1e-12 absolute (fp32 storage of the reference's
  fp64 quotient);
* accumulation: 1e-5 relative (the required bound); elevation: 1e-9
  relative + 1e-6 m (fp64 state, fp32 increments);
* process grids: 1e-5 relative; gelifluction and incision, whose formulas
  cancel (geli = soilT - ero, fa*cs^2/1e4 - Qthreshold), and the diagnostics
  dz, weatherC, weatherP add 1e-6 of the field's largest magnitude;
* budget totals: 1e-5 relative.
The headline configurations are compared with the oracle at full size: one
step of the 4096x4096 grid, the 8192x8192 routing stress grid (directions,
basins, accumulation and contributing counts) and the largest DEMs of the
batched ensemble stepped inside the batch.  Those tests print, per field, the
distribution of the cell-wise relative error (lines starting ERRDIST), so the
share of cells that rely on the additive term of the process-grid tolerance
is visible.  Size-independent invariants (local accumulation balance, donor
deposition, totals equal to the sums of the grids) are checked beside them.
"""
import numpy as np
import pytest

from parallem_gb300 import scenario as S
from tests.helpers import NODATA, ringed

pytestmark = pytest.mark.gpu

MOD_FIELDS = ("slopeptr", "ero", "inci", "geli", "depo", "stone", "fines", "soilT", "soilM", "soilB", "nut", "totB")
STATE_FIELDS = ("stone", "fines", "soilT", "soilM", "soilB", "nut", "totB")


@pytest.fixture(scope="module")
def libs():
    from oracle import oracle
    from parallem_gb300 import build, lem
    oracle.build()
    build.build()
    lem.load()
    return oracle, lem


def pair(libs, dem, rain=800.0, temp=10.0, params=None, soil=None):
    oracle, lem = libs
    st = S.initial_state(dem, 30.0, rain, temp, soil=soil)
    kw = {} if params is None else params
    o = oracle.OracleModel(dem, 30.0, st, rain, temp, params=oracle.make_params(**kw))
    g = lem.Model(dem, 30.0, rain, temp, params=lem.make_params(**kw))
    g.set_state(st)
    return o, g, st["mask"] == 1


def resync(o, g):
    """GPU state := oracle state (identical inputs for the next comparison)."""
    g.set("dem", o["dem"])
    g.set_state({f: o[f] for f in STATE_FIELDS} | {"slopes": o["slopes"], "outlet": o.outlet})


def close(name, gv, ov, mask, rtol=1e-5, afrac=1e-8, atol=0.0):
    cells = np.flatnonzero(np.broadcast_to(mask, np.shape(gv)))
    gv, ov = np.asarray(gv)[mask], np.asarray(ov)[mask]
    both_nan = np.isnan(gv) & np.isnan(ov)
    scale = np.nanmax(np.abs(ov)) if ov.size else 0.0
    err = np.where(both_nan, 0.0, np.abs(gv - ov))
    bad = ~(err <= rtol * np.abs(ov) + afrac * scale + atol) & ~both_nan
    if bad.any():
        w = int(np.nanargmax(np.where(bad, err, -1.0)))
        raise AssertionError(f"{name}: {int(bad.sum())} of {bad.size} outside tolerance, max err "
                             f"{np.nanmax(err):.3e} (scale {scale:.3e}); worst at flat index {int(cells[w])}: "
                             f"gpu {gv[w]!r}, oracle {ov[w]!r}")


def check_fd(o, g, mask):
    np.testing.assert_array_equal(g.get("sfd"), o["sfd"])
    np.testing.assert_array_equal(g.get("fd"), o["fd"])
    t = g.totals()
    assert t["sinkcount"] == o.s.sinkcount
    assert t["initial_sinks"] == o.s.init_sinks and t["initial_flats"] == o.s.init_flats
    gs, os_ = g.get("slopes"), o["slopes"]
    np.testing.assert_array_equal(gs != 0, os_ != 0)
    # fp32 slopes: 2e-6 relative, plus 1e-12 absolute for near-flat drops whose
    # fp32 estimate carries the 2^-44 |z| split error
    close("slopes", gs, os_, np.broadcast_to(mask[..., None], gs.shape), rtol=2e-6, afrac=0.0, atol=1e-12)
    check_partition(g.get("watershed"), o["watershed"], mask, o.s.sinkcount)


def check_partition(ws_g, ws_o, mask, sinkcount):
    """The basin partitions are the same up to label numbering: the pairs
    (GPU label, oracle label) are as many as the labels on either side."""
    if not sinkcount:
        return
    a, b = ws_g[mask].astype(np.int64), ws_o[mask].astype(np.int64)
    pairs = np.unique((a << 32) | (b & 0xFFFFFFFF))
    assert pairs.size == np.unique(a).size == np.unique(b).size


def check_fa(o, g, mask, contrib=False):
    close("runoff", g.get("runoff"), o["runoff"], mask, rtol=1e-6)
    close("soilM", g.get("soilM"), o["soilM"], mask, rtol=1e-6)
    close("fa", g.get("fa"), o["fa"], mask, rtol=1e-5, afrac=0.0)
    t = g.totals()
    assert t["fa_uncomputed"] == o.s.fa_uncomputed
    if contrib:
        np.testing.assert_array_equal(g.get("contrib"), o["contrib"])


def error_stats(fields, g_get, o_get, mask, rtol=1e-5):
    """Per field: cells compared, largest and 99.9th-percentile relative error,
    and the share of cells whose error exceeds rtol * |oracle| (the cells that
    rely on the additive term of the process-grid tolerance)."""
    out = {}
    for f in fields:
        gv, ov = np.asarray(g_get(f))[mask], np.asarray(o_get(f))[mask]
        ok = ~(np.isnan(gv) & np.isnan(ov))
        gv, ov = gv[ok], ov[ok]
        err = np.abs(gv - ov)
        rel = err / np.maximum(np.abs(ov), 1e-300)
        out[f] = {"cells": int(ov.size), "max_rel": float(rel.max()) if rel.size else 0.0,
                  "p999_rel": float(np.quantile(rel, 0.999)) if rel.size else 0.0,
                  "share_above_rtol": float((err > rtol * np.abs(ov)).mean()) if rel.size else 0.0}
    return out


def report(name, stats):
    import json
    print(f"ERRDIST {name} {json.dumps(stats, sort_keys=True)}")


# Process grids whose formulas cancel: gelifluction is capped at soilT - ero and
# incision starts at fa*cs^2/1e4 - Qthreshold, so near those points a 1e-7
# relative input difference is a much larger relative output difference.  They
# keep an additive term of 1e-6 of the field's largest magnitude; every other
# process grid is held to 1e-5 relative alone.  (Measured at the headline sizes:
# 0.004-0.04 % of cells of these two need the additive term, none of the rest.)
CANCELLING = ("geli", "inci")


def check_mod(o, g, mask, diag=False):
    for f in MOD_FIELDS:
        close(f, g.get(f), o[f], mask, afrac=1e-6 if f in CANCELLING else 0.0)
    if diag:
        for f in ("dz", "wC", "wP"):
            close(f, g.get(f), o[f], mask, afrac=1e-6)
    # elevation: fp64 state updated by fp32 increments; 1e-9 relative plus 1e-6 m
    close("dem", g.get("dem"), o["dem"], mask, rtol=1e-9, afrac=0.0, atol=1e-6)
    t = g.totals()
    for k_g, k_o in (("tot_e", "totE"), ("tot_i", "totI"), ("tot_g", "totG"), ("tot_d", "totD"),
                     ("tot_weather_c", "totWC"), ("tot_weather_p", "totWP"), ("tot_bio", "totbio"),
                     ("fa_max", "FA_max")):
        a, b = t[k_g], getattr(o.s, k_o)
        assert abs(a - b) <= 1e-5 * abs(b) + 1e-12 or (np.isnan(a) and np.isnan(b)), (k_g, a, b)
    assert t["sed_uncomputed"] == o.s.sed_uncomputed
    assert t["outlet"] == o.outlet


def run_steps(libs, dem, steps, rain, temp, recompute, params=None, flags=0, soil=None):
    o, g, mask = pair(libs, dem, rain[0], temp[0], params, soil)
    from parallem_gb300 import lem
    for i in range(steps):
        if recompute:
            g.set_climate(rain[i], temp[i], True)
            o.s.last_rain, o.s.last_temp = o.s.rain, o.s.temp
            o.s.rain, o.s.temp = float(rain[i]), float(temp[i])
            from oracle.oracle import lib, C
            lib().oracle_set_climate(C.byref(o.s), 0)
        g.flow_direction()
        o.flow_direction()
        check_fd(o, g, mask)
        g.flow_accumulation(flags)
        o.flow_accumulation(flags)
        check_fa(o, g, mask, contrib=bool(flags & lem.STEP_CONTRIB))
        g.erosion(flags)
        o.erosion()
        check_mod(o, g, mask, diag=bool(flags & lem.STEP_KEEP_DIAGNOSTICS))
        g.synchronize()
        resync(o, g)
    return o, g


def test_small_config_three_steps(libs):
    from parallem_gb300 import lem
    sc = S.config_small(1)
    run_steps(libs, sc.dem, 3, sc.rain, sc.temp, sc.recompute,
              flags=lem.STEP_CONTRIB | lem.STEP_KEEP_DIAGNOSTICS)


def test_climate_series_recomputed_each_step(libs):
    sc = S.config_large(2, n=256, steps=3)
    run_steps(libs, sc.dem, 3, sc.rain, sc.temp, True)


def test_quantised_flats_and_nested_depressions(libs):
    dem = S.make_dem(192, 0.7, 800.0, 0.03, 10, 4, 13, flats_frac=0.15, depressions=40)
    run_steps(libs, dem, 2, np.full(2, 900.0), np.full(2, 9.0), False)


@pytest.mark.parametrize("props", [0, 1])
def test_mfd_modes(libs, props):
    dem = S.make_dem(128, 0.8, 600.0, 0.05, 10, 2, 17)
    run_steps(libs, dem, 2, np.full(2, 800.0), np.full(2, 10.0), False,
              params=dict(flow_direction_type=1, mfd_proportions=props))


def test_grid_without_nodata_ring(libs):
    rng = np.random.default_rng(5)
    dem = S.spectral_dem(48, 64, 0.8, 300.0, rng).astype(np.float64)
    run_steps(libs, dem, 2, np.full(2, 800.0), np.full(2, 10.0), False)


def test_outlet_relocation_flag(libs):
    from parallem_gb300 import lem
    dem = S.make_dem(96, 0.8, 400.0, 0.05, 10, 2, 23)
    run_steps(libs, dem, 2, np.full(2, 800.0), np.full(2, 10.0), False, flags=lem.STEP_SET_OUTLET_FROM_FA)


@pytest.mark.parametrize("shape", [(1, 1), (1, 16), (3, 3), (2, 40), (16, 16)])
def test_tiny_and_degenerate_grids(libs, shape):
    rng = np.random.default_rng(shape[0] * 100 + shape[1])
    dem = rng.uniform(100.0, 120.0, size=shape)
    run_steps(libs, dem, 2, np.full(2, 800.0), np.full(2, 10.0), False)


def test_all_flat_grid_and_single_pit(libs):
    flat = ringed(np.full((12, 12), 250.0), 2)
    run_steps(libs, flat, 2, np.full(2, 800.0), np.full(2, 10.0), False)
    pit = ringed(np.array([[9, 5, 9], [9, 1, 9], [9, 9, 9.0]]) + 300.0, 2)
    run_steps(libs, pit, 2, np.full(2, 800.0), np.full(2, 10.0), False)


def test_negative_soil_thickness_propagates_nan_like_the_reference(libs):
    # createSoilTfromformula gives negative thickness below 400 m; conc_erosion
    # then divides by a zero incision (eroincidep.cu:333-336)
    dem = S.make_dem(64, 0.8, 600.0, 0.05, 5, 1, 29)
    o, g, mask = pair(libs, dem, 800.0, 10.0)
    st = S.initial_state(dem, 30.0, 800.0, 10.0, soil_from_formula=True)
    o.a["soilT"][...] = st["soilT"]
    g.set("soilT", st["soilT"])
    for m in (o, g):
        m.flow_direction()
        m.flow_accumulation()
    g.erosion()
    o.erosion()
    np.testing.assert_array_equal(np.isnan(g.get("inci"))[mask], np.isnan(o["inci"])[mask])


def test_deterministic_repeat(libs):
    oracle, lem = libs
    sc = S.config_large(4, n=1024, steps=1)
    st = S.initial_state(sc.dem, 30.0, 900.0, 9.0)
    outs = []
    for _ in range(2):
        g = lem.Model(sc.dem, 30.0, 900.0, 9.0)
        g.set_state(st)
        g.step(sc.rain[0], sc.temp[0], True)
        outs.append({f: g.get(f) for f in ("fd", "fa", "depo", "stone", "dem")})
        g.close()
    for f in outs[0]:
        np.testing.assert_array_equal(outs[0][f], outs[1][f], err_msg=f)


def _donor_sum(fd, val, masked_ok):
    """sum over donors in the reference's order E,SE,S,SW,W,NW,N,NE (float64)."""
    H, W = fd.shape
    acc = np.zeros((H, W))
    pad = np.pad(val, 1)
    code = np.pad(fd, 1, constant_values=0)
    for dy, dx, bit in ((0, 1, 16), (1, 1, 32), (1, 0, 64), (1, -1, 128), (0, -1, 1), (-1, -1, 2), (-1, 0, 4),
                        (-1, 1, 8)):
        n_code = code[1 + dy:1 + dy + H, 1 + dx:1 + dx + W]
        n_val = pad[1 + dy:1 + dy + H, 1 + dx:1 + dx + W]
        acc += np.where((n_code & bit) != 0, n_val, 0.0)
    return acc


def test_full_size_invariants_4096(libs):
    """One C2 step at 4096x4096: accumulation balances cell by cell, counts are
    exact, deposition follows from the donors, totals equal the grid sums."""
    oracle, lem = libs
    sc = S.config_large(2, n=4096, steps=1)
    st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    g = lem.Model(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    g.set_state(st)
    g.set_climate(sc.rain[0], sc.temp[0], True)
    g.flow_direction()
    g.flow_accumulation(lem.STEP_CONTRIB)
    g.synchronize()
    mask = st["mask"] == 1
    fd = g.get("fd")
    fa, w, cnt = g.get("fa"), g.get("runoff"), g.get("contrib")
    t = g.totals()
    assert t["fa_uncomputed"] >= 0
    done = mask.copy()
    if t["fa_uncomputed"]:
        done &= ~np.isclose(fa, w, rtol=0, atol=0)  # cells left at fa = w (cycles) are excluded
    fd_m = np.where(mask, fd, fd & 0xFF)
    balance = w + _donor_sum(fd_m, np.where(mask, fa, 0.0), True)
    rel = np.abs(fa - balance) / np.maximum(np.abs(fa), 1e-30)
    assert rel[done].max() < 1e-5
    cbal = 1 + _donor_sum(fd_m, np.where(mask, cnt, 0).astype(np.float64), True)
    assert np.array_equal(cnt[done], cbal[done].astype(np.int64))
    g.erosion()
    g.synchronize()
    t = g.totals()
    ero = g.get("ero")
    assert abs(t["tot_e"] - ero.sum()) <= 1e-5 * abs(ero.sum())
    assert np.isfinite(g.get("dem")[mask]).all()


def test_full_size_tiled_waves_4096(libs):
    """One C2 step at 4096x4096 on the tiled waves (no contributing counts): the
    accumulation balances cell by cell (1e-5), and every routed cell's
    deposition is its donors' formula (mfd_accum.cu:222, fp32: 1e-5)."""
    oracle, lem = libs
    sc = S.config_large(2, n=4096, steps=1)
    st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    g = lem.Model(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    g.set_state(st)
    g.step(sc.rain[0], sc.temp[0], True)
    g.synchronize()
    mask = st["mask"] == 1
    fd = g.get("fd")
    fa, w = g.get("fa"), g.get("runoff")
    t = g.totals()
    done = mask.copy()
    if t["fa_uncomputed"]:
        done &= ~np.isclose(fa, w, rtol=0, atol=0)
    fd_m = np.where(mask, fd, fd & 0xFF)
    balance = w + _donor_sum(fd_m, np.where(mask, fa, 0.0), True)
    rel = np.abs(fa - balance) / np.maximum(np.abs(fa), 1e-30)
    assert rel[done].max() < 1e-5
    ero, inci, geli, depo = (g.get(f) for f in ("ero", "inci", "geli", "depo"))
    p = S.DEFAULT_PAR
    ddk, dck, dgk = min(p["ddk"], 0.95), min(p["dck"], 0.9), p["dgk"]
    sed_mask = mask.copy()
    sed_mask[0, :] = sed_mask[:, 0] = False
    src = np.where(sed_mask, 1.0, 0.0)
    ad = _donor_sum(fd_m, np.where(mask, ero, 0.0) * (1 - ddk), True)
    ac = _donor_sum(fd_m, np.where(mask, inci, 0.0) * (1 - dck), True)
    ag = _donor_sum(fd_m, np.where(mask, geli, 0.0) * (1 - dgk), True)
    want = (ad + ero) * ddk + (ac + inci) * dck + (ag + geli) * dgk
    routed = sed_mask & (depo != np.float32(1e-5)) & (src > 0)
    err = np.abs(depo - want)[routed]
    assert (err <= 1e-5 * np.abs(want[routed]) + 1e-9).all()
    assert routed.sum() > 0.9 * mask.sum()
    g.close()


def check_step(o, g, mask, name):
    """After one whole step from the same state: codes and counts bit-exact,
    accumulation 1e-5, process grids and totals as check_mod."""
    np.testing.assert_array_equal(g.get("sfd"), o["sfd"])
    np.testing.assert_array_equal(g.get("fd"), o["fd"])
    t = g.totals()
    assert t["sinkcount"] == o.s.sinkcount
    assert t["initial_sinks"] == o.s.init_sinks and t["initial_flats"] == o.s.init_flats
    assert t["fa_uncomputed"] == o.s.fa_uncomputed
    close("fa", g.get("fa"), o["fa"], mask, rtol=1e-5, afrac=0.0)
    close("runoff", g.get("runoff"), o["runoff"], mask, rtol=1e-6)
    check_mod(o, g, mask)
    report(name, error_stats(("fa",) + MOD_FIELDS + ("dem",), g.get, o.__getitem__, mask))


def test_c2_full_step_4096_matches_the_oracle(libs):
    """One step of the single large grid (4096x4096, Hurst 0.7, 0-1500 m, 2 %
    nodata, 5000 pits, 300 plateaus, per-step climate) from the same state on
    both sides: direction codes, slopes, sink counts and the basin partition
    bit-exact or as check_fd; the tiled accumulation at 1e-5, then the global
    walk with contributing-cell counts bit-exact; every process grid, the DEM
    and the totals as check_mod."""
    oracle, lem = libs
    sc = S.config_large(2, n=4096, steps=1)
    o, g, mask = pair(libs, sc.dem, sc.init_rain, sc.init_temp)
    soil_m = g.get("soilM")
    g.set_climate(sc.rain[0], sc.temp[0], True)
    o.s.last_rain, o.s.last_temp = o.s.rain, o.s.temp
    o.s.rain, o.s.temp = float(sc.rain[0]), float(sc.temp[0])
    from oracle.oracle import C, lib
    lib().oracle_set_climate(C.byref(o.s), 0)
    g.flow_direction()
    o.flow_direction()
    check_fd(o, g, mask)
    g.flow_accumulation(0)  # the tiled path of the bench step
    o.flow_accumulation(lem.STEP_CONTRIB)
    check_fa(o, g, mask)
    g.set("soilM", soil_m)  # runoff updates soil moisture: run the walk from the same state
    g.flow_accumulation(lem.STEP_CONTRIB)
    check_fa(o, g, mask, contrib=True)
    g.erosion()
    o.erosion()
    check_mod(o, g, mask)
    report("c2_4096_one_step", error_stats(("fa",) + MOD_FIELDS + ("dem",), g.get, o.__getitem__, mask))
    g.close()


def test_c3_routing_stress_8192_matches_the_oracle(libs):
    """The routing stress configuration (8192x8192, 10 % of cells in 1 m flats,
    50k nested depressions): direction codes, sink count and basin partition
    bit-exact with the oracle; the tiled accumulation at 1e-5; the global walk's
    int32 contributing-cell counts bit-exact."""
    oracle, lem = libs
    sc = S.config_routing(3, n=8192)
    st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    mask = st["mask"] == 1
    o = oracle.OracleModel(sc.dem, 30.0, st, sc.init_rain, sc.init_temp)
    g = lem.Model(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    g.set_state(st)
    g.flow_direction()
    o.flow_direction()
    np.testing.assert_array_equal(g.get("sfd"), o["sfd"])
    np.testing.assert_array_equal(g.get("fd"), o["fd"])
    t = g.totals()
    assert t["sinkcount"] == o.s.sinkcount
    assert t["initial_sinks"] == o.s.init_sinks and t["initial_flats"] == o.s.init_flats
    assert t["plateau_sweeps"] > 0 and t["flood_edges"] > 0
    check_partition(g.get("watershed"), o["watershed"], mask, o.s.sinkcount)
    g.flow_accumulation(0)  # tiled
    o.flow_accumulation(lem.STEP_CONTRIB)
    close("fa", g.get("fa"), o["fa"], mask, rtol=1e-5, afrac=0.0)
    assert g.totals()["fa_uncomputed"] == o.s.fa_uncomputed
    g.set("soilM", st["soilM"])  # runoff changes soil moisture; the walk starts from the same state
    g.flow_accumulation(lem.STEP_CONTRIB)  # global walk
    np.testing.assert_array_equal(g.get("contrib"), o["contrib"])
    close("fa", g.get("fa"), o["fa"], mask, rtol=1e-5, afrac=0.0)
    report("c3_8192_routing", error_stats(("fa",), g.get, o.__getitem__, mask))
    g.close()


class _InBatch:
    """One DEM of a batch with the Model interface the checks use."""

    def __init__(self, b, i):
        self.b, self.i = b, i

    def get(self, f):
        return self.b.get(self.i, f)

    def totals(self):
        return self.b.totals(self.i)


def test_c4_largest_ensemble_dems_stepped_in_the_batch_match_the_oracle(libs):
    """The three largest DEMs of the batched ensemble (64 DEMs, sides
    log-uniform in [256, 2048]) packed into one canvas with two small ones and
    stepped by lem_step_batch; each DEM's step equals the oracle's step of that
    DEM alone (codes bit-exact, accumulation 1e-5, process grids as check_mod)."""
    oracle, lem = libs
    sizes = S.ensemble_sides(4, 64, steps=200)
    order = sorted(range(64), key=lambda i: -sizes[i])
    pick = order[:3] + order[-2:]
    ens = S.config_ensemble(4, count=64, steps=200, only=pick)  # the DEMs of the bench's ensemble
    from parallem_gb300.packing import TilePacker
    W = 4096
    Hc = 1024
    while True:
        p = TilePacker(W, Hc)
        if all(p.alloc(ens[i].dem.shape[1], ens[i].dem.shape[0]) is not None for i in pick):
            break
        Hc += 512
    b = lem.Batch(W, Hc, 30.0, max_dems=8)
    members = []
    for i in pick:
        sc = ens[i]
        st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
        k = b.add(sc.dem, sc.init_rain, sc.init_temp)
        b.set_state(k, st)
        b.set_climate(k, float(sc.rain[0]), float(sc.temp[0]), True)
        o = oracle.OracleModel(sc.dem, 30.0, st, sc.init_rain, sc.init_temp)
        members.append((i, k, o, st["mask"] == 1))
    b.step()
    b.synchronize()
    for i, k, o, mask in members[:3]:
        sc = ens[i]
        o.step(float(sc.rain[0]), float(sc.temp[0]), True)
        check_step(o, _InBatch(b, k), mask, f"c4_dem{i}_{sc.dem.shape[0]}")
    b.close()
