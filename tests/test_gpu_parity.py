"""Parity of the CUDA path (through the C ABI) with the FP64 oracle.

Every comparison starts both sides from the same state and runs one stage or
one step.  Tolerances (stated per check):
* direction codes, sink counts, contributing-cell counts: bit-exact;
* slopes: 2e-6 relative + 1e-12 absolute (fp32 storage of the reference's
  fp64 quotient);
* accumulation: 1e-5 relative (the required bound); elevation: 1e-9
  relative + 1e-6 m (fp64 state, fp32 increments);
* process grids: |gpu - oracle| <= 1e-5 |oracle| + 1e-6 max|oracle| (fp32
  arithmetic; differences such as geli = soilT - ero and dz cancel);
* budget totals: 1e-5 relative.
At sizes the oracle cannot finish quickly the checks are size-independent
invariants of the outputs (local accumulation balance, donor deposition,
totals equal to the sums of the grids).
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
    gv, ov = np.asarray(gv)[mask], np.asarray(ov)[mask]
    both_nan = np.isnan(gv) & np.isnan(ov)
    scale = np.nanmax(np.abs(ov)) if ov.size else 0.0
    err = np.where(both_nan, 0.0, np.abs(gv - ov))
    bad = ~(err <= rtol * np.abs(ov) + afrac * scale + atol) & ~both_nan
    assert not bad.any(), (f"{name}: {int(bad.sum())} of {bad.size} outside tolerance, max err "
                           f"{np.nanmax(err):.3e} (scale {scale:.3e})")


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
    ws_g, ws_o = g.get("watershed"), o["watershed"]
    if o.s.sinkcount:
        pairs = set(zip(ws_g[mask].tolist(), ws_o[mask].tolist()))
        assert len(pairs) == len(set(ws_o[mask].tolist())) == len(set(ws_g[mask].tolist()))


def check_fa(o, g, mask, contrib=False):
    close("runoff", g.get("runoff"), o["runoff"], mask, rtol=1e-6)
    close("soilM", g.get("soilM"), o["soilM"], mask, rtol=1e-6)
    close("fa", g.get("fa"), o["fa"], mask, rtol=1e-5, afrac=0.0)
    t = g.totals()
    assert t["fa_uncomputed"] == o.s.fa_uncomputed
    if contrib:
        np.testing.assert_array_equal(g.get("contrib"), o["contrib"])


def check_mod(o, g, mask, diag=False):
    # fp32 process arithmetic: 1e-5 of the value plus 1e-6 of the field's largest
    # magnitude (differences such as geli = soilT - ero or dz cancel)
    for f in MOD_FIELDS:
        close(f, g.get(f), o[f], mask, afrac=1e-6)
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


def test_routing_stress_8192_tiled_and_walk_agree(libs):
    """The routing stress configuration (8192x8192, 10 % of cells in 1 m flats,
    50k nested depressions): the tiled accumulation and the global wave give
    the same accumulation from the same directions (1e-5), and the
    contributing-cell counts balance exactly."""
    oracle, lem = libs
    sc = S.config_routing(3, n=8192)
    st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    g = lem.Model(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    g.set_state(st)
    g.flow_direction()
    g.flow_accumulation(0)  # tiled
    fa_tiled = g.get("fa")
    t = g.totals()
    assert t["plateau_sweeps"] > 0 and t["flood_edges"] > 0
    g.set_state({f: st[f] for f in ("soilM",)})  # runoff changes soil moisture; start both from the same state
    g.flow_accumulation(lem.STEP_CONTRIB)  # global wave
    fa_walk, cnt = g.get("fa"), g.get("contrib")
    mask = st["mask"] == 1
    both_nan = np.isnan(fa_tiled) & np.isnan(fa_walk)
    err = np.where(both_nan, 0.0, np.abs(fa_tiled - fa_walk))
    assert (err[mask] <= 1e-5 * np.abs(fa_walk[mask])).all()
    fd = g.get("fd")
    fd_m = np.where(mask, fd, fd & 0xFF)
    done = mask & (cnt > 0)
    cbal = 1 + _donor_sum(fd_m, np.where(mask, cnt, 0).astype(np.float64), True)
    assert np.array_equal(cnt[done], cbal[done].astype(np.int64))
    g.close()
