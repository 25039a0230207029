"""Pins the FP64 oracle to the reference's own kernels (CPU, no GPU).

oracle/_ref/libref.so is built by oracle/ref_build.py from the kernel bodies in
the reference sources and runs them as one sequential schedule.  From identical
inputs, each stage of the oracle must agree with it:

* flow direction: identical plateau distances, sink counts and basin
  partitions; direction codes identical except at plateau ties, where the
  reference's choice depends on the thread schedule (newflow.cu:328-347) and
  both answers must point at a neighbour that attains the cell's distance;
* flow accumulation and the process stage: bit-identical fp64 grids and totals.

The tests skip where the reference sources are absent (e.g. on the GPU host).
"""
import numpy as np
import pytest

from parallem_gb300 import scenario as S

DX = [0, 1, 1, 1, 0, -1, -1, -1]
DY = [-1, -1, 0, 1, 1, 1, 0, -1]
CODE = [64, 128, 1, 2, 4, 8, 16, 32]
STATE = ("dem", "slopes", "stone", "fines", "soilT", "soilM", "soilB", "nut", "totB", "depo", "prop")


@pytest.fixture(scope="module")
def ref():
    from oracle import oracle
    oracle.build()
    if oracle.ref_lib() is None:
        pytest.skip("reference sources not present")
    return oracle


def _points_to_tie(zr, sp, y, x, code):
    if code not in CODE:
        return False
    d = CODE.index(code)
    ny, nx = y + DY[d], x + DX[d]
    dc = np.float32(1.0 if d % 2 == 0 else 1.41)
    return zr[ny, nx] == zr[y, x] and np.float32(sp[ny, nx] + dc) == sp[y, x]


def _same_partition(a, b, mask):
    pairs = set(zip(a[mask].tolist(), b[mask].tolist()))
    return len(pairs) == len(set(a[mask].tolist())) == len(set(b[mask].tolist()))


def _copy(dst, src, fields):
    for f in fields:
        dst.a[f][...] = src.a[f]
    dst.s.outlet = src.s.outlet


# (dem, recompute climate, strict): a DEM without flats has no tie in the first
# plateau pass, so its basin partition and raised DEM must match exactly; with
# flats a tie may send a plateau to a different sink (a schedule choice).
CASES = {
    "noflat96": lambda: (S.make_dem(96, 0.8, 400.0, 0.05, 20, 0, 7), False, True),
    "fbm96": lambda: (S.make_dem(96, 0.8, 400.0, 0.05, 20, 3, 7), False, False),
    "flats64": lambda: (S.make_dem(64, 0.7, 300.0, 0.06, 5, 2, 11, flats_frac=0.2, depressions=12), False, False),
    "climate80": lambda: (S.make_dem(80, 0.7, 1500.0, 0.05, 15, 0, 5), True, True),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("flow_type,props", [(0, 0), (1, 0), (1, 1)])
def test_stagewise_against_reference_kernels(ref, case, flow_type, props):
    dem, recompute, strict = CASES[case]()
    p = ref.make_params(flow_direction_type=flow_type, mfd_proportions=props)
    rain, temp = (900.0, 9.0)
    st = S.initial_state(dem, 30.0, rain, temp)
    o = ref.OracleModel(dem, 30.0, st, rain, temp, params=ref.make_params(flow_direction_type=flow_type,
                                                                           mfd_proportions=props))
    r = ref.RefModel(dem, 30.0, st, rain, temp, params=p)
    mask = st["mask"] == 1
    ties = 0
    rng = np.random.default_rng(3)
    for step in range(2):
        if recompute:
            rr, tt = float(rng.lognormal(np.log(900), 0.3)), float(rng.normal(9, 2))
            for m in (o, r):
                m.s.last_rain, m.s.last_temp = m.s.rain, m.s.temp
                m.s.rain, m.s.temp = rr, tt
                ref.lib().oracle_set_climate(ref.C.byref(m.s), 0)
        r.flow_direction()
        o.flow_direction()
        assert r.s.init_sinks == o.s.init_sinks and r.s.init_flats == o.s.init_flats
        if strict:
            assert _same_partition(r["watershed"], o["watershed"], mask)
            np.testing.assert_array_equal(r["dem_routed"], o["dem_routed"])
            np.testing.assert_array_equal(r["shortest_paths"], o["shortest_paths"])
            assert r.s.sinkcount == o.s.sinkcount
        elif not np.array_equal(r["dem_routed"], o["dem_routed"]):
            _copy(r, o, ("fd", "sfd", "slopes", "dem"))  # a tie changed a spill: continue from the oracle
            r.flow_accumulation()
            o.flow_accumulation()
            r.erosion()
            o.erosion()
            _copy(o, r, STATE)
            continue
        for y, x in np.argwhere(r["sfd"] != o["sfd"]):
            assert _points_to_tie(o["dem_routed"], o["shortest_paths"], y, x, int(r["sfd"][y, x]))
            assert _points_to_tie(o["dem_routed"], o["shortest_paths"], y, x, int(o["sfd"][y, x]))
            ties += 1
        # plateau slopes: the reference may leave 1e-4 on directions a cell
        # routed through before its final one; every other entry is identical
        ds = r["slopes"] != o["slopes"]
        assert np.all((r["slopes"][ds] == 0.0001) | (o["slopes"][ds] == 0.0001))
        # the rest of the step from identical inputs: bit-identical
        _copy(r, o, ("fd", "sfd", "slopes", "dem"))
        r.flow_accumulation()
        o.flow_accumulation()
        for f in ("runoff", "soilM", "fa", "prop"):
            np.testing.assert_array_equal(r[f], o[f], err_msg=f)
        assert r.s.FA_max == o.s.FA_max and r.s.fa_uncomputed == o.s.fa_uncomputed
        r.erosion()
        o.erosion()
        for f in ("slopeptr", "ero", "inci", "geli", "depo", "dz", "wC", "wP", "stone", "fines", "soilT", "soilM",
                  "soilB", "nut", "totB", "dem", "slopes"):
            np.testing.assert_array_equal(r[f], o[f], err_msg=f)
        for k in ("totE", "totI", "totG", "totD", "totWC", "totWP", "totbio", "sed_uncomputed"):
            a, b = getattr(r.s, k), getattr(o.s, k)
            assert a == b or (np.isnan(a) and np.isnan(b)), k  # calcprops' 0/0 props give NaN in both
        _copy(o, r, STATE)
    # the tie rate stays small; it is reported in the design notes
    assert ties <= 0.02 * 2 * mask.sum()
