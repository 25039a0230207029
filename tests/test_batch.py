"""Batches (lem_create_batch): DEMs of uneven sizes stepped together in one
canvas give the grids of the same DEMs stepped alone, bit for bit; budget
totals agree to 1e-9 relative (their fp64 block sums are added in another
order).  Also DEMs that join and leave between steps, and per-DEM step flags.
"""
import numpy as np
import pytest

from parallem_gb300 import scenario as S

pytestmark = pytest.mark.gpu

GRIDS = ("fd", "sfd", "fa", "runoff", "dem", "stone", "fines", "soilT", "soilM", "soilB", "nut", "totB", "ero",
         "inci", "geli", "depo", "slopeptr", "slopes")
TOT = ("tot_e", "tot_i", "tot_g", "tot_d", "tot_weather_c", "tot_weather_p", "tot_bio", "fa_max")
INT_TOT = ("sinkcount", "outlet", "initial_sinks", "initial_flats", "fa_uncomputed", "sed_uncomputed")


@pytest.fixture(scope="module")
def lem():
    from parallem_gb300 import build, lem
    build.build()
    lem.load()
    return lem


def scenario(n_rows, n_cols, seed, relief=600.0):
    dem = S.make_dem(max(n_rows, n_cols), 0.75, relief, 0.04, 10, 2, seed)[:n_rows, :n_cols].copy()
    dem[:2, :] = dem[-2:, :] = -9999.0  # a nodata ring on the cropped edges too
    dem[:, :2] = dem[:, -2:] = -9999.0
    st = S.initial_state(dem, 30.0, 900.0, 9.0)
    rng = np.random.default_rng(seed + 7)
    clim = [(float(rng.lognormal(np.log(900), 0.3)), float(rng.normal(9, 2))) for _ in range(3)]
    return dem, st, clim


def run_alone(lem, dem, st, clim, flags0=0):
    m = lem.Model(dem, 30.0, 900.0, 9.0)
    m.set_state(st)
    for j, (r, t) in enumerate(clim):
        m.step(r, t, True, flags0 if j == 0 else 0)
    out = {f: m.get(f) for f in GRIDS}
    out["totals"] = m.totals()
    m.close()
    return out


def check_same(a, b, name):
    for f in GRIDS:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f"{name}: {f}")
    for k in TOT:
        x, y = a["totals"][k], b["totals"][k]
        assert (np.isnan(x) and np.isnan(y)) or abs(x - y) <= 1e-9 * abs(y) + 1e-12, f"{name}: {k} {x} {y}"
    for k in INT_TOT:
        assert a["totals"][k] == b["totals"][k], f"{name}: {k}"


def test_batch_equals_alone(lem):
    cases = [scenario(96, 80, 41), scenario(130, 128, 42), scenario(70, 150, 43)]
    b = lem.Batch(512, 256, 30.0, max_dems=8)
    ids = []
    for dem, st, _ in cases:
        i = b.add(dem, 900.0, 9.0)
        assert i is not None
        b.set_state(i, st)
        ids.append(i)
    b.set_step_flags(ids[1], lem.STEP_SET_OUTLET_FROM_FA)  # the second DEM starts like lem.cpp's first iteration
    for j in range(3):
        for i, (_, _, clim) in zip(ids, cases):
            b.set_climate(i, clim[j][0], clim[j][1], True)
        b.step()
    b.synchronize()
    for n, (i, (dem, st, clim)) in enumerate(zip(ids, cases)):
        got = {f: b.get(i, f) for f in GRIDS}
        got["totals"] = b.totals(i)
        want = run_alone(lem, dem, st, clim, lem.STEP_SET_OUTLET_FROM_FA if n == 1 else 0)
        check_same(got, want, f"dem {n}")
    # the budget rows of all DEMs after one synchronisation are the rows read one by one
    rows = b.totals_n(ids[::-1])
    for i, row in zip(ids[::-1], rows):
        one = b.totals(i)
        assert all((row[k] == one[k]) or (row[k] != row[k] and one[k] != one[k]) for k in one), i
    b.close()


def test_batch_join_and_leave(lem):
    a, c, d = scenario(90, 90, 51), scenario(100, 64, 52), scenario(60, 60, 53)
    b = lem.Batch(256, 128, 30.0, max_dems=4)
    ia = b.add(a[0], 900.0, 9.0)
    b.set_state(ia, a[1])
    ic = b.add(c[0], 900.0, 9.0)
    b.set_state(ic, c[1])
    b.set_climate(ia, a[2][0][0], a[2][0][1], True)
    b.set_climate(ic, c[2][0][0], c[2][0][1], True)
    b.step()
    b.remove(ia)  # a leaves; d joins in its place and runs beside c's second step
    idd = b.add(d[0], 900.0, 9.0)
    b.set_state(idd, d[1])
    b.set_climate(idd, d[2][0][0], d[2][0][1], True)
    b.set_climate(ic, c[2][1][0], c[2][1][1], True)
    b.step()
    got_d = {f: b.get(idd, f) for f in GRIDS}
    got_d["totals"] = b.totals(idd)
    check_same(got_d, run_alone(lem, d[0], d[1], d[2][:1]), "joined")
    got_c = {f: b.get(ic, f) for f in GRIDS}
    got_c["totals"] = b.totals(ic)
    check_same(got_c, run_alone(lem, c[0], c[1], c[2][:2]), "stayed")
    b.close()


def test_batch_rejects_bad_placement(lem):
    dem, st, _ = scenario(64, 64, 61)
    b = lem.Batch(256, 128, 30.0, max_dems=2)
    with pytest.raises(lem.LemError):
        b.add(dem, 900.0, 9.0, at=(16, 0))  # not on a tile boundary
    i = b.add(dem, 900.0, 9.0, at=(0, 0))
    with pytest.raises(lem.LemError):
        b.add(dem, 900.0, 9.0, at=(32, 32))  # overlaps the first DEM's tiles
    bad = dem.copy()
    bad[0, 10] = 5.0  # no nodata ring
    with pytest.raises(lem.LemError):
        b.add(bad, 900.0, 9.0, at=(128, 0))
    b.remove(i)
    b.close()
