"""Restart snapshots (lem_snapshot_*): the steps after loading a snapshot equal
the steps after saving it, bit for bit, for a single grid and for a DEM of a
batch; a snapshot of another size is refused."""
import numpy as np
import pytest

from parallem_gb300 import scenario as S

pytestmark = pytest.mark.gpu
GRIDS = ("fd", "fa", "dem", "stone", "fines", "soilT", "soilM", "soilB", "nut", "totB", "depo", "slopes")


def test_single_grid_restart():
    from parallem_gb300 import build, lem
    build.build()
    sc = S.config_large(6, n=192, steps=4)
    st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    a = lem.Model(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    a.set_state(st)
    for i in range(2):
        a.step(sc.rain[i], sc.temp[i], True)
    snap = a.snapshot()
    for i in range(2, 4):
        a.step(sc.rain[i], sc.temp[i], True)
    b = lem.Model(sc.dem, 30.0, sc.init_rain, sc.init_temp, upload=False)
    b.restore(snap)
    for i in range(2, 4):
        b.step(sc.rain[i], sc.temp[i], True)
    for f in GRIDS:
        np.testing.assert_array_equal(a.get(f), b.get(f), err_msg=f)
    assert a.totals()["outlet"] == b.totals()["outlet"]
    small = lem.Model(sc.dem[:96, :96], 30.0, sc.init_rain, sc.init_temp, upload=False)
    with pytest.raises(lem.LemError):
        small.restore(snap)
    for m in (a, b, small):
        m.close()


def test_batch_dem_restart_into_single_grid():
    from parallem_gb300 import build, lem
    build.build()
    sc = S.config_large(7, n=128, steps=3)
    st = S.initial_state(sc.dem, 30.0, sc.init_rain, sc.init_temp)
    bt = lem.Batch(256, 256, 30.0, max_dems=2)
    i = bt.add(sc.dem, sc.init_rain, sc.init_temp, at=(128, 64))
    bt.set_state(i, st)
    bt.set_climate(i, sc.rain[0], sc.temp[0], True)
    bt.step()
    snap = bt.snapshot(i)
    bt.set_climate(i, sc.rain[1], sc.temp[1], True)
    bt.step()
    m = lem.Model(sc.dem, 30.0, sc.init_rain, sc.init_temp, upload=False)
    m.restore(snap)
    m.step(sc.rain[1], sc.temp[1], True)
    for f in GRIDS:
        np.testing.assert_array_equal(bt.get(i, f), m.get(f), err_msg=f)
    bt.close()
    m.close()
