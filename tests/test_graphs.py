"""CUDA-graph steps (lem_set_graphs): a timestep launched as one captured graph
gives the grids of eager steps bit for bit, for a single grid and for a batch
whose DEMs join and leave between steps (each change of the visited tiles or
chunks captures a new graph), and issues the same kernel launches.
"""
import numpy as np
import pytest

from parallem_gb300 import scenario as S

from test_batch import GRIDS, check_same, scenario

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lem():
    from parallem_gb300 import build, lem
    build.build()
    lem.load()
    return lem


def _single(lem, graphs, flags0):
    dem = S.make_dem(192, 0.75, 600.0, 0.04, 40, 4, 71)
    st = S.initial_state(dem, 30.0, 900.0, 9.0)
    rng = np.random.default_rng(72)
    m = lem.Model(dem, 30.0, 900.0, 9.0)
    m.set_state(st)
    m.graphs(graphs)
    n0 = m.launches
    for j in range(4):
        m.step(float(rng.lognormal(np.log(900), 0.3)), float(rng.normal(9, 2)), True, flags0 if j == 0 else 0)
    m.synchronize()
    out = {f: m.get(f) for f in GRIDS}
    out["totals"] = m.totals()
    n = m.launches - n0
    m.close()
    return out, n


@pytest.mark.parametrize("flags0", [0, 0x1])
def test_single_grid_graph_equals_eager(lem, flags0):
    eager, n_eager = _single(lem, False, flags0)
    graph, n_graph = _single(lem, True, flags0)
    check_same(graph, eager, "graph")
    assert n_graph == n_eager


def _batch(lem, graphs):
    a, c, d = scenario(90, 90, 81), scenario(100, 64, 82), scenario(60, 60, 83)
    b = lem.Batch(256, 128, 30.0, max_dems=4)
    b.graphs(graphs)
    ia = b.add(a[0], 900.0, 9.0)
    b.set_state(ia, a[1])
    ic = b.add(c[0], 900.0, 9.0)
    b.set_state(ic, c[1])
    for j in range(2):
        b.set_climate(ia, a[2][j][0], a[2][j][1], True)
        b.set_climate(ic, c[2][j][0], c[2][j][1], True)
        b.step()
    b.remove(ia)
    idd = b.add(d[0], 900.0, 9.0)
    b.set_state(idd, d[1])
    b.set_step_flags(idd, lem.STEP_SET_OUTLET_FROM_FA)
    b.set_climate(idd, d[2][0][0], d[2][0][1], True)
    b.set_climate(ic, c[2][2][0], c[2][2][1], True)
    b.step()
    out = {}
    for name, i in (("c", ic), ("d", idd)):
        g = {f: b.get(i, f) for f in GRIDS}
        g["totals"] = b.totals(i)
        out[name] = g
    b.close()
    return out


def test_batch_graph_equals_eager_across_joins(lem):
    eager = _batch(lem, False)
    graph = _batch(lem, True)
    for k in ("c", "d"):
        check_same(graph[k], eager[k], f"graph {k}")


def test_autotuned_schedule_gives_the_same_grids(lem):
    """Steps under every candidate schedule of the autotuner (cooperative blocks
    per SM) give the grids of the default schedule, and the schedule kept
    afterwards is one of the candidates."""
    def run(tune):
        dem = S.make_dem(160, 0.75, 800.0, 0.04, 30, 3, 91)
        st = S.initial_state(dem, 30.0, 900.0, 9.0)
        rng = np.random.default_rng(92)
        m = lem.Model(dem, 30.0, 900.0, 9.0)
        m.set_state(st)
        m.graphs(True)
        if tune:
            m.autotune(3)
            assert m.tuning()["state"] == "tuning"
        for j in range(14):
            m.step(float(rng.lognormal(np.log(900), 0.3)), float(rng.normal(9, 2)), True, 0x1 if j == 0 else 0)
        m.synchronize()
        out = {f: m.get(f) for f in GRIDS}
        out["totals"] = m.totals()
        t = m.tuning()
        m.close()
        return out, t

    plain, t0 = run(False)
    tuned, t1 = run(True)
    check_same(tuned, plain, "autotuned")
    assert t0["state"] == "default" and t1["state"] == "tuned" and t1["steps_left"] == 0
    assert all(b > 0 for b in t1["coop_blocks"].values())
    assert t1["tuned_ms"] <= t1["default_ms"] + 1e-9


def test_every_flow_direction_tile_shape_gives_the_same_steps(lem):
    """The autotuner's candidate steps run the TMA flow-direction kernel with
    tiles of 8, 16, 32 and again 8 rows; each of those steps equals, bit for
    bit, the same step under the default schedule.  A width that is not a
    multiple of 16 takes the plain-load kernel, and the same DEM inside a
    32-aligned batch canvas takes the TMA kernel: those agree too."""
    dem = S.make_dem(256, 0.75, 600.0, 0.04, 60, 6, 91)
    st = S.initial_state(dem, 30.0, 900.0, 9.0)
    rng = np.random.default_rng(92)
    clim = [(float(rng.lognormal(np.log(900), 0.3)), float(rng.normal(9, 2))) for _ in range(5)]
    a = lem.Model(dem, 30.0, 900.0, 9.0)
    b = lem.Model(dem, 30.0, 900.0, 9.0)
    for m in (a, b):
        m.set_state(st)
    assert b.tuning()["flowdirs_tile_rows"] in (8, 16, 32)  # a width of 256 takes the TMA kernel
    b.autotune(1)  # one unmeasured step, then the four candidates
    for rain, temp in clim:
        a.step(rain, temp, True)
        b.step(rain, temp, True)
        for f in ("fd", "sfd", "slopes", "fa", "dem", "stone"):
            np.testing.assert_array_equal(a.get(f), b.get(f), err_msg=f)
    assert b.tuning()["state"] == "tuned"
    a.close()
    b.close()
    # a width of 250 (not a multiple of 16): the plain-load kernel, against the TMA kernel on the canvas
    d2 = dem[:, :250].copy()
    d2[:, -2:] = S.NODATA
    st2 = S.initial_state(d2, 30.0, 900.0, 9.0)
    c = lem.Model(d2, 30.0, 900.0, 9.0)
    c.set_state(st2)
    assert c.tuning()["flowdirs_tile_rows"] == 0
    bt = lem.Batch(512, 512, 30.0, max_dems=4)
    i = bt.add(d2, 900.0, 9.0)
    bt.set_state(i, st2)
    for rain, temp in clim[:2]:
        c.step(rain, temp, True)
        bt.set_climate(i, rain, temp, True)
        bt.step()
        for f in ("fd", "sfd", "slopes", "fa", "dem"):
            np.testing.assert_array_equal(c.get(f), bt.get(i, f), err_msg=f)
    c.close()
    bt.close()
