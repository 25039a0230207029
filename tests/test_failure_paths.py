"""Failure detection in the forms this path allows: bounded device loops that
return an error status to the host, and a full table that says so.

The reference's loops run until their change flags clear, without a bound
(plateau sweeps FD_kernels/routeflow.cu:854-872, merge and label loops
routeflow.cu:285-302,314-338, accumulation FA_kernels/mfd_simple.cu:204-226),
and its basin-pair hash table drops entries silently when a bucket overflows
(FD_kernels/newflow.cu:860-872).  Here every device loop stops after
lem_limits.max_rounds rounds and lem_synchronize returns LEM_ERR_NOCONVERGE; a
basin-pair table of 2^edge_table_log2 slots that fills up makes it return
LEM_ERR_CAPACITY.  In both cases the handle stays usable: after the limits are
restored the next stage gives the oracle's direction codes again.

The cyclic-code case is the reference's own behaviour, not an error: cells
whose donors never finish keep fa = w (mfd_simple.cu:72), and the handle path
reports them in fa_uncomputed exactly as the oracle counts them.
"""
import numpy as np
import pytest

from parallem_gb300 import scenario as S
from tests.helpers import NODATA, ringed

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def libs():
    from oracle import oracle
    from parallem_gb300 import build, lem
    oracle.build()
    build.build()
    lem.load()
    return oracle, lem


def _pair(libs, dem):
    oracle, lem = libs
    st = S.initial_state(dem, 30.0, 800.0, 10.0)
    o = oracle.OracleModel(dem, 30.0, st, 800.0, 10.0)
    g = lem.Model(dem, 30.0, 800.0, 10.0)
    g.set_state(st)
    return o, g, st


def _wide_flat(n=160):
    """A tilted surface with a flat shelf that spans several 32x32 tiles, so
    its plateau distances need many relaxation rounds across tiles."""
    y, x = np.mgrid[0:n, 0:n]
    z = 300.0 + 0.5 * x + 0.25 * y
    z[20:140, 30:150] = 340.0  # the shelf: 120 x 120 cells at one height
    return ringed(z, 2)


def test_plateau_round_cap_returns_noconverge_and_the_handle_recovers(libs):
    oracle, lem = libs
    dem = _wide_flat()
    o, g, _ = _pair(libs, dem)
    g.limits(max_rounds=1)
    g.flow_direction()
    with pytest.raises(lem.LemError) as e:
        g.synchronize()
    assert e.value.code == 3  # LEM_ERR_NOCONVERGE
    g.limits()  # defaults again; the same stage from the same DEM now completes
    g.flow_direction()
    g.synchronize()
    o.flow_direction()
    np.testing.assert_array_equal(g.get("fd"), o["fd"])
    np.testing.assert_array_equal(g.get("sfd"), o["sfd"])


def test_flooding_round_cap_returns_noconverge_and_the_handle_recovers(libs):
    oracle, lem = libs
    # nested depressions and quantised flats: the label merge, the pointer
    # jumping, the spill relaxation and the plateau sweeps all need rounds
    dem = S.make_dem(192, 0.7, 800.0, 0.03, 10, 4, 13, flats_frac=0.15, depressions=40)
    o, g, _ = _pair(libs, dem)
    g.limits(max_rounds=2)
    g.flow_direction()
    with pytest.raises(lem.LemError) as e:
        g.synchronize()
    assert e.value.code == 3
    g.limits()
    g.flow_direction()
    g.synchronize()
    o.flow_direction()
    np.testing.assert_array_equal(g.get("fd"), o["fd"])
    assert g.totals()["sinkcount"] == o.s.sinkcount


def test_full_basin_pair_table_returns_capacity(libs):
    oracle, lem = libs
    dem = S.make_dem(256, 0.8, 400.0, 0.05, 200, 0, 41)  # 200 pits: hundreds of basin pairs
    o, g, _ = _pair(libs, dem)
    g.limits(edge_table_log2=4)  # 16 slots
    g.flow_direction()
    with pytest.raises(lem.LemError) as e:
        g.synchronize()
    assert e.value.code == 2  # LEM_ERR_CAPACITY
    g.limits()
    g.flow_direction()
    g.synchronize()
    o.flow_direction()
    np.testing.assert_array_equal(g.get("fd"), o["fd"])
    assert g.totals()["sinkcount"] == o.s.sinkcount


def _cyclic_codes(n=24):
    """A grid whose codes all drain west to the nodata ring, except a 2-cycle
    (two cells pointing at each other) fed by a chain of three cells."""
    dem = ringed(np.full((n, n), 200.0), 1)
    fd = np.where(dem == NODATA, -9999, 16).astype(np.int32)  # every cell flows west
    r = 12
    fd[r, 10] = 1    # E: points at (r, 11)
    fd[r, 11] = 16   # W: points back at (r, 10)
    fd[r, 14] = 16   # a chain (r, 14) -> (r, 13) -> (r, 12) -> (r, 11) enters the cycle
    fd[r, 13] = 16
    fd[r, 12] = 16
    return dem, fd


def test_cyclic_codes_complete_like_the_reference(libs):
    oracle, lem = libs
    dem, fd = _cyclic_codes()
    o, g, st = _pair(libs, dem)
    o.set_arrays(fd=fd, sfd=fd)
    g.set("fd", fd)
    g.set("sfd", fd)
    for flags in (0, lem.STEP_CONTRIB):
        g.set_state({"soilM": st["soilM"]})
        o.set_arrays(soilM=st["soilM"])
        g.flow_accumulation(flags)
        g.synchronize()
        o.flow_accumulation(flags)
        mask = st["mask"] == 1
        fa, w = g.get("fa"), g.get("runoff")
        np.testing.assert_allclose(fa[mask], o["fa"][mask], rtol=1e-5, atol=0)
        t = g.totals()
        assert t["fa_uncomputed"] == o.s.fa_uncomputed
        # the two cells of the cycle are never finished; the chain that feeds it is
        assert t["fa_uncomputed"] == 2
        r = 12
        assert fa[r, 10] == pytest.approx(w[r, 10], rel=1e-6) and fa[r, 11] == pytest.approx(w[r, 11], rel=1e-6)
        if flags & lem.STEP_CONTRIB:
            np.testing.assert_array_equal(g.get("contrib"), o["contrib"])
