"""Known-answer tests of the FP64 oracle on hand-built grids.

Each expectation is worked out from the reference kernels it names; they pin
the oracle's reading of the reference before it is used to check the GPU path.
"""
import numpy as np
import pytest

from tests.helpers import CODE, NODATA, oracle_model, ringed


def centre_codes(z3x3):
    m = oracle_model(np.array(z3x3, dtype=np.float64))
    m.flow_direction()
    return m, int(m["sfd"][1, 1])


def test_flowdirs_steepest_descent_and_mfd_mask():
    # newflow.cu:92-140: N drop 1 (1/30), NE drop 2 (2/42.3), E drop .5, SE drop 3 (3/42.3)
    z = [[10, 9, 8], [12, 10, 9.5], [11, 10, 7]]
    from oracle.oracle import OracleModel  # noqa: F401
    m = oracle_model(np.array(z, dtype=np.float64))
    from oracle import oracle as O
    O.lib().oracle_flow_direction  # noqa: B018
    # run FlowDirs only through the public stage and read the pass-1 slopes
    m.flow_direction()
    slopes = m["slopes"][1, 1]
    L1, L2 = np.float64(np.float32(30) * np.float32(1.0)), np.float64(np.float32(30) * np.float32(1.41))
    assert slopes[0] == pytest.approx((10 - 9) / L1, rel=1e-15)
    assert slopes[1] == pytest.approx((10 - 8) / L2, rel=1e-15)
    assert slopes[2] == pytest.approx((10 - 9.5) / L1, rel=1e-15)
    assert slopes[3] == pytest.approx((10 - 7) / L2, rel=1e-15)
    assert list(slopes[4:]) == [0, 0, 0, 0]


def test_flowdirs_first_maximum_wins_ties():
    # two cardinal neighbours with the same drop: N (d=0) comes first
    m, sfd = centre_codes([[20, 9, 20], [20, 10, 20], [20, 9, 20]])
    assert sfd == CODE[0]
    m, sfd = centre_codes([[20, 20, 20], [9, 10, 9], [20, 20, 20]])
    assert sfd == CODE[2]  # E (d=2) before W (d=6)


def test_flowdirs_diagonal_length_is_float_1_41():
    # drop 1 cardinal vs drop 1.41 diagonal: 1.41/fl32(30*1.41f) > 1/30 by rounding
    m, sfd = centre_codes([[20, 20, 8.59], [20, 10, 9], [20, 20, 20]])
    L2 = np.float64(np.float32(30) * np.float32(1.41))
    expect = CODE[1] if (10 - 8.59) / L2 > (10 - 9) / 30.0 else CODE[2]
    assert sfd == expect


def test_flowdirs_sink_and_flat_counters():
    m, sfd = centre_codes([[20, 20, 20], [20, 10, 20], [20, 20, 20]])
    assert sfd == 0 and m.s.init_sinks == 1
    m, sfd = centre_codes([[10, 10, 10], [10, 10, 10], [10, 10, 10]])
    assert sfd == 0 and m.s.init_flats == 1 and m.s.init_sinks == 0


def test_nodata_neighbour_is_never_downslope():
    m, sfd = centre_codes([[NODATA, 20, 20], [20, 10, 20], [20, 20, 20]])
    assert sfd == 0


def test_plateau_routing_distances_and_cycle_at_the_outlet():
    # one row: a flat of six cells draining east into a lower cell
    dem = ringed(np.array([[5, 5, 5, 5, 5, 5, 4.0]]))
    m = oracle_model(dem)
    m.flow_direction()
    row = m["sfd"][1, 1:8]
    assert list(row[:6]) == [CODE[2]] * 6   # every flat cell routes east
    sp = m["shortest_paths"][1, 1:7]
    assert list(sp) == [5.0, 4.0, 3.0, 2.0, 1.0, 0.0]   # the last flat cell drains directly
    # the outlet (lowest cell) is forced to flow west (routeflow.cu:953): a 2-cycle
    assert m.outlet == 1 * dem.shape[1] + 7
    assert m["fd"][1, 7] == 16
    m.flow_accumulation()
    fa, w = m["fa"][1, 1:8], m["runoff"][1, 1:8]
    np.testing.assert_allclose(fa[:5], np.cumsum(w[:5]), rtol=1e-14)
    assert fa[5] == w[5] and fa[6] == w[6]    # the cycle never completes (mfd_simple.cu:72)
    assert m.s.fa_uncomputed == 2


def test_sediment_blocked_by_masked_south_neighbour():
    # MFDsedbud never completes masked cells (mfd_accum.cu:46,76): a masked
    # neighbour whose -9999 code has the bit pointing back blocks the cell
    dem = ringed(np.array([[5, 5, 5, 5, 5, 5, 4.0]]))
    m = oracle_model(dem)
    m.flow_direction()
    m.flow_accumulation()
    m.erosion()
    assert m.s.sed_uncomputed == 7
    assert np.all(m["depo"][1, 1:8] == 0.00001)


def test_pit_is_flooded_to_its_spill_height():
    interior = np.array([[9, 5, 9], [9, 1, 9], [9, 9, 9.0]])
    dem = ringed(interior)
    m = oracle_model(dem)
    m.flow_direction()
    ws = m["watershed"]
    assert len(set(ws[1:4, 1:4].ravel())) == 1 and ws[2, 2] > 0
    assert m.s.sinkcount == 2                      # labels {pit, 0} on boundary edges
    # after raising the pit to 5 (the lowest rim cell) both 5-cells are a flat
    # with no exit, so they stay sinks; the 9-cells drain into them
    assert m["sfd"][2, 2] == 0 and m["sfd"][1, 2] == 0
    assert m["sfd"][3, 2] == CODE[0]               # south-middle 9 flows north into the raised pit


def test_fd_epilogue_mfd_mode_falls_back_to_sfd():
    from oracle.oracle import make_params
    z = np.array([[10, 9, 8], [12, 10, 9.5], [11, 10, 7]], dtype=np.float64)
    m = oracle_model(z, params=make_params(flow_direction_type=1))
    m.flow_direction()
    assert m["fd"][1, 1] == CODE[0] + CODE[1] + CODE[2] + CODE[3]
