"""lem_accumulate_flow_noalloc: flow accumulation that allocates nothing.

It exists for callers that may not allocate device memory (a host program that
passes only buffers from its own device arena, a memory-budgeted service that
must not call cudaMalloc on its request path).  Its scratch is one static
device array shared by every call, so these tests check that consecutive calls
on different grids each give the accumulation of the FP64 oracle and of the
handle path (the existing entry point) within the accumulation tolerance of the
parity tests (1e-5 relative); that codes with a cycle give the oracle's values
(the cycle's cells keep their own weight) and the status that says cells were
left unreached; and that a grid larger than the array is refused before any
work.  This file is collected last; it passes alone or after the other tests.
"""
import numpy as np
import pytest

from tests.helpers import NODATA, ringed

pytestmark = pytest.mark.gpu


def _handle_path_and_oracle(seed: int, n: int) -> dict:
    from oracle import oracle
    from parallem_gb300 import lem
    from parallem_gb300 import scenario as S
    dem = S.make_dem(n, 0.8, 400.0, 0.05, 20, 3, seed)
    st = S.initial_state(dem, 30.0, 800.0, 10.0)
    g = lem.Model(dem, 30.0, 800.0, 10.0)
    g.set_state(st)
    g.flow_direction()
    g.flow_accumulation()
    g.synchronize()
    out = {f: g.get(f) for f in ("fd", "runoff", "dem", "fa")}
    g.close()
    o = oracle.OracleModel(dem, 30.0, st, 800.0, 10.0)
    o.flow_direction()
    o.flow_accumulation()
    out["oracle"] = {f: o[f].copy() for f in ("fd", "runoff", "fa")}
    out["unreached"] = o.s.fa_uncomputed  # e.g. a 2-cycle at the outlet, whose code is forced to 16
    return out


def _noalloc(L, fd, w, dem):
    import torch
    dev = torch.device("cuda", 0)
    h, wd = dem.shape
    t_fd = torch.from_numpy(np.ascontiguousarray(fd, dtype=np.int32)).to(dev)
    t_w = torch.from_numpy(np.ascontiguousarray(w, dtype=np.float64)).to(dev)
    t_dem = torch.from_numpy(np.ascontiguousarray(dem, dtype=np.float64)).to(dev)
    out = torch.full((h, wd), -1.0, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc = L.lem_accumulate_flow_noalloc(t_fd.data_ptr(), t_w.data_ptr(), t_dem.data_ptr(), out.data_ptr(), wd, h,
                                       None)
    return rc, out.cpu().numpy()


def test_noalloc_matches_the_oracle_and_the_handle_path_on_consecutive_calls():
    pytest.importorskip("torch")
    from oracle import oracle
    from parallem_gb300 import build, lem
    oracle.build()
    build.build()
    L = lem.load()
    for seed, n in ((31, 256), (37, 384), (31, 256)):
        ref = _handle_path_and_oracle(seed, n)
        inside = ref["dem"] != -9999
        # LEM_ERR_NOCONVERGE exactly when the oracle leaves cells unreached; d_fa is written either way
        want = 3 if ref["unreached"] else 0
        # from the oracle's own codes and weights: correctmfdflow directly
        o = ref["oracle"]
        rc, fa = _noalloc(L, o["fd"], o["runoff"], ref["dem"])
        assert rc == want, lem.STATUS.get(rc, rc)
        np.testing.assert_allclose(fa[inside], o["fa"][inside], rtol=1e-5, atol=0)
        assert np.all(fa[~inside] == 0.0)
        # from the handle path's codes and weights: the existing entry point
        rc, fa = _noalloc(L, ref["fd"], ref["runoff"], ref["dem"])
        assert rc == want, lem.STATUS.get(rc, rc)
        np.testing.assert_allclose(fa[inside], ref["fa"][inside], rtol=1e-5, atol=0)
        assert np.all(fa[~inside] == 0.0)


def test_noalloc_cycle_keeps_the_weights_and_reports_unreached_cells():
    pytest.importorskip("torch")
    from oracle import oracle
    from parallem_gb300 import build, lem
    from parallem_gb300 import scenario as S
    oracle.build()
    build.build()
    L = lem.load()
    n = 24
    dem = ringed(np.full((n, n), 200.0), 1)
    fd = np.where(dem == NODATA, -9999, 16).astype(np.int32)  # every cell flows west
    r = 12
    fd[r, 10], fd[r, 11] = 1, 16  # (r, 10) -> (r, 11) -> (r, 10): a 2-cycle; row r east of it feeds it
    st = S.initial_state(dem, 30.0, 800.0, 10.0)
    o = oracle.OracleModel(dem, 30.0, st, 800.0, 10.0)
    o.set_arrays(fd=fd, sfd=fd)
    o.flow_accumulation()
    assert o.s.fa_uncomputed == 2
    inside = dem != NODATA
    for _ in range(2):  # twice in a row: the shared scratch starts clean each call
        rc, fa = _noalloc(L, fd, o["runoff"], dem)
        assert rc == 3  # LEM_ERR_NOCONVERGE: two cells were never reached; d_fa is still written
        np.testing.assert_allclose(fa[inside], o["fa"][inside], rtol=1e-5, atol=0)
        assert fa[r, 10] == pytest.approx(o["runoff"][r, 10], rel=1e-6)


def test_noalloc_refuses_grids_larger_than_its_scratch():
    from parallem_gb300 import build, lem
    build.build()
    L = lem.load()
    n = 1025  # 1025 * 1025 cells > LEM_NOALLOC_MAX_CELLS (2**20)
    rc = L.lem_accumulate_flow_noalloc(1, 1, 1, 1, n, n, None)  # refused before any pointer is touched
    assert rc == 2  # LEM_ERR_CAPACITY
