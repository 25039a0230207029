"""lem_accumulate_flow_noalloc: flow accumulation that allocates nothing.

It exists for callers that may not allocate device memory (a host program that
passes only buffers from its own device arena, a memory-budgeted service that
must not call cudaMalloc on its request path).  Its scratch is one static
device array shared by every call, so these tests check that consecutive calls
on different grids each give the accumulation of the handle path (the existing
entry point) within the accumulation tolerance of the parity tests (1e-5
relative), and that a grid larger than the array is refused before any work.
This file is collected last; it passes alone or after the other tests.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _handle_path(seed: int, n: int) -> dict:
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
    return out


def test_noalloc_matches_the_handle_path_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    from parallem_gb300 import build, lem
    build.build()
    L = lem.load()
    dev = torch.device("cuda", 0)
    for seed, n in ((31, 256), (37, 384), (31, 256)):
        ref = _handle_path(seed, n)
        fd = torch.from_numpy(ref["fd"]).to(dev)
        w = torch.from_numpy(ref["runoff"]).to(dev)
        dem = torch.from_numpy(ref["dem"]).to(dev)
        out = torch.full((n, n), -1.0, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = L.lem_accumulate_flow_noalloc(fd.data_ptr(), w.data_ptr(), dem.data_ptr(), out.data_ptr(), n, n, None)
        assert rc == 0, lem.STATUS.get(rc, rc)
        fa = out.cpu().numpy()
        inside = ref["dem"] != -9999
        np.testing.assert_allclose(fa[inside], ref["fa"][inside], rtol=1e-5, atol=0)
        assert np.all(fa[~inside] == 0.0)


def test_noalloc_refuses_grids_larger_than_its_scratch():
    from parallem_gb300 import build, lem
    build.build()
    L = lem.load()
    n = 1025  # 1025 * 1025 cells > LEM_NOALLOC_MAX_CELLS (2**20)
    rc = L.lem_accumulate_flow_noalloc(1, 1, 1, 1, n, n, None)  # refused before any pointer is touched
    assert rc == 2  # LEM_ERR_CAPACITY
