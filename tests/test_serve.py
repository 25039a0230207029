"""Serving (parallem_gb300.serve): continuous batching over one batch handle.

gpu: requests with staggered arrivals, admitted while others run, each give
the grids of the same request run alone on its own handle, bit for bit.
cpu: the tile packer that places DEMs in the canvas.
"""
import numpy as np
import pytest

from parallem_gb300.packing import TilePacker


def test_packer_places_without_overlap_and_reuses_freed_room():
    p = TilePacker(512, 256)
    rects = [p.alloc(w, h) for w, h in ((100, 40), (64, 200), (300, 100), (33, 33))]
    assert all(r is not None for r in rects)
    occ = np.zeros((256 // 32, 512 // 32), int)
    for x0, y0, bw, bh in rects:
        assert x0 % 32 == 0 and y0 % 32 == 0
        occ[y0 // 32:y0 // 32 + bh, x0 // 32:x0 // 32 + bw] += 1
    assert occ.max() == 1 and occ.sum() == p.occ.sum()
    assert p.alloc(512, 256) is None
    for r in rects:
        p.free(r)
    assert p.used_fraction() == 0.0 and p.alloc(512, 256) == (0, 0, 16, 8)


@pytest.mark.gpu
def test_served_requests_equal_alone():
    from parallem_gb300 import build
    from parallem_gb300 import serve as SV
    build.build()
    rng = np.random.default_rng(5)
    # three arrive together, three while those run
    reqs = [SV.make_request(i, rng, arrival=0.0 if i < 3 else 0.005 * i, side_lo=64, side_hi=200, steps_lo=2,
                            steps_hi=6) for i in range(6)]
    srv = SV.Server(512, 512, budget_bytes=150e9, max_dems=16)
    stats = srv.run(reqs)
    srv.close()
    assert stats["requests"] == len(reqs)
    assert stats["batch_steps"] < sum(r.steps for r in reqs)  # the work overlapped
    for r in reqs:
        alone = SV.run_alone(r)
        for f in r.outputs:
            np.testing.assert_array_equal(r.result[f], alone[f], err_msg=f"request {r.rid}: {f}")
