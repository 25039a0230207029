"""Serving (parallem_gb300.serve): continuous batching over one batch handle.

cpu: the tile packer that places DEMs in the canvas; the server's admission
logic on a stand-in batch (no GPU): refusal of requests that can never run,
queueing under the HBM budget, cancellation of a waiting and of a running
request, and results that stream back after their DEM has left the batch.
gpu: requests with staggered arrivals, admitted while others run, each give
the grids of the same request run alone on its own handle, bit for bit (their
grids come back through the asynchronous export); a request larger than the
canvas is refused while the others are served.
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


class FakeExport:
    def __init__(self, shape, names):
        self.shape, self.names, self.polls = shape, names, 0

    def ready(self):
        self.polls += 1
        return self.polls > 1  # the copy finishes one loop iteration later

    def wait(self):
        return {f: np.zeros(self.shape) for f in self.names}


class FakeBatch:
    """The batch interface the server uses, on the host only."""

    def __init__(self, W, H, bytes_per_cell=100, on_step=None):
        self.packer = TilePacker(W, H)
        self.W, self.H, self.bpc = W, H, bytes_per_cell
        self.ids, self.next, self.steps, self.removed, self.max_active = {}, 0, 0, [], 0
        self.on_step = on_step

    def graphs(self, on):
        pass

    def device_bytes(self):
        return self.W * self.H * self.bpc

    def add(self, dem, rain, temp):
        r = self.packer.alloc(dem.shape[1], dem.shape[0])
        if r is None:
            return None
        i, self.next = self.next, self.next + 1
        self.ids[i] = (r, dem.shape)
        self.max_active = max(self.max_active, len(self.ids))
        return i

    def set_state(self, i, st):
        pass

    def set_step_flags(self, i, f):
        pass

    def set_climate(self, i, rain, temp, recompute):
        pass

    def step(self):
        self.steps += 1
        if self.on_step:
            self.on_step(self.steps)

    def export(self, i, names):
        return FakeExport(self.ids[i][1], names)

    def remove(self, i):
        self.packer.free(self.ids.pop(i)[0])
        self.removed.append(i)

    def close(self):
        pass


def _req(rid, side, steps, arrival=0.0, **kw):
    from parallem_gb300 import serve as SV
    dem = np.full((side, side), 100.0)
    st = {"mask": np.ones((side, side), np.int32)}
    return SV.Request(rid, dem, st, np.full(steps, 900.0), np.full(steps, 9.0), steps, arrival, **kw)


def test_refuses_requests_that_can_never_run():
    from parallem_gb300 import serve as SV
    b = FakeBatch(256, 256)
    srv = SV.Server(256, 256, budget_bytes=4e6, batch=b)
    too_wide = _req(0, 300, 3)                        # larger than the canvas
    too_big = _req(1, 250, 3, outputs=("slopes",) * 3)  # its reservation exceeds the budget
    fine = _req(2, 64, 3)
    stats = srv.run([too_wide, too_big, fine])
    assert too_wide.status == "refused" and "canvas" in too_wide.reason
    assert too_big.status == "refused" and "budget" in too_big.reason
    assert fine.status == "done" and stats["requests"] == 1 and stats["refused"] == 2
    assert b.steps == 3 and srv.reserved == 0


def test_budget_queues_requests_until_memory_frees():
    from parallem_gb300 import serve as SV
    b = FakeBatch(512, 512)
    one = SV.Server(512, 512, batch=FakeBatch(512, 512)).reservation(_req(9, 200, 1))
    srv = SV.Server(512, 512, budget_bytes=1.5 * one, batch=b)  # room for one such request at a time
    reqs = [_req(i, 200, 4) for i in range(3)]
    stats = srv.run(reqs)
    assert stats["requests"] == 3 and all(r.status == "done" for r in reqs)
    assert b.max_active == 1 and b.steps == 12  # no overlap: the budget, not the canvas, held them back
    assert reqs[1].admitted >= reqs[0].admitted and reqs[2].admitted >= reqs[1].admitted
    assert srv.reserved == 0


def test_cancels_a_waiting_and_a_running_request():
    from parallem_gb300 import serve as SV
    srv = None

    def on_step(n):
        if n == 3:
            srv.cancel(0)  # running: leaves at the next step boundary
            srv.cancel(2)  # still waiting for room: dropped

    b = FakeBatch(256, 256, on_step=on_step)
    srv = SV.Server(256, 256, budget_bytes=150e9, batch=b)
    running = _req(0, 200, 50)   # takes most of the canvas
    short = _req(1, 32, 6)
    waiting = _req(2, 200, 5)    # no room while `running` holds its region
    stats = srv.run([running, short, waiting])
    assert running.status == "cancelled" and not running.result
    assert waiting.status == "cancelled" and waiting.admitted < 0
    assert short.status == "done"
    assert 0 in b.removed and stats["cancelled"] == 2 and stats["requests"] == 1
    assert b.steps < 50 and srv.reserved == 0


@pytest.mark.gpu
def test_served_requests_equal_alone():
    from parallem_gb300 import build
    from parallem_gb300 import serve as SV
    build.build()
    rng = np.random.default_rng(5)
    # three arrive together, three while those run
    reqs = [SV.make_request(i, rng, arrival=0.0 if i < 3 else 0.005 * i, side_lo=64, side_hi=200, steps_lo=2,
                            steps_hi=6) for i in range(6)]
    huge = SV.make_request(6, rng, arrival=0.0, side_lo=600, side_hi=600, steps_lo=2, steps_hi=2)
    srv = SV.Server(512, 512, budget_bytes=150e9, max_dems=16)
    assert srv.bytes_per_cell > 50  # measured from the handle's allocations
    stats = srv.run(reqs + [huge])
    srv.close()
    assert huge.status == "refused"
    assert stats["requests"] == len(reqs)
    assert stats["batch_steps"] < sum(r.steps for r in reqs)  # the work overlapped
    for r in reqs:
        assert r.status == "done"
        alone = SV.run_alone(r)
        for f in r.outputs:
            np.testing.assert_array_equal(r.result[f], alone[f], err_msg=f"request {r.rid}: {f}")
