"""
Serving loop: admission, budget and slot accounting on the host (fake
executor, no GPU), and on the GPU the same result for a request alone and in
a mix of concurrent packs.
"""

import math

import numpy as np
import pytest

from dxtb_gb300.serving import Request, Server, latency_summary, poisson_requests


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


class FakeExecutor:
    """Each pack takes `cost` seconds of fake time per molecule of its largest member."""

    def __init__(self, clock, cost=1e-3):
        self.clock = clock
        self.cost = cost
        self.launched = []

    def nbytes(self, r):
        return 1000 * len(r.numbers)

    def launch(self, reqs, slot):
        self.launched.append(([r.rid for r in reqs], slot, self.clock()))
        dur = self.cost * max(len(r.numbers) for r in reqs)
        return {"t": self.clock() + dur, "reqs": reqs}

    def ready(self, h):
        return self.clock() >= h["t"]

    def collect(self, h):
        return [(-float(len(r.numbers)), None, 5, 0) for r in h["reqs"]]

    def norb(self, r):
        return 2 * len(r.numbers)


def _req(rid, method="gfn2", nat=10, t=0.0):
    return Request(rid, method, np.ones(nat, dtype=np.int64), np.zeros((nat, 3)), arrival=t)


def test_fifo_method_grouping_and_pack_cap():
    clk = FakeClock()
    ex = FakeExecutor(clk)
    srv = Server(ex, hbm_budget=1e9, slots=2, max_pack=3, clock=clk)
    for i, m in enumerate(["gfn2", "gfn1", "gfn2", "gfn2", "gfn2", "gfn1"]):
        srv.submit(_req(i, m))
    srv.pump()
    # slot 0: oldest is gfn2 -> gfn2 requests 0, 2, 3 (cap 3); slot 1: next oldest is gfn1 -> 1, 5
    assert ex.launched[0][0] == [0, 2, 3]
    assert ex.launched[1][0] == [1, 5]
    assert [r.rid for r in srv.queue] == [4]
    assert len(srv.inflight) == 2 and not srv.free_slots


def test_budget_limits_admission_and_releases():
    clk = FakeClock()
    ex = FakeExecutor(clk)
    srv = Server(ex, hbm_budget=25_000, slots=4, max_pack=8, clock=clk)
    for i in range(4):
        srv.submit(_req(i, nat=10))      # 10 kB each
    srv.pump()
    assert ex.launched[0][0] == [0, 1]  # 20 kB fits, the third would not
    assert srv.used == 20_000
    srv.pump()
    assert len(ex.launched) == 1        # no memory: the queue waits
    clk.t = 1.0
    out = srv.pump()
    assert sorted(r.rid for r in out) == [0, 1]
    assert ex.launched[1][0] == [2, 3]
    assert srv.stats.max_bytes <= 25_000


def test_oversized_request_is_rejected_not_blocking():
    clk = FakeClock()
    ex = FakeExecutor(clk)
    srv = Server(ex, hbm_budget=15_000, slots=1, max_pack=8, clock=clk)
    srv.submit(_req(0, nat=20))          # 20 kB > budget
    srv.submit(_req(1, nat=5))
    out = srv.pump()
    assert len(out) == 1 and out[0].rid == 0 and out[0].error and math.isnan(out[0].energy)
    assert ex.launched[0][0] == [1]


def test_slots_bound_inflight_packs():
    clk = FakeClock()
    ex = FakeExecutor(clk)
    srv = Server(ex, hbm_budget=1e12, slots=3, max_pack=1, clock=clk)
    for i in range(10):
        srv.submit(_req(i))
    done = []
    while not srv.idle:
        done += srv.pump()
        assert len(srv.inflight) <= 3
        clk.t += 0.004
    assert sorted(r.rid for r in done) == list(range(10))
    assert srv.stats.max_inflight == 3
    # FIFO: admission times are non-decreasing in request id
    adm = [r.admitted for r in sorted(done, key=lambda r: r.rid)]
    assert adm == sorted(adm)


def test_large_lane_keeps_small_requests_moving():
    clk = FakeClock()
    ex = FakeExecutor(clk, cost=1e-3)
    # orbitals = 2 nat; large lane from 200 orbitals (nat >= 100), 1 of 3 slots
    srv = Server(ex, hbm_budget=1e12, slots=3, max_pack=8, large_slots=1, large_n=200, large_pack=2,
                 clock=clk)
    big = [_req(i, nat=300) for i in range(3)]          # 0.3 s each pack
    small = [_req(10 + i, nat=10) for i in range(12)]  # 0.01 s each pack
    for r in big + small:
        srv.submit(r)
    assert [r.rid for r in srv.queues["large"]] == [0, 1, 2]
    srv.pump()
    # the large slot takes at most large_pack big requests; small packs fill the rest
    assert ex.launched[0][0] == [0, 1] and ex.launched[0][1] == 2
    assert all(len(ids) <= 8 and min(ids) >= 10 for ids, _, _ in ex.launched[1:])
    done = {}
    while not srv.idle:
        for x in srv.pump():
            done[x.rid] = x.done
        clk.t += 0.005
    # every small request finishes before the second large pack does
    assert max(done[10 + i] for i in range(12)) < done[2]


def test_size_order_packs_similar_sizes_smallest_first():
    clk = FakeClock()
    ex = FakeExecutor(clk)
    srv = Server(ex, hbm_budget=1e12, slots=1, max_pack=8, order="size", clock=clk)
    for rid, nat in enumerate([40, 10, 30, 12, 25, 100]):
        srv.submit(_req(rid, nat=nat))
    srv.pump()
    # smallest head (nat 10 -> 20 orbitals); only requests of <= 40 orbitals join
    assert ex.launched[0][0] == [1, 3]
    done = []
    while not srv.idle:
        done += srv.pump()
        clk.t += 0.2
    order = [ids for ids, _, _ in ex.launched]
    assert order[1:] == [[4, 2, 0], [5]]  # head 25 atoms (50 orbitals): up to 100 join


def test_longest_first_large_lane():
    """large_order="longest": the large lane admits its largest request
    first, with pack members of at least half its size; the small lane keeps
    its own order."""
    clk = FakeClock()
    ex = FakeExecutor(clk)
    srv = Server(ex, hbm_budget=1e12, slots=2, max_pack=8, large_slots=1, large_n=200,
                 large_pack=2, order="size", large_order="longest", clock=clk)
    for rid, nat in enumerate([120, 300, 100, 160, 10, 5]):
        srv.submit(_req(rid, nat=nat))
    srv.pump()
    # large lane (>= 100 atoms): 300 first, then 160 (>= 150) joins; 120 and 100 wait
    assert ex.launched[0] == ([1, 3], 1, 0.0)
    assert ex.launched[1][0] == [5, 4]  # small lane: smallest first
    while not srv.idle:
        srv.pump()
        clk.t += 0.05
    assert [ids for ids, slot, _ in ex.launched if slot == 1][1] == [0, 2]
    with pytest.raises(ValueError):
        Server(ex, large_order="random")


def test_large_lane_sm_cap():
    """large_sms: in-flight large packs hold at most that many SMs (the team
    size of each molecule); a molecule whose team alone exceeds the cap
    runs when the lane is otherwise empty."""
    clk = FakeClock()
    ex = FakeExecutor(clk)
    ex.team_sms = lambda r: 16 if len(r.numbers) >= 250 else 8
    srv = Server(ex, hbm_budget=1e12, slots=6, max_pack=8, large_slots=5, large_n=200,
                 large_pack=1, order="size", large_order="longest", large_sms=24, clock=clk)
    for rid, nat in enumerate([300, 280, 120, 150, 110, 20]):
        srv.submit(_req(rid, nat=nat))
    srv.pump()
    # the small request on the small slot; large: 300 (16 SMs) first, 280
    # (16) would exceed 24 while a small request runs, 150 (8) fits, 120 waits
    assert [ids for ids, slot, _ in ex.launched if slot == 0] == [[5]]
    assert [ids for ids, slot, _ in ex.launched if slot > 0] == [[0], [3]]
    assert srv.sms_used == 24
    while srv._small_busy():
        srv.pump()
        assert srv.sms_used <= 24
        clk.t += 0.001
    # no small request left: the cap is lifted
    while not srv.idle:
        srv.pump()
        clk.t += 0.01
    assert sorted(ids[0] for ids, _, _ in ex.launched) == [0, 1, 2, 3, 4, 5]
    alone = Server(ex, hbm_budget=1e12, slots=2, max_pack=8, large_slots=1, large_n=200,
                   large_sms=8, clock=clk)
    alone.submit(_req(8, nat=10))
    alone.submit(_req(9, nat=300))
    alone.pump()
    assert [9] in [ids for ids, _, _ in ex.launched] and alone.sms_used == 16


def test_small_requests_borrow_idle_large_slots():
    clk = FakeClock()
    ex = FakeExecutor(clk)
    srv = Server(ex, hbm_budget=1e12, slots=2, max_pack=1, large_slots=1, large_n=200, clock=clk)
    for i in range(3):
        srv.submit(_req(i, nat=10))
    srv.pump()
    assert sorted(slot for _, slot, _ in ex.launched) == [0, 1]  # no large request queued


def test_latency_summary_and_poisson_stream():
    a = poisson_requests(50, 2000.0, seed=4, nat_range=(8, 20))
    b = poisson_requests(50, 2000.0, seed=4, nat_range=(8, 20))
    assert [r.arrival for r in a] == [r.arrival for r in b]
    assert all(np.array_equal(x.numbers, y.numbers) for x, y in zip(a, b))
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) > 0)
    # mean inter-arrival of a rate-2000 stream is 0.5 ms (loose statistical bound)
    assert 0.2e-3 < np.diff(arr).mean() < 1.0e-3
    assert {r.method for r in a} <= {"gfn1", "gfn2"}
    clk = FakeClock()
    ex = FakeExecutor(clk)
    srv = Server(ex, slots=2, max_pack=4, clock=clk)
    for r in a[:8]:
        srv.submit(r)
    out = []
    while not srv.idle:
        out += srv.pump()
        clk.t += 0.001
    s = latency_summary(out)
    assert s["ok"] == 8 and s["p50_ms"] <= s["p99_ms"] <= s["max_ms"]


@pytest.mark.gpu
def test_result_same_alone_and_in_mix():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs CUDA")
    from dxtb_gb300.serving import CudaExecutor

    reqs = poisson_requests(12, 2000.0, seed=7, nat_range=(8, 40))
    # alone: one request per pack, one pack at a time
    ex1 = CudaExecutor(slots=1)
    srv1 = Server(ex1, slots=1, max_pack=1)
    for r in reqs:
        srv1.submit(r)
    alone = {}
    while not srv1.idle:
        for x in srv1.pump():
            alone[x.rid] = x
    # in a mix: everything arrives at once, several packs in flight
    ex2 = CudaExecutor(slots=4)
    srv2 = Server(ex2, slots=4, max_pack=4)
    for r in reqs:
        srv2.submit(r)
    mix = {}
    while not srv2.idle:
        for x in srv2.pump():
            mix[x.rid] = x
    assert srv2.stats.max_inflight > 1
    assert sorted(alone) == sorted(mix) == list(range(len(reqs)))
    for rid in alone:
        a, m = alone[rid], mix[rid]
        assert a.status == 0 and m.status == 0
        assert abs(a.energy - m.energy) <= 1e-8
        assert np.abs(a.forces - m.forces).max() <= 1e-6
        assert a.pack_size == 1


@pytest.mark.gpu
def test_served_results_match_oracle():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs CUDA")
    from dxtb_gb300.serving import CudaExecutor
    from oracle import xtb_oracle as O

    reqs = poisson_requests(4, 2000.0, seed=11, nat_range=(8, 14))
    srv = Server(CudaExecutor(slots=2), slots=2, max_pack=2)
    out = {x.rid: x for x in srv.serve(reqs)}
    for r in reqs:
        ref = O.singlepoint(r.method, r.numbers, r.positions, grad=True, tol=1e-12)
        x = out[r.rid]
        assert x.status == 0
        assert abs(x.energy - ref.energy) <= 1e-8
        assert np.abs(x.forces + ref.extra["gradient"].numpy()).max() <= 1e-6
