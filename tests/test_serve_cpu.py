"""Scheduling logic of the serving loop (lbm/serve.py) with a simulated
backend and clock: admission in arrival order within the HBM budget, every
request advanced by exactly its step count, ticks that never overshoot a
case, and the statistics.  No GPU."""
from dataclasses import dataclass

import pytest

from lbm.serve import Request, poisson_arrivals, serve, serve_sequential


@dataclass
class Case:
    grid: tuple
    steps: int

    @property
    def nodes(self):
        return self.grid[0] * self.grid[1] * self.grid[2]


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 0.0)


class Solver:
    def __init__(self, case):
        self.case = case
        self.steps = 0
        self.open = True


class FakeBackend:
    """Per step, a batch costs (sum of its nodes) / rate seconds of simulated time."""

    def __init__(self, clock, rate=1e9, bytes_per_node=200):
        self.clock, self.rate, self.bpn = clock, rate, bytes_per_node
        self.resident = []
        self.peak_bytes = 0
        self.ticks = []

    def footprint(self, case):
        return case.nodes * self.bpn

    def build(self, case):
        s = Solver(case)
        self.resident.append(s)
        self.peak_bytes = max(self.peak_bytes, sum(self.footprint(x.case) for x in self.resident if x.open))
        return s

    def batch(self, solvers):
        backend = self

        class B:
            def run(self, n):
                assert all(s.open for s in solvers)
                for s in solvers:
                    s.steps += n
                    assert s.steps <= s.case.steps, "a case stepped past its step count"
                backend.ticks.append((n, len(solvers)))
                backend.clock.t += n * sum(s.case.nodes for s in solvers) / backend.rate

            def close(self):
                pass

        return B()

    def run_alone(self, solver, n):
        solver.steps += n
        self.clock.t += n * solver.case.nodes / self.rate

    def finish(self, solver):
        solver.open = False
        return {"steps": solver.steps}, None

    def sync(self):
        pass


def _requests(n=12, seed=3):
    arr = poisson_arrivals(n, rate=4.0, seed=seed)
    grids = [(64, 64, 48), (96, 96, 64), (128, 128, 96)]
    return [Request(i, Case(grids[i % 3], 200 + 150 * (i % 4)), a) for i, a in enumerate(arr)]


def test_poisson_arrivals_are_increasing_and_seeded():
    a = poisson_arrivals(50, 4.0, 7)
    assert a == sorted(a) and a == poisson_arrivals(50, 4.0, 7)
    assert 5.0 < a[-1] < 25.0  # mean gap 0.25 s


@pytest.mark.parametrize("budget_nodes", [10 ** 9, 2_500_000])
def test_every_request_served_exactly_within_budget(budget_nodes):
    clk = Clock()
    be = FakeBackend(clk)
    reqs = _requests()
    res, st = serve(reqs, be, budget_nodes * be.bpn, tick=64, clock=clk, sleep=clk.sleep)
    assert sorted(r.rid for r in res) == [r.rid for r in reqs]
    for r in res:
        assert r.measure["steps"] == r.steps
        assert r.arrival <= r.admitted <= r.finished
    assert be.peak_bytes <= budget_nodes * be.bpn
    assert all(n <= 64 for n, _ in be.ticks)
    assert st["requests"] == len(reqs) and st["p50_s"] <= st["p99_s"] and st["mlups"] > 0


def test_tight_budget_admits_in_arrival_order():
    clk = Clock()
    be = FakeBackend(clk)
    reqs = _requests()
    res, _ = serve(reqs, be, 1_600_000 * be.bpn, tick=64, clock=clk, sleep=clk.sleep)
    by_rid = sorted(res, key=lambda r: r.rid)
    for a, b in zip(by_rid, by_rid[1:]):
        assert a.admitted <= b.admitted


def test_oversized_request_is_rejected():
    clk = Clock()
    be = FakeBackend(clk)
    with pytest.raises(ValueError):
        serve([Request(0, Case((128, 128, 128), 10), 0.0)], be, 1000, clock=clk, sleep=clk.sleep)


def test_batching_never_takes_longer_than_sequential():
    """With a batch cost linear in nodes the batched loop finishes the stream
    no later than one-at-a-time (it overlaps requests that arrive while
    others run); its latencies differ (processor sharing, not FIFO)."""
    reqs = _requests()
    c1 = Clock()
    res_b, st_b = serve(reqs, FakeBackend(c1), 10 ** 12, tick=64, clock=c1, sleep=c1.sleep)
    c2 = Clock()
    res_s, st_s = serve_sequential(reqs, FakeBackend(c2), clock=c2, sleep=c2.sleep)
    assert len(res_b) == len(res_s)
    assert st_b["wall_s"] <= st_s["wall_s"] + 1e-9


def test_slots_cap_the_number_of_resident_cases():
    clk = Clock()
    be = FakeBackend(clk)
    reqs = _requests()
    res, _ = serve(reqs, be, 10 ** 12, tick=64, max_slots=2, clock=clk, sleep=clk.sleep)
    assert len(res) == len(reqs)
    assert max(k for _, k in be.ticks) <= 2


def test_background_setup_serves_every_request():
    clk = Clock()
    be = FakeBackend(clk)
    reqs = _requests()
    res, st = serve(reqs, be, 10 ** 12, tick=64, builders=2, clock=clk, sleep=clk.sleep)
    assert sorted(r.rid for r in res) == [r.rid for r in reqs]
    assert all(r.measure["steps"] == r.steps for r in res)


def test_shortest_remaining_work_first():
    """saturate_nodes: each tick steps the cases with the least remaining work
    until their nodes reach the threshold; every request is still served
    exactly, the GPU time is the same, and short requests finish sooner."""
    reqs = _requests(n=16, seed=5)
    c0 = Clock()
    ps, st_ps = serve(reqs, FakeBackend(c0), budget_bytes=10 ** 12, tick=50, clock=c0, sleep=c0.sleep)
    c1 = Clock()
    b1 = FakeBackend(c1)
    sr, st_sr = serve(reqs, b1, budget_bytes=10 ** 12, tick=50, saturate_nodes=400_000, clock=c1, sleep=c1.sleep)
    assert sorted(r.rid for r in sr) == list(range(len(reqs)))
    for r in sr:
        assert r.measure["steps"] == r.steps
    assert st_sr["wall_s"] == pytest.approx(st_ps["wall_s"], rel=1e-9)
    assert st_sr["mean_s"] < st_ps["mean_s"] and st_sr["p50_s"] <= st_ps["p50_s"]
    # a tick with several resident cases steps only some of them
    assert any(k < max(kk for _, kk in b1.ticks) for _, k in b1.ticks)


def test_select_order():
    from lbm.serve import _select

    class R:
        def __init__(self, nodes):
            self.case = Case((nodes, 1, 1), 0)

    active = {0: [R(100), None, 50], 1: [R(10), None, 100], 2: [R(1000), None, 1], 3: [R(10), None, 10]}
    # remaining work: 0 -> 5000, 1 -> 1000, 2 -> 1000, 3 -> 100
    assert _select(active, None) == (0, 1, 2, 3)
    assert _select(active, 5) == (3,)
    assert _select(active, 15) == (1, 3)
    assert _select(active, 1015) == (1, 2, 3)
    assert _select(active, 10 ** 9) == (0, 1, 2, 3)
