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
        self.nan_at = None  # injected fault: the status word reports NaN from this step on


class FakeBackend:
    """Per step, a batch costs (sum of its nodes) / rate seconds of simulated time."""

    def __init__(self, clock, rate=1e9, bytes_per_node=200, fail_build=(), nan_at=None):
        self.clock, self.rate, self.bpn = clock, rate, bytes_per_node
        self.resident = []
        self.peak_bytes = 0
        self.ticks = []
        self.fail_build = set(fail_build)  # cases (by step count) whose set-up raises
        self.nan_at = dict(nan_at or {})    # step count -> step at which NaN appears

    def footprint(self, case):
        return case.nodes * self.bpn

    def build(self, case):
        if case.steps in self.fail_build:
            raise RuntimeError("injected set-up failure")
        s = Solver(case)
        s.nan_at = self.nan_at.get(case.steps)
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

    def healthy(self, solver):
        return solver.nan_at is None or solver.steps < solver.nan_at

    def discard(self, solver):
        solver.open = False

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


def test_oversized_request_is_rejected_alone():
    """A request larger than the whole budget retires with an error on arrival;
    the others are served."""
    clk = Clock()
    be = FakeBackend(clk)
    reqs = [Request(0, Case((64, 64, 48), 100), 0.0), Request(1, Case((512, 512, 512), 10), 0.1),
            Request(2, Case((64, 64, 48), 120), 0.2)]
    res, st = serve(reqs, be, 64 * 64 * 48 * be.bpn * 2, tick=32, clock=clk, sleep=clk.sleep)
    by = {r.rid: r for r in res}
    assert by[1].error == "exceeds the HBM budget" and by[1].steps == 0
    assert by[0].error is None and by[2].error is None
    assert by[0].measure["steps"] == 100 and by[2].measure["steps"] == 120
    assert st["errors"] == 1


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



@pytest.mark.parametrize("builders", [0, 2])
def test_failed_setup_retires_alone(builders):
    """A set-up that raises retires that request with an error and frees its
    budget; every other request is served exactly."""
    reqs = _requests()
    bad = reqs[4].case.steps  # cases with this step count fail to build
    clk = Clock()
    be = FakeBackend(clk, fail_build=[bad])
    res, st = serve(reqs, be, 10 ** 12, tick=64, builders=builders, clock=clk, sleep=clk.sleep)
    assert sorted(r.rid for r in res) == [r.rid for r in reqs]
    for r in res:
        req = reqs[r.rid]
        if req.case.steps == bad:
            assert r.error.startswith("build failed") and r.steps == 0
        else:
            assert r.error is None and r.measure["steps"] == req.case.steps
    assert st["errors"] == sum(1 for r in reqs if r.case.steps == bad)


def test_non_finite_case_retires_alone():
    """A case whose status word reports NaN after a tick leaves the batch with
    an error; the cases it shared ticks with continue and finish exactly."""
    reqs = _requests()
    bad = reqs[1].case.steps
    clk = Clock()
    be = FakeBackend(clk, nan_at={bad: 100})
    res, st = serve(reqs, be, 10 ** 12, tick=64, clock=clk, sleep=clk.sleep)
    for r in res:
        req = reqs[r.rid]
        if req.case.steps == bad:
            assert r.error == "non-finite phi" and 100 <= r.steps < req.case.steps
        else:
            assert r.error is None and r.measure["steps"] == req.case.steps
    assert st["errors"] >= 1


def test_cancel_and_deadline():
    """A request that is cancelled, or still running past its deadline, leaves
    between ticks with an error; the others are served exactly."""
    reqs = _requests()
    reqs[2] = Request(reqs[2].rid, reqs[2].case, reqs[2].arrival, deadline=0.001)
    clk = Clock()
    be = FakeBackend(clk)
    res, st = serve(reqs, be, 10 ** 12, tick=16, cancelled=lambda rid: rid == 5, clock=clk, sleep=clk.sleep)
    by = {r.rid: r for r in res}
    assert by[5].error == "cancelled" and by[5].steps < reqs[5].case.steps
    assert by[2].error == "deadline exceeded" and by[2].steps < reqs[2].case.steps
    for rid, r in by.items():
        if rid not in (2, 5):
            assert r.error is None and r.measure["steps"] == reqs[rid].case.steps
    assert st["errors"] == 2
