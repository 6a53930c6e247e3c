"""Serving loop for droplet-impact requests: continuous batching on one GPU.

Requests (an ``ImpactCase`` and an arrival time) are admitted in arrival
order as soon as they have arrived and their device footprint fits in the
HBM budget next to the cases already resident.  Resident cases advance
together in ticks of batched steps (``AllenCahnBatch``: one launch of each
step kernel per step for all of them).  A tick is never longer than the
fewest steps any resident case still needs, so a case stops exactly at its
step count.  Finished cases are measured and freed at the end of a tick, and
requests that arrived in the meantime are admitted before the next tick.  A
case's results do not depend on what it shares the GPU with: the batch
keeps every case's arithmetic and reductions separate.

Reported per request: arrival, admission and completion times (seconds from
the start of ``serve``) and the spread diagnostics of the final phi; overall:
p50 / p99 time to completion and aggregate MLUPS (node updates of all
requests / wall time).  ``serve_sequential`` runs the same request stream
through the plain one-case-at-a-time path for comparison.

A request that fails (larger than the budget, a set-up that raises, a
non-finite phi, cancelled, past its deadline) retires alone with
``Result.error`` set; the others continue.

The scheduling logic talks to the GPU through a backend (``GpuBackend``);
tests substitute a simulated one and inject the failures on the host.  The
reference has no serving loop.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Request:
    rid: int
    case: object          # ImpactCase (grid, steps, ...)
    arrival: float        # seconds after the start of serving
    deadline: float = None  # seconds after arrival by which it must finish (None: none)


@dataclass
class Result:
    rid: int
    arrival: float
    admitted: float
    finished: float
    steps: int            # steps taken (the request's count unless it failed)
    nodes: int
    measure: dict = field(default_factory=dict)
    phi: object = None    # final phi on the host, if kept
    error: str = None     # why the request was retired without a result (None: served)

    @property
    def latency(self):
        return self.finished - self.arrival


def poisson_arrivals(n, rate, seed):
    """Arrival times of n requests of a Poisson process with `rate` per second."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n)).tolist()


class GpuBackend:
    """Cases as AllenCahnSolver objects on the current CUDA device."""

    def __init__(self, dtype, device="cuda", keep_phi=False):
        import torch
        self.torch = torch
        self.dtype = dtype
        self.device = device
        self.keep_phi = keep_phi

    def footprint(self, case):
        from .batch import footprint
        return footprint(case.grid, self.dtype)

    def build(self, case):
        from .impact import build_impact_case
        return build_impact_case(case, self.dtype, self.device)

    def batch(self, solvers):
        from .batch import AllenCahnBatch
        return AllenCahnBatch(solvers)

    def run_alone(self, solver, nsteps):
        solver.run(nsteps)

    def finish(self, solver):
        m = solver.measure()
        phi = solver.phi.cpu().numpy() if self.keep_phi else None
        solver.close()
        return m, phi

    def healthy(self, solver):
        """False once the case's status word reports a non-finite sum of phi
        (lbm_status: a small synchronous copy, after the tick's steps)."""
        from . import _native as nat
        return not (solver.status() & nat.STATUS_NAN)

    def discard(self, solver):
        solver.close()

    def sync(self):
        self.torch.cuda.synchronize()


def _stats(results, wall):
    ok = [r for r in results if r.error is None]
    lat = np.array([r.latency for r in ok]) if ok else np.zeros(1)
    updates = float(sum(r.nodes * r.steps for r in results))
    return {"requests": len(results), "errors": len(results) - len(ok), "wall_s": wall,
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "mlups": updates / wall / 1e6 if wall > 0 else 0.0}


def _select(active, saturate_nodes):
    """Resident cases to step in the next tick.  saturate_nodes None: all of
    them (processor sharing).  Otherwise shortest remaining work first
    (nodes x remaining steps, then request id): cases in that order until
    their nodes reach saturate_nodes, so that the GPU stays busy while the
    cases closest to completion go first."""
    keys = sorted(active)
    if saturate_nodes is None:
        return tuple(keys)
    order = sorted(keys, key=lambda k: (active[k][0].case.nodes * active[k][2], k))
    picked, nodes = [], 0
    for k in order:
        picked.append(k)
        nodes += active[k][0].case.nodes
        if nodes >= saturate_nodes:
            break
    return tuple(sorted(picked))


def serve(requests, backend, budget_bytes, tick=100, max_slots=None, builders=0, saturate_nodes=None,
          cancelled=None, clock=time.perf_counter, sleep=time.sleep):
    """Continuous batching of `requests` under an HBM budget and at most
    `max_slots` resident cases (None: no limit).  With builders > 0, admitted
    cases are set up (inputs, geometry, init) by that many host threads while
    the GPU keeps stepping the resident ones; their footprint counts against
    the budget from the start of the set-up.  saturate_nodes (None: every
    resident case advances in every tick) selects shortest-remaining-work-first
    ticks that step only the resident cases closest to completion, at least
    that many nodes of them (see _select).

    A failing request retires with ``Result.error`` set and its memory freed,
    without disturbing the others: a request larger than the whole budget (at
    its arrival), a set-up that raises (``build failed: ...``), a case whose
    status word reports a non-finite phi after a tick (``non-finite phi``), a
    request for which ``cancelled(rid)`` turns true (``cancelled``) and one
    still unfinished past its ``deadline`` (``deadline exceeded``); the last
    three are checked between ticks.  Returns (results in completion order,
    stats)."""
    from concurrent.futures import ThreadPoolExecutor
    pending = sorted(requests, key=lambda r: r.arrival)
    pool = ThreadPoolExecutor(max_workers=builders) if builders > 0 else None
    building = {}      # rid -> (future, request, bytes)
    active = {}        # rid -> [request, solver, remaining steps, bytes, admitted]
    used = 0
    batch = None
    members = ()
    results = []
    t0 = clock()

    def fail(r, adm, steps, why):
        results.append(Result(r.rid, r.arrival, adm, clock() - t0, steps, r.case.nodes, error=why))

    def overdue(r, now):
        return (r.deadline is not None and now > r.arrival + r.deadline) or (cancelled is not None and cancelled(r.rid))

    try:
        while pending or active or building:
            now = clock() - t0
            # requests that can never fit are refused on arrival
            while pending and pending[0].arrival <= now and backend.footprint(pending[0].case) > budget_bytes:
                r = pending.pop(0)
                fail(r, now, 0, "exceeds the HBM budget")
            # admit, in arrival order, what has arrived and fits
            while (pending and pending[0].arrival <= now
                   and used + backend.footprint(pending[0].case) <= budget_bytes
                   and (max_slots is None or len(active) + len(building) < max_slots)):
                r = pending.pop(0)
                b = backend.footprint(r.case)
                used += b
                if pool is None:
                    try:
                        active[r.rid] = [r, backend.build(r.case), int(r.case.steps), b, clock() - t0]
                    except Exception as e:  # a bad request fails alone
                        used -= b
                        fail(r, clock() - t0, 0, f"build failed: {e}")
                else:
                    building[r.rid] = (pool.submit(backend.build, r.case), r, b)
            for rid in [k for k, v in building.items() if v[0].done()]:
                fut, r, b = building.pop(rid)
                try:
                    active[rid] = [r, fut.result(), int(r.case.steps), b, clock() - t0]
                except Exception as e:
                    used -= b
                    fail(r, clock() - t0, 0, f"build failed: {e}")
            # cancelled or overdue requests leave between ticks
            now = clock() - t0
            gone = [k for k, a in active.items() if overdue(a[0], now)]
            if gone:
                if batch is not None:
                    batch.close()
                    batch, members = None, ()
                for k in gone:
                    r, solver, rem, b, adm = active.pop(k)
                    backend.discard(solver)
                    used -= b
                    fail(r, adm, int(r.case.steps) - rem, "cancelled" if cancelled is not None and cancelled(r.rid)
                         else "deadline exceeded")
            if not active:
                if building:
                    sleep(0.002)  # a set-up is in progress
                elif pending:
                    sleep(max(0.0, pending[0].arrival - (clock() - t0)))  # idle until the next arrival
                continue
            key = _select(active, saturate_nodes)
            if key != members:
                if batch is not None:
                    batch.close()
                batch = backend.batch([active[k][1] for k in key])
                members = key
            n = min(tick, min(active[k][2] for k in key))
            batch.run(n)
            done, bad = [], []
            for k in key:
                a = active[k]
                a[2] -= n
                if not backend.healthy(a[1]):
                    bad.append(k)
                elif a[2] == 0:
                    done.append(k)
            if bad:
                batch.close()
                batch, members = None, ()
                for k in bad:
                    r, solver, rem, b, adm = active.pop(k)
                    backend.discard(solver)
                    used -= b
                    fail(r, adm, int(r.case.steps) - rem, "non-finite phi")
            if done:
                # retire: measuring waits for the batch's steps to finish
                batch.close()
                batch, members = None, ()
                for k in done:
                    r, solver, _, b, adm = active.pop(k)
                    m, phi = backend.finish(solver)
                    results.append(Result(r.rid, r.arrival, adm, clock() - t0, int(r.case.steps), r.case.nodes, m,
                                          phi))
                    used -= b
    finally:
        if batch is not None:
            batch.close()
        if pool is not None:
            pool.shutdown(wait=True)
    backend.sync()
    return results, _stats(results, clock() - t0)


def serve_sequential(requests, backend, clock=time.perf_counter, sleep=time.sleep):
    """The same request stream through the plain path: one case at a time,
    in arrival order, each run to completion before the next is built."""
    pending = sorted(requests, key=lambda r: r.arrival)
    results = []
    t0 = clock()
    for r in pending:
        wait = r.arrival - (clock() - t0)
        if wait > 0:
            sleep(wait)
        adm = clock() - t0
        solver = backend.build(r.case)
        backend.run_alone(solver, int(r.case.steps))
        m, phi = backend.finish(solver)
        results.append(Result(r.rid, r.arrival, adm, clock() - t0, int(r.case.steps), r.case.nodes, m, phi))
    backend.sync()
    return results, _stats(results, clock() - t0)
