"""The serving loop on the GPU: requests that arrive while others run are
admitted into the running batch, and every request's final phi is exactly
the phi of the same request run alone."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from lbm.impact import ImpactCase  # noqa: E402
from lbm.serve import GpuBackend, Request, serve, serve_sequential  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return built_lib


def _requests():
    cases = [
        ImpactCase(0, (24, 24, 20), "flat", 5.0, 120.0, -0.03, 40),
        ImpactCase(1, (32, 28, 24), "ridge", 6.0, 150.0, -0.05, 25),
        ImpactCase(2, (28, 28, 28), "convex", 5.5, 100.0, -0.04, 60),
        ImpactCase(3, (30, 26, 22), "concave", 5.0, 162.0, -0.06, 33),
        ImpactCase(4, (26, 30, 24), "ridge", 6.5, 135.0, -0.07, 17),
    ]
    # staggered arrivals: the later ones arrive while the first are running
    return [Request(i, c, 0.02 * i) for i, c in enumerate(cases)]


@pytest.mark.parametrize("dtype,saturate", [(torch.float32, None), (torch.float16, None),
                                             (torch.float16, 30_000)])
def test_served_results_equal_alone(dtype, saturate):
    """Processor sharing, and shortest-remaining-work-first ticks (saturate:
    cases paused while others run), give every request the result it has
    alone."""
    reqs = _requests()
    mix, st = serve(reqs, GpuBackend(dtype, keep_phi=True), budget_bytes=2 * 10 ** 9, tick=8,
                    saturate_nodes=saturate)
    alone, _ = serve_sequential(reqs, GpuBackend(dtype, keep_phi=True))
    assert len(mix) == len(reqs) == len(alone)
    a = {r.rid: r for r in alone}
    for r in mix:
        assert r.steps == a[r.rid].steps
        assert np.array_equal(r.phi, a[r.rid].phi), r.rid
        assert r.measure == a[r.rid].measure
    assert st["p50_s"] <= st["p99_s"] and st["mlups"] > 0


def test_budget_limits_resident_cases():
    """A budget that holds one case at a time still serves every request."""
    from lbm.batch import footprint
    reqs = _requests()
    one = max(footprint(r.case.grid, torch.float32) for r in reqs)
    mix, _ = serve(reqs, GpuBackend(torch.float32), budget_bytes=one, tick=16)
    assert sorted(r.rid for r in mix) == list(range(len(reqs)))
    # one at a time: admission of each waits for the previous completion
    fin = sorted(mix, key=lambda r: r.finished)
    for prev, nxt in zip(fin, fin[1:]):
        assert nxt.admitted >= prev.finished - 1e-6
