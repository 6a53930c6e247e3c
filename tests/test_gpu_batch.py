"""Batched stepping (lbm_batch_*, AllenCahnBatch) against stepping each case
alone: bit-identical phi, u and populations, for float32 (mixing tau_f = 1
cases with a tau_h = 0.57 case, i.e. both update kernels in one batch) and
for the half-precision deviation storage; the batch autotuner leaves the
state unchanged."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from lbm.impact import ImpactCase, impact_config, impact_inputs  # noqa: E402

CASES = [
    ImpactCase(0, (24, 24, 20), "flat", 5.0, 120.0, -0.03, 0),
    ImpactCase(1, (32, 28, 24), "ridge", 6.0, 150.0, -0.05, 0),
    ImpactCase(2, (28, 28, 28), "convex", 5.5, 100.0, -0.04, 0),
    ImpactCase(3, (30, 26, 22), "concave", 5.0, 162.0, -0.06, 0),
]


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return built_lib


def _solver(case, dtype, tau_h=None):
    from lbm.fe_ac_solver import AllenCahnSolver
    cfg = impact_config(case, "cuda")
    if tau_h is not None:
        cfg.tau_h = tau_h
    solid, frac, C, u = impact_inputs(case)
    s = AllenCahnSolver(cfg, dtype=dtype, geo_amplification=1.5, geometric_wetting=True)
    s.set_solid(solid, frac)
    s.init_fields(C, u)
    return s


def _state(s):
    phi, u = s.fields("phi", "u")
    return phi.clone(), u.clone(), s.f.clone(), s.g.clone()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float16])
@pytest.mark.parametrize("steps", [[7], [1, 4, 3]])
def test_batch_matches_cases_alone(dtype, steps):
    from lbm.batch import AllenCahnBatch
    taus = [None, 0.57, None, None]
    alone = [_solver(c, dtype, t) for c, t in zip(CASES, taus)]
    for s in alone:
        s.run(sum(steps))
    mixed = [_solver(c, dtype, t) for c, t in zip(CASES, taus)]
    b = AllenCahnBatch(mixed)
    for n in steps:
        b.run(n)
    torch.cuda.synchronize()
    for a, m in zip(alone, mixed):
        for x, y in zip(_state(a), _state(m)):
            assert torch.equal(x, y)
        assert a.scalars() == m.scalars()
    b.close()


def test_batch_autotune_leaves_state_unchanged():
    from lbm.batch import AllenCahnBatch
    a = [_solver(c, torch.float32) for c in CASES]
    m = [_solver(c, torch.float32) for c in CASES]
    ba, bm = AllenCahnBatch(a), AllenCahnBatch(m)
    ba.run(3)
    bm.run(3)
    per, ms = bm.autotune(reps=2)
    assert per in (1, 2, 4, 8, 12, 16, 24, 32) and ms > 0
    ba.run(5)
    bm.run(5)
    for x, y in zip(a, m):
        assert torch.equal(x.phi, y.phi) and torch.equal(x.u, y.u)


def test_batch_measure_per_case():
    from lbm.batch import AllenCahnBatch
    m = [_solver(c, torch.float32) for c in CASES]
    b = AllenCahnBatch(m)
    b.run(10)
    for s in m:
        d = s.measure()
        assert d["count"] > 0 and not d["has_nan"]
        assert d["volume"] == pytest.approx(s.scalars()[0], rel=1e-2)


def test_injected_case_in_batch_matches_alone():
    """A case injected between batch calls continues bit-identically to the
    same case stepped alone."""
    from lbm.batch import AllenCahnBatch
    a = [_solver(c, torch.float32) for c in CASES[:3]]
    m = [_solver(c, torch.float32) for c in CASES[:3]]
    for s in a:
        s.run(4)
    b = AllenCahnBatch(m)
    b.run(4)
    for s in (a[1], m[1]):
        s.inject_droplet((16.0, 14.0, 19.0), 4.0, 4.0, u_impact=(0.0, 0.01, -0.02))
    for s in a:
        s.run(5)
    b.run(5)
    for x, y in zip(a, m):
        for p, q in zip(_state(x), _state(y)):
            assert torch.equal(p, q)


def test_batch_with_amplification_field():
    """A case with a per-node amplification field gives the same results alone
    and in a batch (its descriptor carries the field)."""
    from lbm.batch import AllenCahnBatch
    from lbm.fe_ac_solver import AllenCahnSolver

    def make(case, field):
        cfg = impact_config(case, "cuda")
        solid, frac, C, u = impact_inputs(case)
        amp = 1.5
        if field:
            nx, ny, nz = case.grid
            amp = np.broadcast_to(np.linspace(0.5, 2.5, nx, dtype=np.float32)[:, None, None], (nx, ny, nz)).copy()
        s = AllenCahnSolver(cfg, dtype=torch.float32, geo_amplification=amp, geometric_wetting=True)
        s.set_solid(solid, frac)
        s.init_fields(C, u)
        return s

    alone = [make(CASES[1], True), make(CASES[3], False)]
    for s in alone:
        s.run(6)
    mixed = [make(CASES[1], True), make(CASES[3], False)]
    b = AllenCahnBatch(mixed)
    b.run(6)
    for a, m in zip(alone, mixed):
        for x, y in zip(_state(a), _state(m)):
            assert torch.equal(x, y)
    # the field changes the result (it is not ignored)
    plain = make(CASES[1], False)
    plain.run(6)
    assert not torch.equal(plain.phi, alone[0].phi)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float16])
def test_launch_shapes_give_identical_results(dtype):
    """Every phi-kernel work size and update-kernel block the autotuners pick
    from gives the same bits."""
    ref = _solver(CASES[1], dtype)
    ref.run(6)
    for per, bs in ((4, 128), (12, 256), (32, 128)):
        s = _solver(CASES[1], dtype)
        s.set_launch_shape(per, bs)
        assert s.launch_shape() == (per, bs)
        s.run(6)
        for x, y in zip(_state(ref), _state(s)):
            assert torch.equal(x, y), (per, bs)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float16])
def test_cooperative_single_launch_matches_two_launches(dtype):
    """The batched step as one cooperative launch (phi work, grid barrier,
    update work) gives the two-launch step's results, mixing tau_f == 1 cases
    with a tau_h = 0.57 case."""
    from lbm.batch import AllenCahnBatch
    taus = [None, 0.57, None, None]
    two = [_solver(c, dtype, t) for c, t in zip(CASES, taus)]
    one = [_solver(c, dtype, t) for c, t in zip(CASES, taus)]
    b2, b1 = AllenCahnBatch(two), AllenCahnBatch(one)
    b1.set_cooperative(True)
    for n in (1, 5, 2):
        b2.run(n)
        b1.run(n)
    torch.cuda.synchronize()
    for a, m in zip(two, one):
        for x, y in zip(_state(a), _state(m)):
            assert torch.equal(x, y)
    b1.close()
    b2.close()
