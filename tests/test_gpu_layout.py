"""The paired storage layout (nodes x and x + nx/2 of the same (y, z) in one
word of every state array, stepped one pair per thread with packed loads,
stores and f32x2 arithmetic; an option of 3-D float32 / float16 grids with
even nx) against the default linear layout (one element per node, stepped one
node per thread) on the same inputs, through the C ABI: the same fields within
a few float32 ulps over every golden case's solver options and equally close
to the float64 run after 40 steps, the same fields read back in the reference
layout, batches mixing both layouts equal to their cases alone bit for bit,
and the layout's argument checks."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from _cases import CASES, config, inputs  # noqa: E402

# 3-D golden cases (even nx): every wetting mode, partial nodes, discrete
# normals, per-node alpha, direct wetting, the gradient-of-mu sources, Liang
# forcing with gravity, tau_l != tau_g
LAYOUT_CASES = [n for n, c in CASES.items() if c["grid"][2] > 1 and c["grid"][0] % 2 == 0 and "long" not in n
                and not n.startswith("cfg1")]


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")


def _solver(name, dtype, paired, tau_h=None):
    from lbm.fe_ac_solver import AllenCahnSolver
    case = CASES[name]
    solid, frac, C, u = inputs(case)
    cfg = config(case, "cuda")
    if tau_h is not None:
        cfg.tau_h = tau_h
    s = AllenCahnSolver(cfg, dtype=dtype, **case["kw"])
    s.set_solid(solid, frac)
    s.set_layout(paired)
    s.init_fields(C, u)
    assert s.paired == paired
    return s


def _maxdiff(a, b):
    return (a.double() - b.double()).abs().max().item()


def _f64(name, tau_h=None):
    return _solver(name, torch.float64, False, tau_h)


@pytest.mark.parametrize("name", LAYOUT_CASES)
def test_paired_matches_linear(name):
    """Float32: phi within 2e-6 after 1 and 5 steps (the bound of the parity
    tests against the reference), u and P alike; after 40 steps both layouts
    as close to the float64 run as each other (rounding differences grow at
    the same rate in either: the paired error at most twice the linear one,
    or 1e-5), populations read back alike and the same spread extents."""
    if CASES[name]["kw"].get("interface_mode") == "cahn-hilliard" or CASES[name]["kw"].get("mu_drive", 0) > 0:
        pytest.skip("gradient-of-mu modes: covered by test_paired_matches_linear_gradient_mu")
    a = _solver(name, torch.float32, True)
    b = _solver(name, torch.float32, False)
    r = _f64(name)
    for n in (1, 4):
        a.run(n)
        b.run(n)
        pa, ua, Pa = a.fields("phi", "u", "P")
        pb, ub, Pb = b.fields("phi", "u", "P")
        assert _maxdiff(pa, pb) <= 2e-6, (n, _maxdiff(pa, pb))
        assert _maxdiff(ua, ub) <= 2e-5
        assert _maxdiff(Pa, Pb) <= 2e-5
    a.run(35)
    b.run(35)
    r.run(40)
    da, db = _maxdiff(a.phi, r.phi), _maxdiff(b.phi, r.phi)
    assert da <= max(2 * db, 1e-5), (da, db)
    assert _maxdiff(a.u, r.u) <= max(2 * _maxdiff(b.u, r.u), 1e-4)
    assert a.status() == 0 and b.status() == 0
    ma, mb = a.measure(), b.measure()
    for key in ("Dx", "Dy", "Dz"):
        assert abs(ma[key] - mb[key]) <= 1, key
    assert ma["volume"] == pytest.approx(mb["volume"], rel=1e-5)


def _close_to_f64(a, b, r, steps):
    for n in (1, 4):
        a.run(n)
        b.run(n)
        assert _maxdiff(a.phi, b.phi) <= 2e-6, (n, _maxdiff(a.phi, b.phi))
        assert _maxdiff(a.u, b.u) <= 2e-5
    a.run(steps - 5)
    b.run(steps - 5)
    r.run(steps)
    da, db = _maxdiff(a.phi, r.phi), _maxdiff(b.phi, r.phi)
    assert da <= max(2 * db, 1e-5), (da, db)


@pytest.mark.parametrize("name", ["ch_flat_q120", "mudrive_ridge_l150"])
def test_paired_matches_linear_gradient_mu(name):
    _close_to_f64(_solver(name, torch.float32, True), _solver(name, torch.float32, False), _f64(name), 40)


def test_paired_matches_linear_tau_f_not_one():
    """tau_h = 0.57: the phase-field collision re-reads f (the second update kernel)."""
    _close_to_f64(_solver("ridge_l162", torch.float32, True, tau_h=0.57),
                  _solver("ridge_l162", torch.float32, False, tau_h=0.57), _f64("ridge_l162", tau_h=0.57), 20)


@pytest.mark.parametrize("name", ["ridge_l162", "convex_l150", "concave_q100_tau"])
def test_paired_matches_linear_half(name):
    """Half-precision deviation storage: both layouts equally close to the
    float64 run after 20 steps (the half form's own rounding dominates)."""
    a = _solver(name, torch.float16, True)
    b = _solver(name, torch.float16, False)
    r = _f64(name)
    a.run(20)
    b.run(20)
    r.run(20)
    da, db = _maxdiff(a.phi, r.phi), _maxdiff(b.phi, r.phi)
    assert da <= max(2 * db, 1e-4), (da, db)
    assert a.status() == 0 and b.status() == 0


def test_layout_defaults_and_checks():
    from lbm import _native as nat
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.fe_config import FEConfig
    for (nx, ny, nz), dt, allowed in (((24, 20, 16), torch.float32, True), ((24, 20, 16), torch.float16, True),
                                      ((24, 20, 16), torch.float64, False), ((25, 20, 16), torch.float32, False),
                                      ((24, 20, 1), torch.float32, False)):
        cfg = FEConfig(nx=nx, ny=ny, nz=nz, rho_l=1.0, rho_g=1.0 / 828.0, sigma=0.01, xi=4.0, tau_l=0.53,
                       tau_g=0.53, theta_eq=120.0, device="cuda")
        s = AllenCahnSolver(cfg, dtype=dt)
        assert not s.paired  # the linear layout is the default
        if allowed:
            s.set_layout(True)
            assert s.paired
        else:
            with pytest.raises(nat.LbmError):
                s.set_layout(True)
        s.set_layout(False)
        shape = (nx, ny) if nz == 1 else (nx, ny, nz)
        s.set_solid(np.zeros(shape, bool))
        s.init_fields(np.full(shape, 0.5, np.float32))
        with pytest.raises(nat.LbmError):  # after init_fields
            s.set_layout(False)
        s.close()


def test_odd_and_even_nx_grids_step():
    """An odd-nx grid in the linear layout and the next even grid in the
    paired layout both stay finite and conserve the corrected mass."""
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.impact import ImpactCase, impact_config, impact_inputs
    for grid in ((27, 26, 22), (28, 26, 22)):
        c = ImpactCase(5, grid, "ridge", 5.0, 140.0, -0.04, 0)
        solid, frac, C, u = impact_inputs(c)
        s = AllenCahnSolver(impact_config(c, "cuda"), dtype=torch.float32, geo_amplification=1.5,
                            geometric_wetting=True)
        s.set_solid(solid, frac)
        s.set_layout(grid[0] % 2 == 0)
        s.init_fields(C, u)
        s.run(30)
        m = s.measure()
        assert s.status() == 0 and not m["has_nan"]
        assert m["volume"] == pytest.approx(s.phi_mass_init, rel=1e-4)
        s.close()


def test_batch_mixing_layouts_matches_cases_alone():
    """A batch of paired and linear cases (both phi kernels and the update
    kernels of both layouts in one step) gives each case's results alone."""
    from lbm.batch import AllenCahnBatch
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.impact import ImpactCase, impact_config, impact_inputs
    cases = [(ImpactCase(0, (24, 24, 20), "flat", 5.0, 120.0, -0.03, 0), True, None),
             (ImpactCase(1, (32, 28, 24), "ridge", 6.0, 150.0, -0.05, 0), False, None),
             (ImpactCase(2, (27, 28, 28), "convex", 5.5, 100.0, -0.04, 0), False, 0.57),
             (ImpactCase(3, (30, 26, 22), "concave", 5.0, 162.0, -0.06, 0), True, 0.57)]

    def make(c, paired, tau_h):
        cfg = impact_config(c, "cuda")
        if tau_h is not None:
            cfg.tau_h = tau_h
        solid, frac, C, u = impact_inputs(c)
        s = AllenCahnSolver(cfg, dtype=torch.float32, geo_amplification=1.5, geometric_wetting=True)
        s.set_solid(solid, frac)
        if c.grid[0] % 2 == 0:
            s.set_layout(paired)
        s.init_fields(C, u)
        return s

    alone = [make(*c) for c in cases]
    for s in alone:
        s.run(9)
    mixed = [make(*c) for c in cases]
    b = AllenCahnBatch(mixed)
    b.run(1)
    b.run(8)
    torch.cuda.synchronize()
    for a, m in zip(alone, mixed):
        assert torch.equal(a.phi, m.phi) and torch.equal(a.u, m.u)
        assert torch.equal(a.f, m.f) and torch.equal(a.g, m.g)
    b.close()


def test_checkpoint_refuses_other_layout():
    a = _solver("ridge_l162", torch.float32, True)
    a.run(3)
    st = a.state_dict()
    b = _solver("ridge_l162", torch.float32, False)
    with pytest.raises(Exception):
        b.load_state_dict(st)
    c = _solver("ridge_l162", torch.float32, True)
    c.load_state_dict(st)
    a.run(4)
    c.run(4)
    assert torch.equal(a.phi, c.phi) and torch.equal(a.f, c.f)
