"""CUDA path against the reference (golden fixtures) and the numpy oracle,
through the C ABI (AllenCahnSolver -> liblbm_gb300.so).

Tolerances: float32 -- a few float ulps per step for the short runs (the
GPU contracts multiply-adds into FMAs and sums in a fixed order; torch's CPU
sum order differs), and the stated parity bound max|dphi| <= 1e-4, relative
L2 on u <= 1e-3 for the long runs; float64 -- 1e-12."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from _cases import CASES, all_cases, config, golden, inputs, rel_l2  # noqa: E402
from oracle.ac_oracle import OracleSolver, measure_spread  # noqa: E402

# float64: the stress tensor is formed from population moments minus the
# analytic equilibrium part (Pi - P cs2 - u u), whose cancellation costs a few
# more float64 ulps than the reference's per-population differences.
SHORT = {"float32": (3e-6, 5e-5, 1e-8, 2e-6, 1e-6), "float64": (1e-11, 1e-10, 1e-15, 1e-11, 1e-11)}


def _gpu(name, dn):
    from lbm.fe_ac_solver import AllenCahnSolver
    case = CASES[name]
    solid, frac, C, u = inputs(case)
    s = AllenCahnSolver(config(case, "cuda"), dtype=getattr(torch, dn), **case["kw"])
    s.set_solid(solid, frac)
    s.init_fields(C, u)
    return case, s


def _np(t):
    return t.detach().cpu().numpy()


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return built_lib


@pytest.mark.parametrize("name,dn", all_cases(long=False))
def test_init_and_geometry(name, dn):
    case, s = _gpu(name, dn)
    gd = golden(name, dn)
    if "is_boundary" in gd:
        assert np.array_equal(_np(s.wetting.is_boundary), gd["is_boundary"])
        assert np.array_equal(_np(s.wetting.wall_normal), gd["wall_normal"])
        assert np.array_equal(_np(s.wetting.wall_weight), gd["wall_weight"])
    assert np.array_equal(_np(s.phi), gd["init_phi"])
    assert np.abs(_np(s.mu_phi) - gd["init_mu"]).max() <= SHORT[dn][3]
    assert np.abs(_np(s.p) - gd["init_p"]).max() <= SHORT[dn][4]
    assert s.phi_mass_init == pytest.approx(float(gd["phi_mass_init"]), rel=1e-6 if dn == "float32" else 1e-13)
    if "init_f" in gd:
        assert np.abs(_np(s.f) - gd["init_f"]).max() <= 1e-7
        assert np.abs(_np(s.g) - gd["init_g"]).max() <= 1e-9


@pytest.mark.parametrize("name,dn", all_cases(long=False))
def test_steps_vs_reference_and_oracle(name, dn):
    case, s = _gpu(name, dn)
    gd = golden(name, dn)
    solid, frac, C, u = inputs(case)
    o = OracleSolver(config(case), dtype=np.dtype(dn), **case["kw"])
    o.set_solid(solid, frac)
    o.init_fields(C, u)
    tp, tu, tP, tmu, trho = SHORT[dn]
    ck = sorted(case["ckpt"])
    for k in range(1, ck[-1] + 1):
        s.step()
        o.step()
        if k in ck:
            phi, vel = _np(s.phi), _np(s.u)
            assert np.abs(phi - gd[f"s{k}_phi"]).max() <= tp, ("ref phi", k)
            assert rel_l2(vel, gd[f"s{k}_u"]) <= tu, ("ref u", k)
            assert np.abs(phi - o.phi).max() <= tp, ("oracle phi", k)
            assert rel_l2(vel, o.u) <= tu, ("oracle u", k)
            if f"s{k}_P" in gd:
                assert np.abs(_np(s.P) - gd[f"s{k}_P"]).max() <= tP
                assert np.abs(_np(s.p) - gd[f"s{k}_P"] / 3.0).max() <= tP
                assert np.abs(_np(s.mu_phi) - gd[f"s{k}_mu"]).max() <= tmu
                assert np.abs(_np(s.rho) - gd[f"s{k}_rho"]).max() <= trho
    # populations in the reference layout after the last step
    tf = 5e-7 if dn == "float32" else 1e-11
    assert np.abs(_np(s.f) - o.f).max() <= tf
    assert np.abs(_np(s.g) - o.g).max() <= tf


@pytest.mark.parametrize("tile", [(4, 4, 8), (6, 5, 7), (12, 12, 28)])
def test_results_independent_of_tiling(tile):
    """Tile shapes of the fused kernel give identical results (the sum of phi
    is an exact fixed-point sum, independent of the order of the partial
    sums); the fused kernel and the two-kernel step (the default) agree to a
    few float32 ulps (the compiler contracts multiply-adds differently in
    the two kernels)."""
    from lbm import _native as nat
    case, a = _gpu("ridge_l162", "float32")
    _, b = _gpu("ridge_l162", "float32")
    _, c = _gpu("ridge_l162", "float32")
    nat.check(b._lib.lbm_set_tile(b._h, *tile), "lbm_set_tile")
    nat.check(c._lib.lbm_set_tile(c._h, 5, 6, 9), "lbm_set_tile")
    a.run(20)
    b.run(20)
    c.run(20)
    assert torch.equal(b.phi, c.phi) and torch.equal(b.u, c.u)
    assert (a.phi - b.phi).abs().max().item() <= 2e-6
    assert rel_l2(_np(a.u), _np(b.u)) <= 1e-5


@pytest.mark.parametrize("name", ["flat_q120_long", "ridge_l162_long", "ridge2d_long"])
def test_long_runs_vs_reference(name):
    case, s = _gpu(name, "float32")
    gd = golden(name, "float32")
    n = sorted(case["ckpt"])[-1]
    masses = []
    for k in range(1, n + 1):
        s.step()
        if k % case["every"] == 0:
            masses.append(float(s.phi.double().sum()))
    assert np.abs(_np(s.phi) - gd[f"s{n}_phi"]).max() <= 1e-4
    assert rel_l2(_np(s.u), gd[f"s{n}_u"]) <= 1e-3
    np.testing.assert_allclose(masses, gd["mass_every"], rtol=1e-6)


@pytest.mark.parametrize("dn", ["float32", "float64"])
def test_flat64_full_run_vs_reference(dn):
    """64x64x48 flat-wall theta=120 static droplet, 500 steps (the reference's
    CPU-runnable case), against the reference's own 500-step output."""
    case, s = _gpu("cfg1_flat64", dn)
    gd = golden("cfg1_flat64", dn)
    masses = []
    for k in range(1, 501):
        s.step()
        if k % 50 == 0:
            masses.append(float(s.phi.double().sum()))
    phi = _np(s.phi)
    assert np.abs(phi - gd["s500_phi"]).max() <= (1e-4 if dn == "float32" else 1e-9)
    if dn == "float32":
        assert rel_l2(_np(s.u), gd["s500_u"]) <= 1e-3
    np.testing.assert_allclose(masses, gd["mass_every"], rtol=1e-6)
    # each mass-corrected step keeps sum(phi) within 1e-6 of the reference's
    m = s.measure()
    ref = measure_spread(gd["s500_phi"], gd["solid"])
    assert (m["Dx"], m["Dy"], m["Dz"]) == (ref["Dx"], ref["Dy"], ref["Dz"])
    assert m["volume"] == pytest.approx(ref["volume"], rel=1e-6)


def test_measure_matches_oracle():
    case, s = _gpu("ridge_l162", "float32")
    for _ in range(5):
        s.step()
    phi = _np(s.phi)
    m = s.measure()
    ref = measure_spread(phi, _np(s.solid))
    for k in ("Dx", "Dy", "Dz", "k", "count"):
        assert m[k] == ref[k], k
    assert m["volume"] == pytest.approx(ref["volume"], rel=1e-12)
    assert m["C_max"] == pytest.approx(ref["C_max"], rel=0, abs=0)
    assert m["z_com"] == pytest.approx(ref["z_com"], rel=1e-12)
    assert not m["has_nan"]


def test_autotune_leaves_state_unchanged():
    """The autotuner times candidates without advancing the state: the next
    steps with its choice continue from the same state (bit-identical when
    it keeps the two-kernel step, within a few ulps when it picks the fused
    kernel)."""
    case, a = _gpu("ridge_l162", "float32")
    _, b = _gpu("ridge_l162", "float32")
    a.run(3)
    b.run(3)
    assert torch.equal(a.phi, b.phi) and torch.equal(a.u, b.u)
    tile, ms = b.autotune(reps=2)
    assert (tile == (0, 0, 0) or all(t >= 2 for t in tile)) and ms > 0
    assert b.scalars()[3] == a.scalars()[3]
    a.run(10)
    b.run(10)
    if tile == (0, 0, 0):
        assert torch.equal(a.phi, b.phi) and torch.equal(a.u, b.u)
    else:
        assert (a.phi - b.phi).abs().max().item() <= 2e-6


@pytest.mark.parametrize("dim", [3, 2])
@pytest.mark.parametrize("dn", ["float32", "float64"])
def test_inject_droplet_vs_reference_and_oracle(dn, dim):
    """Mid-run droplet injection (lbm/fe_ac_solver.py:645-732) on the GPU
    against the reference's own outputs (tests/golden/make_golden_inject.py)
    and the oracle: fields and populations right after the injection, then
    4 more steps (looser: the blend of two overlapping droplets leaves a line
    where the lattice gradient nearly cancels inside the interface, and the
    sharpening direction there is set by rounding)."""
    import os
    from lbm.fe_ac_solver import AllenCahnSolver
    from make_golden_inject import INJECT_CASE, INJECT_CASE_2D
    from _cases import GOLDEN
    case = INJECT_CASE if dim == 3 else INJECT_CASE_2D
    gd = np.load(os.path.join(GOLDEN, f"inject_ridge{'' if dim == 3 else '2d'}_{dn}.npz"))
    solid, frac, C, u = inputs(case)
    s = AllenCahnSolver(config(case, "cuda"), dtype=getattr(torch, dn), **case["kw"])
    s.set_solid(solid, frac)
    s.init_fields(C, u)
    o = OracleSolver(config(case), dtype=np.dtype(dn), **case["kw"])
    o.set_solid(solid, frac)
    o.init_fields(C, u)
    for _ in range(case["before"]):
        s.step()
        o.step()
    inj = case["inject"]
    core = s.inject_droplet(inj["center"], inj["radius"], inj["xi"], u_impact=inj["u_impact"])
    assert core == o.inject_droplet(inj["center"], inj["radius"], inj["xi"], u_impact=inj["u_impact"])
    tp = 3e-6 if dn == "float32" else 1e-11
    phi, vel = _np(s.phi), _np(s.u)
    assert np.abs(phi - gd["inj_phi"]).max() <= tp
    assert np.abs(phi - o.phi).max() <= tp
    assert rel_l2(vel, gd["inj_u"]) <= (5e-5 if dn == "float32" else 1e-10)
    if "inj_f" in gd:
        assert np.abs(_np(s.f) - gd["inj_f"]).max() <= 5e-7
        assert np.abs(_np(s.g) - gd["inj_g"]).max() <= 5e-7
    assert s.phi_mass_init == pytest.approx(float(gd["inj_phi_mass_init"]), rel=1e-6 if dn == "float32" else 1e-12)
    for _ in range(case["after"]):
        s.step()
        o.step()
    assert np.abs(_np(s.phi) - gd["after_phi"]).max() <= (2e-4 if dn == "float32" else 1e-9)
    assert rel_l2(_np(s.u), gd["after_u"]) <= (1e-3 if dn == "float32" else 1e-8)


@pytest.mark.parametrize("dn", ["float32", "float64"])
def test_reduce_matches_fields(dn):
    """lbm_reduce (sum of phi, momentum sum rho u, phi > 0.5 extents, C_max in
    float64 on the device) against the same sums over the fields on the host."""
    case, s = _gpu("ridge_l162", dn)
    s.run(6)
    r = s.reduce()
    phi, vel = _np(s.phi).astype(np.float64), _np(s.u).astype(np.float64)
    solid = _np(s.solid)
    phi_c = np.where(solid, 0.0, phi)
    cfg = s.config
    rho = phi * cfg.rho_l + (1.0 - phi) * cfg.rho_g
    mom = (rho[None] * vel).reshape(3, -1).sum(axis=1)
    scale = np.abs(rho[None] * vel).reshape(3, -1).sum(axis=1)
    assert r["sum_phi"] == pytest.approx(phi_c.sum(), rel=1e-12)
    assert np.all(np.abs(np.array(r["momentum"]) - mom) <= 1e-10 * scale + 1e-300)
    idx = np.argwhere(phi_c > 0.5)
    ext = []
    for d in range(3):
        ext += [int(idx[:, d].min()), int(idx[:, d].max())]
    assert r["extents"] == tuple(ext)
    assert r["C_max"] == pytest.approx(float(phi_c.max()), rel=1e-7)
    # an empty phi > 0.5 set reports -1 extents
    case2, e = _gpu("flat_q120", dn)
    e.init_fields(np.full(e.shape, 0.25, np.float32))
    assert e.reduce()["extents"] == (-1,) * 6
