"""Size-independent properties of the CUDA path at the full 150x150x107
ridge size (the drop-in GPU case), where the CPU reference is too slow to run
to completion: conservation, range, determinism, float32 vs float64, and the
API's error behaviour."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _ridge(dtype, relax=0.3):
    from geometry.substrate import create_substrate_with_fraction
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.fe_config import FEConfig
    from lbm.fe_droplet import create_fe_droplet_with_impact
    cfg = FEConfig(nx=150, ny=150, nz=107, rho_l=1.0, rho_g=1.0 / 828.0, sigma=0.01424, xi=4.0,
                   tau_l=0.53, tau_g=0.53, theta_eq=162.0, device="cuda")
    s = AllenCahnSolver(cfg, dtype=dtype, geo_amplification=1.5, geometric_wetting=True, boundary_relax=relax)
    solid, frac = create_substrate_with_fraction(150, 150, 107, "ridge", R_star=1.0, R_d=22.5)
    s.set_solid(solid, frac)
    C, _, u = create_fe_droplet_with_impact(150, 150, 107, center=(75, 75, 80), radius=22.5, xi=4.0,
                                            u_impact=(0, 0, -0.05))
    s.init_fields(C, u)
    return s


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")


def _ref150():
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ridge150_ref_float32.npz")
    return np.load(path)


def _ridge_perturbed(seed):
    """The same case with every initial phi moved by -1, 0 or +1 float32 ulp."""
    from geometry.substrate import create_substrate_with_fraction
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.fe_droplet import create_fe_droplet_with_impact
    s0 = _ridge(torch.float32)
    cfg = s0.config
    del s0
    C, _, u = create_fe_droplet_with_impact(150, 150, 107, center=(75, 75, 80), radius=22.5, xi=4.0,
                                            u_impact=(0, 0, -0.05))
    r = np.random.default_rng(seed).integers(-1, 2, C.shape)
    Cp = np.where(r > 0, np.nextafter(C, np.float32(2)), np.where(r < 0, np.nextafter(C, np.float32(-1)), C))
    s = AllenCahnSolver(cfg, dtype=torch.float32, geo_amplification=1.5, geometric_wetting=True)
    solid, frac = create_substrate_with_fraction(150, 150, 107, "ridge", R_star=1.0, R_d=22.5)
    s.set_solid(solid, frac)
    s.init_fields(Cp.astype(np.float32), u)
    return s


def test_first_steps_vs_oracle_full_size():
    """At the full size the dynamics amplify a 1-ulp change ~10x per 10
    steps (the reference does the same against itself), so pointwise parity
    is checked over the first steps from identical inputs."""
    from oracle.ac_oracle import OracleSolver
    from geometry.substrate import create_substrate_with_fraction
    from lbm.fe_droplet import create_fe_droplet_with_impact
    s = _ridge(torch.float32)
    o = OracleSolver(s.config, dtype=np.float32, geo_amplification=1.5, geometric_wetting=True)
    solid, frac = create_substrate_with_fraction(150, 150, 107, "ridge", R_star=1.0, R_d=22.5)
    o.set_solid(solid, frac)
    C, _, u = create_fe_droplet_with_impact(150, 150, 107, center=(75, 75, 80), radius=22.5, xi=4.0,
                                            u_impact=(0, 0, -0.05))
    o.init_fields(C, u)
    for k in range(3):
        s.step()
        o.step()
        assert np.abs(s.phi.cpu().numpy() - o.phi).max() <= 2e-6, k
        vel = s.u.cpu().numpy()
        assert np.linalg.norm(vel - o.u) / np.linalg.norm(o.u) <= 2e-5, k


def test_reference_history_within_perturbation_ensemble():
    """sum(phi), spread extents and interface z-centre of the reference's own
    full-size run, every 50 steps, lie inside the envelope of GPU runs whose
    inputs differ by one float32 ulp (the spread a rounding-level difference
    produces in this case)."""
    ref = _ref150()
    hist = ref["hist"]
    last = int(hist[-1, 0])
    members = [_ridge(torch.float32)] + [_ridge_perturbed(seed) for seed in range(5)]
    rec = {int(k): [] for k in hist[:, 0]}
    for k in range(50, last + 1, 50):
        for m in members:
            m.run(50)
            d = m.measure()
            rec[k].append((float(m.phi.double().sum()), d["Dx"], d["Dy"], d["Dz"], d["z_com"]))
    for row in hist:
        k = int(row[0])
        e = np.array(rec[k])
        lo, hi = e.min(0), e.max(0)
        span = hi - lo
        # mass: envelope widened by its own width and 2e-6 relative
        tol_m = span[0] + 2e-6 * abs(row[1])
        assert lo[0] - tol_m <= row[1] <= hi[0] + tol_m, (k, row[1], lo[0], hi[0])
        for j, col in ((1, 2), (2, 3), (3, 4)):  # Dx, Dy, Dz within the envelope +- 1 node
            assert lo[j] - 1 <= row[col] <= hi[j] + 1, (k, j, row[col], lo[j], hi[j])
        assert lo[4] - span[4] - 0.05 <= row[6] <= hi[4] + span[4] + 0.05, (k, row[6], lo[4], hi[4])
    for m in members:
        assert m.status() == 0


def test_deterministic_and_run_equals_steps():
    a = _ridge(torch.float32)
    b = _ridge(torch.float32)
    for _ in range(30):
        a.step()
    b.run(30)
    pa, ua = a.fields("phi", "u")
    pb, ub = b.fields("phi", "u")
    assert torch.equal(pa, pb) and torch.equal(ua, ub)
    assert torch.equal(a.f, b.f) and torch.equal(a.g, b.g)


def test_float32_against_float64_instance():
    """Error of the float32 form against the float64 form of the same kernel
    (the float64 form is the oracle at sizes the CPU cannot run): below 1e-6
    over the first 10 steps, and after 300 steps no larger than the spread
    that a one-ulp change of the float32 inputs produces by itself."""
    s32 = _ridge(torch.float32)
    s64 = _ridge(torch.float64)
    sp = _ridge_perturbed(7)
    s32.run(10)
    s64.run(10)
    assert (s32.phi.double() - s64.phi).abs().max().item() <= 1e-6
    s32.run(290)
    s64.run(290)
    sp.run(300)
    d64 = (s32.phi.double() - s64.phi).abs().max().item()
    dulp = (s32.phi - sp.phi).abs().max().item()
    assert d64 <= 10 * max(dulp, 1e-6), (d64, dulp)


def test_geometry_matches_oracle_at_full_size():
    from oracle.ac_oracle import OracleWetting
    from geometry.substrate import create_substrate_with_fraction
    s = _ridge(torch.float32)
    solid, frac = create_substrate_with_fraction(150, 150, 107, "ridge", R_star=1.0, R_d=22.5)
    cfg = s.config
    w = OracleWetting(solid, cfg.phi_c, cfg.kappa, cfg.sigma, cfg.theta_eq, "linear", solid_fraction=frac)
    assert np.array_equal(s.wetting.is_boundary.cpu().numpy(), w.is_boundary)
    assert np.array_equal(s.wetting.wall_normal.cpu().numpy(), w.wall_normal)
    assert np.array_equal(s.wetting.wall_weight.cpu().numpy(), w.wall_weight)
    assert np.array_equal(s.wetting.near_wall_mask.cpu().numpy(), w.near_wall_mask)


def test_api_errors():
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.fe_config import FEConfig
    cfg = FEConfig(nx=16, ny=16, nz=12, rho_l=1.0, rho_g=1.0 / 828.0, sigma=0.01, xi=4.0, tau_l=0.53,
                   tau_g=0.53, theta_eq=120.0, device="cuda")
    s = AllenCahnSolver(cfg, dtype=torch.float32)
    with pytest.raises(RuntimeError):
        s.step()
    # the gradient-of-mu modes: float32 / float64 only, two-kernel step only, not batched
    from lbm import _native as nat
    from lbm.batch import AllenCahnBatch
    for kw in (dict(interface_mode="cahn-hilliard"), dict(mu_drive=0.1)):
        with pytest.raises(NotImplementedError):
            AllenCahnSolver(cfg, dtype=torch.float16, **kw)
        ch = AllenCahnSolver(cfg, dtype=torch.float32, **kw)
        ch.set_solid(np.zeros((16, 16, 12), bool))
        ch.init_fields(np.full((16, 16, 12), 0.5, np.float32))
        with pytest.raises(nat.LbmError):
            ch.set_tile(4, 4, 6)
        with pytest.raises(nat.LbmError):
            AllenCahnBatch([ch])
    with pytest.raises(ValueError):
        AllenCahnSolver(cfg, interface_mode="phase-field")
    with pytest.raises(ValueError):  # a per-node amplification field must have the grid's shape
        AllenCahnSolver(cfg, geo_amplification=torch.ones(16, 16, 11))
    with pytest.raises(ValueError):
        s.set_solid(np.zeros((4, 4, 4), bool))
