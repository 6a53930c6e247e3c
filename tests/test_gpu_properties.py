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


def test_mass_range_and_no_nan():
    s = _ridge(torch.float32)
    m0 = s.phi_mass_init
    for k in range(1, 201):
        s.step()
        if k % 20 == 0:
            phi = s.phi
            assert float(phi.min()) >= 0.0 and float(phi.max()) <= 1.0
            rel = abs(float(phi.double().sum()) - m0) / m0
            assert rel <= 1e-5, (k, rel)
            _, last_sum, corr, _ = s.scalars()
            assert abs(corr - 1.0) <= 1e-3
    assert s.status() == 0
    m = s.measure()
    assert not m["has_nan"] and m["count"] > 0


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
    (the float64 form is the oracle at sizes the CPU cannot run)."""
    s32 = _ridge(torch.float32)
    s64 = _ridge(torch.float64)
    s32.run(300)
    s64.run(300)
    d = (s32.phi.double() - s64.phi).abs().max().item()
    du = ((s32.u.double() - s64.u).norm() / s64.u.norm()).item()
    assert d <= 1e-4, d
    assert du <= 1e-3, du


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
    for kw in (dict(interface_mode="cahn-hilliard"), dict(mu_drive=0.1), dict(direct_wetting=True),
               dict(geo_amplification=torch.ones(16, 16, 12))):
        with pytest.raises(NotImplementedError):
            AllenCahnSolver(cfg, **kw)
    with pytest.raises(ValueError):
        s.set_solid(np.zeros((4, 4, 4), bool))
