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


def _ref150(dtype_name="float32"):
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"ridge150_ref_{dtype_name}.npz")
    if dtype_name == "float64" and not os.path.exists(path):
        pytest.skip("the reference's float64 run of the case is not in tests/golden")
    return np.load(path)


def _perturbed_phi(seed):
    """The initial phi with every value moved by -1, 0 or +1 float32 ulp."""
    from lbm.fe_droplet import create_fe_droplet_with_impact
    C, _, u = create_fe_droplet_with_impact(150, 150, 107, center=(75, 75, 80), radius=22.5, xi=4.0,
                                            u_impact=(0, 0, -0.05))
    r = np.random.default_rng(seed).integers(-1, 2, C.shape)
    Cp = np.where(r > 0, np.nextafter(C, np.float32(2)), np.where(r < 0, np.nextafter(C, np.float32(-1)), C))
    return Cp.astype(np.float32), u


def _ridge_perturbed(seed, dtype=torch.float32):
    """The same case with every initial phi moved by -1, 0 or +1 float32 ulp."""
    from geometry.substrate import create_substrate_with_fraction
    from lbm.fe_ac_solver import AllenCahnSolver
    s0 = _ridge(dtype)
    cfg = s0.config
    s0.close()
    Cp, u = _perturbed_phi(seed)
    s = AllenCahnSolver(cfg, dtype=dtype, geo_amplification=1.5, geometric_wetting=True)
    solid, frac = create_substrate_with_fraction(150, 150, 107, "ridge", R_star=1.0, R_d=22.5)
    s.set_solid(solid, frac)
    s.init_fields(Cp, u)
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


STEPS = 2000
SNAPS = (100, 500, 2000)
MEMBERS = 12       # runs per precision in the one-ulp ensemble
SNAP_MEMBERS = 6   # of which phi is kept at the snapshot steps


@pytest.fixture(scope="module")
def ensemble():
    """The full 2000-step run on the GPU, in float32, in float64 and with
    half-precision population storage: from the generator's inputs and from
    eleven one-ulp perturbations of them in each form.  Every 50 steps: float64 sum of phi, Dx, Dy, Dz and the
    interface z-centre of each member; at the snapshot steps phi of the first
    SNAP_MEMBERS members of each precision, and u of both unperturbed runs (on
    the host)."""
    m32 = [_ridge(torch.float32)] + [_ridge_perturbed(seed) for seed in range(MEMBERS - 1)]
    m64 = [_ridge(torch.float64)] + [_ridge_perturbed(seed, torch.float64) for seed in range(MEMBERS - 1)]
    m16 = [_ridge(torch.float16)] + [_ridge_perturbed(seed, torch.float16) for seed in range(MEMBERS - 1)]
    hist = {32: {}, 64: {}, 16: {}}
    snaps = {}
    for k in range(50, STEPS + 1, 50):
        for bits, members in ((32, m32), (64, m64), (16, m16)):
            rows = []
            for m in members:
                m.run(50)
                d = m.measure()
                rows.append((float(m.phi.double().sum()), d["Dx"], d["Dy"], d["Dz"], d["z_com"]))
            hist[bits][k] = np.array(rows)
        if k in SNAPS:
            snaps[k] = {"phi32": [m.phi.double().cpu().numpy() for m in m32[:SNAP_MEMBERS]],
                        "phi64": [m.phi.cpu().numpy() for m in m64[:SNAP_MEMBERS]],
                        "u32": m32[0].u.double().cpu().numpy(), "u64": m64[0].u.cpu().numpy()}
    status = [m.status() for m in m32 + m64 + m16]
    for m in m32 + m64 + m16:
        m.close()
    return {"hist": hist, "snaps": snaps, "status": status}


def _check_history(ref_hist, env):
    """The reference's row at every checkpoint against the ensemble's members
    there: sum(phi) within three standard deviations of the members' mean,
    the deviation widened by 2e-6 relative (the reference sums phi for its
    mass correction in its own precision and order, which moves its sum by
    ~1e-7 relative from the first steps on); Dx, Dy, Dz within the members'
    range +- 1 node; the z-centre within their range widened by its width and
    0.05.  The reference's run is one more run with rounding-level different
    arithmetic, i.e. one more draw from the distribution the members sample."""
    for row in ref_hist:
        k = int(row[0])
        e = env[k]
        lo, hi = e.min(0), e.max(0)
        span = hi - lo
        mean, sd = e[:, 0].mean(), e[:, 0].std(ddof=1)
        tol_m = 3.0 * (sd + 2e-6 * abs(row[1]))
        assert abs(row[1] - mean) <= tol_m, (k, row[1], mean, sd)
        for j, col in ((1, 2), (2, 3), (3, 4)):  # Dx, Dy, Dz within the envelope +- 1 node
            assert lo[j] - 1 <= row[col] <= hi[j] + 1, (k, j, row[col], lo[j], hi[j])
        assert lo[4] - span[4] - 0.05 <= row[6] <= hi[4] + span[4] + 0.05, (k, row[6], lo[4], hi[4])


@pytest.mark.parametrize("dtype_name,bits", [("float32", 32), ("float64", 64), ("float32", 16), ("float64", 16)],
                         ids=["float32", "float64", "float32-vs-half", "float64-vs-half"])
def test_reference_history_within_perturbation_ensemble(ensemble, dtype_name, bits):
    """sum(phi), spread extents and interface z-centre of the reference's own
    run of the whole case (2000 steps) in float32 and in float64, every 50
    steps, lie within the spread of the twelve GPU runs of the same precision
    whose initial phi differ by one float32 ulp (the spread a rounding-level
    difference produces in this case); and within the spread of the twelve
    runs of the half-precision storage form."""
    ref = _ref150(dtype_name)
    assert int(ref["hist"][-1, 0]) == STEPS and len(ref["hist"]) == STEPS // 50
    _check_history(ref["hist"], ensemble["hist"][bits])
    assert all(st == 0 for st in ensemble["status"])


@pytest.mark.parametrize("dtype_name", ["float32", "float64"])
def test_reference_fields_within_perturbation_spread(ensemble, dtype_name):
    """phi of the reference's run at steps 100, 500 and 2000 (stored to 1.5e-5)
    is no farther from the GPU run of the same precision than one-ulp
    perturbed GPU runs are from each other (the largest distance among the
    members, with half again as margin: a few samples of a spread), and the
    norm of u within 1 %."""
    ref = _ref150(dtype_name)
    key = "phi32" if dtype_name == "float32" else "phi64"
    for k in SNAPS:
        sn = ensemble["snaps"][k]
        members = sn[key]
        spread = max(np.abs(a - b).max() for i, a in enumerate(members) for b in members[i + 1:])
        ours = members[0]
        ref_phi = ref[f"s{k}_phi_q"].astype(np.float64) / 65535.0
        d = np.abs(ours - ref_phi).max()
        assert d <= 1.5 * spread + 2e-5, (k, d, spread)
        u = sn["u32"] if dtype_name == "float32" else sn["u64"]
        assert np.linalg.norm(u) == pytest.approx(float(ref[f"s{k}_u_norm"]), rel=1e-2), k


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


def test_float32_against_float64_instance(ensemble):
    """Error of the float32 form against the float64 form of the same kernels
    (the float64 form is the oracle at sizes the CPU cannot run) over the whole
    2000-step run: at steps 100, 500 and 2000 max|dphi| no larger than the
    spread that one-ulp changes of the float32 inputs produce by themselves
    (the largest distance of a perturbed float32 run from the unperturbed one,
    with half again as margin: five samples of a spread); every 50 steps the
    float64 sum of phi no farther from the float32 one than the one-ulp runs'
    sums spread (half again as margin) or 2e-5 relative (the clamp of the mass
    correction leaks mass at a rate that depends on the precision: 1.2e-5
    relative at step 1350 measured) and the spread extents within one node
    of the one-ulp runs' range."""
    s32 = _ridge(torch.float32)
    s64 = _ridge(torch.float64)
    s32.run(10)
    s64.run(10)
    assert (s32.phi.double() - s64.phi).abs().max().item() <= 1e-6
    for k in SNAPS:
        sn = ensemble["snaps"][k]
        base = sn["phi32"][0]
        dulp = max(np.abs(base - m).max() for m in sn["phi32"][1:])
        d64 = np.abs(base - sn["phi64"][0]).max()
        assert d64 <= 1.5 * dulp, (k, d64, dulp)
    for k, e32 in ensemble["hist"][32].items():
        e64 = ensemble["hist"][64][k]
        span = e32.max(0) - e32.min(0)
        tol = max(1.5 * span[0], 2e-5 * e32[0, 0])
        assert abs(e64[0, 0] - e32[0, 0]) <= tol, (k, e64[0, 0], e32[:, 0])
        assert np.all(e64[0, 1:4] >= e32[:, 1:4].min(0) - 1) and np.all(e64[0, 1:4] <= e32[:, 1:4].max(0) + 1), k


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
