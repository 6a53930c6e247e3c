"""The precision form's large single solve (384x384x256 convex hemisphere,
37.7 M nodes) against the reference's own run of its first steps
(tests/golden/convex384_ref_float32.npz, made by
tests/golden/make_golden_convex384.py): the wetting tables bit for bit (their
SHA-256), sum(phi) every step, and phi on every 4th node in x and y after the
last step, for the float32, float64 and half-precision storage forms.

The droplet apex on the symmetry axis is unstable at the rounding level (as
the 150x150x107 impact is): a 1e-5 difference there grows ~100x between steps
10 and 20 (float32 against float64: 4.5e-7 -> 5.2e-5; half storage against
float64: 5e-5 -> 6e-3 at (192, 192, 217)).  So float32 and float64 are held to
the parity bound max|dphi| <= 1e-4 everywhere, and the half form to it on all
but 0.1 % of the nodes (those around the apex), plus, for every form, the
sum(phi) history and the phi > 0.5 extents."""
import hashlib
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "convex384_ref_float32.npz")


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return built_lib


@pytest.fixture(scope="module")
def case():
    from geometry.substrate import create_substrate_with_fraction
    from lbm.fe_config import FEConfig
    from lbm.fe_droplet import create_fe_droplet_with_impact
    nx, ny, nz = 384, 384, 256
    cfg = FEConfig(nx=nx, ny=ny, nz=nz, rho_l=1.0, rho_g=1 / 828.0, sigma=0.01424, xi=4.0, tau_l=0.53,
                   tau_g=0.53, theta_eq=150.0, device="cuda")
    solid, frac = create_substrate_with_fraction(nx, ny, nz, "convex", R_star=60.0 / 45.0, R_d=45.0)
    C, _, u = create_fe_droplet_with_impact(nx, ny, nz, center=(192, 192, 180), radius=45.0, xi=4.0,
                                            u_impact=(0, 0, -0.06))
    return cfg, solid, frac, C, u


def _sha(t):
    return hashlib.sha256(np.ascontiguousarray(t.cpu().numpy()).tobytes()).hexdigest()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float16, torch.float64])
def test_convex384_first_steps_vs_reference(case, dtype):
    from lbm.fe_ac_solver import AllenCahnSolver
    cfg, solid, frac, C, u = case
    gd = np.load(GOLDEN)
    s = AllenCahnSolver(cfg, dtype=dtype, geo_amplification=1.5, geometric_wetting=True)
    s.set_solid(solid, frac)
    s.init_fields(C, u)
    if dtype == torch.float32:
        w = s.wetting
        assert [_sha(w.is_boundary), _sha(w.wall_normal), _sha(w.wall_weight), _sha(w.near_wall_mask)] == \
            [str(x) for x in gd["geo_sha256"]]
    hist = gd["hist"]
    K = int(hist[-1, 0])
    masses = []
    for _ in range(K):
        s.step()
        masses.append(float(s.phi.double().sum()))
    np.testing.assert_allclose(masses, hist[:, 1], rtol=1e-6)
    phi = s.phi[::4, ::4, :].cpu().numpy()
    ref = gd[f"s{K}_phi_sub"]
    err = np.abs(phi.astype(np.float64) - ref)
    if dtype == torch.float16:
        # measured on GB300: 570 of 2,359,296 sampled nodes (0.024 %) beyond 1e-4,
        # the largest 6.1e-3, all around the apex
        assert np.count_nonzero(err > 1e-4) <= 1e-3 * err.size
        assert err.max() <= 1e-2
    else:
        assert err.max() <= 1e-4
    inside, inside_ref = np.argwhere(phi > 0.5), np.argwhere(ref > 0.5)
    assert np.array_equal(inside.min(0), inside_ref.min(0)) and np.array_equal(inside.max(0), inside_ref.max(0))
    assert not s.status()
    s.close()
