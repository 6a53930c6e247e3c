"""Set-ups of the reference's code-verification suite (scripts/verify_mms.py),
shared by tests/test_gpu_verify.py (the GPU path) and
tests/golden/make_golden_verify.py (the reference itself, for the fixture).
Each function takes the solver and config classes and the device, so the
same code runs either implementation."""
import numpy as np
import torch


def _classes():
    """The package's solver (default)."""
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.fe_config import FEConfig
    return AllenCahnSolver, FEConfig


def make_solver(N, nz, ac_scale=1.0, amp=0.0, classes=None, device="cuda"):
    """A flat wall at z = 0 (verify_mms.py:17-45)."""
    Solver, FEConfig = classes or _classes()
    xi, sigma = 4.0, 0.01
    beta = 12.0 * sigma / xi
    kappa = beta * xi ** 2 / 8.0
    cfg = FEConfig(nx=N, ny=N, nz=nz, rho_l=1.0, rho_g=1.0 / 828.0, sigma=sigma, xi=xi, beta=beta, kappa=kappa,
                   M=0.02 / beta, tau_l=0.53, tau_g=0.53, tau_h=0.57, theta_eq=162.0, device=device,
                   max_steps=1, output_interval=2, g_force=(0.0, 0.0, 0.0))
    s = Solver(cfg, dtype=torch.float32, stab_mode="fakhari", boundary_relax=0.0, geometric_wetting=(amp > 0),
               geo_amplification=amp, ac_scale=ac_scale)
    solid = np.zeros((N, N, nz), dtype=bool)
    solid[:, :, 0] = True
    s.set_solid(solid, solid_fraction=solid.astype(np.float32))
    return s, xi, beta, kappa


def droplet(N, nz, xi, R, cz):
    """tanh droplet profile centred at (N/2, N/2, cz) (verify_mms.py:48-60)."""
    cx = cy = N / 2.0
    x = np.arange(N, dtype=np.float32)
    X, Y = np.meshgrid(x, x, indexing="ij")
    rxy = np.sqrt((X - cx) ** 2 + (Y - cy) ** 2)
    phi = np.zeros((N, N, nz), dtype=np.float32)
    for k in range(nz):
        r3 = np.sqrt(rxy ** 2 + (k - cz) ** 2)
        phi[:, :, k] = 0.5 * (1.0 - np.tanh(2.0 * (r3 - R) / xi))
    return phi


def place_droplet(s, N, nz, xi, R, U0):
    phi = droplet(N, nz, xi, R, nz / 2.0 + 2)
    u = np.zeros((3, N, N, nz), dtype=np.float32)
    u[2] = U0 * phi
    s.init_fields(phi, u)


def yz_extents(s):
    phi = s.phi.detach().cpu().numpy()
    sol = s.solid.cpu().numpy()
    c = np.argwhere((phi > 0.5) & ~sol)
    if not c.size:
        return 0.0, 0.0
    return float(c[:, 1].max() - c[:, 1].min() + 1), float(c[:, 2].max() - c[:, 2].min() + 1)


def mass_drift_pct(classes=None, device="cuda"):
    N, nz = 60, 30
    s, xi, _, _ = make_solver(N, nz, classes=classes, device=device)
    s.init_fields(droplet(N, nz, xi, 10.0, nz / 2.0), np.zeros((3, N, N, nz), dtype=np.float32))
    m0 = int((s.phi > 0.5).sum().item())
    for _ in range(200):
        s.step()
    m1 = int((s.phi > 0.5).sum().item())
    return (m1 - m0) / m0 * 100.0


def ablation_k(classes=None, device="cuda"):
    N, nz = 60, 30
    out = []
    for sc in (0.0, 0.5, 1.0, 1.5, 2.0):
        s, xi, _, _ = make_solver(N, nz, ac_scale=sc, classes=classes, device=device)
        place_droplet(s, N, nz, xi, 10.0, -0.03)
        for _ in range(300):
            s.step()
        dx, dy = yz_extents(s)
        out.append(dx / dy if dy > 0 else 0.0)
    return out


def flat_k(classes=None, device="cuda"):
    N, nz = 60, 30
    s, xi, _, _ = make_solver(N, nz, amp=1.5, classes=classes, device=device)
    place_droplet(s, N, nz, xi, 10.0, -0.03)
    for _ in range(300):
        s.step()
    dx, dy = yz_extents(s)
    return dx / dy if dy > 0 else 0.0


def energies(classes=None, device="cuda"):
    N, nz = 40, 20
    s, _, beta, kappa = make_solver(N, nz, classes=classes, device=device)
    np.random.seed(42)
    phi = np.clip((0.5 + 0.2 * np.random.randn(N, N, nz)).astype(np.float32), 0.01, 0.99)
    s.init_fields(phi, np.zeros((3, N, N, nz), dtype=np.float32))

    def energy(p):
        bulk = (beta / 2.0) * np.sum(p ** 2 * (1 - p) ** 2)
        g = [np.gradient(p, axis=a) for a in range(3)]
        return bulk + (kappa / 2.0) * np.sum(g[0] ** 2 + g[1] ** 2 + g[2] ** 2)

    out = []
    for step in range(301):
        if step % 30 == 0:
            out.append(energy(s.phi.detach().cpu().numpy()))
        if step < 300:
            s.step()
    return out


def diameters(classes=None, device="cuda"):
    out = []
    for N in (40, 60, 80):
        nz = max(20, N // 2)
        s, xi, _, _ = make_solver(N, nz, amp=1.5, classes=classes, device=device)
        place_droplet(s, N, nz, xi, N / 4.0, -0.03)
        for _ in range(300):
            s.step()
        out.append(yz_extents(s)[0])
    return out
