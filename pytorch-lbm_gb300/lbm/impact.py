"""Droplet-impact cases of the batched sweep and the serving workload.

``sample_impact_case(seed)`` draws one case (numpy ``default_rng(seed)``):
grid, substrate in {flat, ridge, convex, concave} (R* = 1), droplet radius
R_d ~ U[15, 30], contact angle theta ~ U[90, 162] deg, impact speed
u_z ~ U[-0.08, -0.02], xi = 4, density ratio 828, and a step count.
``build_impact_case`` sets a solver up the way the reference's sweep driver
does (scripts/run_thesis_sweep.py:132-162): the substrate with its smooth
solid fraction, the droplet centred in x and y at surface top + 2 + R_d,
clamped to nz - R_d - 2 (the rim height for a concave substrate).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SWEEP_GRIDS = ((96, 96, 96), (128, 128, 96), (150, 150, 107), (192, 192, 128))
SERVE_GRIDS = SWEEP_GRIDS + ((256, 256, 192),)
SUBSTRATES = ("flat", "ridge", "convex", "concave")


@dataclass
class ImpactCase:
    seed: int
    grid: tuple
    substrate: str
    R_d: float
    theta: float
    u_z: float
    steps: int

    @property
    def nodes(self):
        return int(np.prod(self.grid))


def sample_impact_case(seed, grids=SWEEP_GRIDS, steps=(1500, 1500)):
    """One case drawn with ``numpy.random.default_rng(seed)``; ``steps`` is a
    (low, high) range of the step count (inclusive)."""
    rng = np.random.default_rng(seed)
    grid = tuple(int(x) for x in grids[int(rng.integers(len(grids)))])
    substrate = SUBSTRATES[int(rng.integers(len(SUBSTRATES)))]
    R_d = float(rng.uniform(15.0, 30.0))
    theta = float(rng.uniform(90.0, 162.0))
    u_z = float(rng.uniform(-0.08, -0.02))
    lo, hi = steps
    n = int(lo) if lo == hi else int(rng.integers(int(lo), int(hi) + 1))
    return ImpactCase(seed=int(seed), grid=grid, substrate=substrate, R_d=R_d, theta=theta, u_z=u_z, steps=n)


def surface_top(solid):
    """Index of the topmost solid node per (x, y) column (0 if none), as
    get_surface_height of scripts/run_thesis_sweep.py:45-54."""
    kk = np.arange(solid.shape[-1])
    return np.where(solid, kk, -1).max(axis=-1).clip(min=0)


def impact_inputs(case, xi=4.0):
    """(solid, fraction, phi, u) of a case, built with the package's generators."""
    from geometry.substrate import create_substrate_with_fraction
    from .fe_droplet import create_fe_droplet_with_impact
    nx, ny, nz = case.grid
    flat = case.substrate == "flat"
    solid, frac = create_substrate_with_fraction(nx, ny, nz, case.substrate, R_star=None if flat else 1.0,
                                                 R_d=case.R_d)
    top = surface_top(solid)
    ridge_top = int(top.max()) if case.substrate == "concave" else int(top[nx // 2, ny // 2])
    cz = min(ridge_top + 2.0 + case.R_d, nz - case.R_d - 2)
    C, _, u = create_fe_droplet_with_impact(nx, ny, nz, center=(nx / 2.0, ny / 2.0, cz), radius=case.R_d, xi=xi,
                                            u_impact=(0.0, 0.0, case.u_z))
    return solid, frac, C, u


def impact_config(case, device="cuda"):
    from .fe_config import FEConfig
    nx, ny, nz = case.grid
    return FEConfig(nx=nx, ny=ny, nz=nz, rho_l=1.0, rho_g=1.0 / 828.0, sigma=0.01424, xi=4.0, tau_l=0.53,
                    tau_g=0.53, theta_eq=case.theta, device=device, max_steps=case.steps)


def build_impact_case(case, dtype, device="cuda", geo_amplification=1.5):
    """An initialised AllenCahnSolver for ``case`` (geometric wetting,
    alpha_geo = 1.5)."""
    from .fe_ac_solver import AllenCahnSolver
    solid, frac, C, u = impact_inputs(case)
    s = AllenCahnSolver(impact_config(case, device), dtype=dtype, geo_amplification=geo_amplification,
                        geometric_wetting=True)
    s.set_solid(solid, frac)
    s.init_fields(C, u)
    return s
