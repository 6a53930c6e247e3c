"""FEConfig: parameters of the Allen-Cahn phase-field LBM.

Same fields, defaults and derivations as the reference's dataclass
(pytorch-lbm ``lbm/fe_config.py:27-163``), so caller scripts construct it
unchanged:

  beta  = 12 sigma / xi          (when sigma given and beta == 0)
  sigma = beta xi / 12           (when beta given and sigma == 0)
  kappa = beta xi^2 / 8          (when kappa == 0)
  M     = 0.02 / beta            (when M == 0)
  phi_c = -cos(theta) sqrt(2 kappa beta)   (when phi_c == 0 and theta != 90)

``tau_h`` (the phase-field relaxation time) defaults to 1.0 and ``dtype`` is
informational: the solver takes its own ``dtype`` argument.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Tuple


@dataclass
class FEConfig:
    nx: int = 200
    ny: int = 200
    nz: int = 1
    dx: float = 1e-6
    dt: float = 1e-6
    rho_l: float = 828.0
    rho_g: float = 1.0
    sigma: float = 0.01
    xi: float = 5.0
    beta: float = 0.0
    kappa: float = 0.0
    M: float = 0.0
    beta_A: float = 0.25
    tau_l: float = 0.0
    tau_g: float = 0.6
    tau_h: float = 1.0
    theta_eq: float = 162.0
    phi_c: float = 0.0
    g_force: Tuple[float, ...] = (0.0, 0.0, 0.0)
    max_steps: int = 10000
    output_interval: int = 100
    device: str = "cuda"
    dtype: str = "float32"
    use_fft_pressure: bool = False

    def __post_init__(self):
        if self.sigma > 0.0 and self.beta == 0.0:
            self.beta = 12.0 * self.sigma / self.xi
        elif self.sigma == 0.0 and self.beta > 0.0:
            self.sigma = self.beta * self.xi / 12.0
        if self.kappa == 0.0:
            self.kappa = self.beta * self.xi ** 2 / 8.0
        if self.M == 0.0:
            self.M = 0.02 / self.beta
        if self.phi_c == 0.0 and self.theta_eq != 90.0:
            self.phi_c = -math.cos(math.radians(self.theta_eq)) * math.sqrt(
                2.0 * self.kappa * self.beta)

    @property
    def dim(self) -> int:
        return 2 if self.nz == 1 else 3

    @property
    def grid_shape(self) -> Tuple[int, ...]:
        return (self.nx, self.ny) if self.nz == 1 else (self.nx, self.ny, self.nz)

    @property
    def density_ratio(self) -> float:
        return self.rho_l / self.rho_g

    @property
    def nu_l(self) -> float:
        return (self.tau_l - 0.5) / 3.0

    @property
    def nu_g(self) -> float:
        return (self.tau_g - 0.5) / 3.0

    @property
    def mu_l(self) -> float:
        return self.rho_l * self.nu_l

    @property
    def mu_g(self) -> float:
        return self.rho_g * self.nu_g

    @staticmethod
    def compute_tau_from_oh(Oh: float, D0: float, rho_l: float = 828.0,
                            sigma: float = 0.01) -> float:
        """tau_l = 3 Oh sqrt(rho_l sigma D0) / rho_l + 1/2."""
        return 3.0 * (Oh * math.sqrt(rho_l * sigma * D0) / rho_l) + 0.5

    @classmethod
    def from_paper_params(cls, We: float, Oh: float, D0: float, theta_eq: float = 162.0,
                          rho_l: float = 828.0, rho_g: float = 1.0, xi: float = 5.0,
                          beta_A: float = 0.25, U0: float = 0.05, nx: int = 200,
                          ny: int = 200, nz: int = 1, tau_g: float = 0.6,
                          device: str = "cuda", max_steps: int = 10000,
                          output_interval: int = 100) -> "FEConfig":
        """Config for given Weber / Ohnesorge numbers (sigma = rho_l U0^2 D0 / We)."""
        sigma = rho_l * U0 ** 2 * D0 / We
        beta = 12.0 * sigma / xi
        kappa = beta * xi ** 2 / 8.0
        phi_c = -math.cos(math.radians(theta_eq)) * math.sqrt(2.0 * kappa * beta)
        return cls(nx=nx, ny=ny, nz=nz, rho_l=rho_l, rho_g=rho_g, sigma=sigma, xi=xi,
                   beta=beta, kappa=kappa, M=0.02 / beta, beta_A=beta_A,
                   tau_l=cls.compute_tau_from_oh(Oh, D0, rho_l, sigma), tau_g=tau_g,
                   tau_h=0.5, theta_eq=theta_eq, phi_c=phi_c, max_steps=max_steps,
                   output_interval=output_interval, device=device)

    def print_info(self):
        print(f"FEConfig grid={self.grid_shape} rho_l={self.rho_l} rho_g={self.rho_g} "
              f"sigma={self.sigma:.6f} xi={self.xi} beta={self.beta:.6f} "
              f"kappa={self.kappa:.6f} tau_l={self.tau_l} tau_g={self.tau_g} "
              f"tau_h={self.tau_h} theta_eq={self.theta_eq} phi_c={self.phi_c:.6f}")
