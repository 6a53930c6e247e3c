"""Pins from the reference's own verification scripts and paper, on the
oracle (CPU).  The CUDA path is held to the oracle by the parity tests and
to the reference's validation case by tests/test_gpu_pins.py."""
import math

import numpy as np
import pytest

from oracle.ac_oracle import OracleSolver


class _Cfg:
    """The FEConfig fields the oracle reads, for a wall-free periodic box."""

    def __init__(self, n):
        self.nx = self.ny = self.nz = n
        self.rho_l, self.rho_g = 1.0, 1.0 / 828.0
        self.sigma, self.xi, self.beta, self.kappa, self.phi_c = 0.01, 4.0, 1.0, 1.0, 0.0
        self.tau_l = self.tau_g = 0.53
        self.tau_h = 0.57
        self.theta_eq = 162.0
        self.g_force = (0.0, 0.0, 0.0)


# scripts/mms_spatial.py (the reference's spatial manufactured-solution check
# of its fused gradient operator, float64), run on the reference itself:
# root-mean-square error of the gradient of
# phi = sin(2 pi i / N) cos(2 pi j / N) cos(2 pi k / N); the paper quotes
# 1.33e-3 at N = 32 and 2.09e-5 at N = 128
# (paper_pof/sections/4_experiments.tex:188).
MMS_REFERENCE = {32: 0.0013287554489764936, 64: 0.00016697699016028267, 128: 2.0899705779242237e-05}


def _mms_error(n):
    i = np.arange(n)[:, None, None]
    j = np.arange(n)[None, :, None]
    k = np.arange(n)[None, None, :]
    a = 2 * np.pi / n
    phi = np.sin(a * i) * np.cos(a * j) * np.cos(a * k)
    exact = (a * np.cos(a * i) * np.cos(a * j) * np.cos(a * k),
             -a * np.sin(a * i) * np.sin(a * j) * np.cos(a * k),
             -a * np.sin(a * i) * np.cos(a * j) * np.sin(a * k))
    s = OracleSolver(_Cfg(n), dtype=np.float64, boundary_relax=0.0)
    grad, _ = s._grad_lap(phi)
    e = [np.sqrt(((grad[d] - exact[d]) ** 2).mean()) for d in range(3)]
    return math.sqrt((e[0] ** 2 + e[1] ** 2 + e[2] ** 2) / 3)


def test_mms_gradient_matches_reference_and_paper():
    errs = {n: _mms_error(n) for n in (32, 64, 128)}
    for n, e in errs.items():
        assert e == pytest.approx(MMS_REFERENCE[n], rel=1e-10), n
    assert round(errs[32], 5) == 1.33e-3 and round(errs[128], 7) == 2.09e-5
    # the order the script reports (>= 2 for its "converged" verdict)
    orders = [math.log(errs[a] / errs[b], 2) for a, b in ((32, 64), (64, 128))]
    assert all(o >= 2.0 for o in orders)
