"""The reference's code-verification suite on the GPU path.

scripts/verify_mms.py of the reference checks five properties of its solver
on small flat-wall boxes (60 x 60 x 30 unless stated; sigma = 0.01, xi = 4,
tau = 0.53, tau_h = 0.57, theta = 162, boundary_relax = 0, float32), each
with a pass threshold:

  1. mass conservation: the number of phi > 0.5 nodes of a static droplet
     (R = 10) drifts by less than 2 % over 200 steps (verify_mms.py:71-110);
  2. Allen-Cahn ablation: the spread ratio k after 300 steps of an impact
     (U0 = -0.03) does not increase with ac_scale in 0, 0.5, 1, 1.5, 2
     (0.01 slack; :116-152);
  3. flat-wall symmetry with alpha_geo = 1.5: |k - 1| < 0.15 (:158-189);
  4. energy dissipation: the free energy of a random phi field (40 x 40 x 20,
     numpy seed 42) does not increase over 300 steps, sampled every 30
     (1e-4 slack), and decreases overall (:195-241);
  5. grid convergence: the spreading diameter at N = 60 and 80 (R = N / 4)
     differs by less than 15 % (:247-285).

The set-ups (tests/_verify_cases.py) run through AllenCahnSolver on the GPU
and are compared with the reference's own values on the same set-ups
(tests/golden/verify_mms_ref.json, tests/golden/make_golden_verify.py).
The reference passes checks 1, 3 and 4 and fails 2 and 5 itself: its k
against ac_scale is 1.133, 1.056, 1.105, 1.0, 1.0 (not monotonic), and the
droplet radius of check 5 grows with N, so the diameters 23, 33, 43 differ
by 30 %.  The GPU path gives the reference's values, so it passes and fails
the same checks; the tests assert the values and the outcomes."""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import _verify_cases as vc  # noqa: E402
from _cases import GOLDEN  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return built_lib


@pytest.fixture(scope="module")
def ref():
    with open(os.path.join(GOLDEN, "verify_mms_ref.json")) as fh:
        return json.load(fh)


def test_mass_conservation(ref):
    d = vc.mass_drift_pct()
    assert d == pytest.approx(ref["mass_drift_pct"], abs=0.05)  # within two of the ~4100 phi > 0.5 nodes
    assert abs(d) < 2.0


def test_ac_ablation(ref):
    k = vc.ablation_k()
    assert k == ref["ablation_k"]
    monotonic = all(k[i] >= k[i + 1] - 0.01 for i in range(len(k) - 1))
    assert not monotonic  # as the reference: 1.133, 1.056, 1.105, 1.0, 1.0


def test_symmetry_flat(ref):
    k = vc.flat_k()
    assert k == ref["flat_k"]
    assert abs(k - 1.0) < 0.15


def test_energy_dissipation(ref):
    e = vc.energies()
    np.testing.assert_allclose(e, ref["energies"], rtol=1e-5)
    assert all(e[i] >= e[i + 1] - 1e-4 for i in range(len(e) - 1)), e
    assert e[-1] < e[0]


def test_grid_convergence(ref):
    d = vc.diameters()
    assert d == ref["diameters"]
    assert abs(d[-1] - d[-2]) / max(d[-2], 1) >= 0.15  # as the reference: 23, 33, 43
