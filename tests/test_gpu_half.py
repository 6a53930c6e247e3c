"""Accuracy of the half-precision storage form (LBM_F16: populations stored in
float16 as deviations from their rest-state equilibria, float32 arithmetic,
float64 global sums) against the reference's own float64 and float32 runs
(golden fixtures), through the C ABI.

The bound is the parity bound of the float32 form: max|dphi| <= 1e-4 and
relative L2 on u <= 1e-3 after the full run, the history of sum(phi) within
1e-6 relative, and the spread extents equal (so the spread factor error is
0, within the 1 % the precision form is held to)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from _cases import CASES, config, golden, inputs, rel_l2  # noqa: E402
from oracle.ac_oracle import measure_spread  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return built_lib


def _run(name, steps, every=None):
    from lbm.fe_ac_solver import AllenCahnSolver
    case = CASES[name]
    solid, frac, C, u = inputs(case)
    s = AllenCahnSolver(config(case, "cuda"), dtype=torch.float16, **case["kw"])
    s.set_solid(solid, frac)
    s.init_fields(C, u)
    masses = []
    for k in range(1, steps + 1):
        s.step()
        if every and k % every == 0:
            masses.append(float(s.phi.double().sum()))
    return s, masses


@pytest.mark.parametrize("name,steps,every,ref", [
    ("cfg1_flat64", 500, 50, "float64"),       # the 64x64x48 static droplet, full run, against float64
    ("ridge_l162", 5, None, "float64"),
    ("flat_q120", 5, None, "float64"),
    ("ridge_l162_long", 100, 10, "float32"),
    ("flat_q120_long", 100, 10, "float32"),
])
def test_half_storage_within_parity_bound(name, steps, every, ref):
    s, masses = _run(name, steps, every)
    gd = golden(name, ref)
    phi = s.phi.cpu().numpy()
    ref_phi = gd[f"s{steps}_phi"]
    assert s.phi.dtype == torch.float32  # fields are float32 in this form
    assert np.abs(phi - ref_phi).max() <= 1e-4
    if f"s{steps}_u" in gd:
        assert rel_l2(s.u.cpu().numpy(), gd[f"s{steps}_u"]) <= 1e-3
    if masses:
        np.testing.assert_allclose(masses, gd["mass_every"], rtol=1e-6)
    a = measure_spread(phi, gd["solid"])
    b = measure_spread(ref_phi, gd["solid"])
    assert (a["Dx"], a["Dy"], a["Dz"]) == (b["Dx"], b["Dy"], b["Dz"])
    assert a["volume"] == pytest.approx(b["volume"], rel=1e-6)
