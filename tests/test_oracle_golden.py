"""The numpy oracle against the reference's own outputs (golden fixtures).

Pins oracle/ac_oracle.py: setup tables bit-exact, init fields exact, step
fields within a few ulps (torch's CPU reduction order is size/thread
dependent, so bit equality is out of reach for summed quantities)."""
import numpy as np
import pytest

from _cases import CASES, all_cases, config, golden, inputs, rel_l2
from oracle.ac_oracle import OracleSolver

TOL = {  # (phi abs, u rel L2, P abs, mu abs, rho abs)
    ("float32", "short"): (2e-6, 5e-5, 1e-8, 1e-6, 1e-6),
    ("float64", "short"): (1e-13, 1e-12, 1e-17, 1e-13, 1e-13),
    ("float32", "long"): (1e-5, 1e-4, None, None, None),
}


def _run(name, dn):
    case = CASES[name]
    gd = golden(name, dn)
    solid, frac, C, u = inputs(case)
    s = OracleSolver(config(case), dtype=np.dtype(dn), **case["kw"])
    s.set_solid(solid, frac)
    s.init_fields(C, u)
    return case, gd, s


@pytest.mark.parametrize("name,dn", all_cases(long=False))
def test_setup_tables_bit_exact(name, dn):
    case, gd, s = _run(name, dn)
    if s.wetting is not None:
        assert np.array_equal(s.wetting.is_boundary, gd["is_boundary"])
        assert np.array_equal(s.wetting.wall_normal, gd["wall_normal"])
        assert np.array_equal(s.wetting.wall_weight, gd["wall_weight"])
        assert np.array_equal(s.wetting.near_wall_mask, gd["near_wall"])
    else:
        assert "is_boundary" not in gd
    if "partial" in gd:
        assert np.array_equal(s.partial, gd["partial"])
    assert np.array_equal(s.phi, gd["init_phi"])
    assert np.array_equal(s.mu_phi, gd["init_mu"])
    assert np.array_equal(s.p, gd["init_p"])
    if "init_f" in gd:
        assert np.array_equal(s.f, gd["init_f"])
        assert np.array_equal(s.g, gd["init_g"])


@pytest.mark.parametrize("name,dn", all_cases(long=False))
def test_steps_match_reference(name, dn):
    case, gd, s = _run(name, dn)
    tp, tu, tP, tmu, trho = TOL[(dn, "short")]
    ck = sorted(case["ckpt"])
    for k in range(1, ck[-1] + 1):
        s.step()
        if k in ck:
            assert np.abs(s.phi - gd[f"s{k}_phi"]).max() <= tp, k
            assert rel_l2(s.u, gd[f"s{k}_u"]) <= tu, k
            if f"s{k}_P" in gd:
                assert np.abs(s.P - gd[f"s{k}_P"]).max() <= tP
                assert np.abs(s.mu_phi - gd[f"s{k}_mu"]).max() <= tmu
                assert np.abs(s.rho - gd[f"s{k}_rho"]).max() <= trho


@pytest.mark.parametrize("name", ["flat_q120_long", "ridge_l162_long"])
def test_long_runs_match_reference(name):
    case, gd, s = _run(name, "float32")
    tp, tu = TOL[("float32", "long")][:2]
    n = sorted(case["ckpt"])[-1]
    masses = []
    for k in range(1, n + 1):
        s.step()
        if k % case["every"] == 0:
            masses.append(float(s.phi.astype(np.float64).sum()))
    assert np.abs(s.phi - gd[f"s{n}_phi"]).max() <= tp
    assert rel_l2(s.u, gd[f"s{n}_u"]) <= tu
    np.testing.assert_allclose(masses, gd["mass_every"], rtol=1e-6)
