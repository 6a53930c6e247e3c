"""Package input generators and FEConfig against the reference's (golden digests)."""
import hashlib

import numpy as np
import pytest

from _cases import CASES, config, golden, inputs


@pytest.mark.parametrize("name", list(CASES))
def test_inputs_bit_identical(name):
    case = CASES[name]
    gd = golden(name, case["dtypes"][0])
    solid, frac, C, u = inputs(case)
    assert np.array_equal(solid, gd["solid"])
    if frac is not None:
        assert str(frac.dtype) == str(gd["fraction_dtype"])
        assert hashlib.sha256(np.ascontiguousarray(frac).tobytes()).hexdigest() == str(gd["fraction_sha256"])
    assert hashlib.sha256(np.ascontiguousarray(C).tobytes()).hexdigest() == str(gd["init_C_sha256"])
    assert hashlib.sha256(np.ascontiguousarray(u).tobytes()).hexdigest() == str(gd["init_u_sha256"])


@pytest.mark.parametrize("name", list(CASES))
def test_config_derivation(name):
    case = CASES[name]
    gd = golden(name, case["dtypes"][0])
    cfg = config(case)
    assert np.array_equal(np.array([cfg.beta, cfg.kappa, cfg.phi_c, cfg.M, cfg.sigma]), gd["cfg_derived"])


def test_lattice_tables():
    """The package's lattices carry the reference's population layout (the
    oracle's D3Q19 tables, lbm/lattice.py:10-96) and the derived attributes."""
    import numpy as np
    import torch
    import lbm
    from oracle.ac_oracle import E, OPP, W32
    d3 = lbm.D3Q19()
    assert np.array_equal(d3.e.numpy(), E.astype(np.float32)) and np.array_equal(d3.w.numpy(), W32)
    assert np.array_equal(d3.opp.numpy(), OPP) and d3.q == 19 and d3.dim == 3
    assert torch.equal(d3.ew, d3.e * d3.w[:, None]) and np.array_equal(d3.stream_shifts, -E)
    from oracle.ac_oracle import E2, OPP2, W2_32
    d2 = lbm.D2Q9()
    assert d2.q == 9 and d2.dim == 2 and abs(float(d2.w.double().sum()) - 1.0) < 1e-7
    assert np.array_equal(d2.e.numpy()[d2.opp.numpy()], -d2.e.numpy())
    assert np.array_equal(d2.e.numpy(), E2.astype(np.float32)) and np.array_equal(d2.w.numpy(), W2_32)
    assert np.array_equal(d2.opp.numpy(), OPP2)
