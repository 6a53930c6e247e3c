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
