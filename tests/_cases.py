"""Inputs of the golden cases (tests/golden/make_golden.py CASES), built with
the package's own generators (bit-identical to the reference's)."""
import os

import numpy as np

from geometry.substrate import create_substrate, create_substrate_with_fraction
from lbm.fe_config import FEConfig
from lbm.fe_droplet import create_fe_droplet_with_impact
from make_golden import BASE_CFG, CASES

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def inputs(case):
    nx, ny, nz = case["grid"]
    sub = case["substrate"]
    if sub[0] == "flat_z2":
        # two wall layers at the bottom of the last axis (z in 3-D, y in 2-D)
        solid = np.zeros((nx, ny) if nz == 1 else (nx, ny, nz), dtype=bool)
        solid[..., :2] = True
        frac = solid.astype(np.float32)
    elif sub[0] == "fraction":
        solid, frac = create_substrate_with_fraction(nx, ny, nz, sub[1], R_star=sub[2], R_d=sub[3])
    else:
        solid = create_substrate(nx, ny, nz, sub[1], R_star=sub[2], R_d=sub[3])
        frac = None
    d = case["drop"]
    C, _, u = create_fe_droplet_with_impact(nx, ny, nz, center=d["center"], radius=d["radius"], xi=4.0,
                                            u_impact=d["u"])
    return solid, frac, C, u


def config(case, device="cpu"):
    nx, ny, nz = case["grid"]
    return FEConfig(nx=nx, ny=ny, nz=nz, device=device, **{**BASE_CFG, **case["cfg"]})


def golden(name, dtype_name):
    return np.load(os.path.join(GOLDEN, f"{name}_{dtype_name}.npz"))


def all_cases(long=True):
    out = []
    for name, case in CASES.items():
        if not long and ("long" in name or name.startswith("cfg1")):
            continue
        for dn in case["dtypes"]:
            out.append((name, dn))
    return out


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(np.asarray(b, np.float64)), 1e-300))
