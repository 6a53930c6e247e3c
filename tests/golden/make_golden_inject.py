"""Golden fixtures of the reference's mid-run droplet injection
(AllenCahnSolver.inject_droplet, lbm/fe_ac_solver.py:645-732), made by
running the reference itself on the CPU:

    python tests/golden/make_golden_inject.py --reference /path/to/pytorch-lbm

Case: 32x28x30 grid, ridge substrate with solid fraction (R* = 1, R_d = 6),
droplet R = 6 at (16, 14, 20) with u = (0, 0, -0.03), theta = 150 deg,
alpha_geo = 1.5, boundary_relax = 0.3 (the default); 4 steps, then a second
droplet R = 5 at (11, 12, 21) with u = (0.01, 0, -0.02) overlapping the
first, then 4 more steps.  Stored: fields and populations right after the
injection (and, in float32, the populations) and the fields after the
further steps (float32 and float64).
"""
import argparse
import contextlib
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import BASE_CFG, build_inputs  # noqa: E402

INJECT_CASE = dict(
    grid=(32, 28, 30), substrate=("fraction", "ridge", 1.0, 6.0),
    drop=dict(center=(16, 14, 20), radius=6.0, u=(0.0, 0.0, -0.03)),
    cfg=dict(theta_eq=150.0), kw=dict(geo_amplification=1.5, geometric_wetting=True),
    before=4, after=4,
    inject=dict(center=(11.0, 12.0, 21.0), radius=5.0, xi=4.0, u_impact=(0.01, 0.0, -0.02)),
)


def run(ref, dtype_name):
    import torch
    case = INJECT_CASE
    nx, ny, nz = case["grid"]
    cfg = ref["FEConfig"](nx=nx, ny=ny, nz=nz, device="cpu", **{**BASE_CFG, **case["cfg"]})
    solid, frac, C, u = build_inputs(ref, case)
    out = {}
    with contextlib.redirect_stdout(io.StringIO()):
        s = ref["Solver"](cfg, dtype=getattr(torch, dtype_name), **case["kw"])
        s.set_solid(solid, solid_fraction=frac)
        s.init_fields(C, u)
        for _ in range(case["before"]):
            s.step()
        inj = case["inject"]
        s.inject_droplet(inj["center"], inj["radius"], inj["xi"], u_impact=inj["u_impact"])
    out["inj_phi"] = s.phi.numpy().copy()
    out["inj_u"] = s.u.numpy().copy()
    if dtype_name == "float32":
        out["inj_f"] = s.f.numpy().copy()
        out["inj_g"] = s.g.numpy().copy()
    out["inj_phi_mass_init"] = np.array(s.phi_mass_init)
    for _ in range(case["after"]):
        s.step()
    out["after_phi"] = s.phi.numpy().copy()
    out["after_u"] = s.u.numpy().copy()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    args = ap.parse_args()
    sys.path.insert(0, args.reference)
    import torch
    torch.set_num_threads(os.cpu_count())
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.fe_config import FEConfig
    from lbm import fe_droplet
    from geometry import substrate
    ref = dict(Solver=AllenCahnSolver, FEConfig=FEConfig, droplet=fe_droplet, substrate=substrate)
    for dn in ("float32", "float64"):
        np.savez_compressed(os.path.join(HERE, f"inject_ridge_{dn}.npz"), **run(ref, dn))
        print("wrote", dn, flush=True)


if __name__ == "__main__":
    main()
