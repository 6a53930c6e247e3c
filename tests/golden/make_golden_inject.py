"""Golden fixtures of the reference's mid-run droplet injection
(AllenCahnSolver.inject_droplet, lbm/fe_ac_solver.py:645-732), made by
running the reference itself on the CPU:

    python tests/golden/make_golden_inject.py --reference /path/to/pytorch-lbm [--case 3d|2d]

Case: 32x28x30 grid, ridge substrate with solid fraction (R* = 1, R_d = 6),
droplet R = 6 at (16, 14, 20) with u = (0, 0, -0.03), theta = 150 deg,
alpha_geo = 1.5, boundary_relax = 0.3 (the default); 4 steps, then a second
droplet R = 5 at (11, 12, 21) with u = (0.01, 0, -0.02) overlapping the
first, then 4 more steps.  Stored: fields and populations right after the
injection (and, in float32, the populations) and the fields after the
further steps (float32 and float64).

2-D case (INJECT_CASE_2D, D2Q9): 64x48 grid, ridge with solid fraction
(R* = 1, R_d = 8), droplet R = 8 at (32, 19) with u = (0, -0.03), the same
options; a second droplet R = 6 at (24, 24) with u = (0.01, -0.02).
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

INJECT_CASE_2D = dict(
    grid=(64, 48, 1), substrate=("fraction", "ridge", 1.0, 8.0),
    drop=dict(center=(32, 19), radius=8.0, u=(0.0, -0.03)),
    cfg=dict(theta_eq=150.0), kw=dict(geo_amplification=1.5, geometric_wetting=True),
    before=4, after=4,
    inject=dict(center=(24.0, 24.0), radius=6.0, xi=4.0, u_impact=(0.01, -0.02)),
)


def run(ref, dtype_name, case=INJECT_CASE):
    import torch
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
    ap.add_argument("--case", default="3d", choices=["3d", "2d"])
    args = ap.parse_args()
    sys.path.insert(0, args.reference)
    import torch
    torch.set_num_threads(os.cpu_count())
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.fe_config import FEConfig
    from lbm import fe_droplet
    from geometry import substrate
    ref = dict(Solver=AllenCahnSolver, FEConfig=FEConfig, droplet=fe_droplet, substrate=substrate)
    case, stem = (INJECT_CASE, "inject_ridge") if args.case == "3d" else (INJECT_CASE_2D, "inject_ridge2d")
    for dn in ("float32", "float64"):
        np.savez_compressed(os.path.join(HERE, f"{stem}_{dn}.npz"), **run(ref, dn, case))
        print("wrote", stem, dn, flush=True)


if __name__ == "__main__":
    main()
