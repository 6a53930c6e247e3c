"""How fast the 150x150x107 ridge droplet impact amplifies a rounding-level
change, measured on pytorch-lbm's own AllenCahnSolver (imported read-only from
--reference, CPU).

Two reference runs of the drop-in GPU case (ridge R* = 1, R_d = 22.5 with
smooth solid fraction, droplet R = 22.5 at (75, 75, 80), u = (0, 0, -0.05),
theta = 162, alpha_geo = 1.5, float32): one from the generator's initial phi,
one with every initial phi moved by -1, 0 or +1 float32 ulp (the seeded
perturbation the GPU ensemble tests use, seed 0).  Writes max|dphi| between
the two every 10 steps up to --steps to ridge150_ulp_divergence.json beside
this file, with the thread count used.

    python tests/golden/make_ulp_divergence.py --reference /path/to/pytorch-lbm [--steps 60]

About 2.5 minutes with 8 threads.
"""
import argparse
import contextlib
import io
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def perturbed(C, seed):
    r = np.random.default_rng(seed).integers(-1, 2, C.shape)
    return np.where(r > 0, np.nextafter(C, np.float32(2)),
                    np.where(r < 0, np.nextafter(C, np.float32(-1)), C)).astype(np.float32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args()
    sys.path.insert(0, a.reference)
    import torch
    torch.set_num_threads(os.cpu_count())
    from geometry.substrate import create_substrate_with_fraction
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.fe_config import FEConfig
    from lbm.fe_droplet import create_fe_droplet_with_impact
    cfg = FEConfig(nx=150, ny=150, nz=107, rho_l=1.0, rho_g=1 / 828.0, sigma=0.01424, xi=4.0, tau_l=0.53,
                   tau_g=0.53, theta_eq=162.0, device="cpu", max_steps=a.steps)
    solid, frac = create_substrate_with_fraction(150, 150, 107, "ridge", R_star=1.0, R_d=22.5)
    C, _, u = create_fe_droplet_with_impact(150, 150, 107, center=(75, 75, 80), radius=22.5, xi=4.0,
                                            u_impact=(0, 0, -0.05))
    runs = []
    with contextlib.redirect_stdout(io.StringIO()):
        for phi0 in (C, perturbed(C, a.seed)):
            s = AllenCahnSolver(cfg, dtype=torch.float32, geo_amplification=1.5, geometric_wetting=True)
            s.set_solid(solid, frac)
            s.init_fields(phi0, u)
            runs.append(s)
    table = []
    for k in range(1, a.steps + 1):
        for s in runs:
            s.step()
        if k % 10 == 0:
            d = float((runs[0].phi - runs[1].phi).abs().max())
            table.append({"step": k, "max_abs_dphi": d})
            print(k, d, flush=True)
    out = {"case": "ridge 150x150x107, theta 162, alpha_geo 1.5, float32",
           "perturbation": f"initial phi moved by -1/0/+1 float32 ulp per node, numpy default_rng({a.seed})",
           "threads": torch.get_num_threads(), "torch": torch.__version__, "table": table}
    path = os.path.join(HERE, "ridge150_ulp_divergence.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1)
    print(path)


if __name__ == "__main__":
    main()
