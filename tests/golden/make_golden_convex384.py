"""Golden fixture of the 384x384x256 convex-hemisphere case (the precision
form's large single solve), truncated to its first steps.

Runs pytorch-lbm's own AllenCahnSolver (imported read-only from --reference,
CPU, all host threads, float32: ~20 s per step) on the case --
create_substrate_with_fraction(384, 384, 256, 'convex', R_star=60/45, R_d=45),
droplet R = 45 at (192, 192, 180), u = (0, 0, -0.06), theta = 150,
alpha_geo = 1.5, sigma = 0.01424, tau_l = tau_g = 0.53 -- and stores a compact
fixture (the full fields are 37.7 M nodes):

  geo_sha256  SHA-256 of the wetting tables the solver computes
              (is_boundary, wall_normal, wall_weight, near_wall_mask)
  hist        every step: sum(phi) (float64 sum of the solver's phi) and max phi
  sK_phi_sub  phi at the last step on every 4th node in x and y (float32)
  sK_u_norm   ||u||_2 at that step (float64)

    python tests/golden/make_golden_convex384.py --reference /path/to/pytorch-lbm [--steps 20]
"""
import argparse
import contextlib
import hashlib
import io
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GRID = (384, 384, 256)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    ap.add_argument("--steps", type=int, default=20)
    args = ap.parse_args()
    sys.path.insert(0, args.reference)
    import torch
    torch.set_num_threads(os.cpu_count())
    from geometry.substrate import create_substrate_with_fraction
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.fe_config import FEConfig
    from lbm.fe_droplet import create_fe_droplet_with_impact
    nx, ny, nz = GRID
    cfg = FEConfig(nx=nx, ny=ny, nz=nz, rho_l=1.0, rho_g=1 / 828.0, sigma=0.01424, xi=4.0, tau_l=0.53,
                   tau_g=0.53, theta_eq=150.0, device="cpu", max_steps=args.steps)
    t = time.time()
    with contextlib.redirect_stdout(io.StringIO()):
        s = AllenCahnSolver(cfg, dtype=torch.float32, geo_amplification=1.5, geometric_wetting=True)
        solid, frac = create_substrate_with_fraction(nx, ny, nz, "convex", R_star=60.0 / 45.0, R_d=45.0)
        s.set_solid(solid, solid_fraction=frac)
        C, _, u = create_fe_droplet_with_impact(nx, ny, nz, center=(192, 192, 180), radius=45.0, xi=4.0,
                                                u_impact=(0, 0, -0.06))
        s.init_fields(C, u)
    w = s.wetting
    out = {"geo_sha256": np.array([sha(w.is_boundary.numpy()), sha(w.wall_normal.numpy()),
                                   sha(w.wall_weight.numpy()), sha(w.near_wall_mask.numpy())]),
           "init_mass": np.array(float(s.phi.double().sum()))}
    print(f"set-up {time.time() - t:.0f}s", flush=True)
    hist = []
    for k in range(1, args.steps + 1):
        s.step()
        hist.append([k, float(s.phi.double().sum()), float(s.phi.max())])
        print(hist[-1], f"{time.time() - t:.0f}s", flush=True)
    out["hist"] = np.array(hist)
    K = args.steps
    out[f"s{K}_phi_sub"] = np.ascontiguousarray(s.phi.numpy()[::4, ::4, :])
    out[f"s{K}_u_norm"] = np.array(np.linalg.norm(s.u.numpy().astype(np.float64)))
    np.savez_compressed(os.path.join(HERE, "convex384_ref_float32.npz"), **out)


if __name__ == "__main__":
    main()
