"""Golden fixture of the 150x150x107 ridge droplet-impact case (2000 steps).

Runs pytorch-lbm's own AllenCahnSolver (imported read-only from --reference,
CPU, all host threads: about 40 min in float32 and several hours in float64
on an 8-thread host) on the drop-in GPU
case -- ridge R* = 1, R_d = 22.5 with smooth solid fraction, droplet R = 22.5 at
(75, 75, 80), u = (0, 0, -0.05), theta = 162, alpha_geo = 1.5, sigma = 0.01424,
tau_l = tau_g = 0.53, other solver arguments at their defaults -- and stores a
compact fixture:

  hist     every 50 steps: step, sum(phi) (float64 sum of the solver's phi),
           Dx, Dy, Dz, k = Dx/Dy, z centre of the phi > 0.5 fluid set, max phi
  sK_phi_q phi at steps K in (100, 500, 2000) quantised to uint16 (phi * 65535,
           rounded; resolution 1.5e-5, far below the 1e-4 parity bound)
  sK_u_norm  ||u||_2 at those steps (float64)

    python tests/golden/make_golden_ridge150.py --reference /path/to/pytorch-lbm [--dtype float32]
    python tests/golden/make_golden_ridge150.py --from-npz RUN.npz --dtype float32

--from-npz converts the raw output of an earlier run of this script's
--raw-out option instead of re-running the reference.
"""
import argparse
import contextlib
import io
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CKPT = (1, 10, 100, 500, 1000, 2000)
KEEP = (100, 500, 2000)


def run_reference(ref_path, dtype_name, raw_out):
    sys.path.insert(0, ref_path)
    import torch
    torch.set_num_threads(os.cpu_count())
    from geometry.substrate import create_substrate_with_fraction
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.fe_config import FEConfig
    from lbm.fe_droplet import create_fe_droplet_with_impact
    cfg = FEConfig(nx=150, ny=150, nz=107, rho_l=1.0, rho_g=1 / 828.0, sigma=0.01424, xi=4.0, tau_l=0.53,
                   tau_g=0.53, theta_eq=162.0, device="cpu", max_steps=2000)
    with contextlib.redirect_stdout(io.StringIO()):
        s = AllenCahnSolver(cfg, dtype=getattr(torch, dtype_name), geo_amplification=1.5, geometric_wetting=True)
        solid, frac = create_substrate_with_fraction(150, 150, 107, "ridge", R_star=1.0, R_d=22.5)
        s.set_solid(solid, solid_fraction=frac)
        C, _, u = create_fe_droplet_with_impact(150, 150, 107, center=(75, 75, 80), radius=22.5, xi=4.0,
                                                u_impact=(0, 0, -0.05))
        s.init_fields(C, u)
    out, hist, t = {}, [], time.time()
    for k in range(1, 2001):
        s.step()
        if k % 50 == 0:
            ph = s.phi.numpy()
            co = np.argwhere((ph > 0.5) & ~solid)
            Dx, Dy, Dz = (float(np.ptp(co[:, a]) + 1) for a in range(3))
            hist.append([k, float(s.phi.double().sum()), Dx, Dy, Dz, Dx / Dy, float(co[:, 2].mean()),
                         float(ph.max())])
            print(dtype_name, hist[-1], f"{time.time() - t:.0f}s", flush=True)
        if k in CKPT:
            out[f"s{k}_phi"] = s.phi.numpy().copy()
            out[f"s{k}_u"] = s.u.numpy().copy()
            np.savez(raw_out, hist=np.array(hist), **out)
    return raw_out


def compact(raw_npz, dtype_name):
    d = np.load(raw_npz)
    out = {"hist": d["hist"]}
    for k in KEEP:
        if f"s{k}_phi" in d:
            out[f"s{k}_phi_q"] = np.round(np.clip(d[f"s{k}_phi"], 0, 1) * 65535.0).astype(np.uint16)
            out[f"s{k}_u_norm"] = np.array(np.linalg.norm(d[f"s{k}_u"].astype(np.float64)))
    path = os.path.join(HERE, f"ridge150_ref_{dtype_name}.npz")
    np.savez_compressed(path, **out)
    return path


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference")
    ap.add_argument("--from-npz")
    ap.add_argument("--raw-out", default="ridge150_raw.npz")
    ap.add_argument("--dtype", default="float32")
    a = ap.parse_args()
    raw = a.from_npz or run_reference(a.reference, a.dtype, a.raw_out)
    print(compact(raw, a.dtype))


if __name__ == "__main__":
    main()
