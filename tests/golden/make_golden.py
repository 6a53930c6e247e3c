"""Generate the golden fixtures in tests/golden/ by running the reference itself.

Runs pytorch-lbm's own AllenCahnSolver (imported read-only from the path given
by --reference, on the CPU) on small seeded cases and on the 64x64x48
flat-wall static-droplet case, and stores its setup tables and fields.  The
fixtures pin the numpy oracle (tests/test_oracle_golden.py) and the CUDA path
(tests/test_gpu_parity.py); neither test reads the reference at run time.

    python tests/golden/make_golden.py --reference /path/to/pytorch-lbm [--only NAME]

Inputs come from the reference's own generators (geometry/substrate.py,
lbm/fe_droplet.py) with the arguments recorded in CASES; the product's
generators reproduce them bit for bit (tests/test_generators.py).
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


def alpha_ramp(grid, lo, hi):
    """Per-node geometric amplification field rising linearly in x from lo to
    hi (float32): part of the wall has alpha <= 1 (amplification off there),
    part alpha > 1, as in the adaptive-alpha runs of
    scripts/adaptive_alpha_study.py:157-160."""
    nx, ny, nz = grid
    ramp = (np.float32(lo) + np.float32(hi - lo) * np.arange(nx, dtype=np.float32) / np.float32(nx - 1))
    if nz == 1:  # a 2-D grid
        return np.ascontiguousarray(np.broadcast_to(ramp[:, None], (nx, ny)), dtype=np.float32)
    return np.ascontiguousarray(np.broadcast_to(ramp[:, None, None], (nx, ny, nz)), dtype=np.float32)


# name: grid, substrate, droplet, solver kwargs, config overrides, dtypes, checkpoints
CASES = {
    # Short runs (steps 1 and 5) on small grids: every stage's output at step 1.
    "flat_q120": dict(
        grid=(24, 24, 20), substrate=("flat_z2",), drop=dict(center=(12, 12, 7), radius=6.0, u=(0, 0, 0)),
        cfg=dict(theta_eq=120.0), kw=dict(geo_amplification=1.5, geometric_wetting=True),
        dtypes=("float32", "float64"), ckpt=(1, 5), save_f=True),
    "ridge_l162": dict(
        grid=(32, 32, 28), substrate=("fraction", "ridge", 1.0, 6.0), drop=dict(center=(16, 16, 15), radius=6.0, u=(0, 0, -0.05)),
        cfg=dict(theta_eq=162.0), kw=dict(geo_amplification=1.5, geometric_wetting=True),
        dtypes=("float32", "float64"), ckpt=(1, 5), save_f=False),
    "convex_l150": dict(
        grid=(32, 32, 30), substrate=("fraction", "convex", 4.0 / 3.0, 6.0), drop=dict(center=(16, 16, 24), radius=6.0, u=(0, 0, -0.06)),
        cfg=dict(theta_eq=150.0, tau_h=0.57), kw=dict(geo_amplification=1.5, geometric_wetting=True, boundary_relax=0.0),
        dtypes=("float32",), ckpt=(1, 5), save_f=False),
    "concave_q100_tau": dict(
        grid=(32, 32, 24), substrate=("fraction", "concave", 1.0, 8.0), drop=dict(center=(16, 16, 16), radius=6.0, u=(0.01, 0, -0.04)),
        cfg=dict(theta_eq=100.0, tau_g=0.6), kw=dict(),
        dtypes=("float32",), ckpt=(1, 5), save_f=False),
    "discrete_l162": dict(
        grid=(32, 32, 28), substrate=("mask", "ridge", 1.0, 6.0), drop=dict(center=(16, 16, 15), radius=6.0, u=(0, 0, -0.05)),
        cfg=dict(theta_eq=162.0), kw=dict(geo_amplification=1.8, geometric_wetting=True, boundary_relax=0.0),
        dtypes=("float32",), ckpt=(1, 5), save_f=False),
    "ridge_alpha_field": dict(
        grid=(32, 32, 28), substrate=("fraction", "ridge", 1.0, 6.0), drop=dict(center=(16, 16, 15), radius=6.0, u=(0, 0, -0.05)),
        cfg=dict(theta_eq=162.0), kw=dict(geo_amplification=alpha_ramp((32, 32, 28), 0.6, 2.4), geometric_wetting=True),
        dtypes=("float32", "float64"), ckpt=(1, 5), save_f=False),
    "ch_flat_q120": dict(
        grid=(24, 24, 20), substrate=("flat_z2",), drop=dict(center=(12, 12, 7), radius=6.0, u=(0, 0, -0.01)),
        cfg=dict(theta_eq=120.0), kw=dict(interface_mode="cahn-hilliard", geometric_wetting=True),
        dtypes=("float32", "float64"), ckpt=(1, 5), save_f=False),
    "mudrive_ridge_l150": dict(
        grid=(32, 32, 28), substrate=("fraction", "ridge", 1.0, 6.0), drop=dict(center=(16, 16, 15), radius=6.0, u=(0, 0, -0.05)),
        cfg=dict(theta_eq=150.0), kw=dict(mu_drive=0.5, geo_amplification=1.5, geometric_wetting=True),
        dtypes=("float32", "float64"), ckpt=(1, 5), save_f=False),
    "direct_ridge_l150": dict(
        grid=(32, 32, 28), substrate=("fraction", "ridge", 1.0, 6.0), drop=dict(center=(16, 16, 11), radius=6.0, u=(0, 0, -0.05)),
        cfg=dict(theta_eq=150.0), kw=dict(direct_wetting=True, geo_amplification=1.5, geometric_wetting=True),
        dtypes=("float32", "float64"), ckpt=(1, 5), save_f=False),
    "direct_flat_q120": dict(
        grid=(24, 24, 20), substrate=("flat_z2",), drop=dict(center=(12, 12, 7), radius=6.0, u=(0, 0, 0)),
        cfg=dict(theta_eq=120.0), kw=dict(direct_wetting=True, boundary_relax=0.5),
        dtypes=("float32",), ckpt=(1, 5), save_f=False),
    "nowet_liang_grav": dict(
        grid=(24, 24, 20), substrate=("flat_z2",), drop=dict(center=(12, 12, 8), radius=5.0, u=(0, 0, -0.02)),
        cfg=dict(theta_eq=90.0, g_force=(0.0, 0.0, -1e-6)), kw=dict(stab_mode="liang"),
        dtypes=("float32",), ckpt=(1, 5), save_f=False),
    # Longer runs need gas room: in a box only ~2 droplet diameters wide the gas
    # between periodic images keeps phi ~ 1e-2 at points where grad(phi) = 0,
    # and the sharpening normal grad/|grad| there is set by rounding noise.
    "flat_q120_long": dict(
        grid=(44, 44, 32), substrate=("flat_z2",), drop=dict(center=(22, 22, 7), radius=6.0, u=(0, 0, 0)),
        cfg=dict(theta_eq=120.0), kw=dict(geo_amplification=1.5, geometric_wetting=True),
        dtypes=("float32",), ckpt=(100,), save_f=False, every=10),
    "ridge_l162_long": dict(
        grid=(48, 44, 40), substrate=("fraction", "ridge", 1.0, 6.0), drop=dict(center=(24, 22, 15), radius=6.0, u=(0, 0, -0.05)),
        cfg=dict(theta_eq=162.0), kw=dict(geo_amplification=1.5, geometric_wetting=True),
        dtypes=("float32",), ckpt=(100,), save_f=False, every=10),
    # 2-D (nz = 1, D2Q9) grids: the wall at the bottom of y.
    "flat2d_q120": dict(
        grid=(48, 40, 1), substrate=("flat_z2",), drop=dict(center=(24, 11), radius=8.0, u=(0, 0)),
        cfg=dict(theta_eq=120.0), kw=dict(geo_amplification=1.5, geometric_wetting=True),
        dtypes=("float32", "float64"), ckpt=(1, 5), save_f=True),
    "ridge2d_l162": dict(
        grid=(64, 48, 1), substrate=("fraction", "ridge", 1.0, 8.0), drop=dict(center=(32, 19), radius=8.0, u=(0, -0.05)),
        cfg=dict(theta_eq=162.0), kw=dict(geo_amplification=1.5, geometric_wetting=True),
        dtypes=("float32", "float64"), ckpt=(1, 5), save_f=False),
    "discrete2d_l150": dict(
        grid=(64, 48, 1), substrate=("mask", "convex", 4.0 / 3.0, 8.0), drop=dict(center=(32, 30), radius=8.0, u=(0, -0.06)),
        cfg=dict(theta_eq=150.0, tau_h=0.57), kw=dict(geo_amplification=1.5, geometric_wetting=True, boundary_relax=0.0),
        dtypes=("float32",), ckpt=(1, 5), save_f=False),
    "concave2d_q100_tau": dict(
        grid=(64, 48, 1), substrate=("fraction", "concave", 1.0, 10.0), drop=dict(center=(32, 18), radius=8.0, u=(0.01, -0.04)),
        cfg=dict(theta_eq=100.0, tau_g=0.6, g_force=(0.0, -1e-6, 0.0)), kw=dict(stab_mode="liang"),
        dtypes=("float32",), ckpt=(1, 5), save_f=False),
    "ch2d_q120": dict(
        grid=(48, 40, 1), substrate=("flat_z2",), drop=dict(center=(24, 11), radius=8.0, u=(0, -0.01)),
        cfg=dict(theta_eq=120.0), kw=dict(interface_mode="cahn-hilliard", geometric_wetting=True),
        dtypes=("float32", "float64"), ckpt=(1, 5), save_f=False),
    "direct2d_l150": dict(
        grid=(64, 48, 1), substrate=("fraction", "ridge", 1.0, 8.0), drop=dict(center=(32, 15), radius=8.0, u=(0, -0.05)),
        cfg=dict(theta_eq=150.0), kw=dict(direct_wetting=True, mu_drive=0.5, geo_amplification=1.5, geometric_wetting=True),
        dtypes=("float32", "float64"), ckpt=(1, 5), save_f=False),
    "ridge2d_alpha_field": dict(
        grid=(64, 48, 1), substrate=("fraction", "ridge", 1.0, 8.0), drop=dict(center=(32, 19), radius=8.0, u=(0, -0.05)),
        cfg=dict(theta_eq=162.0), kw=dict(geo_amplification=alpha_ramp((64, 48, 1), 0.6, 2.4), geometric_wetting=True),
        dtypes=("float32", "float64"), ckpt=(1, 5), save_f=False),
    "ridge2d_long": dict(
        grid=(128, 64, 1), substrate=("fraction", "ridge", 1.0, 8.0), drop=dict(center=(64, 19), radius=8.0, u=(0, -0.05)),
        cfg=dict(theta_eq=162.0), kw=dict(geo_amplification=1.5, geometric_wetting=True),
        dtypes=("float32",), ckpt=(200,), save_f=False, every=20),
    # The 64x64x48 flat-wall, theta=120 static droplet case, full 500-step run.
    "cfg1_flat64": dict(
        grid=(64, 64, 48), substrate=("flat_z2",), drop=dict(center=(32, 32, 14), radius=12.0, u=(0, 0, 0)),
        cfg=dict(theta_eq=120.0), kw=dict(geo_amplification=1.5, geometric_wetting=True),
        dtypes=("float32", "float64"), ckpt=(500,), save_f=False, every=50, phi_only_f64=True),
}

BASE_CFG = dict(rho_l=1.0, rho_g=1.0 / 828.0, sigma=0.01424, xi=4.0, tau_l=0.53, tau_g=0.53)


def build_inputs(ref, case):
    nx, ny, nz = case["grid"]
    sub = case["substrate"]
    if sub[0] == "flat_z2":
        # two wall layers at the bottom of the last axis (z in 3-D, y in 2-D)
        solid = np.zeros((nx, ny) if nz == 1 else (nx, ny, nz), dtype=bool)
        solid[..., :2] = True
        frac = solid.astype(np.float32)
    elif sub[0] == "fraction":
        solid, frac = ref["substrate"].create_substrate_with_fraction(
            nx, ny, nz, substrate_type=sub[1], R_star=sub[2], R_d=sub[3])
    else:
        solid = ref["substrate"].create_substrate(nx, ny, nz, substrate_type=sub[1],
                                                  R_star=sub[2], R_d=sub[3])
        frac = None
    d = case["drop"]
    C, _, u = ref["droplet"].create_fe_droplet_with_impact(
        nx, ny, nz, center=d["center"], radius=d["radius"], xi=4.0, u_impact=d["u"])
    return solid, frac, C, u


def run_case(ref, name, case, dtype_name):
    import torch
    nx, ny, nz = case["grid"]
    cfg = ref["FEConfig"](nx=nx, ny=ny, nz=nz, device="cpu", **{**BASE_CFG, **case["cfg"]})
    solid, frac, C, u = build_inputs(ref, case)
    dt = getattr(torch, dtype_name)
    out = {}
    # a per-node amplification field goes to the reference as a torch tensor
    kw = {k: (torch.from_numpy(v) if isinstance(v, np.ndarray) else v) for k, v in case["kw"].items()}
    with contextlib.redirect_stdout(io.StringIO()):
        s = ref["Solver"](cfg, dtype=dt, **kw)
        s.set_solid(solid, solid_fraction=frac)
        s.init_fields(C, u)
    out["solid"] = np.asarray(solid, dtype=bool)
    if frac is not None:
        out["fraction_sha256"] = np.array(hashlib.sha256(np.ascontiguousarray(frac).tobytes()).hexdigest())
        out["fraction_dtype"] = np.array(str(np.asarray(frac).dtype))
    out["init_C_sha256"] = np.array(hashlib.sha256(np.ascontiguousarray(C).tobytes()).hexdigest())
    out["init_u_sha256"] = np.array(hashlib.sha256(np.ascontiguousarray(u).tobytes()).hexdigest())
    out["cfg_derived"] = np.array([cfg.beta, cfg.kappa, cfg.phi_c, cfg.M, cfg.sigma])
    w = s.wetting
    if w is not None:
        out["is_boundary"] = w.is_boundary.numpy()
        out["wall_normal"] = w.wall_normal.numpy()
        out["wall_weight"] = w.wall_weight.numpy()
        out["near_wall"] = w.near_wall_mask.numpy()
    if s._has_partial:
        out["partial"] = s._partial_mask.numpy()
    out["init_phi"] = s.phi.numpy()
    out["init_mu"] = s.mu_phi.numpy()
    out["init_p"] = s.p.numpy()
    out["phi_mass_init"] = np.array(s.phi_mass_init)
    if case["save_f"] and dtype_name == "float32":
        out["init_f"] = s.f.numpy()
        out["init_g"] = s.g.numpy()
    ck = sorted(case["ckpt"])
    every = case.get("every")
    slim = dtype_name == "float64" and case.get("phi_only_f64")
    hist = []
    t0 = time.time()
    for k in range(1, ck[-1] + 1):
        s.step()
        if k in ck:
            out[f"s{k}_phi"] = s.phi.numpy().copy()
            if not slim:
                out[f"s{k}_u"] = s.u.numpy().copy()
            if k == ck[0] and not every:
                # every stage's output at the first checkpoint
                out[f"s{k}_P"] = s.P.numpy().copy()
                out[f"s{k}_mu"] = s.mu_phi.numpy().copy()
                out[f"s{k}_rho"] = s.rho.numpy().copy()
        if every and k % every == 0:
            hist.append(float(s.phi.double().sum()))
    if hist:
        out["mass_every"] = np.array(hist)
    print(f"{name}/{dtype_name}: {ck[-1]} steps in {time.time() - t0:.1f}s", flush=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    sys.path.insert(0, args.reference)
    import torch
    torch.set_num_threads(os.cpu_count())
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.fe_config import FEConfig
    from lbm import fe_droplet
    from geometry import substrate
    ref = dict(Solver=AllenCahnSolver, FEConfig=FEConfig, droplet=fe_droplet, substrate=substrate)
    for name, case in CASES.items():
        if args.only and name != args.only:
            continue
        for dn in case["dtypes"]:
            out = run_case(ref, name, case, dn)
            np.savez_compressed(os.path.join(HERE, f"{name}_{dn}.npz"), **out)


if __name__ == "__main__":
    main()
