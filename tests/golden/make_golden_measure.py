"""Golden outputs of the reference's measurement functions (lbm/fe_measure.py).

Runs the reference's own measure_spread_factor and measure_contact_angle
(imported read-only from the path given by --reference) on the phi fields of
the committed golden fixtures and on a 2-D slice of one, and stores the
results in fe_measure_ref.json; tests/test_fe_measure.py checks the package's
lbm.fe_measure against them.

    python tests/golden/make_golden_measure.py --reference /path/to/pytorch-lbm
"""
import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# (fixture, phi key): fields with a wall below, an impact and a static droplet
FIELDS = [("cfg1_flat64_float32.npz", "s500_phi"), ("cfg1_flat64_float64.npz", "s500_phi"),
          ("ridge_l162_long_float32.npz", "s100_phi"), ("flat_q120_long_float32.npz", "s100_phi"),
          ("ridge_l162_float32.npz", "init_phi"), ("convex_l150_float32.npz", "s5_phi")]


def inputs():
    """name -> (phi, solid) of every measured field, 3-D and one 2-D slice."""
    out = {}
    for fn, key in FIELDS:
        z = np.load(os.path.join(HERE, fn))
        out[f"{fn[:-4]}:{key}"] = (z[key], z["solid"])
    phi, solid = out["cfg1_flat64_float32:s500_phi"]
    out["cfg1_flat64_float32:s500_phi:slice_y32"] = (np.ascontiguousarray(phi[:, 32, :]),
                                                     np.ascontiguousarray(solid[:, 32, :]))
    # spherical caps cut by a flat wall (solid z < 2), centre height zc: wetting
    # (zc below the wall top), neutral and non-wetting contact, in 3-D and 2-D
    nx, ny, nz = 48, 44, 32
    x, y, zz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    wall = zz < 2
    for zc in (-3.0, 2.0, 7.5):
        r = np.sqrt((x - 23.3) ** 2 + (y - 21.8) ** 2 + (zz - zc) ** 2)
        cap = (0.5 + 0.5 * np.tanh(2.0 * (12.0 - r) / 4.0)).astype(np.float32)
        cap[wall] = 0.0
        out[f"cap3d_zc{zc}"] = (cap, wall)
        out[f"cap2d_zc{zc}"] = (np.ascontiguousarray(cap[:, 22, :]), np.ascontiguousarray(wall[:, 22, :]))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    args = ap.parse_args()
    sys.path.insert(0, args.reference)
    from lbm.fe_measure import measure_contact_angle, measure_spread_factor
    res = {}
    for name, (phi, solid) in inputs().items():
        sp = measure_spread_factor(phi, solid)
        sp_nomask = measure_spread_factor(phi)
        ca = measure_contact_angle(phi, solid, axis="z" if phi.ndim == 3 else "y")
        res[name] = {"spread": {k: float(v) for k, v in sp.items()},
                     "spread_nomask": {k: float(v) for k, v in sp_nomask.items()},
                     "contact_angle": float(ca)}
    with open(os.path.join(HERE, "fe_measure_ref.json"), "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)
    print(json.dumps(res, indent=1)[:1500])


if __name__ == "__main__":
    main()
