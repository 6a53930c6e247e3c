"""Golden hashes of the reference's ASCII VTK writer (io_utils/vtk_writer.py).

Runs the reference's own write_vtk (imported read-only from the path given by
--reference) on the seeded inputs of vtk_cases() and stores the SHA-256 and
size of each file in vtk_sha256.json; tests/test_vtk_writer.py writes the same
inputs through the package's writer and compares the hashes.

    python tests/golden/make_golden_vtk.py --reference /path/to/pytorch-lbm
"""
import argparse
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def vtk_cases():
    """name -> (rho, u, solid, dx, step, t): a 3-D float32 snapshot with
    special values (NaN, infinities, signed zero, tiny and huge numbers), a
    float64 one without a solid mask, and a 2-D one."""
    rng = np.random.default_rng(20261203)
    rho = rng.uniform(0.0, 1.2, (7, 6, 5)).astype(np.float32)
    u = rng.normal(0.0, 0.03, (3, 7, 6, 5)).astype(np.float32)
    rho[0, 0, 0], rho[1, 2, 3], rho[2, 2, 2], rho[3, 1, 4] = np.nan, np.inf, -np.inf, -0.0
    u[0, 0, 0, 1], u[1, 4, 4, 4], u[2, 6, 5, 4] = 1e-42, 3.4e38, -np.nan
    solid = rng.uniform(0, 1, (7, 6, 5)) < 0.3
    cases = {"f32_3d": (rho, u, solid, 1.0, 150, 150.0)}
    rho64 = rng.uniform(0.0, 1.0, (4, 5, 6))
    u64 = rng.normal(0.0, 0.1, (3, 4, 5, 6))
    cases["f64_3d_nosolid"] = (rho64, u64, None, 0.5, 0, 0.0)
    rho2 = rng.uniform(0.0, 1.0, (9, 8)).astype(np.float32)
    u2 = rng.normal(0.0, 0.05, (2, 9, 8)).astype(np.float32)
    solid2 = np.zeros((9, 8), dtype=bool)
    solid2[:, :2] = True
    cases["f32_2d"] = (rho2, u2, solid2, 1.0, 7, 3.5e-3)
    return cases


def sha256_file(path):
    with open(path, "rb") as f:
        data = f.read()
    return hashlib.sha256(data).hexdigest(), len(data)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    args = ap.parse_args()
    sys.path.insert(0, args.reference)
    from io_utils.vtk_writer import write_vtk
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for name, (rho, u, solid, dx, step, t) in vtk_cases().items():
            path = os.path.join(d, name + ".vtk")
            write_vtk(path, rho, u, solid=solid, dx=dx, step=step, t=t)
            h, n = sha256_file(path)
            out[name] = {"sha256": h, "bytes": n}
    with open(os.path.join(HERE, "vtk_sha256.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(out)


if __name__ == "__main__":
    main()
