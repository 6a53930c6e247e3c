"""Fixture of the reference's code-verification suite: runs the set-ups of
scripts/verify_mms.py (tests/_verify_cases.py) on the reference itself,
imported read-only from --reference, on the CPU, and writes the measured
values to tests/golden/verify_mms_ref.json.

    python tests/golden/make_golden_verify.py --reference /path/to/pytorch-lbm
"""
import argparse
import contextlib
import io
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    args = ap.parse_args()
    sys.path.insert(0, args.reference)
    sys.path.insert(0, os.path.dirname(HERE))
    import torch
    torch.set_num_threads(os.cpu_count())
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.fe_config import FEConfig
    import _verify_cases as vc
    cl = (AllenCahnSolver, FEConfig)
    out = {}
    for name in ("mass_drift_pct", "flat_k", "energies", "ablation_k", "diameters"):
        with contextlib.redirect_stdout(io.StringIO()):
            r = getattr(vc, name)(classes=cl, device="cpu")
        out[name] = [float(x) for x in r] if isinstance(r, list) else float(r)
        print(name, out[name], flush=True)
    with open(os.path.join(HERE, "verify_mms_ref.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main()
