"""Writes rep_powders.npz: the reference's repulsion powder sets crystals/rep{100,144,320,678}
(3 columns: phi, theta, weight; gamma = 0), read with this package's own powder-file reader
(the reference's column rules, powder.cc:333-389).  The seeded c3/c4 workloads draw their
144/320/678-crystallite powders (rep678 holds 677 points) and the 100-crystallite powder of
the large serving jobs from this file.

    python blochlib_gb300/data/make_powders.py   (reference tree: BLOCHLIB_REF, resolved
                                                  by oracle/build_ref.sh)
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
import blochlib_gb300 as bl  # noqa: E402


def main():
    from blochlib_gb300.build import reference_tree
    ref = reference_tree()
    if ref is None:
        sys.exit("reference tree not found (set BLOCHLIB_REF)")
    out = {}
    for n in (100, 144, 320, 678):
        pw = bl.powder.read(ref / "crystals" / f"rep{n}")
        theta, phi, gamma, w = pw.arrays()
        out[f"rep{n}"] = np.stack([phi, theta, gamma, w])
    np.savez_compressed(HERE / "rep_powders.npz", **out)
    for k, v in out.items():
        print(k, v.shape[1], "points")


if __name__ == "__main__":
    main()
