"""Generates tests/golden/structures.npz: atoms of the reference's sample structures.

Reads the MMTF files the reference ships (samples/*.mmtf in its checkout) with sesdf_gb300.mmtf, the
reader that follows the reference's loader, and stores each structure's (N, 4) float32 atoms under
its PDB id. Kept: the entries whose atoms all lie at least ~100 float32 ulps from a reference-grid cell
boundary (the reference's fast-math division then places every atom in the same cell as an IEEE
division); 3EAM and 7DBB have atoms exactly on a boundary and are left out.

    python tests/golden/make_structures.py <reference checkout> [out.npz]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from sesdf_gb300 import mmtf  # noqa: E402

ENTRIES = ("1AGA", "101M", "1VIS", "7SC0")


def main():
    ref = sys.argv[1]
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(HERE, "structures.npz")
    data = {e: mmtf.load(os.path.join(ref, "samples", f"{e}.mmtf")) for e in ENTRIES}
    np.savez_compressed(out, **data)
    for e, a in data.items():
        print(e, a.shape[0], "atoms")


if __name__ == "__main__":
    main()
