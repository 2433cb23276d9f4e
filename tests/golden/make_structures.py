"""Generates tests/golden/structures.npz and tests/golden/structures_ref.npz: atoms of the reference's
sample structures.

Reads the MMTF files the reference ships (samples/*.mmtf in its checkout) with sesdf_gb300.mmtf, the
reader that follows the reference's loader, and stores each structure's (N, 4) float32 atoms under
its PDB id.
* structures.npz (GPU build against the FP64 oracle): the entries whose atoms all lie at least ~100
  float32 ulps from a reference-grid cell boundary (the reference's fast-math division then places
  every atom in the same cell as an IEEE division).
* structures_ref.npz (GPU build against the reference's own kernels, which share the fast-math grid
  division): 3EAM and 7DBB, which have atoms exactly on a cell boundary, and two larger entries, 1AON
  (58,870 atoms) and 7RGD (65,008 atoms, up to 119 neighbours per atom, next to the 128-slot rows).

    python tests/golden/make_structures.py <reference checkout>
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from sesdf_gb300 import mmtf  # noqa: E402

SETS = {"structures.npz": ("1AGA", "101M", "1VIS", "7SC0"),
        "structures_ref.npz": ("3EAM", "7DBB", "1AON", "7RGD")}


def main():
    ref = sys.argv[1]
    for name, entries in SETS.items():
        data = {e: mmtf.load(os.path.join(ref, "samples", f"{e}.mmtf")) for e in entries}
        np.savez_compressed(os.path.join(HERE, name), **data)
        for e, a in data.items():
            print(name, e, a.shape[0], "atoms")


if __name__ == "__main__":
    main()
