"""The oracle pinned against the reference's own CUDA kernels (golden fixtures).

tests/golden/*.npz hold outputs of the reference kernels, built from the
reference's sources and run on a GB300 by tests/golden/make_golden.py. Every
difference between them and the FP64 oracle must lie in the degeneracy band
(tests/refcompare.py states the band widths); geometry agrees to 1e-4 A.
"""
import glob
import os

import numpy as np
import pytest

import refcompare
from oracle import oracle

GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "*.npz"))
                if p.endswith(("_full.npz", "_exterior.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference_kernels(path):
    g = dict(np.load(path))
    name = os.path.basename(path)[:-4]
    mode = "full" if name.endswith("_full") else "exterior"
    atoms, box, rp = g["atoms"], g["box"], float(g["probe_radius"])
    cap = int(g["max_nbr"]) if "max_nbr" in g else 128
    o = oracle.run(atoms, rp, mode, box=box, max_nbr=cap)
    rep = refcompare.compare(atoms, rp, mode, g, o)
    print(name, rep)
    assert rep["nbr_unexplained"] == 0
    assert rep["status_unexplained"] == 0
    assert rep["probe_unexplained"] == 0
    assert rep["probe_pos_over_1e-4"] == 0, rep
    if mode == "full":
        assert rep["segment_unexplained"] == 0
        assert rep["full_unexplained"] == 0
        assert rep["sector_max_err"] < 1e-4
    else:
        assert rep["tori_unexplained"] == 0
        assert rep["tori_max_err"] < 1e-4


def test_golden_fixtures_present():
    names = {os.path.basename(p)[:-4] for p in GOLDEN}
    assert "globule2k_full" in names and "globule2k_exterior" in names
    # probe 2.4 A on the reference's 288-slot library
    assert {"globule2k_rp24_full", "globule2k_rp24_exterior", "1AGA_rp24_full", "101M_rp24_full"} <= names
