"""The FP64 error report (sesdf_gb300/precision.py) on the oracle's own outputs (CPU).

precision.py re-evaluates a build's probe positions, convex sectors and exterior tori in double precision and is
what the benchmark's error statement of the 1M-atom builds rests on. Applied to the FP64 oracle, it must find
the oracle's double-precision geometry (which follows the reference's formulas, e.g. the intersection of the
circles (i, j) and (i, k) of sesdf/include/bcs/sesdf/operations.inl:384-398, where precision.py uses the closed
form of the same point) equal to its own up to double rounding, and the float32 positions within rounding.
"""
import numpy as np
import pytest

from oracle import oracle
from sesdf_gb300 import precision, synth

RP = 1.4


def rows(o):
    """CSR neighbour lists and statuses of the oracle as [n, cap] rows, with the counts."""
    noff = o["noff"]
    cnt = np.diff(noff).astype(np.int64)
    cap = max(int(cnt.max()) if len(cnt) else 1, 1)
    n = len(cnt)
    ids = np.zeros((n, cap), np.uint32)
    st = np.zeros((n, cap), np.uint8)
    for i in range(n):
        ids[i, :cnt[i]] = o["nbr"][noff[i]:noff[i + 1]]
        st[i, :cnt[i]] = o["status"][noff[i]:noff[i + 1]]
    return ids, cnt, st


@pytest.fixture(scope="module")
def globule():
    return synth.globule(2000, 1000)


def test_probe_positions(globule):
    o = oracle.run(globule, RP, "full")
    assert len(o["ids"]) > 1000
    exact = precision.probe_error(o["atoms"], o["ids"], o["posd"], RP)
    rounded = precision.probe_error(o["atoms"], o["ids"], o["posf"], RP)
    # the closed form and the reference's circle intersection give one point in double precision
    assert exact["max_err_A"] < 1e-9 and exact["over_1e-4"] == 0
    # float32 storage: half an ulp of coordinates below 64 A
    assert 0.0 < rounded["max_err_A"] <= 2.0 ** -18 and rounded["over_1e-4"] == 0


def test_sectors(globule):
    o = oracle.run(globule, RP, "full")
    ids, cnt, st = rows(o)
    rep = precision.sector_error(o["atoms"], ids, cnt, st, o["sectors"], RP)
    assert rep["sectors"] == len(o["sectors"]) > 10000
    assert rep["axis_max_err"] < 1e-9 and rep["cos_max_err"] < 1e-9


def test_exterior_tori(globule):
    o = oracle.run(globule, RP, "exterior")
    ids, cnt, st = rows(o)
    t = np.asarray(o["tori"], np.float64).reshape(-1, 12)
    rep = precision.tori_error(o["atoms"], ids, cnt, st, t[:, 0:4], t[:, 4:8], t[:, 8:12], RP)
    assert rep["tori"] == len(t) > 1000
    assert rep["max_err"] < 1e-9
