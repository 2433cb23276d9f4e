"""Circles evaluated once (CPU): the oracle, like the GPU build, gives circle (i, j), j < i, of two complete
neighbour lists the status of (j, i) instead of evaluating it from atom i. The reference evaluates both
(sesdf/src/sesdf/operations.cu:126-204). This checks, on the oracle's own outputs, that evaluating every such
lower circle directly from atom i in double precision (computeCirclesVisibilityStatus restated) gives the
mirrored status, except where one of the tests lies inside the float32 band of tests/refcompare.py.
"""
import numpy as np
import pytest

import refcompare
from cases import hand_cases
from oracle import oracle
from sesdf_gb300 import synth

RP = 1.4


def direct_status(pos, rad, i, j, nbrs, rp):
    """Status of circle (i, j) evaluated from atom i over its neighbours (operations.cu:126-204 in FP64)."""
    c, n, r = refcompare.circle_geometry(pos[i], rad[i], pos[j], rad[j], rp)
    tol = refcompare._f(1e-4)
    visible, complete = True, True
    for k in nbrs:
        if k == j:
            continue
        Rk = rad[k] + rp
        v = c - pos[k]
        dist = np.sqrt(np.dot(v, v))
        second = np.dot(v, n)
        cos = second / dist
        sin = np.sqrt(1.0 - cos * cos)
        first = sin * dist + r
        if first * first + second * second - Rk * Rk < tol:
            visible = False
            break
        if complete:
            first = -sin * dist + r
            if first * first + second * second - Rk * Rk < tol:
                complete = False
    return int(visible) * (1 + int(complete))


def lower_circles(o, cap):
    noff, nbr = o["noff"], o["nbr"]
    cnt = np.diff(noff)
    for i in range(o["n"]):
        if cnt[i] >= cap:
            continue
        for s in range(noff[i], noff[i + 1]):
            j = int(nbr[s])
            if j < i and cnt[j] < cap:
                yield i, j, s


def check(atoms, cap=128):
    with np.errstate(invalid="ignore", divide="ignore"):
        o = oracle.run(atoms, RP, "full", max_nbr=cap)
        pos = o["atoms"][:, :3].astype(np.float64)
        rad = o["atoms"][:, 3].astype(np.float64)
        noff, nbr, st = o["noff"], o["nbr"], o["status"]
        rows = [set(int(x) for x in nbr[noff[a]:noff[a + 1]]) for a in range(o["n"])]
        checked = differ = 0
        for i, j, s in lower_circles(o, cap):
            checked += 1
            want = direct_status(pos, rad, i, j, sorted(rows[i]), RP)
            if want != int(st[s]):
                differ += 1
                margin = refcompare.status_margin(pos, rad, i, j, sorted(rows[i] | rows[j]), RP)
                assert margin < refcompare.WIDE, (i, j, want, int(st[s]), margin)
    return checked, differ


@pytest.mark.parametrize("n,seed", [(2000, 1000), (1500, 7)])
def test_mirrored_statuses_equal_direct_evaluation(n, seed):
    checked, differ = check(synth.globule(n, seed))
    assert checked > 10 * n  # most lower circles are mirrored
    assert differ == 0


def test_mirrored_statuses_on_hand_cases():
    # degenerate inputs (collinear stacks, tangent and co-spherical atoms): differences only in the band
    for name, atoms in hand_cases().items():
        check(atoms)


def test_truncated_lists_keep_both_evaluations():
    # with 40 neighbour slots some lists are cut: their circles are not mirrored, and the others still agree
    atoms = synth.globule(1500, 7)
    checked, differ = check(atoms, cap=40)
    o = oracle.run(atoms, RP, "full", max_nbr=40)
    full = int(np.count_nonzero(np.diff(o["noff"]) >= 40))
    assert full > 0 and checked > 0 and differ == 0
