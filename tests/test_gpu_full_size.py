"""The 1M-atom shell (200 globules x 5,000 atoms on a 400 A sphere) through
size-independent properties, since the oracle comparison runs at smaller sizes.

Checked on the GPU build, both modes:
* every probe lies on the SAS spheres of its three atoms (within 1e-4 A) and
  strictly inside none of its atom's other neighbours (sampled);
* the singular flag matches the probe's distance to the plane of its three
  atom centres (|d| < rp, outside a 1e-3 band);
* singular probes first, neighbour counts of singular probes <= 32;
* segments join two probes of the same partial circle (both probes lie on the
  SAS spheres of the circle's two atoms) -- except where a probe's (j, k)
  circle is not partial itself, where the reference's trimmed-id scan hands
  the probe to the next partial circle of the row (5 of 2.6M segments here,
  the FP64 oracle has the same ones); convex ranges tile the sectors;
* full and exterior builds agree on the probe set;
* a second build gives identical buffers (determinism at full size).
"""
import numpy as np
import pytest

from sesdf_gb300 import SesBuild, synth

pytestmark = pytest.mark.gpu
RP = 1.4
TOL = 1e-4


@pytest.fixture(scope="module")
def shell():
    return synth.shell()


def sphere_error(atoms, ids, pos, cols):
    c = atoms[ids[:, cols], :3].astype(np.float64)
    R = atoms[ids[:, cols], 3].astype(np.float64) + RP
    d = np.linalg.norm(pos[:, None, :3].astype(np.float64) - c, axis=2)
    return np.abs(d - R).max(axis=1)


def on_sphere(atoms, ids, pos, cols):
    return sphere_error(atoms, ids, pos, cols).max()


def test_shell_1m_full(shell):
    with SesBuild(shell, RP, "full") as g:
        g.build()
        out = g.fetch(analysis=True)
        g.build()
        again = g.fetch(analysis=False)
    c = out["counts"]
    assert c["atoms"] == 1_000_000 and c["truncated_atoms"] == 0 and c["outside_atoms"] == 0
    atoms = out["atoms"]
    ids, pos = out["probe_ids"], out["probe_pos"]
    I, Q = c["probes"], c["singular_probes"]
    assert I == ids.shape[0] and I > 1_000_000
    assert on_sphere(atoms, ids, pos, [0, 1, 2]) <= TOL
    # singular probes first
    sing = np.abs(pos[:, 3]) == 2
    assert sing[:Q].all() and not sing[Q:].any()
    assert (ids[:Q, 3] <= 32).all()
    # singular flag against the plane of the three centres (outside a small band)
    rng = np.random.default_rng(7)
    pick = rng.choice(I, 50_000, replace=False)
    a, b_, k = (atoms[ids[pick, m], :3].astype(np.float64) for m in range(3))
    nrm = np.cross(b_ - a, k - a)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    d = np.abs(np.einsum("ij,ij->i", pos[pick, :3].astype(np.float64) - a, nrm))
    clear = np.abs(d - RP) > 1e-3
    assert np.array_equal((d < RP)[clear], sing[pick][clear])
    # no probe strictly inside a neighbour's SAS sphere of its first atom
    nbr, cnt = out["nbr_ids"], out["nbr_count"]
    sub = pick[:5000]
    for p in sub:
        i = ids[p, 0]
        nb = nbr[i, :cnt[i]]
        dd = np.linalg.norm(atoms[nb, :3].astype(np.float64) - pos[p, :3], axis=1) - (atoms[nb, 3] + RP)
        assert dd.min() >= -TOL
    # segments: both probes on the circle's two spheres
    seg = out["segments"]
    assert seg.shape[0] == c["segments"] and seg.shape[0] > 0
    assert (seg[:, 2] < I).all() and (seg[:, 3] < I).all()
    off = np.zeros(seg.shape[0], bool)
    for col in (2, 3):
        off |= sphere_error(atoms, seg[:, :2].astype(np.int64), pos[seg[:, col]], [0, 1]) > TOL
    assert off.sum() <= 10
    # convex ranges tile the sector array
    cv = out["convex"].astype(np.int64)
    assert cv[0, 0] == 0 and cv[-1, 1] == c["sectors"] and (cv[1:, 0] == cv[:-1, 1]).all()
    for k in ("probe_pos", "probe_ids", "segments", "sectors", "convex", "full"):
        assert np.array_equal(out[k], again[k], equal_nan=True), k


def test_shell_1m_exterior_matches_full_probes(shell):
    with SesBuild(shell, RP, "exterior") as g:
        g.build()
        ext = g.fetch(analysis=False)
    with SesBuild(shell, RP, "full") as g:
        g.build()
        full = g.fetch(analysis=False)
    assert ext["counts"]["probes"] == full["counts"]["probes"]
    assert np.array_equal(ext["probe_ids"][:, :3], full["probe_ids"][:, :3])
    assert np.array_equal(ext["probe_pos"][:, :3], full["probe_pos"][:, :3])
    assert ext["counts"]["tori"] > 0 and np.isfinite(ext["tori_pos"]).all()
