"""The FP64 oracle on its own (CPU): geometric invariants of its outputs.

The reference has no tests or fixtures (its only check is the census of
app/circles/main.cu:13-87); these invariants are the ones that census and the
reference's kernels imply."""
import numpy as np
import pytest

from cases import hand_cases
from oracle import oracle
from sesdf_gb300 import synth

RP = 1.4


def check_invariants(atoms, o):
    n = atoms.shape[0]
    perm, srt = o["perm"], o["atoms"]
    assert sorted(perm.tolist()) == list(range(n))
    assert np.array_equal(srt, atoms[perm])
    noff, nbr, st = o["noff"], o["nbr"], o["status"]
    # neighbour lists ascending, no self, symmetric, predicate holds
    pairs = set()
    for i in range(n):
        row = nbr[noff[i]:noff[i + 1]]
        assert np.all(np.diff(row.astype(np.int64)) > 0)
        assert i not in row
        for j in row:
            pairs.add((i, int(j)))
            d2 = np.sum((srt[i, :3].astype(np.float64) - srt[j, :3]) ** 2)
            R = (srt[i, 3] + np.float64(np.float32(RP))) + (srt[j, 3] + np.float64(np.float32(RP)))
            assert d2 - R * R <= 1e-4 + 1e-9
    assert all((j, i) in pairs for (i, j) in pairs)
    assert set(np.unique(st).tolist()) <= {0, 1, 2}
    return pairs


@pytest.mark.parametrize("name", sorted(hand_cases().keys()))
@pytest.mark.parametrize("mode", ["full", "exterior"])
def test_hand_cases(name, mode):
    atoms = hand_cases()[name]
    o = oracle.run(atoms, RP, mode)
    check_invariants(atoms, o)


def probe_checks(o, rp=RP):
    srt = o["atoms"].astype(np.float64)
    ids, posd = o["ids"], o["posd"]
    for q in range(len(ids)):
        x = posd[q, :3]
        for t in ids[q, :3]:
            R = srt[t, 3] + np.float64(np.float32(rp))
            assert abs(np.linalg.norm(x - srt[t, :3]) - R) < 1e-6
    # singular probes first
    w = o["cids"][:, 3]
    Q = o["Q"]
    assert np.all(np.abs(w[:Q]) == 2) and np.all(np.abs(w[Q:]) == 1)


def test_globule_full():
    atoms = synth.globule(2000, 1000)
    o = oracle.run(atoms, RP, "full")
    check_invariants(atoms, o)
    probe_checks(o)
    # probes lie outside every other SAS sphere
    srt = o["atoms"].astype(np.float64)
    R = srt[:, 3] + np.float64(np.float32(RP))
    for q in range(0, len(o["ids"]), 7):
        x = o["posd"][q, :3]
        d = np.linalg.norm(srt[:, :3] - x, axis=1) - R
        others = np.setdiff1d(np.arange(len(srt)), o["ids"][q, :3])
        assert np.all(d[others] > -1e-9)
    # sector ranges partition the sector buffer; counts match visible circles
    cv = o["convex"]
    assert cv[0, 0] == 0 and cv[-1, 1] == len(o["sectors"])
    assert np.all(cv[1:, 0] == cv[:-1, 1])
    vis = np.array([np.count_nonzero(o["status"][o["noff"][i]:o["noff"][i + 1]]) for i in range(len(cv))])
    assert np.array_equal(cv[:, 1] - cv[:, 0], vis)
    # segments only on partial circles (app/circles/main.cu:52-55), from probes on that circle
    seg = o["segments"]
    slot_of = {}
    for i in range(len(cv)):
        for s in range(o["noff"][i], o["noff"][i + 1]):
            slot_of[(i, int(o["nbr"][s]))] = s
    for s in seg:
        assert o["status"][slot_of[(int(s[0]), int(s[1]))]] == 1
        for q in s[2:]:
            assert {int(s[0]), int(s[1])} <= set(o["ids"][q, :3].tolist())
    # every partial circle carries an even number of probes when counted with its segments
    assert len(seg) == int(np.sum(np.minimum(o["ccount"], 32) // 2))


def test_globule_exterior_tori():
    atoms = synth.globule(2000, 1000)
    o = oracle.run(atoms, RP, "exterior")
    check_invariants(atoms, o)
    probe_checks(o)
    st = o["status"]
    # j < i slots stay 0; tori are the status-2 slots
    assert o["tori"].shape[0] == int(np.sum(st == 2))
    # torus radius = circle radius, axis unit
    assert np.allclose(np.linalg.norm(o["tori"][:, 4:7], axis=1), 1.0)
    assert np.all(o["tori"][:, 7] == np.float64(np.float32(RP)))


def test_full_and_exterior_share_probes():
    atoms = synth.globule(2000, 1000)
    f = oracle.run(atoms, RP, "full")
    e = oracle.run(atoms, RP, "exterior")
    assert np.array_equal(f["posf"][:, :3], e["posf"][:, :3])
    assert np.array_equal(f["ids"][:, :3], e["ids"][:, :3])


def test_aabb_matches_reference_rule():
    atoms = synth.globule(500, 3)
    box = oracle.aabb(atoms)
    assert np.array_equal(box[:3], (atoms[:, :3] - atoms[:, 3:4]).min(0))
    assert np.array_equal(box[3:], (atoms[:, :3] + atoms[:, 3:4]).max(0))
