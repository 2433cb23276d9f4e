"""Canonical forms of SES build outputs, for comparisons between implementations.

Sorted ids (reference-grid order) are mapped back to input ids with each side's
permutation; probes are keyed by their sorted input-id triplet and the side of
the triplet's plane they lie on; segments by their circle and probe keys.
Works on the dicts produced by oracle.run, SesBuild.fetch and RefBuild.fetch.
"""
from __future__ import annotations

import numpy as np


def neighbor_sets(perm, nbr_count, nbr_rows) -> dict:
    """input id -> frozenset of neighbour input ids."""
    out = {}
    for s in range(len(perm)):
        row = nbr_rows[s][: nbr_count[s]]
        out[int(perm[s])] = frozenset(int(perm[j]) for j in row)
    return out


def csr_rows(noff, nbr):
    counts = np.diff(noff)
    rows = [nbr[noff[i]:noff[i + 1]] for i in range(len(counts))]
    return counts, rows


def status_map(perm, nbr_count, nbr_rows, status_rows, exterior: bool = False) -> dict:
    """(input i, input j) -> status of the directed circle; exterior keeps only sorted i < j."""
    out = {}
    for s in range(len(perm)):
        for q in range(nbr_count[s]):
            j = int(nbr_rows[s][q])
            if exterior and not s < j:
                continue
            out[(int(perm[s]), int(perm[j]))] = int(status_rows[s][q])
    return out


def side(atoms_in, trip, x) -> int:
    a, b, c = (np.asarray(atoms_in[t, :3], np.float64) for t in trip)
    d = np.dot(np.cross(b - a, c - a), np.asarray(x[:3], np.float64) - a)
    return 1 if d > 0 else (-1 if d < 0 else 0)


def probe_keys(atoms_in, perm, ids, pos) -> list:
    """Key per probe: (sorted input-id triplet, side of the plane)."""
    keys = []
    for q in range(len(ids)):
        trip = tuple(sorted(int(perm[t]) for t in ids[q][:3]))
        keys.append((trip, side(atoms_in, trip, pos[q])))
    return keys


def segment_set(perm, segments, keys) -> set:
    out = set()
    for s in segments:
        circle = frozenset((int(perm[s[0]]), int(perm[s[1]])))
        out.add((circle, frozenset((keys[int(s[2])], keys[int(s[3])]))))
    return out


def pair_set(perm, pairs) -> set:
    return {frozenset((int(perm[p[0]]), int(perm[p[1]]))) for p in pairs}


def written_probe_nbrs(probe_nbrs, probe_ids, q_count) -> np.ndarray:
    """The written entries of the singular probes' 32-entry neighbour blocks (probe q's first
    probe_ids[q, 3] entries, q < q_count), concatenated; the rest of a block is never written."""
    blocks = np.asarray(probe_nbrs, np.float32).reshape(-1, 32, 4)
    rows = [blocks[q, :max(0, min(32, int(probe_ids[q, 3])))] for q in range(int(q_count))]
    return np.concatenate(rows) if rows else np.zeros((0, 4), np.float32)
