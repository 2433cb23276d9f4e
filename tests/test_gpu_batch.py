"""Batched builds (sesgb_create_batch) against one build per molecule.

Molecule m's slice of a batch must equal, buffer for buffer and bit for bit,
what a SesBuild of that molecule alone produces: same reference-grid order,
same sectors, complete circles, probes (singular first within the molecule),
probe neighbours, segments or tori, and molecule-local ids throughout. The
batch mixes sizes (including an empty molecule, a single atom and a hand-made
degenerate cluster) so that the per-molecule grids, offsets and the
singular-first partition are exercised at their edges.
"""
import numpy as np
import pytest

import canon
from cases import hand_cases
from sesdf_gb300 import SesBatch, SesBuild, synth

pytestmark = pytest.mark.gpu
RP = 1.4


def molecules():
    hc = hand_cases()
    return [synth.globule(1200, 1301), hc["cluster40"], np.zeros((0, 4), np.float32), synth.globule(300, 1302),
            hc["single"], synth.globule(2500, 1303), hc["octahedron"], synth.globule(700, 1304)]


def plain(atoms, mode):
    with SesBuild(atoms, RP, mode) as g:
        g.build()
        out = g.fetch(analysis=True)
    return out


BUFFERS = {"full": ["atoms", "probe_pos", "probe_ids", "probe_nbrs", "convex", "sectors", "segments", "full", "perm"],
           "exterior": ["atoms", "probe_pos", "probe_ids", "probe_nbrs", "tori_pos", "tori_axis", "tori_vs", "perm"]}


def compare(batch, mols, mode):
    for m, atoms in enumerate(mols):
        got = batch.molecule(m)
        want = plain(atoms, mode)
        rec, c = got["record"], want["counts"]
        assert rec["atoms"] == atoms.shape[0]
        assert rec["probes"] == c["probes"] and rec["singular_probes"] == c["singular_probes"], m
        if mode == "full":
            assert (rec["sectors"], rec["full_circles"], rec["segments"]) == (c["sectors"], c["full_circles"], c["segments"])
        else:
            assert rec["tori"] == c["tori"]
        for k in BUFFERS[mode]:
            a, b = got[k], want[k]
            assert a.shape == b.shape, (m, k, a.shape, b.shape)
            if k == "probe_nbrs":  # only the written part of each neighbour block
                a = canon.written_probe_nbrs(a, got["probe_ids"], rec["singular_probes"])
                b = canon.written_probe_nbrs(b, want["probe_ids"], c["singular_probes"])
            assert np.array_equal(a, b, equal_nan=True), (m, k)


@pytest.mark.parametrize("mode", ["full", "exterior"])
def test_batch_matches_plain_builds(mode):
    mols = molecules()
    with SesBatch(mols, RP, mode) as b:
        assert b.molecules == len(mols)
        b.build()
        compare(b, mols, mode)


def test_batch_graph_replay_and_frames():
    # jittered frames of one molecule, rebuilt in a graph with new coordinates
    base = synth.globule(1500, 1401)
    frames = [synth.jitter(base, 0.3, 1402 + f) for f in range(5)]
    with SesBatch(frames, RP, "full", graph=True) as b:
        b.build()
        b.build()  # replay
        compare(b, frames, "full")


@pytest.mark.parametrize("mode", ["full", "exterior"])
def test_batch_regrow_from_minimal_capacities(mode):
    # the first batch build overflows every count-dependent buffer; after the regrow and the
    # second build each molecule's slice still equals its own build
    mols = molecules()
    with SesBatch(mols, RP, mode, min_capacity=True) as b:
        b.build()
        assert b.counts()["rebuilds"] >= 1
        compare(b, mols, mode)
