"""Parity of the GPU build (through the C ABI) with the FP64 oracle.

Topology (neighbour lists, statuses, circles, probes, segments, singular
neighbours) must be identical; probe positions are compared bit for bit (both
sides solve in double precision with the same operations and round to float32);
sectors and tori, which the GPU computes in float32, within 1e-4 A (rad).
"""
import os

import numpy as np
import pytest

import canon
from cases import hand_cases
from oracle import oracle
from sesdf_gb300 import SesBuild, synth

pytestmark = pytest.mark.gpu
RP = 1.4
GEOM_TOL = 1e-4  # A (and rad for sector angles)


def same_buffers(got, want, what=""):
    """Every fetched buffer equal (the neighbour blocks of singular probes: their written entries)."""
    Q = want["counts"]["singular_probes"]
    for k in want:
        if k == "counts":
            continue
        a, b = got[k], want[k]
        if k == "probe_nbrs":
            a = canon.written_probe_nbrs(a, got["probe_ids"], Q)
            b = canon.written_probe_nbrs(b, want["probe_ids"], Q)
        assert np.array_equal(a, b, equal_nan=True), (what, k)


def run_both(atoms, mode, rp=RP):
    with SesBuild(atoms, rp, mode) as g:
        g.build()
        out = g.fetch()
    o = oracle.run(atoms, rp, mode)
    return out, o


def compare(atoms, out, o, mode):
    n = atoms.shape[0]
    c = out["counts"]
    assert c["atoms"] == n
    assert c["truncated_atoms"] == o["counters"]["nbr_truncated"]
    assert c["outside_atoms"] == 0
    # stable reference-grid order: same permutation
    assert np.array_equal(out["perm"], o["perm"]), "sorted order differs"
    assert np.array_equal(out["atoms"], o["atoms"])
    # neighbour lists and statuses, slot for slot
    cnt = np.diff(o["noff"])
    assert np.array_equal(out["nbr_count"], cnt)
    for i in range(n):
        row = o["nbr"][o["noff"][i]:o["noff"][i + 1]]
        assert np.array_equal(out["nbr_ids"][i, :cnt[i]], row), f"neighbours of {i}"
        assert np.array_equal(out["status"][i, :cnt[i]], o["status"][o["noff"][i]:o["noff"][i + 1]]), f"status of {i}"
    assert c["pairs"] == len(o["nbr"])
    assert c["partial_circles"] == len(o["trim_slot"])
    # probes: ids, positions (bit for bit), singular partition
    assert c["probes"] == len(o["ids"]) and c["singular_probes"] == o["Q"]
    assert np.array_equal(out["probe_ids"][:, :3], o["ids"][:, :3])
    assert np.array_equal(out["probe_ids"][:, 3], o["ids"][:, 3]), "singular neighbour counts"
    assert np.array_equal(out["probe_pos"], o["posf"])
    # singular neighbours: same sets (list order follows the reference-grid hash)
    Q = o["Q"]
    gn = out["probe_nbrs"].reshape(Q, 32, 4)
    on = o["snbr"].reshape(Q, 32, 4)
    for q in range(Q):
        k = o["ids"][q, 3]
        a = sorted(map(tuple, gn[q, :k].tolist()))
        b = sorted(map(tuple, on[q, :k].tolist()))
        assert a == b, f"neighbours of singular probe {q}"
    if mode == "full":
        assert np.array_equal(out["full"], o["full"])
        assert np.array_equal(out["convex"], o["convex"])
        assert out["sectors"].shape == o["sectors"].shape
        if len(o["sectors"]):
            sg = out["sectors"].astype(np.float64)
            assert np.max(np.abs(sg[:, :3] - o["sectors"][:, :3])) < GEOM_TOL
            # the half angle through its cosine (ill-conditioned next to 0 and pi)
            assert np.max(np.abs(np.cos(sg[:, 3]) - np.cos(o["sectors"][:, 3]))) < GEOM_TOL
        assert np.array_equal(out["segments"], o["segments"])
        g2t = out["global_to_trimmed"]
        cap = out["nbr_ids"].shape[1]
        for i in range(n):
            assert np.array_equal(g2t[i * cap:i * cap + cnt[i]], o["slot_trim"][o["noff"][i]:o["noff"][i + 1]])
    else:
        T = o["tori"].shape[0]
        assert c["tori"] == T
        if T:
            tor = np.concatenate([out["tori_pos"], out["tori_axis"], out["tori_vs"]], axis=1).astype(np.float64)
            # the reference's NaN (axes parallel to z, tangent spheres) is not compared
            ok = np.isfinite(o["tori"]).all(axis=1)
            if ok.any():
                assert np.max(np.abs(tor[ok] - o["tori"][ok])) < GEOM_TOL


@pytest.mark.parametrize("name", sorted(hand_cases().keys()))
@pytest.mark.parametrize("mode", ["full", "exterior"])
def test_hand_cases(name, mode):
    atoms = hand_cases()[name]
    out, o = run_both(atoms, mode)
    compare(atoms, out, o, mode)


@pytest.mark.parametrize("mode", ["full", "exterior"])
def test_globule_2k(mode):
    atoms = synth.globule(2000, 1000)
    out, o = run_both(atoms, mode)
    compare(atoms, out, o, mode)


@pytest.mark.parametrize("mode", ["full", "exterior"])
def test_globule_20k(mode):
    atoms = synth.globule(20000, 1500)
    out, o = run_both(atoms, mode)
    compare(atoms, out, o, mode)


STRUCTURES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "structures.npz")


@pytest.mark.parametrize("entry", ["1AGA", "101M", "1VIS", "7SC0"])
@pytest.mark.parametrize("mode", ["full", "exterior"])
def test_sample_structures(entry, mode):
    """The reference's own sample structures (MMTF, read as its loader does; coordinates on a
    0.001 A grid, so exact ties in the predicates are common)."""
    with np.load(STRUCTURES) as s:
        atoms = s[entry]
    out, o = run_both(atoms, mode)
    compare(atoms, out, o, mode)


def test_probe_radius_24():
    # the reference's second benchmark configuration (probe 2.4 A, 288 slots,
    # sesdf/CMakeLists.txt:96-117)
    atoms = synth.globule(2000, 1001)
    with SesBuild(atoms, 2.4, "full", max_neighbor_per_atom=288) as g:
        g.build()
        out = g.fetch()
    o = oracle.run(atoms, 2.4, "full", max_nbr=288)
    compare(atoms, out, o, "full")


@pytest.mark.parametrize("mode", ["full", "exterior"])
def test_neighbor_truncation(mode):
    # 32 neighbour slots per atom where most atoms of the globule have 35-42: rows keep their first 32
    # neighbours in visit order (sorted id), as the reference's neighbour search does when its slots are
    # full (sesdf/src/sesdf/operations.cu:111-116), and the truncated atoms are counted
    atoms = synth.globule(2000, 1000)
    with SesBuild(atoms, RP, mode, max_neighbor_per_atom=32) as g:
        g.build()
        out = g.fetch()
    o = oracle.run(atoms, RP, mode, max_nbr=32)
    assert o["counters"]["nbr_truncated"] > 500
    compare(atoms, out, o, mode)


@pytest.mark.parametrize("mode", ["full", "exterior"])
def test_regrow_from_minimal_capacities(mode):
    # every count-dependent buffer starts at its minimum: the first build overflows them all, the
    # library regrows each to the counts it met and builds again; the result must be the default
    # build's, and a second build must fit without another rebuild
    atoms = synth.globule(20000, 1500)
    with SesBuild(atoms, RP, mode) as g:
        g.build()
        want = g.fetch()
    with SesBuild(atoms, RP, mode, min_capacity=True) as g:
        g.build()
        got = g.fetch()
        first = g.counts()["rebuilds"]
        g.build()
        again = g.fetch()
        second = g.counts()["rebuilds"]
    assert first >= 1 and second == first
    assert want["counts"]["rebuilds"] == 0
    same_buffers(got, want)
    same_buffers(again, want)


@pytest.mark.slow
@pytest.mark.parametrize("mode", ["full", "exterior"])
def test_assembly_100k(mode):
    atoms = synth.assembly()
    out, o = run_both(atoms, mode)
    compare(atoms, out, o, mode)


def test_repeated_builds_are_identical():
    atoms = synth.globule(3000, 77)
    with SesBuild(atoms, RP, "full") as g:
        g.build()
        a = g.fetch()
        g.build()
        b = g.fetch()
    for k in ("perm", "nbr_count", "probe_pos", "probe_ids", "segments", "sectors", "full"):
        assert np.array_equal(a[k], b[k]), k


def test_graph_replay_matches():
    atoms = synth.globule(3000, 78)
    with SesBuild(atoms, RP, "full") as g:
        g.build()
        a = g.fetch()
    with SesBuild(atoms, RP, "full", graph=True) as g:
        for _ in range(3):
            g.build()
        b = g.fetch()
    for k in ("perm", "probe_pos", "probe_ids", "segments", "sectors"):
        assert np.array_equal(a[k], b[k]), k


def test_set_atoms_moves_surface():
    base = synth.globule(2000, 1000)
    moved = synth.jitter(base, 0.3, 5)
    with SesBuild(base, RP, "full") as g:
        g.build()
        g.set_atoms(moved)
        g.build()
        out = g.fetch()
    o = oracle.run(moved, RP, "full", box=g.box)
    compare(moved, out, o, "full")


def test_profiled_graph_stage_times():
    # stage events recorded inside the replayed graph add up to the build
    import torch
    atoms = synth.globule(5000, 79)
    with SesBuild(atoms, RP, "full", graph=True, profile=True) as g:
        d = torch.from_numpy(atoms).cuda()
        s = torch.cuda.current_stream()
        for _ in range(3):
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0.record(s)
            g.build_async(d.data_ptr(), s.cuda_stream)
            t1.record(s)
            g.finish()
        torch.cuda.synchronize()
        st = g.stage_times()
        total = t0.elapsed_time(t1)
    assert all(v >= 0 for v in st.values())
    assert 0.5 * total <= sum(st.values()) <= 1.01 * total + 0.05


@pytest.mark.parametrize("mode", ["full", "exterior"])
def test_tuning_knobs_change_no_result(mode):
    # every tuning knob (neighbour-grid cell size, block shapes, persistent probe screen) is a
    # speed choice: each setting must give the default build's buffers exactly
    from sesdf_gb300.autotune import KNOBS
    atoms = synth.globule(5000, 81)
    with SesBuild(atoms, RP, mode) as g:
        g.build()
        want = g.fetch()
        default = g.tuning()
        assert default == {"neighbor_cell_span": 2, "neighbor_warps": 8, "visibility_warps": 1, "probe_warps": 1,
                           "probe_queue": 0}
        for knob, values in KNOBS.items():
            for v in values:
                g.set_tuning(**dict(default, **{knob: v}))
                g.build()
                same_buffers(g.fetch(), want, (knob, v))
        with pytest.raises(Exception):
            g.set_tuning(neighbor_warps=3)


def test_cutoff_cells_match_oracle():
    # the 27-cell neighbour search (cells of the full pair cutoff) against the oracle
    atoms = synth.globule(2000, 1000)
    with SesBuild(atoms, RP, "full") as g:
        g.set_tuning(neighbor_cell_span=1)
        g.build()
        out = g.fetch()
    compare(atoms, out, oracle.run(atoms, RP, "full"), "full")
