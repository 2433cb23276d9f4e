"""Generates the golden fixtures: outputs of the reference's own CUDA kernels.

Runs on a machine with a GPU and the reference harness built (oracle/_ref/, see
oracle/Makefile): for each input it builds the reference's full-surface and
exterior-only surfaces through oracle/refharness.py and stores the outputs in
compact form (neighbour lists as CSR) in <outdir>/<case>_<mode>.npz, together
with the input atoms, box and probe radius.

    python tests/golden/make_golden.py <outdir> [case ...]

The cases ending in _rp24 use the reference's second benchmark configuration: probe
radius 2.4 A on its 288-slot library (sesdf288, sesdf/CMakeLists.txt:96-117).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from cases import hand_cases  # noqa: E402
from oracle import oracle, refharness  # noqa: E402
from sesdf_gb300 import synth  # noqa: E402

RP = 1.4
RP_WIDE, CAP_WIDE = 2.4, 288


def golden_inputs():
    cases = {k: v for k, v in hand_cases().items() if v.shape[0] > 0}
    cases["globule2k"] = synth.globule(2000, 1000)
    # the reference's own sample structures (tests/golden/structures.npz, made by make_structures.py)
    with np.load(os.path.join(HERE, "structures.npz")) as s:
        for e in ("1AGA", "101M"):
            cases[e] = s[e]
    return cases


def golden_inputs_wide():
    """Probe 2.4 A, 288 neighbour slots per atom."""
    with np.load(os.path.join(HERE, "structures.npz")) as s:
        return {"globule2k_rp24": synth.globule(2000, 1000), "1AGA_rp24": s["1AGA"], "101M_rp24": s["101M"]}


def check_reference_limits(atoms, rp, cap):
    """The reference's probe kernel keeps an atom's probes in a block buffer of `cap` entries
    without a bound check (operations.inl:230-486, groupIntersectionsIds): an input runs on it only
    when the oracle finds no atom owning more probes than that."""
    o = oracle.run(atoms, rp, "full", max_nbr=cap)
    ids = np.asarray(o["ids"]).reshape(-1, 4)
    most = int(np.bincount(ids[:, 0], minlength=atoms.shape[0]).max()) if len(ids) else 0
    if most > cap:
        raise RuntimeError(f"an atom owns {most} probes (reference block buffer: {cap})")


def compact_neighbors(nbrs, ids, Q):
    blocks = np.asarray(nbrs, np.float32).reshape(-1, 32, 4)
    rows = [blocks[q, :max(0, min(32, int(ids[q, 3])))] for q in range(int(Q))]
    return np.concatenate(rows) if rows else np.zeros((0, 4), np.float32)


def compact(ref: dict, mode: str, cap: int) -> dict:
    c = ref["counts"]
    cnt = ref["nbr_count"].astype(np.uint32)
    rows = [ref["nbr_ids"][i, :cnt[i]] for i in range(len(cnt))]
    srows = [ref["status"][i, :cnt[i]] for i in range(len(cnt))]
    out = {
        "perm": ref["perm"], "atoms_sorted": ref["atoms"], "nbr_count": cnt,
        "nbr": np.concatenate(rows) if rows else np.zeros(0, np.uint32),
        "status": np.concatenate(srows) if srows else np.zeros(0, np.uint8),
        "probe_ids": ref["probe_ids"], "probe_pos": ref["probe_pos"],
        # only the filled part of each probe's 32-entry neighbour block (the rest is unwritten memory)
        "probe_nbrs": compact_neighbors(ref["probe_nbrs"], ref["probe_ids"], c["Q"]),
        "counts": np.array([c[k] for k in refharness.COUNT_NAMES], np.uint64),
    }
    if mode == "full":
        for k in ("convex", "full", "sectors", "segments"):
            out[k] = ref[k]
        g2t = ref["global_to_trimmed"]
        out["slot_trim"] = np.concatenate([g2t[i * cap:i * cap + cnt[i]] for i in range(len(cnt))]) if len(cnt) else np.zeros(0, np.uint32)
    else:
        for k in ("tori_pos", "tori_axis", "tori_vs"):
            out[k] = ref[k]
    return out


def main():
    outdir = sys.argv[1]
    only = set(sys.argv[2:])
    os.makedirs(outdir, exist_ok=True)
    runs = [(name, atoms, RP, refharness.MAX_NBR) for name, atoms in golden_inputs().items()]
    runs += [(name, atoms, RP_WIDE, CAP_WIDE) for name, atoms in golden_inputs_wide().items()]
    for name, atoms, rp, cap in runs:
        if only and name not in only:
            continue
        check_reference_limits(atoms, rp, cap)
        for mode in ("full", "exterior"):
            r = refharness.RefBuild(atoms, rp, mode, max_nbr=cap)
            r.build()
            ref = r.fetch()
            r.close()
            data = compact(ref, mode, cap)
            box = r.box
            np.savez_compressed(os.path.join(outdir, f"{name}_{mode}.npz"), atoms=atoms, box=box,
                                probe_radius=np.float32(rp), max_nbr=np.uint32(cap), **data)
            print(name, mode, {k: int(v) for k, v in zip(refharness.COUNT_NAMES, data["counts"])}, flush=True)


if __name__ == "__main__":
    main()
