"""Comparison of the reference's own kernels with the FP64 oracle, band-aware.

The reference evaluates its predicates in float32 with --use_fast_math
(sesdf/CMakeLists.txt:117-125); the oracle evaluates the same expressions in
double precision. They may disagree only where a predicate's margin is within
the float32 error of the reference's arithmetic (the degeneracy band). Every
difference found is checked against that band and reported as "explained" when
its FP64 margin lies inside it, together with the cases that depend on it
(probes on a circle whose status differs, segments of such circles).

Band widths (|FP64 margin| below which a disagreement is explained):
  neighbour   |d^2 - R^2 - 1e-4|            < 64 eps32 (d^2 + R^2)
  visibility  |complete - R_k^2 - 1e-4|      < 2^-10 (complete + R_k^2)     (float32 sqrt(1-cos^2) amplifies)
  circle      |R_i^2 - |c_i - c|^2|          < 2^-10 R_i^2                  (tangent SAS spheres: radius^2 ~ 0)
  occlusion   ||c_l - x|^2 - R_l^2|          < 2^-10 (|c_l - x|^2 + R_l^2)  (float32 triplet solve)
  singular    |d^2 - rp^2 + 1e-4|            < 2^-10 (d^2 + rp^2)
  probe pair  |t| (x1 = x2)                  < 2^-10 R_i^2
  probe order two probes of a circle closer than 4x the reference's own position error (|ref - FP64|)
              can change places in the circle's order, and with it the pairs of its segments
"""
from __future__ import annotations

import numpy as np

import canon
from sesdf_gb300 import precision

EPS32 = 2.0 ** -23
WIDE = 2.0 ** -10


def _f(x):
    return np.float64(np.float32(x))


def circle_geometry(ci, ri, cj, rj, rp):
    R1, R2 = ri + rp, rj + rp
    d = np.dot(ci - cj, ci - cj)
    t = (R1 * R1 - R2 * R2 + d) / (2 * d)
    c = ci + (cj - ci) * t
    r = np.sqrt(max(R1 * R1 - np.dot(ci - c, ci - c), 0.0))
    n = (cj - ci) / np.sqrt(np.dot(cj - ci, cj - ci))
    return c, n, r


def status_margin(pos, rad, i, j, nbrs, rp):
    """Smallest |margin| over k of the two visibility predicates of circle (i, j); 0 when the circle
    itself hangs on the band (SAS spheres of i and j tangent: its radius is the root of a difference
    of nearly equal numbers, NaN on one side and a tiny circle on the other)."""
    R1, R2 = rad[i] + rp, rad[j] + rp
    dij = np.dot(pos[i] - pos[j], pos[i] - pos[j])
    t = (R1 * R1 - R2 * R2 + dij) / (2 * dij)
    cc = pos[i] + (pos[j] - pos[i]) * t
    r2 = R1 * R1 - np.dot(pos[i] - cc, pos[i] - cc)
    if abs(r2) < WIDE * R1 * R1:
        return 0.0
    c, n, r = circle_geometry(pos[i], rad[i], pos[j], rad[j], rp)
    best = np.inf
    for k in nbrs:
        if k == j:
            continue
        v = c - pos[k]
        dist = np.sqrt(np.dot(v, v))
        s = np.dot(v, n)
        p = np.sqrt(max(dist * dist - s * s, 0.0))
        if dist == 0.0 or p < 1e-2 * dist:
            # k on the circle's axis: the reference's sqrt(1 - cos^2) is NaN or
            # loses half its digits in float32 (operations.cu:172-179)
            return 0.0
        Rk2 = (rad[k] + rp) ** 2
        for sign in (1.0, -1.0):
            comp = (sign * p + r) ** 2 + s * s
            m = abs(comp - Rk2 - _f(1e-4))
            best = min(best, m / (comp + Rk2))
    return best


def probe_solutions(pos, rad, i, j, k, rp):
    ci, cj, ck = pos[i], pos[j], pos[k]
    cij, nij, _ = circle_geometry(ci, rad[i], cj, rad[j], rp)
    cik, nik, _ = circle_geometry(ci, rad[i], ck, rad[k], rp)
    u = nik - nij * np.dot(nik, nij)
    den = np.dot(u, nik)
    xc = cij + u * (np.dot(cik - cij, nik) / den)
    Ri2 = (rad[i] + rp) ** 2
    t = Ri2 - np.dot(xc - ci, xc - ci)
    if not t >= 0:
        return None, t / Ri2
    nn = np.cross(nij, nik)
    nn = nn / np.linalg.norm(nn)
    return (xc + nn * np.sqrt(t), xc - nn * np.sqrt(t)), t / Ri2


def occlusion_margin(pos, rad, x, i, exclude, nbrs, rp):
    best = np.inf
    for l in nbrs:
        if l in exclude:
            continue
        e = pos[l] - x
        ee = np.dot(e, e)
        Rl2 = (rad[l] + rp) ** 2
        best = min(best, abs(ee - Rl2) / (ee + Rl2))
    return best


def compare(atoms_in: np.ndarray, rp: float, mode: str, ref: dict, o: dict) -> dict:
    """ref: reference outputs (compact golden form); o: oracle.run output. Returns a report."""
    rpd = _f(rp)
    n = atoms_in.shape[0]
    pos = atoms_in[:, :3].astype(np.float64)
    rad = atoms_in[:, 3].astype(np.float64)
    rep = {"perm_mismatch": int(np.count_nonzero(ref["perm"] != o["perm"]))}

    # neighbours (input ids)
    roff = np.concatenate([[0], np.cumsum(ref["nbr_count"].astype(np.int64))])
    rrows = [ref["nbr"][roff[s]:roff[s + 1]] for s in range(n)]
    ocnt, orows = canon.csr_rows(o["noff"], o["nbr"])
    rn = canon.neighbor_sets(ref["perm"], ref["nbr_count"], rrows)
    on = canon.neighbor_sets(o["perm"], ocnt, orows)
    bad_pairs = set()
    unexplained = 0
    for a in range(n):
        for b in rn[a] ^ on[a]:
            d2 = np.dot(pos[a] - pos[b], pos[a] - pos[b])
            R = (rad[a] + rpd) + (rad[b] + rpd)
            m = abs(d2 - R * R - _f(1e-4))
            bad_pairs.add(frozenset((a, b)))
            if m >= 64 * EPS32 * (d2 + R * R):
                unexplained += 1
    rep["nbr_mismatch"] = len(bad_pairs)
    rep["nbr_unexplained"] = unexplained

    # statuses of directed circles (input ids)
    srows_r = [ref["status"][roff[s]:roff[s + 1]] for s in range(n)]
    srows_o = [o["status"][o["noff"][s]:o["noff"][s + 1]] for s in range(n)]
    ext = mode == "exterior"
    sr = canon.status_map(ref["perm"], ref["nbr_count"], rrows, srows_r, ext)
    so = canon.status_map(o["perm"], ocnt, orows, srows_o, ext)
    tainted = set()
    st_bad = st_unexp = 0
    for key in set(sr) | set(so):
        if sr.get(key) == so.get(key):
            continue
        a, b = key
        if frozenset(key) in bad_pairs:
            tainted.add(frozenset(key))
            st_bad += 1
            continue
        if ext and ( key not in sr or key not in so ):
            # sorted order decides which direction is evaluated
            continue
        st_bad += 1
        tainted.add(frozenset(key))
        # the oracle evaluates a circle of two complete lists from its lower atom only: any
        # atom of either list can decide it
        if status_margin(pos, rad, a, b, sorted(set(on[a]) | set(on[b])), rpd) >= WIDE:
            st_unexp += 1
    rep["status_mismatch"] = st_bad
    rep["status_unexplained"] = st_unexp

    # probes
    rk = canon.probe_keys(atoms_in, ref["perm"], ref["probe_ids"], ref["probe_pos"])
    ok = canon.probe_keys(atoms_in, o["perm"], o["ids"], o["posf"])
    rmap = {k: q for q, k in enumerate(rk)}
    omap = {k: q for q, k in enumerate(ok)}
    pr_bad = pr_unexp = 0
    bad_probes = set()
    for key in set(rmap) ^ set(omap):
        pr_bad += 1
        bad_probes.add(key)
        trip = key[0]
        circles = [frozenset((trip[0], trip[1])), frozenset((trip[0], trip[2])), frozenset((trip[1], trip[2]))]
        if any(c in tainted or c in bad_pairs for c in circles):
            continue
        # margins of the triplet solve and of the occlusion test
        explained = False
        for owner in trip:
            others = [t for t in trip if t != owner]
            sol, tnorm = probe_solutions(pos, rad, owner, others[0], others[1], rpd)
            if sol is None or abs(tnorm) < WIDE:
                explained = True
                break
            for x in sol:
                if canon.side(atoms_in, trip, x) != key[1]:
                    continue
                if occlusion_margin(pos, rad, x, owner, set(trip), on[owner], rpd) < WIDE:
                    explained = True
        if not explained:
            pr_unexp += 1
    rep["probe_mismatch"] = pr_bad
    rep["probe_unexplained"] = pr_unexp
    if ext and st_unexp:
        # exterior statuses are read after probes promoted their circles to tori;
        # a probe present on one side only changes its three circles
        probe_circles = set()
        for key in bad_probes:
            t = key[0]
            probe_circles |= {frozenset((t[0], t[1])), frozenset((t[0], t[2])), frozenset((t[1], t[2]))}
        st_unexp = 0
        for key in set(sr) | set(so):
            if sr.get(key) == so.get(key) or key not in sr or key not in so:
                continue
            fk = frozenset(key)
            if fk in bad_pairs or fk in probe_circles:
                continue
            if status_margin(pos, rad, key[0], key[1], sorted(on[key[0]]), rpd) >= WIDE:
                st_unexp += 1
        rep["status_unexplained"] = st_unexp
    common = sorted(set(rmap) & set(omap))
    if common:
        rq = np.array([rmap[k] for k in common])
        oq = np.array([omap[k] for k in common])
        err = np.abs(ref["probe_pos"][rq, :3].astype(np.float64) - o["posd"][oq, :3])
        rep["probe_pos_max_err"] = float(err.max())
        rep["probe_pos_over_1e-4"] = int(np.count_nonzero(err.max(axis=1) > 1e-4))
        rsing = np.abs(ref["probe_pos"][rq, 3]) == 2 if not ext else None
        osing = np.abs(o["cids"][oq, 3]) == 2
        if rsing is None:
            # exterior: w of a singular probe holds its neighbour-block index; singular
            # probes are the first Q
            rsing = rq < ref["counts"][5]
        rep["singular_mismatch"] = int(np.count_nonzero(rsing != osing))
    else:
        rep["probe_pos_max_err"] = 0.0
        rep["probe_pos_over_1e-4"] = 0
        rep["singular_mismatch"] = 0
    rep["probes_common"] = len(common)

    if mode == "full":
        # sectors per directed circle (input ids), in each side's slot order
        def sector_map(perm, cnt, rows, st_rows, sectors):
            out, q = {}, 0
            for s in range(n):
                for e in range(cnt[s]):
                    if st_rows[s][e] != 0:
                        out[(int(perm[s]), int(perm[rows[s][e]]))] = sectors[q]
                        q += 1
            return out
        sm_r = sector_map(ref["perm"], ref["nbr_count"], rrows, srows_r, ref["sectors"])
        sm_o = sector_map(o["perm"], ocnt, orows, srows_o, o["sectors"])
        common_s = set(sm_r) & set(sm_o)
        # axis error, and half-angle error compared through its cosine (the angle
        # itself is ill-conditioned next to 0 and pi, e.g. for tangent spheres)
        rep["sector_axis_max_err"] = float(max((np.max(np.abs(np.asarray(sm_r[k][:3], np.float64) - sm_o[k][:3]))
                                                for k in common_s), default=0.0))
        rep["sector_cos_max_err"] = float(max((abs(np.cos(np.float64(sm_r[k][3])) - np.cos(sm_o[k][3])) for k in common_s),
                                              default=0.0))
        rep["sector_max_err"] = max(rep["sector_axis_max_err"], rep["sector_cos_max_err"])
        # complete circles
        fr = canon.pair_set(ref["perm"], ref["full"])
        fo = canon.pair_set(o["perm"], o["full"])
        rep["full_mismatch"] = len(fr ^ fo)
        rep["full_unexplained"] = len([c for c in fr ^ fo if c not in tainted])
        # segments: per circle, the set of probe pairs
        sg_r = canon.segment_set(ref["perm"], ref["segments"], rk)
        sg_o = canon.segment_set(o["perm"], o["segments"], ok)
        seg_bad = sg_r ^ sg_o
        unexp = 0
        for circle, pair in seg_bad:
            if circle in tainted or any(p in bad_probes for p in pair):
                continue
            unexp += 1
        rep["segment_mismatch"] = len(seg_bad)
        rep["segment_unexplained"] = unexp
        rep["segments_ref"] = len(ref["segments"])
    else:
        # tori per circle: compare where both sides have one
        def tori_map(perm, cnt, rows, st_rows, tp, ta, tv):
            out, q = {}, 0
            for s in range(n):
                for e in range(cnt[s]):
                    if st_rows[s][e] == 2:
                        out[frozenset((int(perm[s]), int(perm[rows[s][e]])))] = np.concatenate([tp[q], ta[q], tv[q]])
                        q += 1
            return out
        srows_r2 = srows_r
        srows_o2 = [o["status"][o["noff"][s]:o["noff"][s + 1]] for s in range(n)]
        tm_r = tori_map(ref["perm"], ref["nbr_count"], rrows, srows_r2, ref["tori_pos"], ref["tori_axis"], ref["tori_vs"])
        T = o["tori"]
        tm_o = tori_map(o["perm"], ocnt, orows, srows_o2, T[:, 0:4], T[:, 4:8], T[:, 8:12])
        rep["tori_mismatch"] = len(set(tm_r) ^ set(tm_o))
        pc = set()
        for key in bad_probes:
            t = key[0]
            pc |= {frozenset((t[0], t[1])), frozenset((t[0], t[2])), frozenset((t[1], t[2]))}
        rep["tori_unexplained"] = len([c for c in set(tm_r) ^ set(tm_o) if c not in tainted and c not in pc
                                       and c not in bad_pairs])
        errs = [np.max(np.abs(np.asarray(tm_r[k], np.float64) - tm_o[k])) for k in set(tm_r) & set(tm_o)
                if np.all(np.isfinite(tm_o[k])) and np.all(np.isfinite(tm_r[k]))]
        rep["tori_max_err"] = float(max(errs, default=0.0))
    return rep


# ---------------------------------------------------------------------------------------------------------
# GPU build against the reference's kernels, in sorted-id space (vectorised, for 10^5 - 10^6 atoms)


def _probe_keys_sorted(atoms, ids, pos, n):
    """int64 key per probe: sorted triplet of sorted ids and the side of the centres' plane."""
    trip = np.sort(np.asarray(ids)[:, :3].astype(np.int64), axis=1)
    a = np.asarray(atoms, np.float64)
    ca, cb, cc = (a[trip[:, m], :3] for m in range(3))
    d = np.einsum("ij,ij->i", np.cross(cb - ca, cc - ca), np.asarray(pos, np.float64)[:, :3] - ca)
    side = np.sign(d).astype(np.int64) + 1
    return ((trip[:, 0] * n + trip[:, 1]) * n + trip[:, 2]) * 4 + side


def _decode_probe_key(key, n):
    side = int(key % 4) - 1
    t = key // 4
    c = int(t % n)
    t //= n
    return (int(t // n), int(t % n), c), side


def _slot_keys(nbr_ids, nbr_count, n):
    cap = nbr_ids.shape[1]
    live = np.arange(cap)[None, :] < np.asarray(nbr_count)[:, None]
    i, s = np.nonzero(live)
    j = nbr_ids[i, s].astype(np.int64)
    return i.astype(np.int64) * n + j, i, s


def compare_sorted(ref: dict, gpu: dict, rp: float, mode: str) -> dict:
    """GPU build (SesBuild.fetch) against the reference's kernels (RefBuild.fetch) on the same atoms.

    Both sort the atoms with the same fast-math reference-grid division, so every id is compared in
    sorted-id space. Each difference is checked against the float32 band of the predicate that decides
    it (module docstring; margins in double precision from the float32 atoms) and counted as explained
    when inside it, with the cases that follow from it (statuses of circles whose neighbour pair
    differs, probes on such circles, segments of such probes)."""
    rpd = _f(rp)
    rep = {"perm_mismatch": int(np.count_nonzero(ref["perm"] != gpu["perm"])),
           "atoms_mismatch": int(np.count_nonzero(np.any(ref["atoms"] != gpu["atoms"], axis=1)))}
    if rep["perm_mismatch"] or rep["atoms_mismatch"]:
        return rep
    atoms = gpu["atoms"]
    n = atoms.shape[0]
    pos = atoms[:, :3].astype(np.float64)
    rad = atoms[:, 3].astype(np.float64)
    ext = mode == "exterior"

    # neighbour pairs
    kr, ir, sr_ = _slot_keys(ref["nbr_ids"], ref["nbr_count"], n)
    kg, ig, sg_ = _slot_keys(gpu["nbr_ids"], gpu["nbr_count"], n)
    diff = np.setxor1d(kr, kg)
    a, b = diff // n, diff % n
    d2 = np.einsum("ij,ij->i", pos[a] - pos[b], pos[a] - pos[b])
    R = (rad[a] + rpd) + (rad[b] + rpd)
    m = np.abs(d2 - R * R - _f(1e-4))
    bad_pairs = set(zip(np.minimum(a, b).tolist(), np.maximum(a, b).tolist()))
    rep["pairs"] = int(len(kg))
    rep["nbr_mismatch"] = len(bad_pairs)
    rep["nbr_unexplained"] = int(np.count_nonzero(m >= 64 * EPS32 * (d2 + R * R)))

    def nbrs_of(i):
        return [int(x) for x in gpu["nbr_ids"][i, :gpu["nbr_count"][i]]]

    # statuses of the directed circles both sides hold
    common, xr, xg = np.intersect1d(kr, kg, return_indices=True)
    str_ = ref["status"][ir[xr], sr_[xr]]
    stg = gpu["status"][ig[xg], sg_[xg]]
    ci_, cj_ = common // n, common % n
    keep = ci_ < cj_ if ext else np.ones(len(common), bool)
    bad = np.nonzero(keep & (str_ != stg))[0]
    # a circle's status depends on every neighbour of its atom: an atom whose neighbour list differs
    # between the two sides (a neighbour decided inside the band) explains all of its circles
    bad_atoms = {x for pr in bad_pairs for x in pr}
    # exterior statuses are read after the probes promoted their circles to status 2, so there a
    # circle is a cause for its probes only when its own visibility margin is inside the band
    tainted = set()
    out_of_band = []
    cases = []
    for q in bad.tolist():
        i, j = int(ci_[q]), int(cj_[q])
        c = (min(i, j), max(i, j))
        # the full build evaluates a circle of two complete lists from its lower atom only, so the
        # neighbours of both atoms can decide it
        margin = 0.0 if i in bad_atoms or (not ext and j in bad_atoms) else \
            status_margin(pos, rad, i, j, sorted(set(nbrs_of(i)) | set(nbrs_of(j))), rpd)
        inband = margin < WIDE
        if inband or not ext:
            tainted.add(c)
        if not inband:
            out_of_band.append(c)
            if len(cases) < 20:
                cases.append({"i": int(gpu["perm"][i]), "j": int(gpu["perm"][j]), "ref": int(str_[q]), "gpu": int(stg[q]),
                              "margin": float(margin)})
    rep["status_mismatch"] = int(len(bad))
    rep["status_unexplained"] = len(out_of_band)
    rep["status_cases"] = cases

    # probes
    pkr = _probe_keys_sorted(atoms, ref["probe_ids"], ref["probe_pos"], n)
    pkg = _probe_keys_sorted(atoms, gpu["probe_ids"], gpu["probe_pos"], n)
    pdiff = np.setxor1d(pkr, pkg)
    bad_probe_circles = set()
    pr_unexp = 0
    for key in pdiff.tolist():
        trip, side = _decode_probe_key(key, n)
        circles = [(trip[0], trip[1]), (trip[0], trip[2]), (trip[1], trip[2])]
        bad_probe_circles |= set(circles)
        if any(c in tainted or c in bad_pairs for c in circles):
            continue
        explained = False
        for owner in trip:
            others = [t for t in trip if t != owner]
            sol, tnorm = probe_solutions(pos, rad, owner, others[0], others[1], rpd)
            if sol is None or abs(tnorm) < WIDE:
                explained = True
                break
            for x in sol:
                if canon.side(atoms, trip, x) != side:
                    continue
                if occlusion_margin(pos, rad, x, owner, set(trip), nbrs_of(owner), rpd) < WIDE:
                    explained = True
        if not explained:
            pr_unexp += 1
    rep["probes"] = int(len(pkg))
    rep["probe_mismatch"] = int(len(pdiff))
    rep["probe_unexplained"] = pr_unexp
    if ext:
        # a probe found on one side only changes the statuses of its three circles
        rep["status_unexplained"] = len([c for c in out_of_band if c not in bad_probe_circles and c not in bad_pairs])
    rep["ref_probe_vs_fp64"] = precision.probe_error(atoms, ref["probe_ids"], ref["probe_pos"], rp)
    _, qr, qg = np.intersect1d(pkr, pkg, return_indices=True)
    if len(qr):
        err = np.abs(ref["probe_pos"][qr, :3].astype(np.float64) - gpu["probe_pos"][qg, :3].astype(np.float64))
        rep["probe_pos_max_diff"] = float(err.max())
        rep["probe_pos_over_1e-4"] = int(np.count_nonzero(err.max(axis=1) > 1e-4))
        if ext:
            rs, gs = qr < ref["counts"]["Q"], qg < gpu["counts"]["singular_probes"]
        else:
            rs, gs = np.abs(ref["probe_pos"][qr, 3]) == 2, np.abs(gpu["probe_pos"][qg, 3]) == 2
        rep["singular_mismatch"] = int(np.count_nonzero(rs != gs))
    else:
        rep["probe_pos_max_diff"], rep["probe_pos_over_1e-4"], rep["singular_mismatch"] = 0.0, 0, 0

    def circle_tainted(i, j):
        c = (min(i, j), max(i, j))
        return c in tainted or c in bad_pairs or c in bad_probe_circles

    if not ext:
        # sectors of the visible circles both sides hold, by slot
        def sector_index(side):
            cap = side["nbr_ids"].shape[1]
            live = np.arange(cap)[None, :] < side["nbr_count"][:, None]
            vis = live & (side["status"] != 0)
            idx = np.full(vis.shape, -1, np.int64)
            idx[vis] = np.arange(int(vis.sum()))
            return idx
        sxr, sxg = sector_index(ref), sector_index(gpu)
        a_r, a_g = sxr[ir[xr], sr_[xr]], sxg[ig[xg], sg_[xg]]
        both = (a_r >= 0) & (a_g >= 0)
        sr_v = ref["sectors"][a_r[both]].astype(np.float64)
        sg_v = gpu["sectors"][a_g[both]].astype(np.float64)
        rep["sector_axis_max_diff"] = float(np.abs(sr_v[:, :3] - sg_v[:, :3]).max()) if both.any() else 0.0
        rep["sector_cos_max_diff"] = float(np.abs(np.cos(sr_v[:, 3]) - np.cos(sg_v[:, 3])).max()) if both.any() else 0.0
        # complete circles
        fr = np.sort(ref["full"].astype(np.int64), axis=1)
        fg = np.sort(gpu["full"].astype(np.int64), axis=1)
        fdiff = np.setxor1d(fr[:, 0] * n + fr[:, 1], fg[:, 0] * n + fg[:, 1])
        rep["full_mismatch"] = int(len(fdiff))
        rep["full_unexplained"] = int(sum(1 for k in fdiff.tolist() if not circle_tainted(k // n, k % n)))

        # segments: circle and the unordered pair of probe keys
        def seg_rows(side, pk):
            s = side["segments"].astype(np.int64)
            if len(s) == 0:
                return np.zeros((0, 4), np.int64)
            c = np.sort(s[:, :2], axis=1)
            p = np.sort(np.stack([pk[s[:, 2]], pk[s[:, 3]]], 1), axis=1)
            return np.ascontiguousarray(np.concatenate([c, p], 1))
        rows_r, rows_g = seg_rows(ref, pkr), seg_rows(gpu, pkg)
        vt = np.dtype((np.void, 32))
        sdiff = np.setxor1d(rows_r.view(vt).ravel(), rows_g.view(vt).ravel())
        bad_probe_keys = set(pdiff.tolist())
        gtrip = (pkg // 4)
        g0, g1, g2 = gtrip // (n * n), (gtrip // n) % n, gtrip % n
        rmap_k = dict(zip(pkr[qr].tolist(), qr.tolist())) if len(qr) else {}

        def order_in_band(i, j):
            # the probes of circle (i, j) are paired in their order along the circle: two of them closer
            # than the reference's own position error (its float32 solve) can change places there
            on = np.flatnonzero(((g0 == i) | (g1 == i) | (g2 == i)) & ((g0 == j) | (g1 == j) | (g2 == j)))
            if len(on) < 3:
                return False
            pg = gpu["probe_pos"][on, :3].astype(np.float64)
            err = 1e-4
            for q in on.tolist():
                k = int(pkg[q])
                if k in rmap_k:
                    err = max(err, float(np.abs(ref["probe_pos"][rmap_k[k], :3].astype(np.float64) - pg[on.tolist().index(q)]).max()))
            dmin = min(np.linalg.norm(pg[a] - pg[b]) for a in range(len(on)) for b in range(a + 1, len(on)))
            return dmin < 4.0 * err
        # A probe joins the list of the circle its partial-circle number names. For a circle (j, k)
        # that is not partial on one side (a probe on a circle its atom's visibility pass found
        # hidden or complete: a decision inside the float32 band, since a probe is a visible point
        # of that circle) the number is that of the next partial circle in slot order (the
        # exclusive scan of operations.inl:46-67), so the probe lands in a circle it does not lie
        # on. Every segment of a circle holding such a probe on either side is explained by it.
        def off_circle(rows):
            if len(rows) == 0:
                return set()
            t = rows[:, 2:] // 4
            trip = np.stack([t // (n * n), (t // n) % n, t % n], -1)  # [rows, 2 probes, 3 atoms]
            on = ((trip == rows[:, None, 0:1]).any(-1) & (trip == rows[:, None, 1:2]).any(-1)).all(-1)
            return {(int(a), int(b)) for a, b in rows[~on, :2].tolist()}
        degenerate = off_circle(rows_r) | off_circle(rows_g)
        rep["segment_off_circle_circles"] = len(degenerate)
        unexp = 0
        seg_cases = []
        for v in sdiff:
            r = np.frombuffer(v.tobytes(), np.int64)
            if circle_tainted(int(r[0]), int(r[1])) or int(r[2]) in bad_probe_keys or int(r[3]) in bad_probe_keys:
                continue
            if (int(r[0]), int(r[1])) in degenerate:
                continue
            if order_in_band(int(r[0]), int(r[1])):
                continue
            unexp += 1
            if len(seg_cases) < 10:
                on = np.flatnonzero(((g0 == r[0]) | (g1 == r[0]) | (g2 == r[0])) & ((g0 == r[1]) | (g1 == r[1]) | (g2 == r[1])))
                seg_cases.append({"circle": [int(gpu["perm"][r[0]]), int(gpu["perm"][r[1]])], "side": "ref" if bool((rows_r == r).all(1).any()) else "gpu",
                                  "probes": [list(map(int, gpu["perm"][list(_decode_probe_key(int(k), n)[0])])) + [_decode_probe_key(int(k), n)[1]]
                                             for k in (r[2], r[3])],
                                  "circle_probes_gpu": int(len(on))})
        rep["segment_cases"] = seg_cases
        rep["segments"] = int(len(rows_g))
        rep["segment_mismatch"] = int(len(sdiff))
        rep["segment_unexplained"] = unexp
    else:
        # tori of the circles with status 2 (i < j) both sides hold, by slot
        def tori_index(side):
            cap = side["nbr_ids"].shape[1]
            live = np.arange(cap)[None, :] < side["nbr_count"][:, None]
            t = live & (side["status"] == 2)
            idx = np.full(t.shape, -1, np.int64)
            idx[t] = np.arange(int(t.sum()))
            return idx
        txr, txg = tori_index(ref), tori_index(gpu)
        a_r, a_g = txr[ir[xr], sr_[xr]], txg[ig[xg], sg_[xg]]
        both = (a_r >= 0) & (a_g >= 0) & keep
        tr = np.concatenate([ref["tori_pos"], ref["tori_axis"], ref["tori_vs"]], 1)[a_r[both]].astype(np.float64)
        tg = np.concatenate([gpu["tori_pos"], gpu["tori_axis"], gpu["tori_vs"]], 1)[a_g[both]].astype(np.float64)
        fin = np.isfinite(tr).all(axis=1) & np.isfinite(tg).all(axis=1)
        rep["tori_max_diff"] = float(np.abs(tr[fin] - tg[fin]).max()) if fin.any() else 0.0
        only = keep & ((a_r >= 0) != (a_g >= 0))
        rep["tori_mismatch"] = int(np.count_nonzero(only))
        rep["tori_unexplained"] = int(sum(1 for q in np.nonzero(only)[0].tolist()
                                          if not circle_tainted(int(ci_[q]), int(cj_[q]))))
    rep["unexplained"] = int(sum(v for k, v in rep.items() if k.endswith("_unexplained")))
    rep["band_cases"] = int(sum(v for k, v in rep.items() if k.endswith("_mismatch") and k != "perm_mismatch"))
    return rep
