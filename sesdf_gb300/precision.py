"""Error of a build's geometry against double precision, from its own output buffers.

The build evaluates its bulk arithmetic in float32 and takes double precision only
for the triplet probe solve and for predicates inside the float32 error band. This
module re-evaluates, in float64 from the float32 atoms of the build, the geometry
the build stores and reports how far the stored float32 values are from it:

* probe positions: the two points at distance R_i, R_j, R_k (R = r + rp) from the
  three atom centres of each probe (the point the reference's intersection of the
  circles (i, j) and (i, k) gives, sesdf/include/bcs/sesdf/operations.inl:384-398),
  on the side of the centres' plane the stored point lies on;
* convex sectors: the axis c_ij (unit vector from i to j) and the half angle
  acos(c_ij . (x - c_i) / R_i) of each visible circle, x the circle point along the
  reference's orthogonal vector (operations.inl:175-228, math.cuh:32-38); the angle
  is compared through its cosine, which is well conditioned next to 0 and pi;
* exterior tori: circle centre and radius, axis, visibility sphere
  (sesdf/src/ssesdf/operations.cu:246-285).

Together with the per-predicate counts of double-precision decisions the build
reports (`fp64_decisions`), this is the error statement of one build.
"""
from __future__ import annotations

import numpy as np


def triplet_points(atoms: np.ndarray, ids: np.ndarray, rp: float):
    """Both FP64 points of each atom triplet (ids[:, :3], sorted atom ids): returns (x_plus, x_minus,
    normal, h2) with x = c_i + y0 +- n sqrt(h2 / |n|^2), n = (c_j - c_i) x (c_k - c_i)."""
    a = np.asarray(atoms, np.float64)
    rpd = float(np.float32(rp))
    ci, cj, ck = (a[ids[:, m], :3] for m in range(3))
    Ri, Rj, Rk = (a[ids[:, m], 3] + rpd for m in range(3))
    u, v = cj - ci, ck - ci
    n = np.cross(u, v)
    nn = np.einsum("ij,ij->i", n, n)
    p = 0.5 * (np.einsum("ij,ij->i", u, u) + Ri * Ri - Rj * Rj)
    q = 0.5 * (np.einsum("ij,ij->i", v, v) + Ri * Ri - Rk * Rk)
    with np.errstate(invalid="ignore", divide="ignore"):
        y0 = (p[:, None] * np.cross(v, n) + q[:, None] * np.cross(n, u)) / nn[:, None]
        h2 = Ri * Ri - np.einsum("ij,ij->i", y0, y0)
        t = np.sqrt(np.maximum(h2, 0.0) / nn)
    off = n * t[:, None]
    return ci + y0 + off, ci + y0 - off, n, h2


def probe_error(atoms: np.ndarray, ids: np.ndarray, pos: np.ndarray, rp: float) -> dict:
    """Max and count over 1e-4 A of |stored probe position - FP64 point| (per coordinate)."""
    if len(ids) == 0:
        return {"probes": 0, "max_err_A": 0.0, "over_1e-4": 0}
    ids = np.asarray(ids)[:, :3].astype(np.int64)
    x1, x2, n, _ = triplet_points(atoms, ids, rp)
    p = np.asarray(pos, np.float64)[:, :3]
    ci = np.asarray(atoms, np.float64)[ids[:, 0], :3]
    side = np.einsum("ij,ij->i", p - ci, n) >= 0
    x = np.where(side[:, None], x1, x2)
    err = np.abs(p - x).max(axis=1)
    return {"probes": int(len(ids)), "max_err_A": float(np.nanmax(err)), "over_1e-4": int(np.count_nonzero(err > 1e-4))}


def sector_error(atoms: np.ndarray, nbr_ids: np.ndarray, nbr_count: np.ndarray, status: np.ndarray,
                 sectors: np.ndarray, rp: float) -> dict:
    """Max error of the stored sectors (axis components; cosine of the half angle) against FP64.
    nbr_ids, status: [n, cap] rows; sectors in slot order of the visible circles."""
    a = np.asarray(atoms, np.float64)
    n, cap = nbr_ids.shape
    live = np.arange(cap)[None, :] < np.asarray(nbr_count)[:, None]
    vis = live & (status != 0)
    i = np.nonzero(vis)[0].astype(np.int64)
    j = nbr_ids[vis].astype(np.int64)
    if len(i) == 0:
        return {"sectors": 0, "axis_max_err": 0.0, "cos_max_err": 0.0}
    rpd = float(np.float32(rp))
    ci, cj = a[i, :3], a[j, :3]
    Ri, Rj = a[i, 3] + rpd, a[j, 3] + rpd
    d = cj - ci
    dd = np.einsum("ij,ij->i", d, d)
    t = (Ri * Ri - Rj * Rj + dd) / (2 * dd)
    c = ci + d * t[:, None]
    radius = np.sqrt(np.maximum(Ri * Ri - np.einsum("ij,ij->i", ci - c, ci - c), 0.0))
    axis = d / np.sqrt(dd)[:, None]
    ref = np.zeros_like(axis)
    ref[:, 0] = 1.0
    swap = np.abs(axis[:, 0]) > 1.0 - float(np.float32(1e-4))
    ref[swap] = (0.0, 1.0, 0.0)
    nn = np.cross(axis, ref)
    nn /= np.linalg.norm(nn, axis=1, keepdims=True)
    x = c + nn * radius[:, None]
    cos = np.clip(np.einsum("ij,ij->i", axis, (x - ci) / Ri[:, None]), -1.0, 1.0)
    s = np.asarray(sectors, np.float64)
    return {"sectors": int(len(i)), "axis_max_err": float(np.abs(s[:, :3] - axis).max()),
            "cos_max_err": float(np.abs(np.cos(s[:, 3]) - cos).max())}


def tori_error(atoms: np.ndarray, nbr_ids: np.ndarray, nbr_count: np.ndarray, status: np.ndarray,
               tori_pos: np.ndarray, tori_axis: np.ndarray, tori_vs: np.ndarray, rp: float) -> dict:
    """Max error of the stored exterior tori (fillCircles, sesdf/src/ssesdf/operations.cu:246-285: circle
    centre and radius, axis and probe radius, visibility sphere) against FP64, over the circles with
    status 2 in slot order; tori whose axis is parallel to z (no reference frame, counted by the build as
    degenerate) are left out."""
    a = np.asarray(atoms, np.float64)
    n, cap = nbr_ids.shape
    live = np.arange(cap)[None, :] < np.asarray(nbr_count)[:, None]
    sel = live & (status == 2)
    i = np.nonzero(sel)[0].astype(np.int64)
    j = nbr_ids[sel].astype(np.int64)
    if len(i) == 0:
        return {"tori": 0, "max_err": 0.0, "degenerate": 0}
    rpd = float(np.float32(rp))
    ci, cj, ri = a[i, :3], a[j, :3], a[i, 3]
    Ri, Rj = ri + rpd, a[j, 3] + rpd
    d = ci - cj
    dd = np.einsum("ij,ij->i", d, d)
    t = (Ri * Ri - Rj * Rj + dd) / (2 * dd)
    tc = ci + (cj - ci) * t[:, None]
    radius = np.sqrt(np.maximum(Ri * Ri - np.einsum("ij,ij->i", ci - tc, ci - tc), 0.0))

    def nrm(v):
        return v / np.linalg.norm(v, axis=1, keepdims=True)
    with np.errstate(invalid="ignore", divide="ignore"):
        ta = nrm(tc - ci)
        cz = np.cross(ta, np.array([0.0, 0.0, 1.0]))
        degenerate = np.einsum("ij,ij->i", cz, cz) < 1e-12
        ortho = nrm(cz)
        P = tc + ortho * radius[:, None]
        X = nrm(P - ci) * ri[:, None]
        lpi = np.linalg.norm(P - ci, axis=1)
        lpj = np.linalg.norm(P - cj, axis=1)
        C = (cj - ci) * (lpi / (lpj + lpi))[:, None]
        dist = np.linalg.norm(X - C, axis=1)
        C = C + ci - tc
    want = np.concatenate([tc, radius[:, None], ta, np.full((len(i), 1), rpd), C, dist[:, None]], axis=1)
    got = np.concatenate([tori_pos, tori_axis, tori_vs], axis=1).astype(np.float64)
    ok = ~degenerate & np.isfinite(want).all(axis=1)
    err = np.abs(got[ok] - want[ok])
    return {"tori": int(len(i)), "max_err": float(err.max()) if err.size else 0.0, "degenerate": int(degenerate.sum())}


def error_report(out: dict, rp: float, mode: str) -> dict:
    """Error of one build against FP64 from SesBuild.fetch(analysis=True) output, with the build's
    double-precision decision counts (the degeneracy band) per predicate."""
    rep = {"probes": probe_error(out["atoms"], out["probe_ids"], out["probe_pos"], rp)}
    if mode == "full":
        rep["sectors"] = sector_error(out["atoms"], out["nbr_ids"], out["nbr_count"], out["status"], out["sectors"], rp)
    else:
        rep["tori"] = tori_error(out["atoms"], out["nbr_ids"], out["nbr_count"], out["status"], out["tori_pos"],
                                 out["tori_axis"], out["tori_vs"], rp)
    rep["fp64_decisions"] = dict(zip(FP64_PREDICATES, out["counts"]["fp64_decisions"]))
    rep["band_cases"] = int(sum(out["counts"]["fp64_decisions"]))
    return rep


# order of sesgb_counts.fp64_decisions (include/sesgb.h)
FP64_PREDICATES = ["neighbor", "visibility", "occlusion", "singular_neighbor", "probe_candidate", "segment_order",
                   "probe_position"]
