"""Exterior and cavities: the connected components of the probe-accessible space.

E = probe-centre positions outside every SAS sphere (radius r_i + rp). Its unbounded component is the
exterior; every bounded one is a cavity, a pocket a probe can sit in but not leave. The reference has no
such classification: its exterior-only build (Ssesdf) skips the sector and segment stages and keeps
every probe, cavities included. This module labels E on a voxel grid and assigns every probe of a build
to the component it touches, so that a caller can drop cavity probes or report cavity volumes.

Voxel centres at spacing h are accessible when they lie outside every SAS sphere; components are
6-connected. A channel of E narrower than about h can be missed (two parts then count as separate
components), so the labelling converges as h shrinks. A cavity of some size (the empty core of a closed
shell of atoms) is found at any h up to ~0.3 A; in a packed globule many probes sit in pockets of E
thinner than the grid, which it splits off as one-voxel components or misses (about 5 % of the probes of
a 2,000-atom globule change class between h = 0.25 and 0.2 A). A probe position lies on the boundary of
E (it touches three SAS spheres), so it takes the component of the nearest accessible voxel centre within
two voxels; "probe_resolved" is false where there is none.

``classify_gpu`` is the same classification on the device (``sesgb_cavities``: SAS spheres rasterised
into an occupancy bit grid, lock-free union-find over the accessible voxels, components numbered in the
order of their first voxel, probes of the build assigned by the same nearest-voxel rule); its labels
equal this module's, voxel for voxel, for the same atoms, probe radius and spacing.
"""
from __future__ import annotations

import numpy as np


MAX_VOXELS = 1 << 28  # the labels take 4 bytes per voxel


def accessible_grid(atoms: np.ndarray, probe_radius: float, h: float = 0.25):
    """Boolean grid (nx, ny, nz) of voxel centres outside every SAS sphere, and the centre of voxel 0.
    The grid covers the SAS bounds with two voxels of margin, so its border is exterior."""
    a = np.asarray(atoms, np.float64)
    R = a[:, 3] + probe_radius
    lo = (a[:, :3] - R[:, None]).min(axis=0) - 2 * h
    hi = (a[:, :3] + R[:, None]).max(axis=0) + 2 * h
    dims = np.ceil((hi - lo) / h).astype(np.int64) + 1
    if int(np.prod(dims)) > MAX_VOXELS:
        raise ValueError(f"a {dims.tolist()} grid at h = {h} A exceeds {MAX_VOXELS} voxels: use a larger h")
    occupied = np.zeros(tuple(dims), dtype=bool)
    # rasterise each SAS sphere over its bounding cube of voxels, grouped by radius
    for rad in np.unique(R):
        sel = np.flatnonzero(R == rad)
        k = int(np.ceil(rad / h)) + 1
        off = np.arange(-k, k + 1)
        ox, oy, oz = np.meshgrid(off, off, off, indexing="ij")
        offs = np.stack([ox.ravel(), oy.ravel(), oz.ravel()], axis=1)
        for chunk in np.array_split(sel, max(1, len(sel) // 2048)):
            c = a[chunk, :3]
            base = np.floor((c - lo) / h).astype(np.int64)
            idx = base[:, None, :] + offs[None, :, :]
            idx = np.clip(idx, 0, dims - 1)
            centre = lo + idx * h
            inside = ((centre - c[:, None, :]) ** 2).sum(axis=2) < rad * rad
            v = idx[inside]
            occupied[v[:, 0], v[:, 1], v[:, 2]] = True
    return ~occupied, lo


def label(accessible: np.ndarray):
    """6-connected component labels (0 = not accessible) and the set of labels touching the border."""
    from scipy import ndimage

    lab, n = ndimage.label(accessible)
    border = np.unique(np.concatenate([lab[0].ravel(), lab[-1].ravel(), lab[:, 0].ravel(), lab[:, -1].ravel(),
                                       lab[:, :, 0].ravel(), lab[:, :, -1].ravel()]))
    return lab, n, set(int(x) for x in border if x)


def probe_components(lab: np.ndarray, lo: np.ndarray, h: float, probes: np.ndarray, reach: int = 2):
    """Component label of every probe position: the label of the nearest accessible voxel centre within
    reach voxels of it (0 when there is none)."""
    p = np.asarray(probes, np.float64)[:, :3]
    dims = np.array(lab.shape)
    base = np.round((p - lo) / h).astype(np.int64)
    off = np.arange(-reach, reach + 1)
    ox, oy, oz = np.meshgrid(off, off, off, indexing="ij")
    offs = np.stack([ox.ravel(), oy.ravel(), oz.ravel()], axis=1)
    idx = np.clip(base[:, None, :] + offs[None, :, :], 0, dims - 1)
    d2 = ((lo + idx * h - p[:, None, :]) ** 2).sum(axis=2)
    labs = lab[idx[..., 0], idx[..., 1], idx[..., 2]]
    d2 = np.where(labs > 0, d2, np.inf)
    best = np.argmin(d2, axis=1)
    out = labs[np.arange(len(p)), best]
    return np.where(np.isfinite(d2[np.arange(len(p)), best]), out, 0)


def classify(atoms: np.ndarray, probe_radius: float, probes: np.ndarray | None = None, h: float = 0.25) -> dict:
    """Components of the probe-accessible space of atoms. Returns {"labels" (grid), "origin", "h",
    "exterior" (set of labels), "cavities" (list of labels), "cavity_volume" (A^3 of probe-centre space per
    cavity), and, when probes (k, >=3) are given, "probe_component", "probe_resolved" and
    "probe_in_cavity" (bool [k])}."""
    acc, lo = accessible_grid(atoms, probe_radius, h)
    lab, n, ext = label(acc)
    cav = [k for k in range(1, n + 1) if k not in ext]
    counts = np.bincount(lab.ravel(), minlength=n + 1)
    out = {"labels": lab, "origin": lo, "h": h, "exterior": ext, "cavities": cav,
           "cavity_volume": [float(counts[k]) * h ** 3 for k in cav]}
    if probes is not None:
        comp = probe_components(lab, lo, h, probes)
        out["probe_component"] = comp
        # 0: no accessible voxel centre near the probe (E is thinner than h there)
        out["probe_resolved"] = comp > 0
        out["probe_in_cavity"] = np.isin(comp, cav)
    return out


def classify_gpu(build, h: float = 0.25, with_labels: bool = True) -> dict:
    """classify() of a built SesBuild (one molecule, either mode) on the device: the same keys, the
    probes being the build's own (its concave-patch positions). The grid uses the build's float32
    probe radius."""
    import torch

    k = build.counts()["probes"]
    comp = torch.zeros(max(k, 1), dtype=torch.int32, device="cuda")
    info = build.cavities(h, comp.data_ptr(), torch.cuda.current_stream().cuda_stream)
    n = info["components"]
    vox, bor = build.cavity_components(n)
    ext = {int(x) for x in np.flatnonzero(bor[1:]) + 1}
    cav = [x for x in range(1, n + 1) if x not in ext]
    out = {"origin": info["origin"], "h": h, "exterior": ext, "cavities": cav,
           "cavity_volume": [float(vox[x]) * h ** 3 for x in cav], "dims": info["dims"], "voxels": vox}
    if with_labels:
        out["labels"] = build.cavity_labels().reshape(info["dims"])
    pc = comp.cpu().numpy()[:k]
    out["probe_component"] = pc
    out["probe_resolved"] = pc > 0
    out["probe_in_cavity"] = np.isin(pc, cav)
    return out
