"""Headless SES images by sphere tracing (sesdf_gb300/render.py), driven by the FP64 oracle's signed
distance: hit points lie on the surface within eps (never past it), every ray that meets the surface
is a hit, and the surface lies between the vdW union and the SAS."""
import numpy as np

from cases import hand_cases
from oracle import oracle
from sesdf_gb300 import render, synth

RP = 1.4
EPS = 1e-3


def oracle_fn(atoms):
    o = oracle.run(atoms, RP, "full")
    return lambda p: oracle.sdf(o, p)[:2]


def camera(atoms, width, fov=40.0, view=(0.3, -1.0, 0.5)):
    a = np.asarray(atoms, np.float64)
    lo = (a[:, :3] - a[:, 3:4] - RP).min(axis=0)
    hi = (a[:, :3] + a[:, 3:4] + RP).max(axis=0)
    c = 0.5 * (lo + hi)
    rad = 0.5 * np.linalg.norm(hi - lo)
    v = np.asarray(view, np.float64) / np.linalg.norm(view)
    dist = rad / np.sin(np.radians(fov) / 2)
    eye = c - dist * v
    return eye, render.camera_rays(eye, c, (0, 0, 1), fov, width, width), dist - rad, dist + rad


def test_single_sphere_matches_ray_intersection():
    a = np.array([[0.5, -0.2, 0.1, 1.7]], np.float32)
    fn = oracle_fn(a)
    eye, dirs, t0, t1 = camera(a, 40)
    d = render.sphere_trace(fn, eye, dirs, RP, t0, t1, EPS)
    hit = np.isfinite(d)
    c = a[0, :3].astype(np.float64)
    p = eye + d[hit, None] * dirs[hit]
    gap = np.linalg.norm(p - c, axis=1) - 1.7
    assert gap.min() >= -1e-5 and gap.max() < EPS  # on the sphere within eps, never inside
    oc = eye - c
    b = dirs @ oc
    miss = np.sqrt(np.maximum(oc @ oc - b * b, 0.0)) - 1.7  # closest approach of each ray to the sphere
    assert np.all(hit[miss < 0]) and not np.any(hit & (miss > EPS))
    # the depth image wrapper: same rays, unit normals pointing back at the camera
    depth, nrm = render.depth_image(fn, a, RP, 40, 40, eps=EPS)
    assert np.array_equal(np.isfinite(depth).ravel(), hit)
    n = nrm.reshape(-1, 3)[hit]
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-4)
    assert np.all(np.einsum("ij,ij->i", n, dirs[hit]) < 0)


def test_surface_between_vdw_union_and_sas():
    for atoms in (hand_cases()["tetrahedron"], hand_cases()["cluster40"], synth.globule(300, 11)):
        fn = oracle_fn(atoms)
        eye, dirs, t0, t1 = camera(atoms, 40)
        d = render.sphere_trace(fn, eye, dirs, RP, t0, t1, EPS)
        hit = np.isfinite(d)
        assert hit.any()
        p = eye + d[hit, None] * dirs[hit]
        v, k = fn(p.astype(np.float32))
        assert np.all(np.isin(k, render.INSIDE_SAS)) and v.min() >= -1e-4 and v.max() < EPS
        a = atoms.astype(np.float64)
        dc = np.linalg.norm(p[:, None, :] - a[None, :, :3], axis=2)
        assert np.all((dc - a[None, :, 3]).min(axis=1) >= -1e-4)       # outside the vdW union
        assert np.all((dc - a[None, :, 3] - RP).min(axis=1) <= 1e-4)   # inside the SAS
        # a ray that meets a vdW sphere (passing at least eps inside it) meets the SES no later; the
        # float32 ray directions are unit vectors only to a few ulps, so the entry solves the quadratic
        # with |d|^2 as it is
        d64 = dirs.astype(np.float64)
        dd = np.einsum("ij,ij->i", d64, d64)
        for i in range(a.shape[0]):
            oc = eye - a[i, :3]
            b = d64 @ oc
            disc = b * b - dd * (oc @ oc - a[i, 3] ** 2)
            tv = np.where(disc > 2 * a[i, 3] * EPS, (-b - np.sqrt(np.maximum(disc, 0.0))) / dd, np.inf)
            meets = np.isfinite(tv)
            assert np.all(hit[meets]) and np.all(d[meets] <= tv[meets] + 1e-4)
