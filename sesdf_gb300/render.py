"""Headless depth and normal images of the SES by sphere tracing its signed distance.

The reference draws its primitives through an OpenGL renderer; here the image is an array and needs no
graphics stack: each pixel's ray advances by a step that never crosses the surface, the signed distance
of ``sesgb_sdf`` (``SesBuild.sdf``) being evaluated for all live rays at once per step.

Safe steps. With kind the primitive that decided the value (1 atom outside the SAS, 2 beyond the band
outside, 3 SAS sphere, 4 circle arc, 5 probe, 0 deeper than the band):
  * outside the SAS (kinds 1, 2) the value is min_i(|x - c_i| - r_i) (clamped at the band), so value - rp
    bounds the distance to the SAS, and the SES lies inside the SAS;
  * inside the SAS (kinds 3-5) the value is rp - dist(x, E) with E the probe-centre positions: every SES
    point y has dist(y, E) = rp, so |x - y| >= rp - dist(x, E): the value bounds the distance to the SES.
A ray stops when an inside-SAS value falls below ``eps`` (a hit at depth t) or t passes ``t_far``.
Normals are the normalised central differences of the signed distance at the hit points.

The tracer takes the signed distance as a function of (m, 3) float32 points, so the same code runs on
the GPU build (``gpu_sdf_fn``) and, in the tests, on the FP64 oracle. ``gpu_depth_image`` is the same
image from one device launch (``sesgb_render``: a warp per ray, the signed distance evaluated in the
kernel, no host round trip per step); its ray arithmetic (float32, every operation rounded on its own)
follows this module's operation for operation.
"""
from __future__ import annotations

import numpy as np

INSIDE_SAS = (3, 4, 5)


def camera_basis(eye, target, up):
    """Unit forward, right and up vectors (float64) of a camera at eye looking at target."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, np.float64))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    return f, r, u


def camera_rays(eye, target, up, fov_deg: float, width: int, height: int):
    """Unit ray directions (height*width, 3) float32 of a pinhole camera, row-major from the top left.
    float32 arithmetic, every operation rounded on its own in the order written (the device tracer's)."""
    f, r, u = (v.astype(np.float32) for v in camera_basis(eye, target, up))
    th = np.float32(np.tan(np.radians(fov_deg) / 2.0))
    W, H = np.float32(width), np.float32(height)
    one, two, half = np.float32(1.0), np.float32(2.0), np.float32(0.5)
    ix = np.arange(width, dtype=np.float32)
    iy = np.arange(height, dtype=np.float32)
    xs = ((((two * (ix + half)) / W - one) * th) * W) / H
    ys = (one - (two * (iy + half)) / H) * th
    d = (f[None, None, :] + xs[None, :, None] * r[None, None, :]) + ys[:, None, None] * u[None, None, :]
    ln = np.sqrt((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2])
    d = d / ln[..., None]
    return d.reshape(-1, 3).astype(np.float32)


def sphere_trace(sdf_fn, origin, dirs, probe_radius: float, t_near: float, t_far: float, eps: float = 1e-3,
                 max_steps: int = 256):
    """Depth t (float32 [m], inf where the ray misses) of the first SES point along origin + t * dirs.
    sdf_fn(points float32 [k, 3]) -> (value [k], kind [k]) as numpy arrays."""
    m = dirs.shape[0]
    # the march is in float32 (the build's probe radius, float32 points, steps and depths)
    rp32, eps32 = np.float32(probe_radius), np.float32(eps)
    min_step = np.float32(0.25) * eps32
    t = np.full(m, np.float32(t_near), np.float32)
    t_far32 = np.float32(t_far)
    depth = np.full(m, np.inf, np.float32)
    live = np.arange(m)
    o = np.asarray(origin, np.float64).astype(np.float32)
    d32 = np.asarray(dirs, np.float64).astype(np.float32)
    for _ in range(max_steps):
        if live.size == 0:
            break
        p = o[None, :] + t[live, None] * d32[live]
        v, k = sdf_fn(p)
        v = np.asarray(v, np.float32)
        k = np.asarray(k)
        inside = np.isin(k, INSIDE_SAS)
        hit = inside & (v < eps32)
        depth[live[hit]] = t[live[hit]]
        step = np.where(inside, v, v - rp32)
        # deeper than the band (kind 0) cannot be reached with these steps; such a ray stops as a hit
        hit |= k == 0
        depth[live[k == 0]] = t[live[k == 0]]
        t[live] += np.where(hit, np.float32(0.0), np.maximum(step, min_step)).astype(np.float32)
        live = live[~hit & (t[live] <= t_far32)]
    return depth


def normals(sdf_fn, points, h: float = 1e-2):
    """Unit gradients (float32 [k, 3]) of the signed distance at float32 points by central differences
    (float32 arithmetic, every operation rounded on its own, as the device tracer computes them)."""
    p = np.asarray(points, np.float32)
    h32 = np.float32(h)
    g = np.zeros_like(p)
    for a in range(3):
        qp, qm = p.copy(), p.copy()
        qp[:, a] = p[:, a] + h32
        qm[:, a] = p[:, a] - h32
        vp, _ = sdf_fn(qp)
        vm, _ = sdf_fn(qm)
        g[:, a] = (np.asarray(vp, np.float32) - np.asarray(vm, np.float32)) / (np.float32(2.0) * h32)
    n = np.sqrt((g[:, 0] * g[:, 0] + g[:, 1] * g[:, 1]) + g[:, 2] * g[:, 2])
    return g / np.where(n > 0, n, np.float32(1.0))[:, None]


def framing(atoms, probe_radius: float, view=(0.3, -1.0, 0.5), fov_deg: float = 40.0):
    """Camera framing the SAS bounds of atoms from the direction view: (eye, centre, up, t_near, t_far)."""
    a = np.asarray(atoms, np.float64)
    lo = (a[:, :3] - a[:, 3:4] - probe_radius).min(axis=0)
    hi = (a[:, :3] + a[:, 3:4] + probe_radius).max(axis=0)
    centre = 0.5 * (lo + hi)
    radius = 0.5 * np.linalg.norm(hi - lo)
    v = np.asarray(view, np.float64)
    v /= np.linalg.norm(v)
    dist = radius / np.sin(np.radians(fov_deg) / 2.0)
    eye = centre - dist * v
    up = (0.0, 0.0, 1.0) if abs(v[2]) < 0.9 else (0.0, 1.0, 0.0)
    return eye, centre, up, max(dist - radius, 0.0), dist + radius


def depth_image(sdf_fn, atoms, probe_radius: float, width: int = 128, height: int = 128, view=(0.3, -1.0, 0.5),
                fov_deg: float = 40.0, eps: float = 1e-3, with_normals: bool = True):
    """Depth (height, width) float32 (inf = background) and normals (height, width, 3) float32 (0 where
    the ray misses) of the SES of atoms seen from the direction view, the camera framing the SAS bounds."""
    eye, centre, up, t_near, t_far = framing(atoms, probe_radius, view, fov_deg)
    dirs = camera_rays(eye, centre, up, fov_deg, width, height)
    depth = sphere_trace(sdf_fn, eye, dirs, probe_radius, t_near, t_far, eps)
    nrm = np.zeros((width * height, 3), np.float32)
    hit = np.isfinite(depth)
    if with_normals and hit.any():
        # the hit points as the march computed them (float32)
        o32 = np.asarray(eye, np.float64).astype(np.float32)
        nrm[hit] = normals(sdf_fn, o32[None, :] + depth[hit, None] * dirs[hit])
    return depth.reshape(height, width).astype(np.float32), nrm.reshape(height, width, 3).astype(np.float32)


def gpu_depth_image(build, width: int = 128, height: int = 128, view=(0.3, -1.0, 0.5), fov_deg: float = 40.0,
                    eps: float = 1e-3, with_normals: bool = True, max_steps: int = 256, normal_step: float = 1e-2):
    """depth_image of a built full-surface SesBuild in one device launch (sesgb_render)."""
    import torch
    eye, centre, up, t_near, t_far = framing(build.atoms, build.probe_radius, view, fov_deg)
    f, r, u = camera_basis(eye, centre, up)
    cam = dict(eye=eye, forward=f, right=r, up=u, tan_half_fov=float(np.tan(np.radians(fov_deg) / 2.0)),
               t_near=float(t_near), t_far=float(t_far), eps=float(eps), normal_step=float(normal_step),
               width=width, height=height, max_steps=max_steps)
    depth = torch.empty(width * height, dtype=torch.float32, device="cuda")
    nrm = torch.zeros(width * height * 3, dtype=torch.float32, device="cuda") if with_normals else None
    build.render(cam, depth.data_ptr(), nrm.data_ptr() if nrm is not None else None,
                 torch.cuda.current_stream().cuda_stream)
    d = depth.cpu().numpy().reshape(height, width)
    n = nrm.cpu().numpy().reshape(height, width, 3) if nrm is not None else np.zeros((height, width, 3), np.float32)
    return d, n


def gpu_sdf_fn(build):
    """The signed distance of a built full-surface SesBuild on the GPU, as a function of host points."""
    import torch

    def fn(points):
        q = torch.from_numpy(np.ascontiguousarray(points, np.float32)).cuda()
        out = torch.empty(q.shape[0], dtype=torch.float32, device="cuda")
        kind = torch.empty(q.shape[0], dtype=torch.int32, device="cuda")
        build.sdf(q.data_ptr(), q.shape[0], out.data_ptr(), kind.data_ptr(), torch.cuda.current_stream().cuda_stream)
        return out.cpu().numpy(), kind.cpu().numpy()

    return fn
