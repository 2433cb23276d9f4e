"""Sphere-traced SES images on the GPU signed distance (sesdf_gb300/render.py, gpu_sdf_fn) against the
same tracer on the FP64 oracle: the same pixels hit (a ray grazing the surface within eps may differ),
every GPU hit point on the oracle's surface within eps, depths and normals alike."""
import numpy as np
import pytest

from oracle import oracle
from sesdf_gb300 import SesBuild, render, synth

pytestmark = pytest.mark.gpu
RP = 1.4
EPS = 1e-3


@pytest.mark.parametrize("n,seed", [(300, 11), (2000, 1000)])
def test_depth_image_matches_oracle(n, seed):
    atoms = synth.globule(n, seed)
    o = oracle.run(atoms, RP, "full")
    ofn = lambda p: oracle.sdf(o, p)[:2]  # noqa: E731
    with SesBuild(atoms, RP, "full") as g:
        g.build()
        gfn = render.gpu_sdf_fn(g)
        depth, nrm = render.depth_image(gfn, atoms, RP, 64, 64, eps=EPS)
    want, wnrm = render.depth_image(ofn, atoms, RP, 64, 64, eps=EPS)
    hit, whit = np.isfinite(depth), np.isfinite(want)
    assert hit.sum() > 500
    assert np.mean(hit == whit) >= 0.99
    both = hit & whit
    assert np.quantile(np.abs(depth[both] - want[both]), 0.99) <= 5 * EPS
    dots = np.einsum("ij,ij->i", nrm[both], wnrm[both])
    assert np.mean(dots > 0.99) >= 0.95
    # every GPU hit point lies on the oracle's surface
    a = np.asarray(atoms, np.float64)
    lo = (a[:, :3] - a[:, 3:4] - RP).min(axis=0)
    hi = (a[:, :3] + a[:, 3:4] + RP).max(axis=0)
    c = 0.5 * (lo + hi)
    rad = 0.5 * np.linalg.norm(hi - lo)
    v = np.array((0.3, -1.0, 0.5)) / np.linalg.norm((0.3, -1.0, 0.5))
    dist = rad / np.sin(np.radians(20.0))
    eye = c - dist * v
    dirs = render.camera_rays(eye, c, (0, 0, 1), 40.0, 64, 64)
    p = eye + depth.ravel()[hit.ravel(), None].astype(np.float64) * dirs[hit.ravel()]
    val, kind = ofn(p.astype(np.float32))
    assert np.all(np.isin(kind, render.INSIDE_SAS))
    assert val.min() >= -1e-3 and val.max() < EPS + 1e-3


@pytest.mark.parametrize("n,seed", [(300, 11), (2000, 1000)])
def test_device_trace_matches_host_loop_and_oracle(n, seed):
    """sesgb_render traces every ray in one launch: its image equals, pixel for pixel and bit for bit,
    the host loop of sphere_trace over sesgb_sdf (same ray arithmetic, same signed distance), and so
    the oracle's image as above."""
    atoms = synth.globule(n, seed)
    with SesBuild(atoms, RP, "full") as g:
        g.build()
        loop_depth, loop_nrm = render.depth_image(render.gpu_sdf_fn(g), atoms, RP, 64, 48, eps=EPS)
        depth, nrm = render.gpu_depth_image(g, 64, 48, eps=EPS)
        c = g.counts()
    assert depth.shape == (48, 64) and nrm.shape == (48, 64, 3)
    assert np.array_equal(depth, loop_depth)
    assert np.array_equal(nrm, loop_nrm)
    o = oracle.run(atoms, RP, "full")
    want, _ = render.depth_image(lambda p: oracle.sdf(o, p)[:2], atoms, RP, 64, 48, eps=EPS)
    hit, whit = np.isfinite(depth), np.isfinite(want)
    assert hit.sum() > 300 and np.mean(hit == whit) >= 0.99
    both = hit & whit
    assert np.quantile(np.abs(depth[both] - want[both]), 0.99) <= 5 * EPS
    assert c["atoms"] == n


def test_device_trace_rejects_bad_camera():
    import torch
    from sesdf_gb300 import SesgbError
    atoms = synth.globule(300, 11)
    with SesBuild(atoms, RP, "full") as g:
        g.build()
        out = torch.empty(4, dtype=torch.float32, device="cuda")
        cam = dict(eye=(0, 0, -50), forward=(0, 0, 1), right=(1, 0, 0), up=(0, 1, 0), tan_half_fov=0.3, t_near=0.0,
                   t_far=100.0, eps=0.0, normal_step=1e-2, width=2, height=2, max_steps=16)
        with pytest.raises(SesgbError):
            g.render(cam, out.data_ptr())
