"""SES area of the build's primitives (sesgb_ses_area) and its adjoint against the
FP64 oracle (oracle/area_oracle.c, pinned by closed forms, Monte Carlo and finite
differences in test_oracle_area.py).

Both evaluate the same primitives: the build's topology is identical, and the
oracle takes the float32 probe positions the build stores (the primitives are
those; two nearly coincident probes make the concave area sensitive to that
rounding, so FP64 positions would compare a different surface). The convex,
toroidal and concave parts agree to 1e-4 relative, per-atom areas to
1e-3 A^2 + 1e-4 relative, and the adjoint d area / d (x, y, z, r) to 1e-3 of its
largest component.
"""
import numpy as np
import pytest

from cases import hand_cases
from oracle import oracle
from sesdf_gb300 import SesBuild, synth

pytestmark = pytest.mark.gpu
RP = 1.4


def gpu_area(atoms, grad=False):
    import torch
    with SesBuild(atoms, RP, "full") as g:
        g.build()
        per = torch.zeros(atoms.shape[0], dtype=torch.float32, device="cuda")
        parts = g.ses_area(per.data_ptr())
        gr = None
        if grad:
            ga = torch.empty((atoms.shape[0], 4), dtype=torch.float32, device="cuda")
            g.ses_area_backward(ga.data_ptr())
            torch.cuda.synchronize()
            gr = ga.cpu().numpy().astype(np.float64)
        return parts, per.cpu().numpy().astype(np.float64), gr


def oracle_area(atoms, grad=False):
    o = oracle.run(atoms, RP, "full")
    o["posd"] = o["posf"].astype(np.float64)  # the stored (float32) probe positions
    p, per, g = oracle.area(o, 1.0 if grad else None)
    perm = o["perm"]
    pin = np.zeros_like(per)
    pin[perm] = per  # sorted -> input order
    gin = None
    if g is not None:
        gin = np.zeros_like(g)
        gin[perm] = g
    return p, pin, gin


def _check(atoms, name):
    got, per, _ = gpu_area(atoms)
    want, wper, _ = oracle_area(atoms)
    for k, key in enumerate(("convex", "toroidal", "concave")):
        assert got[key] == pytest.approx(want[k], rel=1e-4, abs=1e-3), (name, key, got, want)
    assert got["total"] == pytest.approx(want.sum(), rel=1e-4, abs=1e-3)
    err = np.abs(per - wper)
    assert np.all(err <= 1e-3 + 1e-4 * np.abs(wper)), (name, err.max(), int(np.argmax(err)))
    assert per.sum() == pytest.approx(got["total"], rel=1e-5)


def test_single_and_two_atoms():
    got, _, _ = gpu_area(np.array([[0, 0, 0, 1.7]], np.float32))
    assert got["convex"] == pytest.approx(4 * np.pi * float(np.float32(1.7)) ** 2, rel=1e-6)
    assert got["toroidal"] == 0 and got["concave"] == 0
    for d, r2 in ((3.04, 1.5), (1.2, 1.55), (5.5, 1.8)):
        _check(np.array([[0, 0, 0, 1.7], [d, 0.3, -0.2, r2]], np.float32), f"pair{d}")


@pytest.mark.parametrize("name", ["pair", "pair_far", "triangle", "tangent", "tetrahedron", "trigonal", "cluster40",
                                  "octahedron", "stack", "square", "collinear", "hexring"])
def test_hand_cases(name):
    _check(hand_cases()[name], name)


@pytest.mark.parametrize("n,seed", [(300, 11), (2000, 1000)])
def test_globules(n, seed):
    _check(synth.globule(n, seed), f"globule{n}")


def test_gradient_matches_oracle():
    """The adjoint against the oracle's FP64 adjoint on the same float32 probe positions: within
    1e-3 relative (Frobenius) and every component within 1e-3 of the largest. Where the adjoint
    is ill-conditioned (torus arc ends at shallow crossings, probe regions with a nearly
    coincident neighbour probe, probes near the plane of their centres) the GPU takes those
    terms in double precision."""
    atoms = synth.globule(2000, 1000)
    _, _, g = gpu_area(atoms, grad=True)
    _, _, go = oracle_area(atoms, grad=True)
    scale = np.abs(go).max()
    err = np.abs(g - go)
    rel = np.linalg.norm(g - go) / np.linalg.norm(go)
    frac = np.mean(err <= 1e-3 * scale)
    print(f"area adjoint, 2,000 atoms: GPU vs oracle {rel:.2e} relative (Frobenius), {frac:.4f} of components within "
          f"1e-3 of the largest, worst {err.max() / scale:.2e}")
    assert rel <= 1e-3 and frac == 1.0, (rel, frac, err.max(), scale, np.unravel_index(np.argmax(err), err.shape))


def test_torch_autograd():
    torch = pytest.importorskip("torch")
    from sesdf_gb300.torch_sdf import ses_area
    atoms = synth.globule(300, 11)
    a = torch.from_numpy(atoms).cuda().requires_grad_(True)
    area = ses_area(a, RP)
    (2.0 * area).backward()
    want, _, go = oracle_area(atoms, grad=True)
    assert float(area.detach()) == pytest.approx(want.sum(), rel=1e-4)
    g = a.grad.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(g - 2.0 * go) <= 1e-3 * np.linalg.norm(2.0 * go)


def test_sdf_workload_globule():
    """The 20,000-atom globule of the SDF workload (seed 1500): parts and the adjoint's bulk."""
    atoms = synth.globule(20000, 1500)
    got, per, g = gpu_area(atoms, grad=True)
    want, wper, go = oracle_area(atoms, grad=True)
    for k, key in enumerate(("convex", "toroidal", "concave")):
        assert got[key] == pytest.approx(want[k], rel=1e-4), (key, got, want)
    assert np.mean(np.abs(per - wper) <= 1e-3 + 1e-4 * np.abs(wper)) >= 0.999
    rel = np.linalg.norm(g - go) / np.linalg.norm(go)
    print(f"area adjoint, 20,000 atoms: GPU vs oracle {rel:.2e} relative (Frobenius)")
    assert rel <= 1e-3
