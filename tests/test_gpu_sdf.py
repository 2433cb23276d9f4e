"""Signed distance to the SES at query points, and its adjoint, against the FP64 oracle.

Values: within 1e-4 A of the oracle (both evaluate the same definition; the
GPU in float32 with the float32-rounded probe positions of the build). The
primitive that decides each value (atom, sphere patch, arc, probe) agrees
except on exact ties. Gradients: the GPU adjoint of sum_q g_q sdf_q with
respect to every atom's (x, y, z, r) against the oracle's analytic gradient
(same active primitives, FP64) and against FP64 central finite differences of
the oracle (h = 1e-4 A, relative tolerance 1e-3).
"""
import numpy as np
import pytest

from cases import hand_cases
from oracle import oracle
from sesdf_gb300 import SesBuild, synth

pytestmark = pytest.mark.gpu
RP = 1.4
TOL = 1e-4


def gpu_sdf(atoms, q, gq=None):
    import torch
    with SesBuild(atoms, RP, "full") as g:
        g.build()
        dq = torch.from_numpy(np.ascontiguousarray(q, np.float32)).cuda()
        out = torch.empty(q.shape[0], dtype=torch.float32, device="cuda")
        kind = torch.empty(q.shape[0], dtype=torch.int32, device="cuda")
        g.sdf(dq.data_ptr(), q.shape[0], out.data_ptr(), kind.data_ptr())
        grad = None
        if gq is not None:
            dg = torch.from_numpy(np.ascontiguousarray(gq, np.float32)).cuda()
            ga = torch.empty((atoms.shape[0], 4), dtype=torch.float32, device="cuda")
            g.sdf_backward(dq.data_ptr(), q.shape[0], dg.data_ptr(), ga.data_ptr())
            grad = ga.cpu().numpy().astype(np.float64)
        torch.cuda.synchronize()
        c = g.counts()
        return out.cpu().numpy(), kind.cpu().numpy(), grad, c


def oracle_sdf(atoms, q, gq=None):
    o = oracle.run(atoms, RP, "full")
    s, k, g = oracle.sdf(o, q, gq=gq)
    if g is not None:
        gin = np.zeros_like(g)
        gin[o["perm"]] = g  # sorted -> input order
        g = gin
    return s, k, g


@pytest.mark.parametrize("name", ["globule2k", "cluster40", "octahedron", "stack", "square"])
def test_sdf_values_match_oracle(name):
    atoms = synth.globule(2000, 1000) if name == "globule2k" else hand_cases()[name]
    q = synth.queries(atoms, 20000 if name == "globule2k" else 4000, 1501)
    got, kind, _, c = gpu_sdf(atoms, q)
    want, wkind, _ = oracle_sdf(atoms, q)
    assert c["outside_atoms"] == 0
    err = np.abs(got.astype(np.float64) - want)
    assert err.max() <= TOL, (name, err.max(), int(np.argmax(err)))
    assert np.mean(kind == wkind) > 0.99
    assert got.min() >= -3.0 - TOL and got.max() <= 3.0 + TOL


def test_sdf_gradient_matches_oracle_and_finite_differences():
    atoms = synth.globule(2000, 1000)
    q = synth.queries(atoms, 20000, 1501)
    rng = np.random.default_rng(1502)
    gq = rng.standard_normal(q.shape[0])
    _, _, g, _ = gpu_sdf(atoms, q, gq)
    _, _, go = oracle_sdf(atoms, q, gq)
    scale = np.abs(go).max()
    assert np.abs(g - go).max() <= 1e-3 * scale
    # FP64 central differences of the oracle on random atoms
    h = 1e-4
    for a in rng.choice(atoms.shape[0], 8, replace=False):
        for comp in range(4):
            ap = atoms.astype(np.float64).copy()
            am = ap.copy()
            ap[a, comp] += h
            am[a, comp] -= h
            ap32, am32 = ap.astype(np.float32), am.astype(np.float32)
            step = float(ap32[a, comp]) - float(am32[a, comp])
            sp, _, _ = oracle_sdf(ap32, q)
            sm, _, _ = oracle_sdf(am32, q)
            fd = (gq @ sp - gq @ sm) / step
            rel = abs(fd - g[a, comp]) / max(abs(fd), 1e-2)
            assert rel <= 1e-3, (a, comp, fd, g[a, comp])


def test_torch_autograd_binding():
    torch = pytest.importorskip("torch")
    from sesdf_gb300.torch_sdf import ses_sdf
    atoms = synth.globule(1500, 1601)
    q = synth.queries(atoms, 5000, 1602)
    a = torch.from_numpy(atoms).cuda().requires_grad_(True)
    s = ses_sdf(a, torch.from_numpy(q).cuda())
    w = torch.linspace(-1.0, 1.0, q.shape[0], device="cuda")
    (s * w).sum().backward()
    _, _, g, _ = gpu_sdf(atoms, q, w.cpu().numpy())
    assert np.allclose(a.grad.cpu().numpy(), g, atol=1e-5 * max(1.0, np.abs(g).max()))
    want, _, _ = oracle_sdf(atoms, q)
    assert np.abs(s.detach().cpu().numpy() - want).max() <= TOL
