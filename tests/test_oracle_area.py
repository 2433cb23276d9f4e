"""The FP64 SES-area oracle (oracle/area_oracle.c) against closed forms, Monte Carlo
and finite differences. The area is the area of the build's primitives (convex sphere
patches, tori over the accessible arcs, concave probe triangles outside the listed
neighbour probes); the reference computes none, so these checks pin it."""
import numpy as np
import pytest

from oracle import oracle
from sesdf_gb300 import synth

RP = 1.4


def _mc_region(cons, rng, n=1_000_000):
    y = rng.normal(size=(n, 3))
    y /= np.linalg.norm(y, axis=1)[:, None]
    ok = np.ones(n, bool)
    for w0, w1, w2, c in cons:
        ok &= y @ np.array([w0, w1, w2]) <= c
    return 4 * np.pi * ok.mean()


def test_region_closed_forms():
    assert oracle.region_area(np.zeros((0, 4)))[0] == pytest.approx(4 * np.pi, rel=1e-14)
    rng = np.random.default_rng(1)
    for c in (-0.9, -0.3, 0.0, 0.5, 0.99):
        w = rng.normal(size=3)
        w /= np.linalg.norm(w)
        a, s = oracle.region_area(np.array([[*w, c]]))
        assert a == pytest.approx(2 * np.pi * (1 + c), rel=1e-12)  # the sphere outside one cap
        assert s[0, 0] == pytest.approx(2 * np.pi, rel=1e-12)
    assert oracle.region_area(np.array([[0, 0, 1, -1.0]]))[0] == 0.0


@pytest.mark.parametrize("through_point", [False, True])
def test_region_monte_carlo(through_point):
    """Random cap sets; with through_point, most circles pass through one common point
    (the corners of a self-intersecting torus look like this)."""
    rng = np.random.default_rng(7 + through_point)
    for _ in range(12):
        M = int(rng.integers(2, 9))
        X = rng.normal(size=3)
        X /= np.linalg.norm(X)
        cons = []
        for m in range(M):
            w = rng.normal(size=3)
            w /= np.linalg.norm(w)
            c = float(w @ X) if through_point and (m < 3 or rng.random() < 0.5) else rng.uniform(-0.2, 0.9)
            cons.append([*w, c])
        cons = np.array(cons)
        a, _ = oracle.region_area(cons)
        assert abs(a - _mc_region(cons, rng)) < 0.04, cons  # 4 sigma of the Monte Carlo estimate


def test_region_derivatives():
    """dA/dc_m = boundary angle of m; dA/dw_m = -integral of y over it (tangential part)."""
    rng = np.random.default_rng(3)
    M = 6
    w = rng.normal(size=(M, 3))
    w /= np.linalg.norm(w, axis=1)[:, None]
    cons = np.concatenate([w, rng.uniform(0.0, 0.9, size=(M, 1))], 1)
    a, s = oracle.region_area(cons)
    h = 1e-6
    for m in range(M):
        cp, cm = cons.copy(), cons.copy()
        cp[m, 3] += h
        cm[m, 3] -= h
        assert (oracle.region_area(cp)[0] - oracle.region_area(cm)[0]) / (2 * h) == pytest.approx(s[m, 0], abs=1e-6)
        P = np.eye(3) - np.outer(cons[m, :3], cons[m, :3])
        fd = []
        for k in range(3):
            cp, cm = cons.copy(), cons.copy()
            cp[m, k] += h
            cm[m, k] -= h
            cp[m, :3] /= np.linalg.norm(cp[m, :3])
            cm[m, :3] /= np.linalg.norm(cm[m, :3])
            fd.append((oracle.region_area(cp)[0] - oracle.region_area(cm)[0]) / (2 * h))
        np.testing.assert_allclose(P @ np.array(fd), P @ -s[m, 1:], atol=1e-6)


def _two_sphere(r1, r2, d, rp):
    """SES of two spheres: two caps and the torus, integrated numerically."""
    R1, R2 = r1 + rp, r2 + rp
    h1 = (R1 * R1 - R2 * R2 + d * d) / (2 * d)
    rho = np.sqrt(R1 * R1 - h1 * h1)
    conv = 2 * np.pi * r1 * r1 * (1 + h1 / R1) + 2 * np.pi * r2 * r2 * (1 + (d - h1) / R2)
    b = np.linspace(-np.arctan2(h1, rho), np.arctan2(d - h1, rho), 400001)
    tor = 2 * np.pi * rp * np.trapezoid(np.maximum(0.0, rho - rp * np.cos(b)), b)
    return conv, tor


def test_atoms_closed_forms():
    p, per, _ = oracle.area(oracle.run(np.array([[0, 0, 0, 1.7]], np.float32), RP, "full"))
    assert p[0] == pytest.approx(4 * np.pi * float(np.float32(1.7)) ** 2, rel=1e-12) and p[1] == 0 and p[2] == 0
    for d, r2 in ((3.04, 1.5), (1.2, 1.55), (5.5, 1.8)):  # regular torus, self-intersecting torus, barely touching
        atoms = np.array([[0, 0, 0, 1.7], [d, 0, 0, r2]], np.float32)
        p, per, _ = oracle.area(oracle.run(atoms, RP, "full"))
        conv, tor = _two_sphere(float(np.float32(1.7)), float(np.float32(r2)), float(np.float32(d)), float(np.float32(RP)))
        assert p[0] == pytest.approx(conv, rel=1e-9)
        assert p[1] == pytest.approx(tor, rel=1e-6)
        assert per.sum() == pytest.approx(p.sum(), rel=1e-12)


def test_area_against_sdf_shell():
    """Independent check: the volume of the shell |sdf| < eps is 2 eps area (12 atoms)."""
    at = synth.globule(12, 3)
    at[:, :3] -= at[:, :3].mean(0)
    o = oracle.run(at.astype(np.float32), RP, "full")
    p, _, _ = oracle.area(o)
    lo = at[:, :3].min(0) - at[:, 3].max() - 0.5
    hi = at[:, :3].max(0) + at[:, 3].max() + 0.5
    rng = np.random.default_rng(0)
    eps, hits, n = 0.02, 0, 0
    for _ in range(8):
        q = (lo + (hi - lo) * rng.random((500_000, 3))).astype(np.float32)
        sd, _, _ = oracle.sdf(o, q)
        hits += np.count_nonzero(np.abs(sd) < eps)
        n += len(q)
    est = hits / n * np.prod(hi - lo) / (2 * eps)
    assert abs(est - p.sum()) < 4 * est / np.sqrt(hits), (est, p)


@pytest.mark.parametrize("n,seed", [(40, 7), (300, 11)])
def test_area_gradient_finite_differences(n, seed):
    """Central differences with h = 2^-12 A (exact in float32 near the origin)."""
    at = synth.globule(n, seed)
    at[:, :3] -= at[:, :3].mean(0)
    at = at.astype(np.float32)
    o = oracle.run(at, RP, "full")
    _, _, g = oracle.area(o, 1.0)
    h = 2.0 ** -12
    rng = np.random.default_rng(seed)
    for _ in range(10):
        s, k = int(rng.integers(0, n)), int(rng.integers(0, 4))
        src = o["perm"][s]
        ap, am = at.copy(), at.copy()
        ap[src, k] += h
        am[src, k] -= h
        fd = (oracle.area(oracle.run(ap, RP, "full"))[0].sum() - oracle.area(oracle.run(am, RP, "full"))[0].sum()) / (2 * h)
        assert g[s, k] == pytest.approx(fd, rel=1e-3, abs=1e-3)
