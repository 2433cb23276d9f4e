"""Exterior and cavities of the probe-accessible space (sesdf_gb300/cavities.py) on inputs whose answer
is known: a closed shell of atoms around an empty core holds one cavity, and the probes of the build on
its inner side are the cavity's, those outside the exterior's."""
import numpy as np

from oracle import oracle
from sesdf_gb300 import cavities, synth

RP = 1.4


def shell(n=320, radius=10.0, r=1.7):
    """Atoms on a sphere (Fibonacci points, ~2 A apart): their SAS spheres close the shell for a probe."""
    k = np.arange(n) + 0.5
    phi = np.arccos(1.0 - 2.0 * k / n)
    th = np.pi * (1.0 + 5.0 ** 0.5) * k
    p = np.stack([np.cos(th) * np.sin(phi), np.sin(th) * np.sin(phi), np.cos(phi)], axis=1) * radius
    return np.concatenate([p, np.full((n, 1), r)], axis=1).astype(np.float32)


def test_shell_has_one_cavity():
    atoms = shell()
    probes = oracle.run(atoms, RP, "full")["posf"][:, :3]
    rad = np.linalg.norm(probes, axis=1)
    assert (rad < 10).any() and (rad > 10).any()
    for h in (0.2, 0.3):
        c = cavities.classify(atoms, RP, probes, h=h)
        assert len(c["cavities"]) == 1 and len(c["exterior"]) == 1
        assert c["probe_resolved"].all()
        assert np.array_equal(c["probe_in_cavity"], rad < 10)
        # probe-centre space of the core: a ball of radius ~ 10 - (1.7 + 1.4), bumpy
        assert abs(c["cavity_volume"][0] / (4.0 / 3.0 * np.pi * 6.9 ** 3) - 1.0) < 0.15


def test_open_shell_has_none():
    atoms = shell()
    keep = atoms[:, 2] < 7.0  # a hole at the top lets a probe in
    c = cavities.classify(atoms[keep], RP, h=0.3)
    assert c["cavities"] == [] and len(c["exterior"]) == 1


def test_single_atom_and_globule():
    c = cavities.classify(np.array([[0, 0, 0, 1.7]], np.float32), RP, h=0.3)
    assert c["cavities"] == [] and len(c["exterior"]) == 1
    atoms = synth.globule(300, 11)
    probes = oracle.run(atoms, RP, "full")["posf"][:, :3]
    c = cavities.classify(atoms, RP, probes, h=0.25)
    lab = c["labels"]
    sizes = np.bincount(lab.ravel())
    ext = max(c["exterior"], key=lambda k: sizes[k])
    assert sizes[ext] == sizes[1:].max()  # the exterior is the largest component
    assert np.mean(c["probe_resolved"]) > 0.9
    assert not np.any(c["probe_in_cavity"] & ~c["probe_resolved"])


def test_grid_size_guard():
    import pytest
    atoms = np.array([[0, 0, 0, 1.7], [400, 0, 0, 1.7], [0, 400, 0, 1.7], [0, 0, 400, 1.7]], np.float32)
    with pytest.raises(ValueError):
        cavities.accessible_grid(atoms, RP, h=0.25)
