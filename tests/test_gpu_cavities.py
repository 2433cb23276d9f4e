"""Exterior and cavities on the GPU (sesgb_cavities, cavities.classify_gpu) against the host labelling
(cavities.classify: numpy rasterisation and scipy's 6-connected labelling). The label grids must be
equal voxel for voxel (components numbered by their first voxel on both sides), and so the exterior
and cavity sets, the cavity volumes and every probe's component."""
import numpy as np
import pytest

from sesdf_gb300 import SesBuild, SesgbError, cavities, synth
from test_cavities import shell

pytestmark = pytest.mark.gpu
RP = 1.4
RPF = float(np.float32(RP))  # the build's float32 probe radius


def both(atoms, mode, h):
    with SesBuild(atoms, RP, mode) as g:
        g.build()
        probes = g.fetch(analysis=False)["probe_pos"][:, :3]
        got = cavities.classify_gpu(g, h)
    want = cavities.classify(atoms, RPF, probes, h=h)
    return got, want, probes


def check(got, want):
    assert got["labels"].shape == want["labels"].shape
    assert np.array_equal(got["origin"], want["origin"])
    assert np.array_equal(got["labels"], want["labels"])
    assert got["exterior"] == want["exterior"] and got["cavities"] == want["cavities"]
    assert got["cavity_volume"] == want["cavity_volume"]
    assert np.array_equal(got["probe_component"], want["probe_component"])
    assert np.array_equal(got["probe_in_cavity"], want["probe_in_cavity"])


@pytest.mark.parametrize("h", [0.2, 0.3])
def test_closed_shell(h):
    atoms = shell()
    got, want, probes = both(atoms, "full", h)
    check(got, want)
    assert len(got["cavities"]) == 1
    assert np.array_equal(got["probe_in_cavity"], np.linalg.norm(probes, axis=1) < 10)


def test_open_shell_exterior_mode():
    atoms = shell()
    atoms = atoms[atoms[:, 2] < 7.0]
    got, want, _ = both(atoms, "exterior", 0.3)
    check(got, want)
    assert got["cavities"] == []


@pytest.mark.parametrize("n,seed,h", [(300, 11, 0.25), (2000, 1000, 0.25), (20000, 1500, 0.5)])
def test_globules(n, seed, h):
    atoms = synth.globule(n, seed)
    got, want, _ = both(atoms, "full", h)
    check(got, want)


def test_grid_size_guard():
    atoms = np.array([[0, 0, 0, 1.7], [400, 0, 0, 1.7], [0, 400, 0, 1.7], [0, 0, 400, 1.7]], np.float32)
    with SesBuild(atoms, RP, "full") as g:
        g.build()
        with pytest.raises(SesgbError, match="fixed limit"):
            g.cavities(0.25)
        assert g.cavities(2.0)["components"] >= 1
