"""The allocation-free sort entry point (sesgb_sort_atoms_noalloc) through the C ABI.

It is meant for callers that cannot allocate device memory when they need the
sort (during a stream capture, under a host-owned memory budget); it keeps its
scratch in a fixed array of the library's device image. Its output must equal
what the regular build produces for the same atoms -- the sorted `atoms` buffer
and the sorted-to-input permutation, compared exactly as the other parity tests
compare integer and reordered data -- on two calls in a row (the second call
reuses the scratch the first one left behind).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RP = 1.4


def regular_build(atoms, box):
    from sesdf_gb300 import SesBuild
    with SesBuild(atoms, RP, "full", box=box) as g:
        g.build()
        out = g.fetch(analysis=True)
    return out["atoms"], out["perm"]


def noalloc_sort(lib, atoms, box):
    import torch
    n = atoms.shape[0]
    d_atoms = torch.from_numpy(atoms).cuda()
    d_sorted = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    d_perm = torch.zeros(n, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    st = lib.sesgb_sort_atoms_noalloc(d_atoms.data_ptr(), n, box.ctypes.data, ctypes.c_float(RP), d_sorted.data_ptr(),
                                      d_perm.data_ptr(), stream.cuda_stream)
    assert st == 0, lib.sesgb_error_string(st)
    torch.cuda.synchronize()
    return d_sorted.cpu().numpy(), d_perm.cpu().numpy().astype(np.uint32)


def test_noalloc_sort_matches_build_twice():
    from sesdf_gb300 import api, synth
    lib = api.load_library()
    first = synth.globule(20000, 1500)
    second = synth.jitter(first, 0.3, 1401)  # a second frame: same size, other order
    box = api.aabb(first)
    for atoms in (first, second):  # two calls in a row share the scratch
        want_atoms, want_perm = regular_build(atoms, box)
        got_atoms, got_perm = noalloc_sort(lib, atoms, box)
        assert np.array_equal(got_perm, want_perm)
        assert np.array_equal(got_atoms, want_atoms)


def test_noalloc_rejects_oversized_input():
    from sesdf_gb300 import api
    lib = api.load_library()
    box = np.zeros(6, np.float32)
    # rejected before anything is launched: no buffers are touched
    st = lib.sesgb_sort_atoms_noalloc(None, api.NOALLOC_MAX_ATOMS + 1, box.ctypes.data, ctypes.c_float(RP), None, None,
                                      None)
    assert st == -7
    assert b"no-allocation" in lib.sesgb_error_string(st)
