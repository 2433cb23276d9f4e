"""The allocation-free sort entry point (sesgb_sort_atoms_noalloc) through the C ABI.

It is meant for callers that cannot allocate device memory when they need the
sort (a plugin whose host owns a fixed device-memory budget, a loop that must
not enter the allocator); it keeps its scratch in a fixed array of the
library's device image. Its output must equal what the regular build produces
for the same atoms -- the sorted `atoms` buffer and the sorted-to-input
permutation, compared exactly as the other parity tests compare integer and
reordered data -- on calls in a row that reuse the scratch the previous call
left behind: the largest accepted size first, then smaller ones (other
histogram and tile counts), one of them sorted in a single radix pass. The
calls in a row must leave the device's free memory and torch's allocation
count unchanged.
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


def lattice(n, seed):
    """n atoms on a jittered 2.8 A lattice (protein-like density), in shuffled order."""
    rng = np.random.default_rng(seed)
    side = int(np.ceil(n ** (1.0 / 3.0)))
    g = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    xyz = g * 2.8 + rng.normal(0.0, 0.3, (n, 3))
    r = rng.choice(np.float32([1.52, 1.55, 1.7, 1.8]), n)
    a = np.c_[xyz, r].astype(np.float32)
    return a[rng.permutation(n)]


class Call:
    """Device buffers of one sort, allocated before any call is timed or checked."""

    def __init__(self, atoms):
        import torch
        from sesdf_gb300 import api
        self.n = atoms.shape[0]
        self.box = api.aabb(atoms)
        self.d_atoms = torch.from_numpy(atoms).cuda()
        self.d_sorted = torch.zeros((self.n, 4), dtype=torch.float32, device="cuda")
        self.d_perm = torch.zeros(self.n, dtype=torch.int32, device="cuda")

    def run(self, lib):
        import torch
        stream = torch.cuda.current_stream()
        st = lib.sesgb_sort_atoms_noalloc(self.d_atoms.data_ptr(), self.n, self.box.ctypes.data, ctypes.c_float(RP),
                                          self.d_sorted.data_ptr(), self.d_perm.data_ptr(), stream.cuda_stream)
        assert st == 0, lib.sesgb_error_string(st)

    def result(self):
        return self.d_sorted.cpu().numpy(), self.d_perm.cpu().numpy().astype(np.uint32)


def test_noalloc_sort_matches_build_in_a_row():
    import torch
    from sesdf_gb300 import api, synth
    lib = api.load_library()
    cases = [lattice(api.NOALLOC_MAX_ATOMS, 11),  # the largest accepted size
             synth.globule(1500, 1500),
             lattice(20, 12),  # one radix pass (odd pass count)
             synth.globule(20000, 1500),
             synth.jitter(synth.globule(20000, 1500), 0.3, 1401)]  # same size again, other order
    want = [regular_build(a, api.aabb(a)) for a in cases]
    calls = [Call(a) for a in cases]
    calls[1].run(lib)  # first call on the device: looks up the scratch array's address
    torch.cuda.synchronize()
    allocated = torch.cuda.memory_allocated()
    free = torch.cuda.mem_get_info()[0]
    for c in calls:
        c.run(lib)
    torch.cuda.synchronize()
    assert torch.cuda.memory_allocated() == allocated
    assert torch.cuda.mem_get_info()[0] == free
    for c, (want_atoms, want_perm) in zip(calls, want):
        got_atoms, got_perm = c.result()
        assert np.array_equal(got_perm, want_perm), c.n
        assert np.array_equal(got_atoms, want_atoms), c.n
    # and once more on the first case, after the smaller ones left their scratch behind
    calls[0].d_perm.zero_()
    calls[0].run(lib)
    got_atoms, got_perm = calls[0].result()
    assert np.array_equal(got_perm, want[0][1]) and np.array_equal(got_atoms, want[0][0])


def test_noalloc_trivial_sizes():
    import torch
    from sesdf_gb300 import api
    lib = api.load_library()
    box = np.float32([-2, -2, -2, 2, 2, 2])
    assert lib.sesgb_sort_atoms_noalloc(None, 0, box.ctypes.data, ctypes.c_float(RP), None, None, None) == 0
    one = Call(np.float32([[0.5, -0.25, 0.0, 1.7]]))
    one.run(lib)
    torch.cuda.synchronize()
    atoms, perm = one.result()
    assert perm.tolist() == [0] and np.array_equal(atoms, np.float32([[0.5, -0.25, 0.0, 1.7]]))


def test_noalloc_rejects_oversized_input():
    from sesdf_gb300 import api
    lib = api.load_library()
    box = np.zeros(6, np.float32)
    # rejected before anything is launched: no buffers are touched
    st = lib.sesgb_sort_atoms_noalloc(None, api.NOALLOC_MAX_ATOMS + 1, box.ctypes.data, ctypes.c_float(RP), None, None,
                                      None)
    assert st == -7
    assert b"no-allocation" in lib.sesgb_error_string(st)
