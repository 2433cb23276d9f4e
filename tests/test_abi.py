"""The C-ABI library loads and exports every entry point include/sesgb.h declares (no GPU needed)."""
import ctypes
import os
import re

import pytest

from sesdf_gb300 import _build, api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "sesgb.h")).read()
    return sorted(set(re.findall(r"\b(sesgb_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    _build.build_cuda()
    return api.load_library()


def test_header_lists_the_binding(lib):
    assert set(declared_functions()) == set(api.EXPORTS)


def test_every_declared_symbol_is_exported(lib):
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_error_strings(lib):
    assert lib.sesgb_error_string(0) == b"ok"
    assert lib.sesgb_error_string(-3) == b"capacity overflow"
    assert lib.sesgb_error_string(-99) == b"unknown status"
    assert lib.sesgb_last_error(None) == b"no context"


def test_invalid_arguments_are_rejected_without_a_gpu(lib):
    h = ctypes.c_void_p()
    # bad mode / missing output pointer: rejected before any CUDA call
    assert lib.sesgb_create(None, 0, None, ctypes.c_float(1.4), 7, None, ctypes.byref(h)) == -1
    assert lib.sesgb_create(None, 0, None, ctypes.c_float(1.4), 0, None, None) == -1
    assert lib.sesgb_build(None, None) == -1
    assert lib.sesgb_get_counts(None, None) == -1


def test_cpp_dropin_symbols(lib):
    # bcs::Sesdf / bcs::Ssesdf are compiled into the same library
    for sym in ("_ZN3bcs5Sesdf5buildEv", "_ZN3bcs6Ssesdf5buildEv", "_ZN3bcs5Sesdf7getDataEv",
                "_ZN3bcs6Ssesdf7getDataEv", "_ZN3bcs5Sesdf14getAtomIndicesEv"):
        assert hasattr(lib, sym), sym


def test_batch_and_sdf_arguments_are_rejected_without_a_gpu(lib):
    import numpy as np
    h = ctypes.c_void_p()
    atoms = np.zeros((4, 4), np.float32)
    # molecule starts must begin at 0 and never decrease
    bad = np.array([1, 2, 4], np.uint32)
    assert lib.sesgb_create_batch(atoms.ctypes.data, bad.ctypes.data, 2, ctypes.c_float(1.4), 0, None,
                                  ctypes.byref(h)) == -1
    dec = np.array([0, 3, 2, 4], np.uint32)
    assert lib.sesgb_create_batch(atoms.ctypes.data, dec.ctypes.data, 3, ctypes.c_float(1.4), 0, None,
                                  ctypes.byref(h)) == -1
    ok = np.array([0, 2, 4], np.uint32)
    assert lib.sesgb_create_batch(atoms.ctypes.data, ok.ctypes.data, 0, ctypes.c_float(1.4), 0, None,
                                  ctypes.byref(h)) == -1  # no molecules
    assert lib.sesgb_create_batch(atoms.ctypes.data, ok.ctypes.data, 2, ctypes.c_float(1.4), 9, None,
                                  ctypes.byref(h)) == -1  # bad mode
    assert lib.sesgb_batch_molecules(None) == 0
    rec = (ctypes.c_uint32 * len(api.MOL_FIELDS))()
    assert lib.sesgb_molecule_record(None, 0, rec) == -1
    assert lib.sesgb_get_full_molecule(None, 0, None) == -1
    assert lib.sesgb_sdf(None, None, 0, None, None, None) == -1
    assert lib.sesgb_sdf_backward(None, None, 0, None, None, None) == -1
    assert len(api.MOL_FIELDS) == 16
