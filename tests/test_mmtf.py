"""The MMTF reader (sesdf_gb300/mmtf.py): MessagePack container, binary codecs, the vdW radius
lookup of the reference's loader, and the committed sample-structure fixture.

Codecs are checked by round trips through encoders written here from the MMTF 1.0 specification and by
literal vectors; where the reference checkout is present, the reader is also checked against the
reference's radius table (sesdf/src/core/molecule.cpp) and its sample files, and the MessagePack
decoder against the msgpack package when that is installed.
"""
import os
import re
import struct

import numpy as np
import pytest

from oracle.refharness import reference_checkout
from sesdf_gb300 import mmtf

HERE = os.path.dirname(os.path.abspath(__file__))
STRUCTURES = os.path.join(HERE, "golden", "structures.npz")


def header(codec, length, param=0):
    return struct.pack(">iii", codec, length, param)


def recursive_encode(values, lo, hi):
    out = []
    for v in values:
        while v >= hi:
            out.append(hi)
            v -= hi
        while v <= lo:
            out.append(lo)
            v -= lo
        out.append(v)
    return out


def run_length_encode(values):
    out = []
    for v in values:
        if out and out[-2] == v:
            out[-1] += 1
        else:
            out += [v, 1]
    return out


def test_msgpack_forms():
    data = (bytes([0x84])                                   # fixmap of 4
            + bytes([0xA1]) + b"a" + bytes([0x05])          # "a": 5
            + bytes([0xA1]) + b"b" + bytes([0xE0])          # "b": -32
            + bytes([0xD9, 3]) + b"key"                     # str8 "key"
            + bytes([0xDC, 0, 3, 0xC0, 0xC3, 0xCB]) + struct.pack(">d", 2.5)  # [nil, true, 2.5]
            + bytes([0xA1]) + b"c" + bytes([0xC4, 2, 1, 2]))  # "c": bin8 b"\x01\x02"
    assert mmtf.unpack_msgpack(data) == {"a": 5, "b": -32, "key": [None, True, 2.5], "c": b"\x01\x02"}
    wide = bytes([0xD2]) + struct.pack(">i", -70000)
    assert mmtf.unpack_msgpack(wide) == -70000
    with pytest.raises(ValueError):
        mmtf.unpack_msgpack(bytes([0xA5]) + b"ab")  # truncated


def test_codec_literals():
    # 10: delta + recursive index (int16) / 1000: 32767 + 1 -> 32768 (one value), then deltas
    raw = [32767, 1, 500, -1500]
    buf = header(10, 3, 1000) + struct.pack(">4h", *raw)
    got = mmtf.decode_codec(buf)
    want = np.array([32768, 33268, 31768], np.float32) / np.float32(1000)
    assert got.dtype == np.float32 and np.array_equal(got, want)
    # 4: int32; 8: run-length + delta; 5: fixed-width strings; 6: run-length chars
    assert mmtf.decode_codec(header(4, 2) + struct.pack(">2i", 7, -9)).tolist() == [7, -9]
    assert mmtf.decode_codec(header(8, 4) + struct.pack(">4i", 1, 3, 5, 1)).tolist() == [1, 2, 3, 8]
    assert mmtf.decode_codec(header(5, 2, 4) + b"A\0\0\0BCD\0").tolist() == ["A", "BCD"]
    assert mmtf.decode_codec(header(6, 3) + struct.pack(">4i", 65, 2, 0, 1)).tolist() == ["A", "A", ""]
    with pytest.raises(ValueError):
        mmtf.decode_codec(header(4, 3) + struct.pack(">2i", 7, -9))  # length mismatch


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_codec_round_trips(seed):
    rng = np.random.default_rng(seed)
    coords = np.cumsum(rng.integers(-40000, 40000, 500))  # deltas beyond the int16 range
    deltas = np.diff(np.concatenate([[0], coords]))
    enc = recursive_encode(deltas.tolist(), -32768, 32767)
    got = mmtf.decode_codec(header(10, len(coords), 1000) + struct.pack(f">{len(enc)}h", *enc))
    assert np.array_equal(got, coords.astype(np.float32) / np.float32(1000))
    ints = rng.integers(-300, 300, 200)
    enc = recursive_encode(ints.tolist(), -128, 127)
    assert np.array_equal(mmtf.decode_codec(header(13, len(ints)) + struct.pack(f">{len(enc)}b", *enc)), ints)
    runs = np.repeat(rng.integers(0, 5, 30), rng.integers(1, 6, 30))
    enc = run_length_encode(runs.tolist())
    assert np.array_equal(mmtf.decode_codec(header(7, len(runs)) + struct.pack(f">{len(enc)}i", *enc)), runs)


def test_radius_lookup():
    assert mmtf.radius_of("C") == np.float32(1.77) and mmtf.radius_of("n") == np.float32(1.66)
    assert mmtf.radius_of("O") == np.float32(1.50) and mmtf.radius_of("S") == np.float32(1.89)
    assert mmtf.radius_of("Fe") == np.float32(2.44) and mmtf.radius_of("ZN") == np.float32(2.39)
    # not an enumerator of the reference's SYMBOL: the UNKNOWN radius
    for s in ("D", "X", "", "UNKNOWN", "COUNT"):
        assert mmtf.radius_of(s) == np.float32(1.20), s


def test_minimal_document():
    """A two-model document: only the first model's atoms, radii from each group's element list."""
    def mp_str(s):
        b = s.encode()
        return bytes([0xA0 | len(b)]) + b

    def mp_bin(b):
        return bytes([0xC4, len(b)]) + b

    xs = header(10, 3, 1000) + struct.pack(">3h", 1000, 500, -250)
    group = bytes([0x81]) + mp_str("elementList") + bytes([0x92]) + mp_str("C") + mp_str("O")
    group1 = bytes([0x81]) + mp_str("elementList") + bytes([0x91]) + mp_str("Zz")
    doc = (bytes([0x87])
           + mp_str("xCoordList") + mp_bin(xs) + mp_str("yCoordList") + mp_bin(xs) + mp_str("zCoordList") + mp_bin(xs)
           + mp_str("groupTypeList") + mp_bin(header(4, 2) + struct.pack(">2i", 0, 1))
           + mp_str("groupList") + bytes([0x92]) + group + group1
           + mp_str("chainsPerModel") + bytes([0x92, 1, 1])
           + mp_str("groupsPerChain") + bytes([0x92, 1, 1]))
    atoms = mmtf.load_bytes(doc)
    assert atoms.shape == (2, 4)
    assert np.array_equal(atoms[:, 0], np.array([1.0, 1.5], np.float32))
    assert np.array_equal(atoms[:, 3], np.array([1.77, 1.50], np.float32))
    import gzip
    assert np.array_equal(mmtf.load_bytes(gzip.compress(doc)), atoms)


def minimal_document(elements=("C", "O"), coords=(1000, 500, -250)):
    def mp_str(s):
        b = s.encode()
        return bytes([0xA0 | len(b)]) + b

    def mp_bin(b):
        return bytes([0xC4, len(b)]) + b

    xs = header(10, len(coords), 1000) + struct.pack(f">{len(coords)}h", *coords)
    group = bytes([0x81]) + mp_str("elementList") + bytes([0x90 | len(elements)]) + b"".join(mp_str(e) for e in elements)
    return (bytes([0x87])
            + mp_str("xCoordList") + mp_bin(xs) + mp_str("yCoordList") + mp_bin(xs) + mp_str("zCoordList") + mp_bin(xs)
            + mp_str("groupTypeList") + mp_bin(header(4, 1) + struct.pack(">i", 0))
            + mp_str("groupList") + bytes([0x91]) + group
            + mp_str("chainsPerModel") + bytes([0x91, 1])
            + mp_str("groupsPerChain") + bytes([0x91, 1]))


def test_native_reader():
    """sesgb_load_mmtf (C++, in the library) reads what the Python reader reads, and reports errors."""
    import ctypes

    from sesdf_gb300 import api
    doc = minimal_document(("C", "fe", "Xx"))
    got = api.load_mmtf(doc)
    assert np.array_equal(got, mmtf.load_bytes(doc))
    assert np.array_equal(got[:, 3], np.array([1.77, 2.44, 1.20], np.float32))
    import gzip
    assert np.array_equal(api.load_mmtf(gzip.compress(doc)), got)
    lib = api.load_library()
    n = ctypes.c_uint32()
    small = np.zeros((1, 4), np.float32)
    assert lib.sesgb_load_mmtf(doc, len(doc), small.ctypes.data, 1, ctypes.byref(n)) == -3 and n.value == 3
    for bad in (b"", b"\x93\x01\x02", doc[:40], b"\xc1" + doc):
        assert lib.sesgb_load_mmtf(bad, len(bad), None, 0, ctypes.byref(n)) == -1, bad[:8]
    with pytest.raises(api.SesgbError):
        api.load_mmtf(b"\x80")


def test_structure_fixture():
    with np.load(STRUCTURES) as s:
        sizes = {k: s[k].shape for k in s.files}
        for k in s.files:
            a = s[k]
            assert a.dtype == np.float32 and np.isfinite(a).all()
            assert set(np.unique(a[:, 3]).tolist()) <= set(mmtf.VDW_RADIUS.tolist())
    assert sizes == {"1AGA": (126, 4), "101M": (1413, 4), "1VIS": (2531, 4), "7SC0": (11638, 4)}


REFERENCE = reference_checkout()


@pytest.mark.skipif(REFERENCE is None or not os.path.isdir(os.path.join(REFERENCE, "samples")),
                    reason="reference checkout absent")
def test_against_reference_checkout():
    # the radius table, as the reference states it
    src = open(os.path.join(REFERENCE, "sesdf/src/core/molecule.cpp")).read()
    vals = re.findall(r"([0-9]+\.[0-9]+)f,? +// ([A-Z]+)", src)
    assert [s for _, s in vals] == mmtf.SYMBOLS
    assert np.array_equal(np.array([float(v) for v, _ in vals], np.float32), mmtf.VDW_RADIUS)
    # the committed fixture is what the reader makes of the reference's samples
    with np.load(STRUCTURES) as s:
        for k in s.files:
            assert np.array_equal(mmtf.load(os.path.join(REFERENCE, "samples", f"{k}.mmtf")), s[k]), k
    from sesdf_gb300 import api
    for path in sorted(os.listdir(os.path.join(REFERENCE, "samples"))):
        if path.endswith(".mmtf"):
            data = open(os.path.join(REFERENCE, "samples", path), "rb").read()
            assert np.array_equal(api.load_mmtf(data), mmtf.load_bytes(data)), path
    msgpack = pytest.importorskip("msgpack")
    data = open(os.path.join(REFERENCE, "samples", "101M.mmtf"), "rb").read()
    assert mmtf.unpack_msgpack(data) == msgpack.unpackb(data, raw=False)
