"""Atoms of a structure file in the MMTF format: (x, y, z, vdW radius) of the first model.

Follows bcs::load (sesdf/src/core/loader.cpp:14-71), which reads a structure through chemfiles: the atoms
of the first frame, residue by residue in file order, each with the radius of its element
(bcs::getRadius, sesdf/src/core/molecule.cpp:9-131). The element symbol is upper-cased and looked up as
the enumerator "A_<symbol>" of bcs::SYMBOL (sesdf/include/bcs/core/molecule.hpp:13-140); a symbol that is
not there takes the UNKNOWN radius. Coordinates are the file's integers divided by the codec parameter in
float32, as the MMTF decoder under chemfiles does.

The container (MessagePack) and the binary codecs are decoded here from the MMTF 1.0 specification; no
third-party package is needed, so the reader also runs where none is installed.
"""
import gzip
import struct

import numpy as np

# bcs::SYMBOL in enumerator order (atomic number = index; 0 is UNKNOWN). The codes past 104 are the
# reference's own (DD, SG, BHJ, ... UUO) and are kept so that the lookup answers the same.
SYMBOLS = (
    "UNKNOWN H HE LI BE B C N O F NE NA MG AL SI P S CL AR K CA SC TI V CR MN FE CO NI CU ZN GA GE AS SE BR KR "
    "RB SR Y ZR NB MO TC RU RH PD AG CD IN SN SB TE I XE CS BA LA CE PR ND PM SM EU GD TB DY HO ER TM YB LU HF "
    "TA W RE OS IR PT AU HG TL PB BI PO AT RN FR RA AC TH PA U NP PU AM CM BK CF ES FM MD NO LR RF DD SG BHJ HS "
    "MT DS RG UUB UUT UUQ UUP UUH UUS UUO"
).split()

# van der Waals radius (A) by the index above, as bcs::getRadius returns it (0 where the reference has none)
VDW_RADIUS = np.array([
    1.20, 1.20, 1.43, 2.12, 1.98, 1.91, 1.77, 1.66, 1.50, 1.46, 1.58, 2.50, 2.51, 2.25, 2.19, 1.90, 1.89, 1.82, 1.83,
    2.73, 2.62, 2.58, 2.46, 2.42, 2.45, 2.45, 2.44, 2.40, 2.40, 2.38, 2.39, 2.32, 2.29, 1.88, 1.82, 1.86, 2.25,
    3.21, 2.84, 2.75, 2.52, 2.56, 2.45, 2.44, 2.46, 2.44, 2.15, 2.53, 2.49, 2.43, 2.42, 2.47, 1.99, 2.04, 2.06,
    3.48, 3.03, 2.98, 2.88, 2.92, 2.95, 0.00, 2.90, 2.87, 2.83, 2.79, 2.87, 2.81, 2.83, 2.79, 2.80, 2.74, 2.63,
    2.53, 2.57, 2.49, 2.48, 2.41, 2.29, 2.32, 2.45, 2.47, 2.60, 2.54, 0.00, 0.00, 0.00, 0.00, 0.00, 2.80, 2.93,
    2.88, 2.71, 2.82, 2.81, 2.83, 3.05, 3.40, 3.05, 2.70, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00,
    0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00,
], dtype=np.float32)
assert len(SYMBOLS) == len(VDW_RADIUS) == 119
_INDEX = {s: k for k, s in enumerate(SYMBOLS) if k > 0}


def radius_of(symbol: str) -> np.float32:
    """bcs::getRadius of the enumerator "A_" + upper-cased symbol; UNKNOWN when there is none."""
    return VDW_RADIUS[_INDEX.get(symbol.upper(), 0)]


# ---- MessagePack ---------------------------------------------------------------------------------
class _Reader:
    def __init__(self, data: bytes):
        self.d = data
        self.p = 0

    def take(self, n: int) -> bytes:
        if self.p + n > len(self.d):
            raise ValueError("truncated MessagePack data")
        b = self.d[self.p:self.p + n]
        self.p += n
        return b

    def unpack(self, fmt: str):
        return struct.unpack(fmt, self.take(struct.calcsize(fmt)))[0]

    def value(self):
        t = self.take(1)[0]
        if t <= 0x7F:
            return t
        if t >= 0xE0:
            return t - 0x100
        if 0x80 <= t <= 0x8F:
            return self.map(t & 0x0F)
        if 0x90 <= t <= 0x9F:
            return [self.value() for _ in range(t & 0x0F)]
        if 0xA0 <= t <= 0xBF:
            return self.take(t & 0x1F).decode("utf-8")
        fixed = {0xCA: ">f", 0xCB: ">d", 0xCC: ">B", 0xCD: ">H", 0xCE: ">I", 0xCF: ">Q",
                 0xD0: ">b", 0xD1: ">h", 0xD2: ">i", 0xD3: ">q"}
        if t in fixed:
            return self.unpack(fixed[t])
        if t == 0xC0:
            return None
        if t in (0xC2, 0xC3):
            return t == 0xC3
        if t in (0xC4, 0xC5, 0xC6):
            return self.take(self.unpack({0xC4: ">B", 0xC5: ">H", 0xC6: ">I"}[t]))
        if t in (0xD9, 0xDA, 0xDB):
            return self.take(self.unpack({0xD9: ">B", 0xDA: ">H", 0xDB: ">I"}[t])).decode("utf-8")
        if t in (0xDC, 0xDD):
            return [self.value() for _ in range(self.unpack(">H" if t == 0xDC else ">I"))]
        if t in (0xDE, 0xDF):
            return self.map(self.unpack(">H" if t == 0xDE else ">I"))
        raise ValueError(f"MessagePack type 0x{t:02x} is not used by MMTF")

    def map(self, n: int) -> dict:
        out = {}
        for _ in range(n):
            k = self.value()
            out[k] = self.value()
        return out


def unpack_msgpack(data: bytes):
    """The first MessagePack object of data (maps, arrays, strings, binaries, numbers, nil, booleans)."""
    return _Reader(data).value()


# ---- MMTF binary codecs (MMTF 1.0: a 12-byte big-endian header codec, length, parameter) -----------
def _run_length(pairs: np.ndarray) -> np.ndarray:
    return np.repeat(pairs[0::2], pairs[1::2])


def _recursive_index(v: np.ndarray, lo: int, hi: int) -> np.ndarray:
    """Values split into runs of the extreme values lo/hi are summed back into one."""
    out = []
    acc = 0
    for x in v.tolist():
        acc += x
        if x != lo and x != hi:
            out.append(acc)
            acc = 0
    return np.array(out, dtype=np.int64)


def decode_codec(buf: bytes) -> np.ndarray:
    codec, length, param = struct.unpack(">iii", buf[:12])
    d = buf[12:]
    if codec == 1:
        out = np.frombuffer(d, ">f4").astype(np.float32)
    elif codec in (2, 3, 4):
        out = np.frombuffer(d, {2: ">i1", 3: ">i2", 4: ">i4"}[codec]).astype(np.int64)
    elif codec == 5:
        out = np.array([d[k * param:(k + 1) * param].split(b"\0")[0].decode() for k in range(length)], dtype=object)
    elif codec == 6:
        out = np.array([chr(c) if c else "" for c in _run_length(np.frombuffer(d, ">i4").astype(np.int64))], dtype=object)
    elif codec == 7:
        out = _run_length(np.frombuffer(d, ">i4").astype(np.int64))
    elif codec == 8:
        out = np.cumsum(_run_length(np.frombuffer(d, ">i4").astype(np.int64)))
    elif codec == 9:
        out = _run_length(np.frombuffer(d, ">i4").astype(np.int64)).astype(np.float32) / np.float32(param)
    elif codec == 10:
        ints = np.cumsum(_recursive_index(np.frombuffer(d, ">i2").astype(np.int64), -32768, 32767))
        out = ints.astype(np.float32) / np.float32(param)
    elif codec == 11:
        out = np.frombuffer(d, ">i2").astype(np.float32) / np.float32(param)
    elif codec == 12:
        out = _recursive_index(np.frombuffer(d, ">i2").astype(np.int64), -32768, 32767).astype(np.float32) / np.float32(param)
    elif codec == 13:
        out = _recursive_index(np.frombuffer(d, ">i1").astype(np.int64), -128, 127)
    elif codec == 14:
        out = _recursive_index(np.frombuffer(d, ">i2").astype(np.int64), -32768, 32767)
    else:
        raise ValueError(f"MMTF codec {codec} is not supported")
    if len(out) != length:
        raise ValueError(f"MMTF codec {codec}: {len(out)} values decoded, header says {length}")
    return out


def _field(doc: dict, key: str):
    v = doc[key]
    return decode_codec(v) if isinstance(v, (bytes, bytearray)) else np.asarray(v)


def load_bytes(data: bytes) -> np.ndarray:
    """(N, 4) float32 atoms of the first model of an MMTF document (gzip-compressed or not)."""
    if data[:2] == b"\x1f\x8b":
        data = gzip.decompress(data)
    doc = unpack_msgpack(data)
    if not isinstance(doc, dict) or "xCoordList" not in doc:
        raise ValueError("not an MMTF document")
    x, y, z = (_field(doc, k) for k in ("xCoordList", "yCoordList", "zCoordList"))
    group_types = _field(doc, "groupTypeList")
    groups = doc["groupList"]
    chains_per_model = np.asarray(doc["chainsPerModel"], dtype=np.int64)
    groups_per_chain = np.asarray(doc["groupsPerChain"], dtype=np.int64)
    n_groups = int(groups_per_chain[:int(chains_per_model[0])].sum()) if len(chains_per_model) else 0
    radii = []
    for g in group_types[:n_groups].tolist():
        radii.extend(radius_of(e) for e in groups[g]["elementList"])
    n = len(radii)
    if n > len(x):
        raise ValueError("MMTF groups hold more atoms than the coordinate lists")
    atoms = np.empty((n, 4), dtype=np.float32)
    atoms[:, 0], atoms[:, 1], atoms[:, 2] = x[:n], y[:n], z[:n]
    atoms[:, 3] = np.array(radii, dtype=np.float32)
    return atoms


def load(path: str) -> np.ndarray:
    """(N, 4) float32 atoms (x, y, z, vdW radius) of the first model of an MMTF file."""
    with open(path, "rb") as f:
        return load_bytes(f.read())
