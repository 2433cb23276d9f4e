"""TEST INFRASTRUCTURE ONLY: Python access to the FP64 CPU oracle (sesdf_oracle.c).

The oracle restates the reference's SES build (PlathC/SESDF, bcs::Sesdf::build at
sesdf/src/sesdf/sesdf.cu:172-264 and bcs::Ssesdf::build at
sesdf/src/ssesdf/ssesdf.cu:133-187) in double precision. Only the tests, the
smoke check and the benchmark's CPU-baseline leg use it; the product path in
sesdf_gb300/ never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sesdf_oracle.c")
SRCS = [SRC, os.path.join(HERE, "area_oracle.c")]
LIB = os.path.join(HERE, "_lib", "liboracle.so")

COUNTERS = [
    "band_neighbor", "band_buried", "band_complete", "band_probe_t", "band_occlusion",
    "band_singular", "band_singular_nbr", "band_angle_tie", "band_ortho", "ill_conditioned",
    "torus_degenerate", "nbr_truncated", "seg_truncated", "snbr_truncated", "grid_outside",
]

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with IEEE double arithmetic (no contraction) and OpenMP."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(s) for s in SRCS):
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
               "-o", LIB + ".tmp"] + SRCS + ["-lm"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def _load():
    global _lib
    with _lock:
        if _lib is None:
            build()
            lib = ctypes.CDLL(LIB)
            lib.ora_build.restype = ctypes.c_void_p
            lib.ora_build.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_float,
                                      ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int]
            lib.ora_array.restype = ctypes.c_int
            lib.ora_array.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p),
                                      ctypes.POINTER(ctypes.c_uint64)]
            lib.ora_free.argtypes = [ctypes.c_void_p]
            lib.ora_aabb.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
            lib.ora_grid.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
            _lib = lib
    return _lib


_DTYPES = {
    "perm": np.uint32, "hash": np.uint32, "atoms": np.float32, "noff": np.uint32, "nbr": np.uint32,
    "status": np.uint8, "status0": np.uint8, "convex": np.uint32, "sectors": np.float64,
    "full": np.uint32, "slot_trim": np.uint32, "trim_slot": np.uint32, "ids": np.int32, "cids": np.int32,
    "posf": np.float32, "posd": np.float64, "ccount": np.uint32, "cstart": np.uint32, "clist": np.uint32,
    "segments": np.uint32, "snbr": np.float32, "snbr_idx": np.uint32, "tori": np.float64, "counters": np.uint64,
}
_SHAPES = {"atoms": 4, "convex": 2, "sectors": 4, "full": 2, "ids": 4, "cids": 4, "posf": 4, "posd": 4,
           "segments": 4, "snbr": 4, "tori": 12}


def aabb(atoms: np.ndarray) -> np.ndarray:
    """getAabb (sesdf/src/core/molecule.cpp:132-143): float32 min/max of xyz -/+ r."""
    a = np.ascontiguousarray(atoms, dtype=np.float32)
    out = np.zeros(6, np.float32)
    _load().ora_aabb(a.ctypes.data, a.shape[0], out.ctypes.data)
    return out


def run(atoms: np.ndarray, probe_radius: float = 1.4, mode: str = "full", box=None, max_nbr: int = 128,
        seg_cap: int = 32, threads: int = 0) -> dict:
    """Runs the oracle and returns its outputs as numpy arrays (copies)."""
    lib = _load()
    a = np.ascontiguousarray(atoms, dtype=np.float32).reshape(-1, 4)
    bx = aabb(a) if box is None else np.ascontiguousarray(box, dtype=np.float32)
    h = lib.ora_build(a.ctypes.data, a.shape[0], bx.ctypes.data, ctypes.c_float(probe_radius),
                      0 if mode == "full" else 1, max_nbr, seg_cap, threads)
    out = {"n": a.shape[0], "mode": mode, "probe_radius": np.float32(probe_radius), "aabb": bx}
    try:
        for name, dt in _DTYPES.items():
            ptr = ctypes.c_void_p()
            cnt = ctypes.c_uint64()
            if lib.ora_array(h, name.encode(), ctypes.byref(ptr), ctypes.byref(cnt)) != 0:
                continue
            n = cnt.value
            if n == 0 or not ptr.value:
                arr = np.zeros(0, dt)
            else:
                buf = (ctypes.c_char * (n * np.dtype(dt).itemsize)).from_address(ptr.value)
                arr = np.frombuffer(buf, dtype=dt).copy()
            if name in _SHAPES:
                arr = arr.reshape(-1, _SHAPES[name])
            out[name] = arr
        origin = np.zeros(3, np.float32)
        cell = np.zeros(3, np.float32)
        gs = np.zeros(1, np.uint32)
        lib.ora_grid(h, origin.ctypes.data, cell.ctypes.data, gs.ctypes.data)
        out["grid_origin"], out["grid_cell"], out["grid_size"] = origin, cell, int(gs[0])
    finally:
        lib.ora_free(h)
    out["counters"] = dict(zip(COUNTERS, [int(c) for c in out["counters"]]))
    out["Q"] = int(np.sum(np.abs(out["cids"][:, 3]) == 2)) if out["cids"].size else 0
    return out


def sdf(built: dict, queries: np.ndarray, band: float = 3.0, gq: np.ndarray | None = None, threads: int = 0):
    """FP64 signed distance to the SES at float32 query points [m, 3] from the outputs of run()
    (full mode). Returns (sdf float64 [m], kind int32 [m], grad float64 [n, 4] in sorted atom order or
    None): grad = sum_q gq[q] d sdf_q / d (x, y, z, r) when gq is given. Test oracle only."""
    lib = _load()
    if not getattr(lib, "_sdf_ready", False):
        P = ctypes.c_void_p
        lib.ora_sdf.argtypes = [P, ctypes.c_uint32, P, P, P, P, P, ctypes.c_uint32, ctypes.c_float, ctypes.c_float, P,
                                ctypes.c_uint32, P, P, P, P, ctypes.c_int]
        lib.ora_sdf.restype = ctypes.c_int
        lib._sdf_ready = True
    atoms = np.ascontiguousarray(built["atoms"], np.float32)
    n = atoms.shape[0]
    q = np.ascontiguousarray(queries, np.float32).reshape(-1, 3)
    m = q.shape[0]
    noff = np.ascontiguousarray(built["noff"], np.uint32)
    nbr = np.ascontiguousarray(built["nbr"], np.uint32)
    status = np.ascontiguousarray(built["status"], np.uint8)
    ids = np.ascontiguousarray(built["ids"], np.int32).reshape(-1, 4)
    posd = np.ascontiguousarray(built["posd"], np.float64).reshape(-1, 4)
    out = np.zeros(m, np.float64)
    kind = np.zeros(m, np.int32)
    g = np.zeros((n, 4), np.float64) if gq is not None else None
    gqa = np.ascontiguousarray(gq, np.float64) if gq is not None else None

    def ptr(a):
        return a.ctypes.data if a is not None and a.size else None
    st = lib.ora_sdf(ptr(atoms), n, ptr(noff), ptr(nbr), ptr(status), ptr(ids), ptr(posd), ids.shape[0],
                     ctypes.c_float(float(built["probe_radius"])), ctypes.c_float(band), ptr(q), m, ptr(gqa),
                     out.ctypes.data, kind.ctypes.data, ptr(g), threads)
    if st != 0:
        raise RuntimeError("ora_sdf failed")
    return out, kind, g


def area(built: dict, g_area=None, threads: int = 0):
    """FP64 SES area of the primitives of a full-surface run(): returns (parts float64 [3] = convex,
    toroidal, concave; per-atom area float64 [n] (sorted order); grad float64 [n, 4] (sorted order) =
    d (g . parts) / d (x, y, z, r) with g = g_area (a scalar weighs the three alike), or None).
    Test oracle only."""
    lib = _load()
    if not getattr(lib, "_area_ready", False):
        P = ctypes.c_void_p
        lib.ora_area.argtypes = [P, ctypes.c_uint32, P, P, P, P, P, ctypes.c_uint32, ctypes.c_uint32, P, ctypes.c_float,
                                 P, P, P, P, ctypes.c_int]
        lib.ora_area.restype = ctypes.c_int
        lib.ora_region_area.argtypes = [P, ctypes.c_int, P]
        lib.ora_region_area.restype = ctypes.c_double
        lib._area_ready = True
    atoms = np.ascontiguousarray(built["atoms"], np.float32)
    n = atoms.shape[0]
    noff = np.ascontiguousarray(built["noff"], np.uint32)
    nbr = np.ascontiguousarray(built["nbr"], np.uint32)
    ids = np.ascontiguousarray(built["ids"], np.int32).reshape(-1, 4)
    posd = np.ascontiguousarray(built["posd"], np.float64).reshape(-1, 4)
    sidx = np.ascontiguousarray(built["snbr_idx"], np.uint32)
    parts = np.zeros(3, np.float64)
    per_atom = np.zeros(n, np.float64)
    g = np.zeros((n, 4), np.float64) if g_area is not None else None
    gw = np.broadcast_to(np.asarray(g_area if g_area is not None else 0.0, np.float64), (3,)).copy()

    def ptr(a):
        return a.ctypes.data if a is not None and a.size else None
    status = np.ascontiguousarray(built["status"], np.uint8)
    ov = lib.ora_area(ptr(atoms), n, ptr(noff), ptr(nbr), ptr(status), ptr(ids), ptr(posd), ids.shape[0], int(built["Q"]),
                      ptr(sidx), ctypes.c_float(float(built["probe_radius"])),
                      gw.ctypes.data, parts.ctypes.data,
                      per_atom.ctypes.data, ptr(g), threads)
    if ov:
        raise RuntimeError(f"ora_area: {ov} region(s) exceeded the arc capacity")
    return parts, per_atom, g


def region_area(cons: np.ndarray):
    """Area of {y on the unit sphere : y . w_m <= c_m} for cons [M, 4] = (w, c); returns
    (area, sums [M, 4] = (boundary angle, integral of y over it)). Test oracle only."""
    lib = _load()
    if not getattr(lib, "_area_ready", False):
        P = ctypes.c_void_p
        lib.ora_region_area.argtypes = [P, ctypes.c_int, P]
        lib.ora_region_area.restype = ctypes.c_double
    c = np.ascontiguousarray(cons, np.float64).reshape(-1, 4)
    s = np.zeros_like(c)
    a = lib.ora_region_area(c.ctypes.data if c.size else None, c.shape[0], s.ctypes.data if s.size else None)
    return a, s
