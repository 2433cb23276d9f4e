"""Seeded synthetic molecules with protein-like density and element mix.

These stand in for the PDB entries the reference benchmarks (app/benchmarks/main.cu:97-113);
the generator itself is native (csrc/synth.c) and deterministic across x86-64 and aarch64.

Workloads:
  globule(2000, 1000)                    2,000-atom compact globule
  assembly()                             100,000 atoms: 20 globules of 5,000 (seeds 1100+g)
  shell()                                1,000,000 atoms: 200 globules (seeds 1200+g) on a 400 A Fibonacci sphere
  batch_sizes()                          256 sizes log-uniform in [500, 50,000] (seed 1300)
  frames()                               64 jittered frames of a 20,000-atom globule (seeds 1400+f)
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _build

_lib = None
_path = None


def use_library(path: str) -> None:
    """Takes the generator from another library that exports the same sesgb_synth_*
    functions (the reference harness links synth.c in, so that a process timing the
    reference loads nothing of this package's native code)."""
    global _lib, _path
    _lib, _path = None, path


def _load():
    global _lib
    if _lib is None:
        path = _path or _build.build_synth()
        lib = ctypes.CDLL(path)
        lib.sesgb_synth_globule.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_void_p]
        lib.sesgb_synth_globule.restype = ctypes.c_int
        lib.sesgb_synth_queries.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                            ctypes.c_float, ctypes.c_void_p]
        lib.sesgb_synth_queries.restype = ctypes.c_uint32
        lib.sesgb_synth_assembly.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64,
                                             ctypes.c_void_p]
        lib.sesgb_synth_shell.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double,
                                          ctypes.c_void_p]
        lib.sesgb_synth_jitter.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_double, ctypes.c_uint64]
        lib.sesgb_synth_jitter.restype = None
        lib.sesgb_synth_uniform.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p]
        lib.sesgb_synth_uniform.restype = None
        _lib = lib
    return _lib


def globule(n: int, seed: int) -> np.ndarray:
    a = np.zeros((n, 4), np.float32)
    if n and _load().sesgb_synth_globule(n, seed, a.ctypes.data) < 0:
        raise RuntimeError("globule generation failed")
    return a


def assembly(globules: int = 20, per: int = 5000, seed0: int = 1100, placement_seed: int = 1100) -> np.ndarray:
    a = np.zeros((globules * per, 4), np.float32)
    if _load().sesgb_synth_assembly(globules, per, seed0, placement_seed, a.ctypes.data) != 0:
        raise RuntimeError("assembly generation failed")
    return a


def shell(globules: int = 200, per: int = 5000, seed0: int = 1200, radius: float = 400.0) -> np.ndarray:
    a = np.zeros((globules * per, 4), np.float32)
    if _load().sesgb_synth_shell(globules, per, seed0, radius, a.ctypes.data) != 0:
        raise RuntimeError("shell generation failed")
    return a


def uniform(seed: int, count: int) -> np.ndarray:
    out = np.zeros(count, np.float64)
    _load().sesgb_synth_uniform(seed, count, out.ctypes.data)
    return out


def batch_sizes(count: int = 256, lo: int = 500, hi: int = 50000, seed: int = 1300) -> np.ndarray:
    u = uniform(seed, count)
    return np.array([int(round(math.exp(math.log(lo) + x * (math.log(hi) - math.log(lo))))) for x in u], np.int64)


def jitter(atoms: np.ndarray, sigma: float, seed: int) -> np.ndarray:
    a = np.ascontiguousarray(atoms, np.float32).copy()
    _load().sesgb_synth_jitter(a.ctypes.data, a.shape[0], sigma, seed)
    return a


def frames(count: int = 64, n: int = 20000, seed: int = 1400, sigma: float = 0.3):
    base = globule(n, seed)
    return [jitter(base, sigma, seed + f) for f in range(count)]


def queries(atoms: np.ndarray, m: int, seed: int, band: float = 3.0) -> np.ndarray:
    """m query points uniform in the atoms' bounding box, kept within `band` of the vdW surface (float32 [m, 3])."""
    lib = _load()
    a = np.ascontiguousarray(atoms, np.float32).reshape(-1, 4)
    out = np.zeros((m, 3), np.float32)
    got = lib.sesgb_synth_queries(a.ctypes.data, a.shape[0], m, seed, ctypes.c_float(band), out.ctypes.data)
    return out[:got]


def sdf_workload():
    """20,000-atom globule (seed 1500) and 1,000,000 query points within 3 A of its vdW surface (seed 1501)."""
    atoms = globule(20000, 1500)
    return atoms, queries(atoms, 1_000_000, 1501)


WORKLOADS = {
    "globule2k": lambda: globule(2000, 1000),
    "assembly100k": assembly,
    "shell1m": shell,
}
