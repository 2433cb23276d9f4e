"""TEST INFRASTRUCTURE ONLY: the reference's own CUDA kernels, run through the
restated host driver (oracle/ref/ref_driver.cu). Used to pin the oracle (golden
fixtures) and as the benchmark's reference arm; never part of the product path.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
CUBIN = os.path.join(OUT, "ref_kernels.cubin")
LIB = os.path.join(OUT, "libsesref.so")


def reference_checkout() -> str | None:
    """The reference checkout the cubin is compiled from: $SESDF_REFERENCE, else a
    checkout named `reference` beside this repository; None when neither exists
    (the prebuilt cubin is used then)."""
    for c in (os.environ.get("SESDF_REFERENCE"), os.path.join(os.path.dirname(HERE), "..", "reference")):
        if c and os.path.isdir(os.path.join(c, "sesdf")):
            return os.path.abspath(c)
    return None

_lib = None


def build_cubin(force: bool = False) -> bool:
    """Compiles the reference kernels when the reference checkout is present."""
    ref = reference_checkout()
    if ref is None:
        return os.path.exists(CUBIN)
    if force and os.path.exists(CUBIN):
        os.remove(CUBIN)
    subprocess.run(["make", "-s", "-C", HERE, "ref-cubin", f"REF={ref}"], check=True)
    return True


def build_driver(force: bool = False) -> str:
    if force and os.path.exists(LIB):
        os.remove(LIB)
    subprocess.run(["make", "-s", "-C", HERE, "ref-driver"], check=True)
    return LIB


def available() -> bool:
    return os.path.exists(CUBIN)


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build_driver()
        lib = ctypes.CDLL(LIB)
        lib.sesref_init.argtypes = [ctypes.c_char_p]
        lib.sesref_error.restype = ctypes.c_char_p
        lib.sesref_create.restype = ctypes.c_void_p
        lib.sesref_create.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_float, ctypes.c_int]
        lib.sesref_create_cap.restype = ctypes.c_void_p
        lib.sesref_create_cap.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_float, ctypes.c_int,
                                          ctypes.c_uint32]
        lib.sesref_build.argtypes = [ctypes.c_void_p]
        lib.sesref_time.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        lib.sesref_counts.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        lib.sesref_counts.restype = None
        lib.sesref_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint64]
        lib.sesref_destroy.argtypes = [ctypes.c_void_p]
        lib.sesref_destroy.restype = None
        st = lib.sesref_init(CUBIN.encode())
        if st != 0:
            raise RuntimeError("reference kernels: " + lib.sesref_error().decode())
        _lib = lib
    return _lib


COUNT_NAMES = ["n", "F", "V", "C1", "I", "Q", "S", "T", "visible"]
MAX_NBR = 128


class RefBuild:
    """One reference object (bcs::Sesdf or bcs::Ssesdf) on the reference kernels."""

    def __init__(self, atoms: np.ndarray, probe_radius: float = 1.4, mode: str = "full", box=None,
                 max_nbr: int = MAX_NBR):
        """max_nbr: neighbour slots per atom, 128 (the reference's sesdf library) or 288 (its sesdf288
        library, sesdf/CMakeLists.txt:96-117)."""
        if max_nbr not in (128, 288):
            raise ValueError("max_nbr: 128 or 288")
        self.lib = _load()
        self.max_nbr = max_nbr
        self.atoms = np.ascontiguousarray(np.asarray(atoms, np.float32).reshape(-1, 4))
        self.mode = mode
        if box is None:
            lo = (self.atoms[:, :3] - self.atoms[:, 3:4]).min(0)
            hi = (self.atoms[:, :3] + self.atoms[:, 3:4]).max(0)
            box = np.concatenate([lo, hi])
        self.box = np.ascontiguousarray(box, np.float32)
        self.h = self.lib.sesref_create_cap(self.atoms.ctypes.data, self.atoms.shape[0], self.box.ctypes.data,
                                            ctypes.c_float(probe_radius), 0 if mode == "full" else 1, max_nbr)
        if not self.h:
            raise RuntimeError("reference object: " + self.lib.sesref_error().decode())

    def build(self):
        if self.lib.sesref_build(self.h) != 0:
            raise RuntimeError("reference build: " + self.lib.sesref_error().decode())

    def time(self, iterations: int) -> np.ndarray:
        ms = np.zeros(iterations, np.float32)
        if self.lib.sesref_time(self.h, iterations, ms.ctypes.data) != 0:
            raise RuntimeError("reference build: " + self.lib.sesref_error().decode())
        return ms

    def counts(self) -> dict:
        c = np.zeros(9, np.uint64)
        self.lib.sesref_counts(self.h, c.ctypes.data)
        return dict(zip(COUNT_NAMES, [int(x) for x in c]))

    def _get(self, name: str, count: int, dtype, width: int = 1) -> np.ndarray:
        out = np.empty((count, width) if width > 1 else count, dtype=dtype)
        st = self.lib.sesref_get(self.h, name.encode(), out.ctypes.data if out.size else None, out.nbytes)
        if st != 0:
            raise RuntimeError(f"reference output {name}: " + self.lib.sesref_error().decode())
        return out

    def fetch(self) -> dict:
        c = self.counts()
        n = c["n"]
        out = {"counts": c, "atoms": self._get("atoms", n, np.float32, 4),
               "perm": self._get("atom_indices", n, np.uint32),
               "nbr_count": self._get("nbr_count", n, np.uint32),
               "nbr_ids": self._get("nbr_ids", n * self.max_nbr, np.uint32).reshape(n, self.max_nbr),
               "status": self._get("status", n * self.max_nbr, np.uint8).reshape(n, self.max_nbr),
               "probe_ids": self._get("int_ids", c["I"], np.int32, 4),
               "probe_pos": self._get("int_pos", c["I"], np.float32, 4),
               "probe_nbrs": self._get("int_nbrs", 32 * c["Q"], np.float32, 4)}
        if self.mode == "full":
            out["global_to_trimmed"] = self._get("global_to_trimmed", n * self.max_nbr + 1, np.uint32)
            out["convex"] = self._get("convex", n, np.uint32, 2)
            out["full"] = self._get("full_circles", c["F"], np.uint32, 2)
            out["sectors"] = self._get("sectors", c["V"], np.float32, 4)
            out["segments"] = self._get("segments", c["S"], np.uint32, 4)
        else:
            t = self._get("tori", 3 * c["T"], np.float32, 4)
            T = c["T"]
            out["tori_pos"], out["tori_axis"], out["tori_vs"] = t[:T], t[T:2 * T], t[2 * T:]
        return out

    def close(self):
        if self.h:
            self.lib.sesref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
