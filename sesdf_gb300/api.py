"""Python mirror of the drop-in API, over the C ABI of include/sesgb.h (ctypes).

`SesBuild` follows bcs::Sesdf / bcs::Ssesdf (sesdf/include/bcs/sesdf/sesdf.hpp:15-88,
sesdf/include/bcs/ssesdf/ssesdf.hpp:14-77): construction from atoms (x, y, z, vdW
radius) and a probe radius, build(), and the output buffers. Outputs stay in
device memory; fetch() copies them to numpy. There is no CPU fallback: without the
CUDA library or a GPU every call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import _build

MODE_FULL = 0
MODE_EXTERIOR = 1
FLAG_GRAPH = 1
FLAG_PROFILE = 2
FLAG_MIN_CAPACITY = 4
FLAG_CUTOFF_CELLS = 8
TUNING_FIELDS = ["neighbor_cell_span", "neighbor_warps", "visibility_warps", "probe_warps", "probe_queue"]

BUF_ATOM_INDICES, BUF_NEIGHBOR_COUNT, BUF_NEIGHBOR_IDS, BUF_VISIBILITY_STATUS, BUF_GLOBAL_TO_TRIMMED = range(5)

# every entry point include/sesgb.h declares
EXPORTS = [
    "sesgb_create", "sesgb_build", "sesgb_build_device", "sesgb_set_host_atoms", "sesgb_get_full",
    "sesgb_get_exterior", "sesgb_get_counts", "sesgb_atom_indices", "sesgb_analysis_buffer", "sesgb_copy_to_host",
    "sesgb_max_neighbor_per_atom", "sesgb_max_intersections_per_circle", "sesgb_max_intersection_neighbors",
    "sesgb_error_string", "sesgb_last_error", "sesgb_destroy", "sesgb_stage_times", "sesgb_stage_name",
    "sesgb_launch_count", "sesgb_build_async", "sesgb_finish", "sesgb_sort_atoms_noalloc",
    "sesgb_create_batch", "sesgb_batch_molecules", "sesgb_molecule_record", "sesgb_get_full_molecule",
    "sesgb_get_exterior_molecule", "sesgb_sdf", "sesgb_sdf_backward", "sesgb_ses_area", "sesgb_ses_area_backward",
    "sesgb_load_mmtf", "sesgb_render", "sesgb_cavities", "sesgb_cavity_labels", "sesgb_cavity_components",
    "sesgb_set_tuning", "sesgb_get_tuning",
]
SDF_BAND = 3.0
MOL_FIELDS = ["atoms", "sectors", "full_circles", "partial_circles", "probes", "singular_probes", "segments", "tori",
              "atom_base", "sector_base", "full_base", "partial_base", "probe_base", "singular_base", "segment_base",
              "tori_base"]
NOALLOC_MAX_ATOMS = 262144


class SesgbError(RuntimeError):
    pass


class Options(ctypes.Structure):
    _fields_ = [("max_neighbor_per_atom", ctypes.c_uint32), ("max_intersections_per_circle", ctypes.c_uint32),
                ("device", ctypes.c_int32), ("flags", ctypes.c_uint32)]


class Camera(ctypes.Structure):
    _fields_ = [("eye", ctypes.c_double * 3), ("forward", ctypes.c_double * 3), ("right", ctypes.c_double * 3),
                ("up", ctypes.c_double * 3), ("tan_half_fov", ctypes.c_double), ("t_near", ctypes.c_double),
                ("t_far", ctypes.c_double), ("eps", ctypes.c_double), ("normal_step", ctypes.c_double),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("max_steps", ctypes.c_uint32)]


class Tuning(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint32) for f in TUNING_FIELDS]


class CavityInfo(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_double * 3), ("voxel", ctypes.c_double), ("dims", ctypes.c_uint32 * 3),
                ("components", ctypes.c_uint32), ("exterior", ctypes.c_uint32), ("cavities", ctypes.c_uint32),
                ("probes", ctypes.c_uint32)]


class FullData(ctypes.Structure):
    _fields_ = [("atomNb", ctypes.c_uint32), ("atoms", ctypes.c_void_p),
                ("convexPatchNb", ctypes.c_uint32), ("convexPatches", ctypes.c_void_p),
                ("sectorNb", ctypes.c_uint32), ("sectors", ctypes.c_void_p),
                ("segmentPatchNb", ctypes.c_uint32), ("segmentPatches", ctypes.c_void_p),
                ("circlePatchNb", ctypes.c_uint32), ("circlePatches", ctypes.c_void_p),
                ("concavePatchNb", ctypes.c_uint32), ("concavePatchesPosition", ctypes.c_void_p),
                ("concavePatchesId", ctypes.c_void_p), ("concavePatchesNeighbors", ctypes.c_void_p),
                ("probeRadius", ctypes.c_float), ("maxConcaveNeighbors", ctypes.c_uint16)]


class ExteriorData(ctypes.Structure):
    _fields_ = [("atomNb", ctypes.c_uint32), ("atoms", ctypes.c_void_p),
                ("circlePatchNb", ctypes.c_uint32), ("circlePosition", ctypes.c_void_p),
                ("circleAxis", ctypes.c_void_p), ("circleVs", ctypes.c_void_p),
                ("concavePatchNb", ctypes.c_uint32), ("concavePatchesPosition", ctypes.c_void_p),
                ("concavePatchesId", ctypes.c_void_p), ("concavePatchesNeighbors", ctypes.c_void_p),
                ("probeRadius", ctypes.c_float), ("maxConcaveNeighbors", ctypes.c_uint16)]


COUNT_FIELDS = ["atoms", "pairs", "sectors", "full_circles", "partial_circles", "candidates", "probes",
                "singular_probes", "segments", "tori", "max_neighbors", "truncated_atoms", "truncated_circles",
                "truncated_probe_neighbors", "degenerate_tori", "outside_atoms"]


class Counts(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint32) for f in COUNT_FIELDS] + [("fp64_decisions", ctypes.c_uint32 * 7),
                                                               ("rebuilds", ctypes.c_uint32)]


_lib = None
_lock = threading.Lock()


def load_library(path: str | None = None) -> ctypes.CDLL:
    """Loads libsesgb.so (built in-tree); raises if it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = path or _build.LIB
        if not os.path.exists(path):
            raise SesgbError(f"CUDA library not built: {path} (run __graft_entry__.build())")
        lib = ctypes.CDLL(path)
        P, U32, I32, F32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_float
        lib.sesgb_create.argtypes = [P, U32, P, F32, I32, ctypes.POINTER(Options), ctypes.POINTER(P)]
        lib.sesgb_build.argtypes = [P, P]
        lib.sesgb_build_device.argtypes = [P, P, P]
        lib.sesgb_set_host_atoms.argtypes = [P, P]
        lib.sesgb_get_full.argtypes = [P, ctypes.POINTER(FullData)]
        lib.sesgb_get_exterior.argtypes = [P, ctypes.POINTER(ExteriorData)]
        lib.sesgb_get_counts.argtypes = [P, ctypes.POINTER(Counts)]
        lib.sesgb_atom_indices.argtypes = [P, P]
        lib.sesgb_analysis_buffer.argtypes = [P, I32, ctypes.POINTER(P), ctypes.POINTER(ctypes.c_uint64)]
        lib.sesgb_copy_to_host.argtypes = [P, P, P, ctypes.c_uint64]
        for f in ("sesgb_max_neighbor_per_atom", "sesgb_max_intersections_per_circle", "sesgb_max_intersection_neighbors"):
            getattr(lib, f).argtypes = [P]
            getattr(lib, f).restype = ctypes.c_uint16
        lib.sesgb_load_mmtf.argtypes = [P, ctypes.c_size_t, P, U32, ctypes.POINTER(U32)]
        lib.sesgb_error_string.argtypes = [I32]
        lib.sesgb_error_string.restype = ctypes.c_char_p
        lib.sesgb_last_error.argtypes = [P]
        lib.sesgb_last_error.restype = ctypes.c_char_p
        lib.sesgb_destroy.argtypes = [P]
        lib.sesgb_destroy.restype = None
        lib.sesgb_stage_times.argtypes = [P, P, U32, ctypes.POINTER(U32)]
        lib.sesgb_stage_name.argtypes = [U32]
        lib.sesgb_stage_name.restype = ctypes.c_char_p
        lib.sesgb_sort_atoms_noalloc.argtypes = [P, U32, P, F32, P, P, P]
        lib.sesgb_build_async.argtypes = [P, P, P]
        lib.sesgb_finish.argtypes = [P]
        lib.sesgb_launch_count.argtypes = []
        lib.sesgb_launch_count.restype = ctypes.c_uint64
        lib.sesgb_create_batch.argtypes = [P, P, U32, F32, I32, ctypes.POINTER(Options), ctypes.POINTER(P)]
        lib.sesgb_batch_molecules.argtypes = [P]
        lib.sesgb_batch_molecules.restype = U32
        lib.sesgb_molecule_record.argtypes = [P, U32, P]
        lib.sesgb_get_full_molecule.argtypes = [P, U32, ctypes.POINTER(FullData)]
        lib.sesgb_get_exterior_molecule.argtypes = [P, U32, ctypes.POINTER(ExteriorData)]
        lib.sesgb_sdf.argtypes = [P, P, U32, P, P, P]
        lib.sesgb_sdf_backward.argtypes = [P, P, U32, P, P, P]
        lib.sesgb_ses_area.argtypes = [P, P, P, P]
        lib.sesgb_ses_area_backward.argtypes = [P, P, P, P]
        lib.sesgb_render.argtypes = [P, ctypes.POINTER(Camera), P, P, P]
        lib.sesgb_cavities.argtypes = [P, ctypes.c_double, ctypes.POINTER(CavityInfo), P, P]
        lib.sesgb_cavity_labels.argtypes = [P, ctypes.POINTER(P), ctypes.POINTER(ctypes.c_uint64)]
        lib.sesgb_cavity_components.argtypes = [P, P, P, U32]
        lib.sesgb_set_tuning.argtypes = [P, ctypes.POINTER(Tuning)]
        lib.sesgb_get_tuning.argtypes = [P, ctypes.POINTER(Tuning)]
        _lib = lib
    return _lib


def launch_count() -> int:
    """Kernels launched by the library in this process."""
    return int(load_library().sesgb_launch_count())


def aabb(atoms: np.ndarray) -> np.ndarray:
    """getAabb (sesdf/src/core/molecule.cpp:132-143) in float32."""
    a = np.asarray(atoms, np.float32).reshape(-1, 4)
    if a.shape[0] == 0:
        return np.zeros(6, np.float32)
    lo = (a[:, :3] - a[:, 3:4]).min(0)
    hi = (a[:, :3] + a[:, 3:4]).max(0)
    return np.concatenate([lo, hi]).astype(np.float32)


def load_mmtf(data: bytes) -> np.ndarray:
    """(N, 4) float32 atoms of the first model of an MMTF document (bytes, gzip-compressed or not)
    through the library's native reader (sesgb_load_mmtf)."""
    import gzip

    if data[:2] == b"\x1f\x8b":
        data = gzip.decompress(data)
    lib = load_library()
    n = ctypes.c_uint32()
    buf = ctypes.create_string_buffer(bytes(data), len(data))
    st = lib.sesgb_load_mmtf(buf, len(data), None, 0, ctypes.byref(n))
    if st == -1:
        raise SesgbError("sesgb_load_mmtf: not a readable MMTF document")
    out = np.zeros((n.value, 4), np.float32)
    if n.value:
        st = lib.sesgb_load_mmtf(buf, len(data), out.ctypes.data, n.value, ctypes.byref(n))
        if st != 0:
            raise SesgbError(f"sesgb_load_mmtf: {lib.sesgb_error_string(st).decode()}")
    return out


class SesBuild:
    """One SES build context (bcs::Sesdf for mode "full", bcs::Ssesdf for "exterior").

    graph=True (default) captures the build's fixed launch sequence in a CUDA graph after
    the first build and replays it (SESGB_FLAG_GRAPH); profile=True records per-stage
    events, also inside the graph."""

    def __init__(self, atoms: np.ndarray, probe_radius: float = 1.4, mode: str = "full", box=None,
                 max_neighbor_per_atom: int = 0, max_intersections_per_circle: int = 0, graph: bool = True,
                 device: int = -1, profile: bool = False, min_capacity: bool = False):
        self._lib = load_library()
        self.atoms = np.ascontiguousarray(np.asarray(atoms, np.float32).reshape(-1, 4))
        self.mode = mode
        self.probe_radius = float(probe_radius)
        bx = None if box is None else np.ascontiguousarray(box, np.float32)
        self.box = aabb(self.atoms) if bx is None else bx
        flags = (FLAG_GRAPH if graph else 0) | (FLAG_PROFILE if profile else 0) | (FLAG_MIN_CAPACITY if min_capacity else 0)
        opt = Options(max_neighbor_per_atom, max_intersections_per_circle, device, flags)
        h = ctypes.c_void_p()
        st = self._lib.sesgb_create(self.atoms.ctypes.data if self.atoms.size else None, self.atoms.shape[0],
                                    self.box.ctypes.data, ctypes.c_float(probe_radius),
                                    MODE_FULL if mode == "full" else MODE_EXTERIOR, ctypes.byref(opt), ctypes.byref(h))
        self._h = h
        self._check(st, "create")

    def _check(self, st: int, what: str):
        if st != 0:
            msg = self._lib.sesgb_error_string(st).decode()
            detail = self._lib.sesgb_last_error(self._h).decode() if self._h else ""
            raise SesgbError(f"{what}: {msg} ({detail})")

    def set_atoms(self, atoms: np.ndarray):
        a = np.ascontiguousarray(np.asarray(atoms, np.float32).reshape(-1, 4))
        if a.shape != self.atoms.shape:
            raise ValueError("atom count is fixed at construction")
        self.atoms = a
        self._check(self._lib.sesgb_set_host_atoms(self._h, a.ctypes.data), "set_atoms")

    def build(self, stream: int | None = None):
        self._check(self._lib.sesgb_build(self._h, stream), "build")

    def build_device(self, device_ptr: int, stream: int | None = None):
        self._check(self._lib.sesgb_build_device(self._h, device_ptr, stream), "build_device")

    def build_async(self, device_ptr: int | None = None, stream: int | None = None):
        """Enqueues a build (device atoms, or the host atoms when None); finish() waits."""
        self._check(self._lib.sesgb_build_async(self._h, device_ptr, stream), "build_async")

    def finish(self):
        self._check(self._lib.sesgb_finish(self._h), "finish")

    def set_host_pointer(self, ptr: int):
        """Reads atoms from raw host memory (e.g. pinned) from now on; caller keeps it alive."""
        self._check(self._lib.sesgb_set_host_atoms(self._h, ptr), "set_host_pointer")

    def counts(self) -> dict:
        c = Counts()
        self._check(self._lib.sesgb_get_counts(self._h, ctypes.byref(c)), "counts")
        d = {f: int(getattr(c, f)) for f in COUNT_FIELDS}
        d["fp64_decisions"] = [int(x) for x in c.fp64_decisions]
        d["rebuilds"] = int(c.rebuilds)
        return d

    def data(self):
        if self.mode == "full":
            d = FullData()
            self._check(self._lib.sesgb_get_full(self._h, ctypes.byref(d)), "getData")
        else:
            d = ExteriorData()
            self._check(self._lib.sesgb_get_exterior(self._h, ctypes.byref(d)), "getData")
        return d

    def _copy(self, ptr, count: int, dtype, width: int = 1) -> np.ndarray:
        out = np.empty((count, width) if width > 1 else count, dtype=dtype)
        if count:
            self._check(self._lib.sesgb_copy_to_host(self._h, ptr, out.ctypes.data, out.nbytes), "copy")
        return out

    def analysis(self, which: int, dtype, width: int = 1) -> np.ndarray:
        p = ctypes.c_void_p()
        nb = ctypes.c_uint64()
        self._check(self._lib.sesgb_analysis_buffer(self._h, which, ctypes.byref(p), ctypes.byref(nb)), "analysis")
        n = nb.value // np.dtype(dtype).itemsize
        return self._copy(p, n, dtype)

    def stage_times(self) -> dict:
        """Milliseconds per stage of the last build (needs profile=True)."""
        ms = (ctypes.c_float * 16)()
        n = ctypes.c_uint32()
        self._check(self._lib.sesgb_stage_times(self._h, ms, 16, ctypes.byref(n)), "stage_times")
        return {self._lib.sesgb_stage_name(k).decode(): float(ms[k]) for k in range(n.value)}

    def sdf(self, queries_ptr: int, m: int, out_ptr: int, kind_ptr: int | None = None, stream: int | None = None):
        """Signed distance to the SES at m float3 query points (device pointers); enqueued on `stream`."""
        self._check(self._lib.sesgb_sdf(self._h, queries_ptr, m, out_ptr, kind_ptr, stream), "sdf")

    def sdf_backward(self, queries_ptr: int, m: int, grad_sdf_ptr: int, grad_atoms_ptr: int, stream: int | None = None):
        """grad_atoms (float4[n], input order) = sum_q grad_sdf[q] d sdf_q / d (x, y, z, r)."""
        self._check(self._lib.sesgb_sdf_backward(self._h, queries_ptr, m, grad_sdf_ptr, grad_atoms_ptr, stream),
                    "sdf_backward")

    def ses_area(self, atom_area_ptr: int | None = None, stream: int | None = None) -> dict:
        """SES area of the primitives of the last full-surface build: {"convex", "toroidal", "concave",
        "total"} in A^2. atom_area_ptr (device float[n], input order): per-atom areas. Synchronises."""
        parts = np.zeros(3, np.float64)
        self._check(self._lib.sesgb_ses_area(self._h, parts.ctypes.data, atom_area_ptr, stream), "ses_area")
        return {"convex": float(parts[0]), "toroidal": float(parts[1]), "concave": float(parts[2]),
                "total": float(parts.sum())}

    def ses_area_backward(self, grad_atoms_ptr: int, grad_parts=(1.0, 1.0, 1.0), stream: int | None = None):
        """grad_atoms (device float4[n], input order) = d (grad_parts . (convex, toroidal, concave)) / d (x, y, z, r)."""
        g = np.ascontiguousarray(np.broadcast_to(np.asarray(grad_parts, np.float32), (3,)))
        self._check(self._lib.sesgb_ses_area_backward(self._h, g.ctypes.data, grad_atoms_ptr, stream), "ses_area_backward")

    def render(self, camera: dict, depth_ptr: int, normals_ptr: int | None = None, stream: int | None = None):
        """Sphere-traced depth (device float[w*h]) and normals (device float3[w*h], optional) of the last
        full-surface build (sesgb_render); camera: the fields of sesgb_camera."""
        c = Camera()
        for k in ("eye", "forward", "right", "up"):
            getattr(c, k)[:] = [float(x) for x in camera[k]]
        for k in ("tan_half_fov", "t_near", "t_far", "eps", "normal_step", "width", "height", "max_steps"):
            setattr(c, k, camera[k])
        self._check(self._lib.sesgb_render(self._h, ctypes.byref(c), depth_ptr, normals_ptr, stream), "render")

    def tuning(self) -> dict:
        """The context's tuning knobs (sesgb_get_tuning)."""
        t = Tuning()
        self._check(self._lib.sesgb_get_tuning(self._h, ctypes.byref(t)), "get_tuning")
        return {f: int(getattr(t, f)) for f in TUNING_FIELDS}

    def set_tuning(self, **knobs):
        """Changes tuning knobs (sesgb_set_tuning); the others keep their values."""
        cur = self.tuning()
        unknown = set(knobs) - set(TUNING_FIELDS)
        if unknown:
            raise ValueError(f"unknown tuning knobs {sorted(unknown)}")
        cur.update({k: int(v) for k, v in knobs.items()})
        t = Tuning(*[cur[f] for f in TUNING_FIELDS])
        self._check(self._lib.sesgb_set_tuning(self._h, ctypes.byref(t)), "set_tuning")

    def cavities(self, voxel: float, probe_component_ptr: int | None = None, stream: int | None = None) -> dict:
        """Components of the probe-accessible space on the device (sesgb_cavities): the grid, the
        component count, exterior and cavity counts; probe_component_ptr (device int32[probes]) receives
        each probe's component. Synchronises."""
        info = CavityInfo()
        self._check(self._lib.sesgb_cavities(self._h, float(voxel), ctypes.byref(info), probe_component_ptr, stream),
                    "cavities")
        return {"origin": np.array(info.origin[:], np.float64), "voxel": info.voxel, "dims": tuple(info.dims[:]),
                "components": info.components, "exterior": info.exterior, "cavities": info.cavities,
                "probes": info.probes}

    def cavity_labels(self) -> np.ndarray:
        """Host copy (int32, flat) of the label grid of the last cavities() call."""
        p = ctypes.c_void_p()
        v = ctypes.c_uint64()
        self._check(self._lib.sesgb_cavity_labels(self._h, ctypes.byref(p), ctypes.byref(v)), "cavity_labels")
        return self._copy(p, v.value, np.int32)

    def cavity_components(self, components: int):
        """(voxel count uint32 [components + 1], border flag uint8 [components + 1]) of the last cavities()."""
        vox = np.zeros(components + 1, np.uint32)
        bor = np.zeros(components + 1, np.uint8)
        self._check(self._lib.sesgb_cavity_components(self._h, vox.ctypes.data, bor.ctypes.data, components + 1),
                    "cavity_components")
        return vox, bor

    @property
    def max_neighbor_per_atom(self) -> int:
        return int(self._lib.sesgb_max_neighbor_per_atom(self._h))

    def _fetch_data(self, d, Q: int) -> dict:
        out = {"atoms": self._copy(d.atoms, d.atomNb, np.float32, 4)}
        out["probe_pos"] = self._copy(d.concavePatchesPosition, d.concavePatchNb, np.float32, 4)
        out["probe_ids"] = self._copy(d.concavePatchesId, d.concavePatchNb, np.int32, 4)
        out["probe_nbrs"] = self._copy(d.concavePatchesNeighbors, 32 * Q, np.float32, 4)
        if self.mode == "full":
            out["convex"] = self._copy(d.convexPatches, d.convexPatchNb, np.uint32, 2)
            out["sectors"] = self._copy(d.sectors, d.sectorNb, np.float32, 4)
            out["segments"] = self._copy(d.segmentPatches, d.segmentPatchNb, np.uint32, 4)
            out["full"] = self._copy(d.circlePatches, d.circlePatchNb, np.uint32, 2)
        else:
            out["tori_pos"] = self._copy(d.circlePosition, d.circlePatchNb, np.float32, 4)
            out["tori_axis"] = self._copy(d.circleAxis, d.circlePatchNb, np.float32, 4)
            out["tori_vs"] = self._copy(d.circleVs, d.circlePatchNb, np.float32, 4)
        return out

    def fetch(self, analysis: bool = True) -> dict:
        """Host copies of every output buffer (and the analysis buffers)."""
        c = self.counts()
        d = self.data()
        out = self._fetch_data(d, c["singular_probes"])
        out["counts"] = c
        if analysis:
            out["perm"] = self.analysis(BUF_ATOM_INDICES, np.uint32)
            out["nbr_count"] = self.analysis(BUF_NEIGHBOR_COUNT, np.uint32)
            cap = self.max_neighbor_per_atom
            out["nbr_ids"] = self.analysis(BUF_NEIGHBOR_IDS, np.uint32)[: d.atomNb * cap].reshape(d.atomNb, cap)
            st = self.analysis(BUF_VISIBILITY_STATUS, np.uint8)
            out["status"] = st[: d.atomNb * cap].reshape(d.atomNb, cap)
            if self.mode == "full":
                out["global_to_trimmed"] = self.analysis(BUF_GLOBAL_TO_TRIMMED, np.uint32)
        return out

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.sesgb_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class SesBatch(SesBuild):
    """Many molecules built together (sesgb_create_batch): one launch sequence for
    the whole batch, molecule m's slice equal to its own SesBuild."""

    def __init__(self, molecules, probe_radius: float = 1.4, mode: str = "full", max_neighbor_per_atom: int = 0,
                 max_intersections_per_circle: int = 0, graph: bool = True, device: int = -1, profile: bool = False,
                 min_capacity: bool = False):
        self._lib = load_library()
        mols = [np.ascontiguousarray(np.asarray(m, np.float32).reshape(-1, 4)) for m in molecules]
        self.starts = np.zeros(len(mols) + 1, np.uint32)
        self.starts[1:] = np.cumsum([m.shape[0] for m in mols])
        self.atoms = np.ascontiguousarray(np.concatenate(mols) if mols else np.zeros((0, 4), np.float32))
        self.mode = mode
        self.probe_radius = float(probe_radius)
        flags = (FLAG_GRAPH if graph else 0) | (FLAG_PROFILE if profile else 0) | (FLAG_MIN_CAPACITY if min_capacity else 0)
        opt = Options(max_neighbor_per_atom, max_intersections_per_circle, device, flags)
        h = ctypes.c_void_p()
        st = self._lib.sesgb_create_batch(self.atoms.ctypes.data if self.atoms.size else None, self.starts.ctypes.data,
                                          len(mols), ctypes.c_float(probe_radius),
                                          MODE_FULL if mode == "full" else MODE_EXTERIOR, ctypes.byref(opt),
                                          ctypes.byref(h))
        self._h = h
        self._check(st, "create_batch")

    @property
    def molecules(self) -> int:
        return int(self._lib.sesgb_batch_molecules(self._h))

    def record(self, m: int) -> dict:
        r = (ctypes.c_uint32 * len(MOL_FIELDS))()
        self._check(self._lib.sesgb_molecule_record(self._h, m, r), "molecule_record")
        return {f: int(r[k]) for k, f in enumerate(MOL_FIELDS)}

    def molecule(self, m: int) -> dict:
        """Host copies of molecule m's output buffers (molecule-local ids)."""
        if self.mode == "full":
            d = FullData()
            self._check(self._lib.sesgb_get_full_molecule(self._h, m, ctypes.byref(d)), "get_full_molecule")
        else:
            d = ExteriorData()
            self._check(self._lib.sesgb_get_exterior_molecule(self._h, m, ctypes.byref(d)), "get_exterior_molecule")
        rec = self.record(m)
        out = self._fetch_data(d, rec["singular_probes"])
        out["record"] = rec
        perm = self.analysis(BUF_ATOM_INDICES, np.uint32)
        out["perm"] = perm[self.starts[m]:self.starts[m + 1]]
        return out
