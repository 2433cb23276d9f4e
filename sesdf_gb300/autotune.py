"""Autotuner for builds of a caller's molecules (one molecule or a batch).

Times a few builds of each candidate setting with CUDA events and keeps the
fastest. The knobs change no result, only speed:

* neighbour-grid cell size: cells of the largest pair cutoff (27-cell stencil)
  or of half of it (125-cell stencil cut to each atom's reach);
* block shapes: warps per block of the neighbour search (2, 4, 8, 16), atoms
  (warps) per block of the visibility pass and of the probe screen (1, 2, 4),
  and the probe screen as a persistent grid over a work counter or one block
  per atom group;
* neighbour-list capacity (max_neighbor_per_atom): only capacities that leave
  the results unchanged are tried -- at least the largest neighbour count met,
  and no more than the default 128 (a larger one would keep neighbours that the
  default build truncates);
* CUDA graph replay of the build.

The search is coordinate-wise: capacity and graph first (they pick the context),
then each tuning knob in turn with the others held at their best so far.
"""
from __future__ import annotations

from .api import SesBatch, SesBuild

DEFAULT_CAP = 128
KNOBS = {
    "neighbor_cell_span": (2, 1),
    "neighbor_warps": (8, 4, 16, 2),
    "visibility_warps": (1, 2, 4),
    "probe_warps": (1, 2, 4),
    "probe_queue": (0, 1),
}


def _time(build, d_atoms, stream, trials: int) -> float:
    import torch
    build.build_async(d_atoms.data_ptr(), stream.cuda_stream)
    build.finish()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    best = float("inf")
    for _ in range(trials):
        t0.record(stream)
        build.build_async(d_atoms.data_ptr(), stream.cuda_stream)
        t1.record(stream)
        build.finish()
        torch.cuda.synchronize()
        best = min(best, t0.elapsed_time(t1))
    return best


def _make(molecules, probe_radius, mode, cap, graph):
    if isinstance(molecules, (list, tuple)):
        return SesBatch(molecules, probe_radius, mode, max_neighbor_per_atom=cap, graph=graph)
    return SesBuild(molecules, probe_radius, mode, max_neighbor_per_atom=cap, graph=graph)


def tune(molecules, probe_radius: float = 1.4, mode: str = "full", trials: int = 3, knobs: dict | None = None) -> dict:
    """molecules: one (n, 4) array (a single build) or a list of them (a batch). Returns
    {"max_neighbor_per_atom", "graph", "tuning": {knob: value}, "ms", "max_neighbors", "tried": [...]}."""
    import torch
    stream = torch.cuda.current_stream()
    knobs = KNOBS if knobs is None else knobs
    with _make(molecules, probe_radius, mode, 0, True) as probe:
        d_atoms = torch.from_numpy(probe.atoms).cuda()
        probe.build_async(d_atoms.data_ptr(), stream.cuda_stream)
        probe.finish()
        most = probe.counts()["max_neighbors"]
    caps = {DEFAULT_CAP}
    if most <= DEFAULT_CAP:
        caps.add(max(32, -(-most // 32) * 32))
    tried = []
    best = None
    for cap in sorted(caps):
        for graph in (False, True):
            with _make(molecules, probe_radius, mode, cap, graph) as b:
                ms = _time(b, d_atoms, stream, trials)
            tried.append({"max_neighbor_per_atom": cap, "graph": graph, "ms": round(ms, 4)})
            if best is None or ms < best["ms"]:
                best = {"max_neighbor_per_atom": cap, "graph": graph, "ms": ms}
    with _make(molecules, probe_radius, mode, best["max_neighbor_per_atom"], best["graph"]) as b:
        setting = b.tuning()
        base_ms = best["ms"]
        for knob, values in knobs.items():
            for v in values:
                if v == setting[knob]:
                    continue
                trial = dict(setting, **{knob: v})
                b.set_tuning(**trial)
                ms = _time(b, d_atoms, stream, trials)
                tried.append({"tuning": trial, "ms": round(ms, 4)})
                if ms < base_ms:
                    base_ms, setting = ms, trial
            b.set_tuning(**setting)
    return {"max_neighbor_per_atom": best["max_neighbor_per_atom"], "graph": best["graph"], "tuning": setting,
            "ms": round(base_ms, 4), "max_neighbors": most, "tried": tried}


def tune_batch(molecules, probe_radius: float = 1.4, mode: str = "full", trials: int = 3) -> dict:
    """tune() of a batch of molecules."""
    return tune(list(molecules), probe_radius, mode, trials)
