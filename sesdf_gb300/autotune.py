"""Autotuner for batched builds.

Picks, for one batch of molecules, the neighbour-list capacity
(max_neighbor_per_atom) and whether the build replays as a CUDA graph, by
timing a few builds of each candidate with CUDA events. Only capacities that
leave the results unchanged are tried: at least the largest neighbour count
of the batch, and no more than the default 128 (a larger one would keep
neighbours that the default build truncates). Kernel block shapes are fixed
by the register and shared-memory budgets of the kernels and are not tuned.
"""
from __future__ import annotations

from .api import SesBatch

DEFAULT_CAP = 128


def _time(batch: SesBatch, d_atoms, stream, trials: int) -> float:
    import torch
    batch.build_async(d_atoms.data_ptr(), stream.cuda_stream)
    batch.finish()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    best = float("inf")
    for _ in range(trials):
        t0.record(stream)
        batch.build_async(d_atoms.data_ptr(), stream.cuda_stream)
        t1.record(stream)
        batch.finish()
        torch.cuda.synchronize()
        best = min(best, t0.elapsed_time(t1))
    return best


def tune_batch(molecules, probe_radius: float = 1.4, mode: str = "full", trials: int = 3) -> dict:
    """Returns {"max_neighbor_per_atom", "graph", "ms", "tried": [...]} for the fastest candidate."""
    import torch
    stream = torch.cuda.current_stream()
    with SesBatch(molecules, probe_radius, mode) as probe:
        d_atoms = torch.from_numpy(probe.atoms).cuda()
        probe.build_async(d_atoms.data_ptr(), stream.cuda_stream)
        probe.finish()
        most = probe.counts()["max_neighbors"]
    caps = {DEFAULT_CAP}
    if most <= DEFAULT_CAP:
        caps.add(max(32, -(-most // 32) * 32))
    tried = []
    for cap in sorted(caps):
        for graph in (False, True):
            with SesBatch(molecules, probe_radius, mode, max_neighbor_per_atom=cap, graph=graph) as b:
                ms = _time(b, d_atoms, stream, trials)
            tried.append({"max_neighbor_per_atom": cap, "graph": graph, "ms": round(ms, 4)})
    best = min(tried, key=lambda r: r["ms"])
    return dict(best, tried=tried, max_neighbors=most)
