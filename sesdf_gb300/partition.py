"""Sharding of independent molecules (batches, MD-like frames) over ranks.

One GPU per rank; molecules are independent, so a batch is split into
contiguous molecule ranges of balanced atom counts and each rank builds its
range as one batch (no collective on the data path; only the per-rank counts
and timings are gathered on the host side).
"""
from __future__ import annotations

import numpy as np


def split_by_atoms(sizes, ranks: int) -> list[tuple[int, int]]:
    """Contiguous [start, end) molecule ranges, one per rank, whose atom totals are as
    even as a prefix cut allows (rank r ends at the first prefix sum >= (r + 1) / ranks
    of the total). Ranges may be empty when there are fewer molecules than ranks."""
    s = np.asarray(sizes, np.int64)
    if ranks < 1:
        raise ValueError("ranks must be >= 1")
    pre = np.concatenate([[0], np.cumsum(s)])
    total = int(pre[-1])
    cuts = [0]
    for r in range(1, ranks):
        target = total * r / ranks
        c = int(np.searchsorted(pre, target, side="left"))
        # the cut closer to the target of the two neighbouring prefix sums
        if c > 0 and abs(pre[c - 1] - target) <= abs(pre[min(c, len(s))] - target):
            c -= 1
        cuts.append(max(cuts[-1], min(c, len(s))))
    cuts.append(len(s))
    return [(cuts[r], cuts[r + 1]) for r in range(ranks)]


def rank_share(sizes, rank: int, ranks: int) -> tuple[int, int]:
    return split_by_atoms(sizes, ranks)[rank]
