"""Database sharding across GPUs/processes.

Subjects are independent, so a database splits into contiguous ordinal-id
ranges with no exchange during the search (H-BLAST splits a volume's subject
groups across cards by byte balance, h_blast.cu:656-870, and splits queries
across processes in scripts/H-BLASTM:212-233).  The only exchange is a host
gather that concatenates the per-shard HSP lists; since shards are contiguous
OID ranges, shifting each shard's subject ids by its base and merging by
(query, subject) keeps the reference order.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np


def partition(lengths: np.ndarray, parts: int) -> list[tuple[int, int]]:
    """Split subjects [0, n) into `parts` contiguous ranges of nearly equal residues."""
    lengths = np.asarray(lengths, dtype=np.int64)
    n = len(lengths)
    if parts < 1:
        raise ValueError("parts must be >= 1")
    cum = np.concatenate([[0], np.cumsum(lengths)])
    total = cum[-1]
    bounds = [0]
    for p in range(1, parts):
        target = total * p / parts
        b = int(np.searchsorted(cum, target, side="left"))
        bounds.append(min(max(b, bounds[-1]), n))
    bounds.append(n)
    return [(bounds[i], bounds[i + 1]) for i in range(parts)]


def merge(parts: Sequence[tuple[int, np.ndarray]]) -> np.ndarray:
    """Merge per-shard HSP arrays (subject ids local to the shard) into one list in
    reference order.  parts = [(subject_base, hsps), ...]."""
    arrs = []
    for base, h in parts:
        h = np.array(h, copy=True)
        h["subject"] += base
        arrs.append(h)
    if not arrs:
        raise ValueError("nothing to merge")
    allh = np.concatenate(arrs)
    order = np.lexsort((allh["q_off"], allh["s_off"], allh["subject"], allh["query"]))
    return allh[order]


def gather_merge(local: np.ndarray, base: int, dst: int = 0):
    """torch.distributed gather of every rank's (base, hsps) to `dst`, merged there.
    Returns the merged array on dst and None elsewhere."""
    import torch.distributed as dist
    world = dist.get_world_size()
    obj = (int(base), local)
    out = [None] * world if dist.get_rank() == dst else None
    dist.gather_object(obj, out, dst=dst)
    if dist.get_rank() != dst:
        return None
    return merge(out)
