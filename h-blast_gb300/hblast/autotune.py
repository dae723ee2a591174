"""Autotuner for the word finder: per query-length bucket, choose the query
group length, the hit mode (chunk mode / offset mode), the CTA size, the
subject chunk a CTA takes (by count: 32, 128 or 512 subjects, about 11, 46 or
184 KB of letters; or by bytes: 4, 16 or 64 KB of subject letters), the
threads per subject (one warp; or 2, 4, 8 warps: that many query groups share
each pass over a subject, 8 warps being one CTA per subject) and the
diagonal-table placement (shared or global memory) by timing searches of the
bucket's queries against the database.  Stage one times the group-length /
mode / CTA candidates; stage two varies the chunk, the threads per subject
and the placement of the best.

Every choice gives identical HSPs (the tests check it); only time changes.
The report lists, per bucket and candidate, the word-finder time, the
achieved subject-stream bandwidth (database bytes / kernel time) and
query x db residues/s.  `search_tuned` then searches a batch bucket by bucket
with the chosen settings and merges the results in reference order.
"""
from __future__ import annotations

import json
from dataclasses import asdict, dataclass, field, replace
from pathlib import Path
from typing import Sequence

import numpy as np

from . import core

DEFAULT_BUCKETS = ((0, 300), (300, 1000), (1000, 4000), (4000, 65001))


@dataclass(frozen=True)
class Choice:
    max_group_len: int      # 1 = one query per group; 0 = library default
    mode: int               # 0 chunk mode, 1 offset mode
    threads: int            # largest CTA size
    tile_subjects: int = 0  # subjects per work unit, 0 = automatic
    global_tables: bool = False
    warps_per_subject: int = 1  # query groups sharing each pass over a subject
    tile_bytes: int = 0     # work unit by subject letters, 0 = automatic


DEFAULT_CANDIDATES = (
    Choice(1, 0, 256), Choice(1000, 0, 256), Choice(2008, 0, 256), Choice(4056, 0, 256),
    Choice(6000, 0, 256), Choice(8152, 1, 256), Choice(16344, 1, 128),
)
STAGE2 = (dict(tile_subjects=32), dict(tile_subjects=128), dict(tile_subjects=512), dict(tile_bytes=4096),
          dict(tile_bytes=16384), dict(tile_bytes=65536), dict(warps_per_subject=2), dict(warps_per_subject=4),
          dict(warps_per_subject=8), dict(global_tables=True))


@dataclass
class BucketResult:
    lo: int
    hi: int
    n_queries: int
    best: Choice | None
    rows: list = field(default_factory=list)   # (choice, ms, GB/s, residues/s)


def time_choice(db: core.Database, pqs: Sequence[core.ProteinQuery], choice: Choice, db_residues: int,
                reps: int = 2) -> float:
    batch = core.Batch.proteins(pqs, max_group_len=choice.max_group_len).set_mode(choice.mode)
    batch.tune(choice.tile_subjects, choice.global_tables).schedule(choice.warps_per_subject, choice.tile_bytes)
    s = core.Searcher(db, batch, core.default_options(num_threadsx=choice.threads))
    try:
        best = float("inf")
        for _ in range(reps + 1):          # first launch warms up
            s.launch(None)
            s.sync()
            best = min(best, s.timing()[0])
        return best
    finally:
        s.close()
        batch.close()


def tune(db: core.Database, queries: Sequence[core.ProteinQuery], db_residues: int,
         buckets=DEFAULT_BUCKETS, candidates=DEFAULT_CANDIDATES, reps: int = 2,
         stage2=STAGE2) -> list[BucketResult]:
    """Rows per bucket: (choice, word-finder ms, subject-stream GB/s, query x db residues/s)."""
    out = []
    for lo, hi in buckets:
        pqs = [q for q in queries if lo <= q.length < hi]
        br = BucketResult(lo, hi, len(pqs), None)
        if pqs:
            qres = sum(q.length for q in pqs)
            best_ms = float("inf")

            def measure(c):
                nonlocal best_ms
                ms = time_choice(db, pqs, c, db_residues, reps)
                gbs = db_residues / (ms * 1e-3) / 1e9
                br.rows.append((asdict(c), ms, gbs, qres * db_residues / (ms * 1e-3)))
                if ms < best_ms:
                    best_ms, br.best = ms, c

            for c in candidates:
                measure(c)
            first = br.best
            for kw in stage2:
                if kw.get("warps_per_subject", 1) * 32 > first.threads:
                    continue          # a pass shared by W groups needs W warps in the CTA
                measure(replace(first, **kw))
        out.append(br)
    return out


def save(results: list[BucketResult], path: str | Path) -> None:
    Path(path).write_text(json.dumps([dict(lo=r.lo, hi=r.hi, n_queries=r.n_queries,
                                           best=asdict(r.best) if r.best else None, rows=r.rows)
                                      for r in results], indent=1))


def load(path: str | Path) -> list[BucketResult]:
    out = []
    for d in json.loads(Path(path).read_text()):
        out.append(BucketResult(d["lo"], d["hi"], d["n_queries"], Choice(**d["best"]) if d["best"] else None,
                                d["rows"]))
    return out


def choice_for(length: int, table: list[BucketResult]) -> Choice:
    for r in table:
        if r.lo <= length < r.hi and r.best is not None:
            return r.best
    return Choice(0, 0, 256)


def search_tuned(db: core.Database, queries: Sequence[core.ProteinQuery],
                 table: list[BucketResult]) -> core.SearchResult:
    """Search each bucket's queries with its tuned settings; merge in reference order."""
    by_choice: dict[Choice, list[int]] = {}
    for i, q in enumerate(queries):
        by_choice.setdefault(choice_for(q.length, table), []).append(i)
    parts, stats = [], [None] * len(queries)
    wf = od = 0.0
    for c, idx in by_choice.items():
        batch = core.Batch.proteins([queries[i] for i in idx], max_group_len=c.max_group_len).set_mode(c.mode)
        batch.tune(c.tile_subjects, c.global_tables).schedule(c.warps_per_subject, c.tile_bytes)
        r = core.search(db, batch, core.default_options(num_threadsx=c.threads))
        h = r.hsps.copy()
        h["query"] = np.asarray(idx, dtype=np.int32)[h["query"]]
        parts.append(h)
        for k, i in enumerate(idx):
            stats[i] = r.stats[k]
        wf += r.wordfinder_ms
        od += r.ordering_ms
        batch.close()
    h = np.concatenate(parts) if parts else np.zeros(0, dtype=core.HSP_DTYPE)
    h = h[np.lexsort((h["q_off"], h["s_off"], h["subject"], h["query"]))]
    return core.SearchResult(h, stats, wf, od)
