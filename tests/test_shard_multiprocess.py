"""N>1 host path on the CPU: two gloo ranks each search one contiguous shard of
the database and rank 0 gathers and merges; the result must equal a single
search of the whole database.  The per-rank search here is the oracle (the CPU
stand-in for each rank's GPU); the code under test is the partition, the
subject-id rebasing and the gather/merge order."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from hblast import shard, synth
from oracle import oracle


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def oracle_hsps(q, db, lo, hi):
    from hblast.core import HSP_DTYPE
    h, subj, _ = oracle.search(oracle.Query.blastp(q), db.residues, db.offsets, subj_range=(lo, hi))
    out = np.zeros(len(h), dtype=HSP_DTYPE)
    out["subject"] = subj - lo
    for f, g in (("q_start", "q_start"), ("s_start", "s_start"), ("q_off", "q_off"), ("s_off", "s_off"),
                 ("len", "len"), ("score", "score"), ("ctx", "context")):
        out[g] = h[f]
    return out


def _rank(rank, world, port, path):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(21)
    q = synth.random_letters(rng, 250)
    db = synth.make_db(rng, 600, 300, 0.6, 30, 5000, 40, [q], 120, 0.5)
    lo, hi = shard.partition(db.lengths, world)[rank]
    local = oracle_hsps(q, db, lo, hi)
    merged = shard.gather_merge(local, lo)
    if rank == 0:
        np.save(path, merged)
    dist.barrier()
    dist.destroy_process_group()


def test_partition_balances_residues():
    lens = np.array([5, 100, 3, 40, 40, 40, 7, 90, 1, 1])
    parts = shard.partition(lens, 3)
    assert parts[0][0] == 0 and parts[-1][1] == len(lens)
    assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
    assert shard.partition(lens, 1) == [(0, 10)]
    assert len(shard.partition(lens, 20)) == 20      # more parts than subjects: empty ranges allowed


@pytest.mark.timeout(300)
def test_two_rank_gather_equals_single_search(built, tmp_path):
    path = str(tmp_path / "merged.npy")
    mp.start_processes(_rank, args=(2, free_port(), path), nprocs=2, join=True, start_method="spawn")
    merged = np.load(path)
    rng = np.random.default_rng(21)
    q = synth.random_letters(rng, 250)
    db = synth.make_db(rng, 600, 300, 0.6, 30, 5000, 40, [q], 120, 0.5)
    full = oracle_hsps(q, db, 0, db.n)
    assert len(full) > 0
    assert np.array_equal(merged, full)
