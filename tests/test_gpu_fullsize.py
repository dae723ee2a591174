"""Full-size workloads on the GPU, checked through properties that do not need
the whole CPU search: reference ordering, determinism, alone == in the mix,
HSP invariants, and bit-exact oracle parity on a random sample of subjects
taken from the full database."""
import numpy as np
import pytest

import hblast
from hblast import synth
from oracle import oracle

pytestmark = pytest.mark.gpu

ORACLE_FIELDS = (("q_start", "q_start"), ("s_start", "s_start"), ("q_off", "q_off"), ("s_off", "s_off"),
                 ("len", "len"), ("score", "score"), ("ctx", "context"))


@pytest.fixture(scope="module")
def batched(built):
    qs, db = synth.batched_blastp(seed=0)          # 64 queries x 2,000,000 subjects
    gdb = hblast.Database(db.residues, db.offsets)
    pqs = [hblast.ProteinQuery.blastp(q) for q in qs]
    batch = hblast.Batch.proteins(pqs)
    res = hblast.search(gdb, batch)
    return qs, db, gdb, pqs, batch, res


def invariants(h, qlens, slens, cutoffs):
    assert np.array_equal(np.lexsort((h["q_off"], h["s_off"], h["subject"], h["query"])), np.arange(len(h)))
    assert (h["score"] >= cutoffs[h["query"]]).all()
    assert (h["len"] > 0).all() and (h["q_start"] >= 0).all() and (h["s_start"] >= 0).all()
    assert (h["s_start"] + h["len"] <= slens[h["subject"]]).all()
    assert (h["q_start"] + h["len"] <= qlens[h["query"]]).all()
    assert np.array_equal(h["q_start"] - h["s_start"], h["q_off"] - h["s_off"])   # one diagonal


def sample_parity(h, pqs, db, subjects):
    """GPU HSPs of `subjects` (ids in db) against the oracle run on just those subjects."""
    subjects = np.sort(subjects)
    sub = [db.subject(int(j)) for j in subjects]
    off = np.zeros(len(sub) + 1, np.int64)
    off[1:] = np.cumsum([len(x) for x in sub])
    res = np.concatenate(sub)
    mask = np.isin(h["subject"], subjects)
    got_all = h[mask]
    for k, pq in enumerate(pqs):
        ref, subj, _ = oracle.search(oracle.Query(pq.sequence, pq.context_offset, pq.context_length,
                                                  pq.x_dropoff, pq.cutoff_score), res, off, nthreads=8)
        got = got_all[got_all["query"] == k]
        assert len(got) == len(ref), k
        assert np.array_equal(got["subject"], subjects[subj]), k
        for f, g in ORACLE_FIELDS:
            assert np.array_equal(got[g], ref[f]), (k, f)


def test_batched_invariants_and_sample_parity(batched):
    qs, db, gdb, pqs, batch, res = batched
    h = res.hsps
    assert len(h) > 1000
    invariants(h, np.array([len(q) for q in qs]), db.lengths, np.full(len(qs), 41))
    rng = np.random.default_rng(99)
    sample = np.unique(np.concatenate([rng.choice(db.n, 1500, replace=False), db.planted[:300]]))
    sample_parity(h, pqs, db, sample)


def test_batched_deterministic(batched):
    qs, db, gdb, pqs, batch, res = batched
    again = hblast.search(gdb, batch)
    assert np.array_equal(again.hsps, res.hsps)
    assert again.stats == res.stats


def test_batched_alone_equals_mix(batched):
    qs, db, gdb, pqs, batch, res = batched
    for k in (0, 17, 63):
        alone = hblast.search(gdb, hblast.Batch.proteins([pqs[k]])).hsps
        got = res.for_query(k).copy()
        got["query"] = 0
        assert np.array_equal(got, alone), k
        assert res.stats[k]["lookup_hits"] > 0


def test_blastx_full_database(batched):
    qs, db, gdb, pqs, batch, res = batched
    nts = synth.blastx_queries(0, db, n_queries=128)
    xd = np.full((128, 6), 16, dtype=np.int32)
    cu = np.full((128, 6), 41, dtype=np.int32)
    r = hblast.search(gdb, hblast.Batch.blastx(nts, xd, cu))
    h = r.hsps
    tq = []
    for nt in nts:
        prot, off, ln = oracle.translate6(nt)
        tq.append(hblast.ProteinQuery(prot, off, ln, [16] * 6, [41] * 6))
    invariants(h, np.array([q.length for q in tq]), db.lengths, np.full(128, 41))
    # most planted ORFs (40..70% identity over 66..300 aa) give an HSP
    assert len(np.unique(h["query"])) >= 64
    rng = np.random.default_rng(7)
    sample_parity(h[h["query"] < 16], tq[:16], db,
                  np.unique(np.concatenate([rng.choice(db.n, 400, replace=False),
                                            h["subject"][h["query"] < 16][:200]])))
