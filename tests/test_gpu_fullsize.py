"""Full-size workloads on the GPU: bit-exact oracle parity on the whole
batched BLASTP workload (64 queries x 2,000,000 subjects, every HSP field and
counter), on all 128 BLASTX queries against a 100,000-subject slice of the
same database, and on the 64 queries concatenated NCBI-style as one query with
64 contexts; plus reference ordering, determinism, alone == in the mix and HSP
invariants.  The oracle runs on every host core (about a minute on 16)."""
import os

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


def oracle_q(pq):
    return oracle.Query(pq.sequence, pq.context_offset, pq.context_length, pq.x_dropoff, pq.cutoff_score)


def full_parity(h, stats, pqs, residues, offsets, subj_range=None):
    """Every HSP and per-query counter of h (GPU, reference order) against the
    oracle over subjects subj_range (default: all) of the same database."""
    refs = oracle.search_many([oracle_q(pq) for pq in pqs], residues, offsets, nthreads=os.cpu_count() or 1,
                              subj_range=subj_range)
    if subj_range is not None:
        h = h[(h["subject"] >= subj_range[0]) & (h["subject"] < subj_range[1])]
    starts = np.searchsorted(h["query"], np.arange(len(pqs) + 1))
    for k, (ref, subj, cnt) in enumerate(refs):
        got = h[starts[k]:starts[k + 1]]
        assert len(got) == len(ref), (k, len(got), len(ref))
        assert np.array_equal(got["subject"], subj), k
        for f, g in ORACLE_FIELDS:
            assert np.array_equal(got[g], ref[f]), (k, f)
        if subj_range is None:
            st = stats[k]
            assert (st["lookup_hits"], st["init_extends"], st["good_init_extends"]) == tuple(int(c) for c in cnt), k
            assert st["subjects_passed"] == len(np.unique(subj)), k
    return sum(len(r[0]) for r in refs)


def test_batched_full_parity(batched):
    """The whole batched workload, every HSP of every query and subject."""
    qs, db, gdb, pqs, batch, res = batched
    n = full_parity(res.hsps, res.stats, pqs, db.residues, db.offsets)
    assert n == len(res.hsps) and n > 1_000_000


def test_concatenated_queries_as_contexts(batched):
    """NCBI's multi-query form: the 64 queries concatenated as ONE query with
    64 contexts (one sentinel between contexts).  Word hits of neighbouring
    contexts share diagonals here, pair across the context boundary when they
    fall inside the window, and left walks run into the sentinels; the GPU
    must reproduce the oracle on the same concatenation bit for bit."""
    qs, db, gdb, pqs, batch, res = batched
    parts, off, ln = [], [], []
    pos = 0
    for k, q in enumerate(qs):
        if k:
            parts.append(np.zeros(1, np.uint8))
            pos += 1
        off.append(pos)
        ln.append(len(q))
        parts.append(q)
        pos += len(q)
    seq = np.concatenate(parts)
    nctx = len(qs)
    cat = hblast.ProteinQuery(seq, off, ln, [16] * nctx, [41] * nctx)
    sub = db.slice(0, 50_000)
    sdb = hblast.Database(sub.residues, sub.offsets)
    r = hblast.search(sdb, hblast.Batch.proteins([cat]))
    assert len(r.hsps) > 1000 and len(np.unique(r.hsps["context"])) == nctx
    full_parity(r.hsps, r.stats, [cat], sub.residues, sub.offsets)
    # the case is exercised: hits of neighbouring contexts pair up, so the
    # concatenation tries more extensions than the 64 queries searched apart
    apart = hblast.search(sdb, hblast.Batch.proteins(pqs))
    assert r.stats[0]["init_extends"] > sum(st["init_extends"] for st in apart.stats)
    sdb.close()


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
    # all 128 queries (six frames each) against the first 100,000 subjects, bit-exact
    full_parity(h, r.stats, tq, db.residues, db.offsets, subj_range=(0, 100_000))
    rng = np.random.default_rng(7)
    sample_parity(h[h["query"] < 16], tq[:16], db,
                  np.unique(np.concatenate([rng.choice(db.n, 400, replace=False),
                                            h["subject"][h["query"] < 16][:200]])))
