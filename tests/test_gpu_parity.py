"""GPU word finder (through the C ABI) against the CPU oracle, bit-exact.

Every HSP field and the per-query counters must be identical; tolerance 0
(integer work).  Sizes are kept where the oracle finishes in seconds (the
plain configuration is whole); the full-size batched and BLASTX workloads are
compared with the oracle in test_gpu_fullsize.py.
"""
import numpy as np
import pytest

import hblast
from hblast import synth
from oracle import oracle
from test_oracle import KNOWN_ANSWERS, enc, hand_lut

pytestmark = pytest.mark.gpu


def oracle_query(pq: hblast.ProteinQuery) -> oracle.Query:
    return oracle.Query(pq.sequence, pq.context_offset, pq.context_length, pq.x_dropoff, pq.cutoff_score)


def check(res: hblast.SearchResult, pqs, residues, offsets, threads=4):
    h = res.hsps
    # reference order: by query, subject, then (s_off, q_off)
    key = np.lexsort((h["q_off"], h["s_off"], h["subject"], h["query"]))
    assert np.array_equal(key, np.arange(len(h)))
    for k, pq in enumerate(pqs):
        ref, subj, cnt = oracle.search(oracle_query(pq), residues, offsets, nthreads=threads)
        got = h[h["query"] == k]
        assert len(got) == len(ref), (k, len(got), len(ref))
        assert np.array_equal(got["subject"], subj), k
        for f, g in (("q_start", "q_start"), ("s_start", "s_start"), ("q_off", "q_off"), ("s_off", "s_off"),
                     ("len", "len"), ("score", "score"), ("ctx", "context")):
            assert np.array_equal(got[g], ref[f]), (k, f)
        st = res.stats[k]
        assert (st["lookup_hits"], st["init_extends"], st["good_init_extends"]) == tuple(int(c) for c in cnt), k
        assert st["subjects_passed"] == len(np.unique(subj))


@pytest.fixture(scope="module")
def small_db(built):
    rng = np.random.default_rng(11)
    qs = [synth.random_letters(rng, n) for n in (300, 57, 1200, 800, 3, 1500, 433, 96)]
    db = synth.make_db(rng, 3000, 300, 0.6, 30, 5000, 0.05, qs, lambda r: r.integers(50, 301),
                       lambda r: r.uniform(0.3, 0.6))
    return qs, db, hblast.Database(db.residues, db.offsets)


def test_plain_single_query(built):
    # the plain configuration as a whole: 1 query of 300 aa vs 20,000 subjects, seed 0
    qs, db = synth.plain_blastp(seed=0, n_subjects=20000)
    gdb = hblast.Database(db.residues, db.offsets)
    pqs = [hblast.ProteinQuery.blastp(q) for q in qs]
    res = hblast.search(gdb, hblast.Batch.proteins(pqs))
    assert len(res.hsps) > 0
    check(res, pqs, db.residues, db.offsets)


@pytest.mark.parametrize("max_group_len", [0, 1, 4000])
def test_batched_queries(small_db, max_group_len):
    qs, db, gdb = small_db
    pqs = [hblast.ProteinQuery.blastp(q) for q in qs]
    res = hblast.search(gdb, hblast.Batch.proteins(pqs, max_group_len=max_group_len))
    check(res, pqs, db.residues, db.offsets)


def test_alone_equals_in_the_mix(small_db):
    qs, db, gdb = small_db
    pqs = [hblast.ProteinQuery.blastp(q) for q in qs]
    mix = hblast.search(gdb, hblast.Batch.proteins(pqs)).hsps
    for k, pq in enumerate(pqs):
        alone = hblast.search(gdb, hblast.Batch.proteins([pq])).hsps
        got = mix[mix["query"] == k].copy()
        got["query"] = 0
        assert np.array_equal(got, alone), k


@pytest.mark.parametrize("qlen", [3000, 9000, 20000])
def test_long_query_tables(built, qlen):
    # 3000, 9000, 20000: 4096-, 16384- and 32768-entry tables in the global
    # scratch (the 200-letter query's group uses a shared table)
    rng = np.random.default_rng(12)
    q = synth.random_letters(rng, qlen)
    db = synth.make_db(rng, 300, 300, 0.6, 30, 5000, 40, [q], lambda r: r.integers(100, 400), 0.5)
    gdb = hblast.Database(db.residues, db.offsets)
    pqs = [hblast.ProteinQuery.blastp(q), hblast.ProteinQuery.blastp(q[:200])]
    res = hblast.search(gdb, hblast.Batch.proteins(pqs))
    check(res, pqs, db.residues, db.offsets)


@pytest.mark.parametrize("mode", [0, 1])
def test_both_hit_modes(small_db, mode):
    qs, db, gdb = small_db
    pqs = [hblast.ProteinQuery.blastp(q) for q in qs]
    res = hblast.search(gdb, hblast.Batch.proteins(pqs).set_mode(mode))
    check(res, pqs, db.residues, db.offsets)


def contexts_query(parts, x_dropoff, cutoff):
    """Several sequences as the contexts of one query (one sentinel between
    contexts), each with its own X-drop and cutoff."""
    seq, off, ln, pos = [], [], [], 0
    for k, p in enumerate(parts):
        if k:
            seq.append(np.zeros(1, np.uint8))
            pos += 1
        off.append(pos)
        ln.append(len(p))
        seq.append(p)
        pos += len(p)
    return hblast.ProteinQuery(np.concatenate(seq), off, ln, x_dropoff, cutoff)


@pytest.mark.parametrize("mode", [0, 1])
def test_per_context_dropoff_and_cutoff(small_db, mode):
    """X-drop and cutoff are per-context inputs (H-BLAST h_blast.cu:977-983):
    contexts of one query with different values, in both hit modes."""
    qs, db, gdb = small_db
    pqs = [contexts_query([qs[0], qs[1], qs[3]], [7, 16, 30], [25, 41, 55]),
           contexts_query([qs[2], qs[5]], [22, 10], [33, 60]),
           contexts_query([qs[6], qs[7], qs[4]], [40, 12, 16], [41, 20, 41])]
    res = hblast.search(gdb, hblast.Batch.proteins(pqs).set_mode(mode))
    assert len(res.hsps) > 0
    check(res, pqs, db.residues, db.offsets)
    # the per-context values matter: the same contexts at 16 / 41 give other HSPs
    flat = [contexts_query([qs[0], qs[1], qs[3]], [16] * 3, [41] * 3)]
    ref = hblast.search(gdb, hblast.Batch.proteins(flat).set_mode(mode))
    assert not np.array_equal(ref.hsps, res.hsps[res.hsps["query"] == 0])


def test_blastx(built):
    rng = np.random.default_rng(13)
    prot_q = synth.random_letters(rng, 400)
    db = synth.make_db(rng, 600, 300, 0.6, 30, 5000, 30, [prot_q], 150, 0.6)
    nts = synth.blastx_queries(5, db, n_queries=4)
    xd = np.full((4, 6), 16, dtype=np.int32)
    cu = np.full((4, 6), 41, dtype=np.int32)
    cu[1] = [30, 35, 41, 41, 38, 33]
    gdb = hblast.Database(db.residues, db.offsets)
    res = hblast.search(gdb, hblast.Batch.blastx(nts, xd, cu))
    pqs = []
    for k, nt in enumerate(nts):
        prot, off, ln = oracle.translate6(nt)
        pqs.append(hblast.ProteinQuery(prot, off, ln, xd[k], cu[k]))
    assert len(res.hsps) > 0
    check(res, pqs, db.residues, db.offsets)


def test_edge_subjects(built):
    rng = np.random.default_rng(14)
    q = synth.random_letters(rng, 120)
    subs = [np.zeros(0, np.uint8), q[:1], q[:2], q[:3], q[:4], q.copy(), np.concatenate([q, q, q]),
            np.full(200, 1, np.uint8), np.full(300, 20, np.uint8), np.array(list(range(1, 28)) * 10, np.uint8),
            synth.random_letters(rng, 40000)]
    lens = [len(s) for s in subs]
    offsets = np.zeros(len(subs) + 1, np.int64)
    offsets[1:] = np.cumsum(lens)
    residues = np.concatenate(subs).astype(np.uint8)
    gdb = hblast.Database(residues, offsets)
    pqs = [hblast.ProteinQuery.blastp(q), hblast.ProteinQuery.blastp(np.full(50, 1, np.uint8), 16, 20),
           hblast.ProteinQuery.blastp(np.full(64, 20, np.uint8), 10, 30)]
    res = hblast.search(gdb, hblast.Batch.proteins(pqs))
    check(res, pqs, residues, offsets)


def test_full_alphabet(built):
    """Queries and subjects drawn from all 27 NCBIstdaa letters (B, Z, X, U,
    *, O and J included, about a quarter of the letters): words over the whole
    28-letter index space and those letters' matrix rows and columns in the
    walks.  A third of the subjects hold a mutated segment of a query, so
    extensions pass the cutoff."""
    rng = np.random.default_rng(15)
    qs = [rng.integers(1, 28, size=n, dtype=np.uint8) for n in (200, 700, 31)]
    subs = []
    for i in range(1500):
        s = rng.integers(1, 28, size=int(rng.integers(20, 400)), dtype=np.uint8)
        if i % 3 == 0:
            q = qs[i % 2]
            a, n = int(rng.integers(0, len(q) - 60)), int(rng.integers(30, 60))
            seg = q[a:a + n].copy()
            mut = rng.random(n) < 0.2
            seg[mut] = rng.integers(1, 28, size=int(mut.sum()), dtype=np.uint8)
            p = int(rng.integers(0, len(s) + 1))
            s = np.concatenate([s[:p], seg, s[p:]])
        subs.append(s)
    offsets = np.zeros(len(subs) + 1, np.int64)
    offsets[1:] = np.cumsum([len(s) for s in subs])
    residues = np.concatenate(subs)
    gdb = hblast.Database(residues, offsets)
    pqs = [hblast.ProteinQuery.blastp(q) for q in qs]
    res = hblast.search(gdb, hblast.Batch.proteins(pqs))
    h = res.hsps
    assert len(h) > 100
    check(res, pqs, residues, offsets)
    # the HSPs run over the non-standard letters
    nonstd = np.isin(residues, [2, 21, 23, 24, 25, 26, 27])
    covered = sum(int(nonstd[offsets[r["subject"]] + r["s_start"]:offsets[r["subject"]] + r["s_start"] + r["len"]].sum())
                  for r in h)
    assert covered > 0


def test_empty_database(built):
    gdb = hblast.Database(np.zeros(0, np.uint8), np.zeros(1, np.int64))
    res = hblast.search(gdb, hblast.Batch.proteins([hblast.ProteinQuery.blastp(np.ones(50, np.uint8))]))
    assert len(res.hsps) == 0 and res.stats[0]["lookup_hits"] == 0


def test_capacity_overflow_relaunch(small_db):
    qs, db, gdb = small_db
    pqs = [hblast.ProteinQuery.blastp(q) for q in qs[:3]]
    batch = hblast.Batch.proteins(pqs)
    full = hblast.search(gdb, batch)
    tiny = hblast.search(gdb, batch, hsp_capacity=1)
    assert len(full.hsps) > 1
    assert np.array_equal(full.hsps, tiny.hsps)


def test_smallbone_table(built):
    from test_host import smallbone_from_csr
    rng = np.random.default_rng(15)
    q = synth.random_letters(rng, 350)
    db = synth.make_db(rng, 500, 300, 0.6, 30, 5000, 25, [q], 120, 0.45)
    cs, oe = oracle.lookup_table(oracle.Query.blastp(q), 11)
    cells, overflow = smallbone_from_csr(cs, oe)
    gdb = hblast.Database(db.residues, db.offsets)
    pq = hblast.ProteinQuery.blastp(q)
    res = hblast.search(gdb, hblast.Batch.from_smallbone(pq, cells, overflow))
    check(res, [pq], db.residues, db.offsets)


@pytest.mark.parametrize("case", KNOWN_ANSWERS, ids=[c[0] for c in KNOWN_ANSWERS])
def test_hand_derived_cases(built, case):
    """The cases worked out by hand in test_oracle.py, on the GPU: the query's
    lookup table is the hand-made one (passed as an NCBI smallbone table) and
    the database is the case's one subject."""
    from test_host import smallbone_from_csr
    name, q, s, cells, xdrop, cutoff, rows, cnt = case
    cells_bb, overflow = smallbone_from_csr(*hand_lut(cells))
    sub = enc(s)
    gdb = hblast.Database(sub, np.array([0, len(sub)], np.int64))
    pq = hblast.ProteinQuery.blastp(enc(q), xdrop, cutoff)
    res = hblast.search(gdb, hblast.Batch.from_smallbone(pq, cells_bb, overflow))
    got = [tuple(int(h[f]) for f in ("q_start", "s_start", "q_off", "s_off", "len", "score", "context"))
           for h in res.hsps]
    st = res.stats[0]
    if rows is not None:
        assert got == rows, name
    for g, w in zip((st["lookup_hits"], st["init_extends"], st["good_init_extends"]), cnt):
        assert w is None or g == w, name
    gdb.close()


def test_launch_shapes_do_not_change_results(small_db):
    qs, db, gdb = small_db
    pqs = [hblast.ProteinQuery.blastp(q) for q in qs]
    batch = hblast.Batch.proteins(pqs)
    base = hblast.search(gdb, batch).hsps
    for threads, blocks in ((32, 1), (64, 7), (256, 1000)):
        o = hblast.default_options(num_threadsx=threads, num_blocksx=blocks)
        assert np.array_equal(hblast.search(gdb, batch, options=o).hsps, base), (threads, blocks)


def test_repeated_launches_replay_graph(small_db):
    """A reused result on a non-default stream replays a captured CUDA graph
    from its second launch on; every launch must give the same HSPs."""
    import torch
    qs, db, gdb = small_db
    batch = hblast.Batch.proteins([hblast.ProteinQuery.blastp(q) for q in qs])
    stream = torch.cuda.Stream()
    s = hblast.Searcher(gdb, batch)
    outs = []
    for _ in range(3):
        s.launch(stream.cuda_stream)
        s.wait()
        outs.append(s.result().hsps)
    s.close()
    ref = hblast.search(gdb, batch).hsps
    for o in outs:
        assert np.array_equal(o, ref)


def test_blastx_seg_masked(built):
    """BLASTX with SEG-masked frames (blastx's default query masking) against
    the oracle run on the same frames masked by the SEG restatement."""
    from seg_ref import seg as seg_ref
    rng = np.random.default_rng(16)
    prot_q = synth.random_letters(rng, 400)
    db = synth.make_db(rng, 600, 300, 0.6, 30, 5000, 30, [prot_q], 150, 0.6)
    nts = synth.blastx_queries(6, db, n_queries=3)
    nts[1][60:210] = np.tile(np.array([2, 1, 3], np.uint8), 50)     # a low-complexity (Ala) run
    xd = np.full((3, 6), 16, dtype=np.int32)
    cu = np.full((3, 6), 41, dtype=np.int32)
    gdb = hblast.Database(db.residues, db.offsets)
    res = hblast.search(gdb, hblast.Batch.blastx(nts, xd, cu, seg=True))
    pqs = []
    for k, nt in enumerate(nts):
        prot, off, ln = oracle.translate6(nt)
        for f in range(6):
            prot[off[f]:off[f] + ln[f]] = seg_ref(prot[off[f]:off[f] + ln[f]])
        pqs.append(hblast.ProteinQuery(prot, off, ln, xd[k], cu[k]))
    assert len(res.hsps) > 0
    check(res, pqs, db.residues, db.offsets)


@pytest.mark.parametrize("threshold,window", [(12, 40), (13, 40), (11, 20), (11, 60)])
def test_word_parameters(small_db, threshold, window):
    """Other neighbourhood thresholds and two-hit windows (-threshold,
    -window_size), against the oracle run with the same parameters."""
    qs, db, gdb = small_db
    pqs = [hblast.ProteinQuery.blastp(q) for q in qs]
    res = hblast.search(gdb, hblast.Batch.proteins(pqs, threshold=threshold, window=window))
    h = res.hsps
    assert len(h) > 0
    for k, pq in enumerate(pqs):
        ref, subj, cnt = oracle.search(oracle_query(pq), db.residues, db.offsets, threshold=threshold,
                                       window=window, nthreads=4)
        got = h[h["query"] == k]
        assert len(got) == len(ref), (k, threshold, window)
        assert np.array_equal(got["subject"], subj), k
        for f, g in (("q_start", "q_start"), ("s_start", "s_start"), ("q_off", "q_off"), ("s_off", "s_off"),
                     ("len", "len"), ("score", "score"), ("ctx", "context")):
            assert np.array_equal(got[g], ref[f]), (k, f)
        st = res.stats[k]
        assert (st["lookup_hits"], st["init_extends"], st["good_init_extends"]) == tuple(int(c) for c in cnt), k
