"""Autotuner: every candidate setting gives the same HSPs, and searching bucket
by bucket with the tuned settings equals one plain search (bit-exact)."""
import numpy as np
import pytest

import hblast
from hblast import autotune, synth

pytestmark = pytest.mark.gpu


def test_tuned_search_equals_default(built, tmp_path):
    rng = np.random.default_rng(51)
    qs = synth.heavy_tailed_queries(3, 24)
    qs[0] = synth.random_letters(rng, 9000)           # a long query (16384-entry global table)
    db = synth.make_db(rng, 3000, 300, 0.6, 30, 5000, 0.05, qs, lambda r: r.integers(50, 301), 0.5)
    gdb = hblast.Database(db.residues, db.offsets)
    pqs = [hblast.ProteinQuery.blastp(q) for q in qs]
    table = autotune.tune(gdb, pqs, int(db.offsets[-1]), reps=1)
    assert any(r.best is not None for r in table)
    for r in table:
        if r.n_queries:
            n1 = len(autotune.DEFAULT_CANDIDATES)
            best1 = min(r.rows[:n1], key=lambda row: row[1])[0]
            n2 = sum(1 for kw in autotune.STAGE2 if kw.get("warps_per_subject", 1) * 32 <= best1["threads"])
            assert len(r.rows) == n1 + n2
            assert all(row[1] > 0 and row[2] > 0 for row in r.rows)
    path = tmp_path / "tuned.json"
    autotune.save(table, path)
    table = autotune.load(path)
    tuned = autotune.search_tuned(gdb, pqs, table)
    plain = hblast.search(gdb, hblast.Batch.proteins(pqs))
    assert np.array_equal(tuned.hsps, plain.hsps)
    assert tuned.stats == plain.stats


def test_tuning_knobs_keep_results(built):
    """Work-unit size and global diagonal tables (hbg_batch_tune) change no HSP."""
    rng = np.random.default_rng(53)
    qs = [synth.random_letters(rng, int(n)) for n in (80, 700, 2500, 9000)]
    db = synth.make_db(rng, 2500, 300, 0.6, 30, 5000, 0.05, qs, lambda r: r.integers(50, 301), 0.5)
    gdb = hblast.Database(db.residues, db.offsets)
    pqs = [hblast.ProteinQuery.blastp(q) for q in qs]
    ref = hblast.search(gdb, hblast.Batch.proteins(pqs))
    for tile, glob in ((8, False), (32, False), (4096, False), (0, True), (64, True)):
        r = hblast.search(gdb, hblast.Batch.proteins(pqs).tune(tile, glob))
        assert np.array_equal(r.hsps, ref.hsps), (tile, glob)
        assert r.stats == ref.stats
    with pytest.raises(hblast.HblastError):
        hblast.Batch.proteins(pqs).tune(5, False)


def test_schedule_knobs_keep_results(built):
    """Warps per subject (groups sharing each pass over a subject, up to one
    CTA) and work units sized in subject bytes change no HSP or counter."""
    rng = np.random.default_rng(57)
    qs = [synth.random_letters(rng, int(n)) for n in rng.integers(40, 1500, size=40)] + \
         [synth.random_letters(rng, 3000), synth.random_letters(rng, 40000 // 10)]
    db = synth.make_db(rng, 3000, 300, 0.6, 30, 5000, 0.05, qs, lambda r: r.integers(50, 301), 0.5)
    gdb = hblast.Database(db.residues, db.offsets)
    pqs = [hblast.ProteinQuery.blastp(q) for q in qs]
    for glen in (0, 2008):
        ref = hblast.search(gdb, hblast.Batch.proteins(pqs, max_group_len=glen))
        assert hblast.Batch.proteins(pqs, max_group_len=glen).info()["n_groups"] >= 5   # tiles of 3 groups leave a partial one
        for team, tb in ((2, 0), (3, 0), (8, 0), (1, 4096), (1, 65536), (8, 16384), (4, 1024)):
            r = hblast.search(gdb, hblast.Batch.proteins(pqs, max_group_len=glen).schedule(team, tb))
            assert np.array_equal(r.hsps, ref.hsps), (glen, team, tb)
            assert r.stats == ref.stats, (glen, team, tb)
    for bad in ((0, 0), (9, 0), (1, 100), (1, 1 << 25)):
        with pytest.raises(hblast.HblastError):
            hblast.Batch.proteins(pqs).schedule(*bad)
