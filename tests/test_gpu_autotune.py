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
            assert len(r.rows) == len(autotune.DEFAULT_CANDIDATES) + len(autotune.STAGE2)
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
