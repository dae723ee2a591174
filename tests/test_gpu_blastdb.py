"""A database opened from NCBI BLAST files (hbg_db_open_blastdb) searches
exactly like the same sequences passed as arrays (hbg_db_open): same
counts, same HSPs bit for bit, for one volume, for an alias of many
volumes, and for a database larger than the 64 MiB staging pieces."""
import numpy as np
import pytest

import hblast
from hblast import blastdb, synth

pytestmark = pytest.mark.gpu


def compare(path, qs, db):
    a = hblast.Database(db.residues, db.offsets)
    b = hblast.Database.from_blastdb(path)
    assert a.info()[:2] == b.info()[:2]
    batch = hblast.Batch.proteins([hblast.ProteinQuery.blastp(q) for q in qs])
    ra, rb = hblast.search(a, batch), hblast.search(b, batch)
    assert len(ra.hsps) > 0
    assert np.array_equal(ra.hsps, rb.hsps)
    assert ra.stats == rb.stats
    a.close()
    b.close()


def test_single_volume_and_alias(built, tmp_path):
    rng = np.random.default_rng(61)
    qs = [synth.random_letters(rng, int(n)) for n in (90, 400, 1200)]
    db = synth.make_db(rng, 5000, 300, 0.6, 30, 5000, 0.05, qs, lambda r: r.integers(50, 301), 0.5)
    blastdb.write_volume(tmp_path / "one", db.residues, db.offsets)
    compare(tmp_path / "one", qs, db)
    names = blastdb.write(tmp_path / "many", db.residues, db.offsets, volume_residues=300_000)
    assert len(names) > 3
    compare(tmp_path / "many", qs, db)


def test_larger_than_staging_pieces(built, tmp_path):
    qs, db = synth.batched_blastp(seed=5, n_queries=4, n_subjects=450_000)
    assert db.offsets[-1] > 2 * (64 << 20)
    blastdb.write(tmp_path / "big", db.residues, db.offsets, volume_residues=100_000_000)
    compare(tmp_path / "big", qs, db)


def test_bad_database_is_an_error(built, tmp_path):
    with pytest.raises(hblast.HblastError, match="neither"):
        hblast.Database.from_blastdb(tmp_path / "absent")
