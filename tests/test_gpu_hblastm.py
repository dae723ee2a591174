"""The H-BLASTM-style front end end to end: FASTA queries against a BLAST
database on disk through the serving loop; every output line equals the
HSPs of a direct search of that query (bit-exact)."""
import numpy as np
import pytest

import hblast
from hblast import blastdb, hblastm, synth
from hblast.synth import LETTERS
from oracle import oracle

pytestmark = pytest.mark.gpu


def lines_of(name, hsps):
    return [f"{name}\t{h['subject']}\t{h['context']}\t{h['q_start']}\t{h['s_start']}\t{h['len']}\t{h['score']}\t"
            f"{h['q_off']}\t{h['s_off']}" for h in hsps]


def test_blastp_and_blastx_files(built, tmp_path):
    rng = np.random.default_rng(71)
    qs = [synth.random_letters(rng, int(n)) for n in (60, 300, 900)]
    db = synth.make_db(rng, 3000, 300, 0.6, 30, 5000, 0.05, qs, lambda r: r.integers(50, 301), 0.5)
    blastdb.write(tmp_path / "db", db.residues, db.offsets, volume_residues=200_000)
    gdb = hblast.Database(db.residues, db.offsets)

    fa = tmp_path / "p.fasta"
    fa.write_text("".join(f">p{i} protein {i}\n" + "".join(LETTERS[c] for c in q) + "\n" for i, q in enumerate(qs)))
    out = tmp_path / "p.tsv"
    assert hblastm.main(["-module", "blastp", "-query", str(fa), "-db", str(tmp_path / "db"), "-out", str(out),
                         "-screen_out", str(tmp_path / "p.log")]) == 0
    want = []
    for i, q in enumerate(qs):
        want += lines_of(f"p{i}", hblast.search(gdb, hblast.Batch.proteins([hblast.ProteinQuery.blastp(q)])).hsps)
    got = out.read_text().splitlines()
    assert len(got) > 0 and got == want

    nts = synth.blastx_queries(5, db, n_queries=3)
    fx = tmp_path / "x.fasta"
    fx.write_text("".join(f">x{i}\n" + "".join("ACGT"[c] for c in nt) + "\n" for i, nt in enumerate(nts)))
    x6, c6 = np.full(6, 16, np.int32), np.full(6, 41, np.int32)
    # blastx masks its frames with SEG by default, as NCBI blastx does; -seg no searches them as they are
    for seg in ("default", "no"):
        outx = tmp_path / f"x_{seg}.tsv"
        args = ["-module", "blastx", "-query", str(fx), "-db", str(tmp_path / "db"), "-out", str(outx),
                "-screen_out", str(tmp_path / "x.log")] + ([] if seg == "default" else ["-seg", "no"])
        assert hblastm.main(args) == 0
        want = []
        for i, nt in enumerate(nts):
            prot, off, ln = oracle.translate6(nt)
            if seg == "default":
                for f in range(6):
                    prot[off[f]:off[f] + ln[f]] = hblast.seg_mask(prot[off[f]:off[f] + ln[f]])
            pq = hblast.ProteinQuery(prot, off, ln, x6, c6)
            want += lines_of(f"x{i}", hblast.search(gdb, hblast.Batch.proteins([pq])).hsps)
        assert len(want) > 0 and outx.read_text().splitlines() == want, seg
