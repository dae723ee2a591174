"""The H-BLASTM-style front end, host side: FASTA reading, letter encoding,
option checks that need no GPU."""
import numpy as np
import pytest

from hblast import hblastm
from hblast.synth import LETTERS


def test_read_fasta(tmp_path):
    f = tmp_path / "q.fasta"
    f.write_text(">sp|P1| first protein\nMKV\nLLA\n\n>second\n  acde \n>\n")
    assert hblastm.read_fasta(f) == [("sp|P1|", "MKVLLA"), ("second", "acde"), ("query_3", "")]
    bad = tmp_path / "bad.fasta"
    bad.write_text("MKV\n>x\nA\n")
    with pytest.raises(ValueError, match="before the first"):
        hblastm.read_fasta(bad)


def test_encoding():
    assert list(hblastm.encode_protein("ARNDcq*U")) == [LETTERS.index(c) for c in "ARNDCQ*U"]
    with pytest.raises(ValueError, match="amino-acid"):
        hblastm.encode_protein("AR1")
    with pytest.raises(ValueError, match="amino-acid"):
        hblastm.encode_protein("A-R")
    assert list(hblastm.encode_nucleotide("ACGTUacgtN")) == [0, 1, 2, 3, 3, 0, 1, 2, 3, 4]
    with pytest.raises(ValueError, match="nucleotide"):
        hblastm.encode_nucleotide("ACGZ")


def test_no_cpu_path_and_card_checks(tmp_path, built):
    q = tmp_path / "q.fasta"
    q.write_text(">a\nMKV\n")
    log = tmp_path / "log"
    assert hblastm.main(["-query", str(q), "-db", "x", "-gpu", "F", "-screen_out", str(log)]) == 2
    assert "no CPU path" in log.read_text()
    assert hblastm.main(["-query", str(q), "-db", "x", "-gpu_cards", "64", "-screen_out", str(log)]) == 2
    assert "visible GPU" in log.read_text()


def test_seg_option():
    a = hblastm.parse(["-query", "q", "-db", "d", "-module", "blastx"])
    assert a.seg is None                       # blastx default: masked (resolved to yes)
    assert hblastm.parse(["-query", "q", "-db", "d", "-seg", "no"]).seg == "no"
    with pytest.raises(SystemExit):
        hblastm.parse(["-query", "q", "-db", "d", "-seg", "maybe"])
