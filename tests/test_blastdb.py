"""NCBI BLAST database ingest (hbg_blastdb_info / hbg_blastdb_read, host only):
round trips through the format-4 writer, multi-volume aliases, and the
checks that reject damaged or unsupported files."""
import struct

import numpy as np
import pytest

import hblast
from hblast import blastdb, synth


def small_db(seed=3, n=300):
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 400, size=n)
    lens[:3] = (0, 1, 2)                      # empty and tiny sequences too
    off = np.zeros(n + 1, dtype=np.int64)
    off[1:] = np.cumsum(lens)
    res = synth.random_letters(rng, int(off[-1]))
    return res, off


def test_single_volume_round_trip(tmp_path):
    res, off = small_db()
    blastdb.write_volume(tmp_path / "one", res, off, title="one volume")
    info = hblast.blastdb_info(tmp_path / "one")
    assert info == dict(n_subjects=len(off) - 1, n_residues=int(off[-1]), max_len=int(np.diff(off).max()),
                        n_volumes=1)
    r2, o2 = hblast.blastdb_read(tmp_path / "one")
    assert np.array_equal(o2, off) and np.array_equal(r2, res)
    psq = (tmp_path / "one.psq").read_bytes()
    assert psq[0] == 0 and len(psq) == int(off[-1]) + len(off)      # leading 0 + one 0 per sequence


def test_alias_of_volumes_keeps_subject_order(tmp_path):
    res, off = small_db(n=500)
    names = blastdb.write(tmp_path / "db", res, off, volume_residues=20000)
    assert len(names) > 3
    info = hblast.blastdb_info(tmp_path / "db")
    assert info["n_volumes"] == len(names) and info["n_subjects"] == 500
    r2, o2 = hblast.blastdb_read(tmp_path / "db")
    assert np.array_equal(o2, off) and np.array_equal(r2, res)


def test_nested_alias_and_quoted_names(tmp_path):
    res, off = small_db(n=40)
    sub = tmp_path / "sub dir"
    sub.mkdir()
    blastdb.write_volume(sub / "a", res, off[:21])
    blastdb.write_volume(tmp_path / "b", res, off[20:])
    (sub / "inner.pal").write_text('DBLIST "a"\n')
    (tmp_path / "outer.pal").write_text('# two levels\nTITLE x\nDBLIST "sub dir/inner" b\n')
    r2, o2 = hblast.blastdb_read(tmp_path / "outer")
    assert np.array_equal(o2, off) and np.array_equal(r2, res)


def test_empty_database(tmp_path):
    blastdb.write_volume(tmp_path / "e", np.zeros(0, np.uint8), np.zeros(1, np.int64))
    assert hblast.blastdb_info(tmp_path / "e")["n_subjects"] == 0
    r2, o2 = hblast.blastdb_read(tmp_path / "e")
    assert len(r2) == 0 and list(o2) == [0]


def _rewrite(path, fn):
    b = bytearray(path.read_bytes())
    fn(b)
    path.write_bytes(bytes(b))


@pytest.mark.parametrize("damage, message", [
    ("version", "format version"),
    ("nucleotide", "not a protein database"),
    ("truncated_pin", "truncated"),
    ("short_psq", "bytes"),
    ("letter", "outside NCBIstdaa"),
    ("inner_zero", "0 byte inside"),
    ("separator", "not followed by a 0 byte"),
    ("total", "residue total"),
    ("longest", "longest"),
    ("missing", "missing"),
    ("subset", "not supported"),
    ("no_dblist", "no DBLIST"),
])
def test_damaged_files_are_rejected(tmp_path, damage, message):
    res, off = small_db(n=50)
    base = tmp_path / "d"
    blastdb.write_volume(base, res, off)
    pin, psq = tmp_path / "d.pin", tmp_path / "d.psq"
    title_end = 12                                # empty title
    date_len = struct.unpack(">I", pin.read_bytes()[title_end:title_end + 4])[0]
    n_at = title_end + 4 + date_len
    name = base
    k = int(np.flatnonzero(np.diff(off) > 0)[1])  # a non-empty sequence
    first = int(off[k]) + k + 1                   # .psq byte of its first letter
    if damage == "version":
        _rewrite(pin, lambda b: b.__setitem__(slice(0, 4), struct.pack(">I", 5)))
    elif damage == "nucleotide":
        _rewrite(pin, lambda b: b.__setitem__(slice(4, 8), struct.pack(">I", 0)))
    elif damage == "truncated_pin":
        _rewrite(pin, lambda b: b.__delitem__(slice(len(b) - 10, len(b))))
    elif damage == "short_psq":
        _rewrite(psq, lambda b: b.__delitem__(slice(len(b) - 1, len(b))))
    elif damage == "letter":
        _rewrite(psq, lambda b: b.__setitem__(first, 30))
    elif damage == "inner_zero":
        _rewrite(psq, lambda b: b.__setitem__(first, 0))
    elif damage == "separator":
        sep = int(off[k + 1]) + k + 1             # the 0 after it
        _rewrite(psq, lambda b: b.__setitem__(sep, 5))
    elif damage == "total":
        _rewrite(pin, lambda b: b.__setitem__(slice(n_at + 4, n_at + 12), struct.pack("<Q", 7)))
    elif damage == "longest":
        _rewrite(pin, lambda b: b.__setitem__(slice(n_at + 12, n_at + 16), struct.pack(">I", 1)))
    elif damage == "missing":
        psq.unlink()
    elif damage == "subset":
        (tmp_path / "s.pal").write_text("DBLIST d\nOIDLIST d.msk\n")
        name = tmp_path / "s"
    elif damage == "no_dblist":
        (tmp_path / "s.pal").write_text("TITLE nothing\n")
        name = tmp_path / "s"
    with pytest.raises(hblast.HblastError, match=message):
        hblast.blastdb_read(name)


def test_big_endian_total_is_accepted(tmp_path):
    res, off = small_db(n=20)
    blastdb.write_volume(tmp_path / "d", res, off)
    pin = tmp_path / "d.pin"
    b = bytearray(pin.read_bytes())
    n_at = 12 + 4 + len(blastdb.DATE)
    b[n_at + 4:n_at + 12] = struct.pack(">Q", int(off[-1]))
    pin.write_bytes(bytes(b))
    assert hblast.blastdb_info(tmp_path / "d")["n_residues"] == int(off[-1])
