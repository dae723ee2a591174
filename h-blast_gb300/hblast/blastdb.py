"""Writer for NCBI BLAST protein databases (format version 4), for building
test and benchmark databases without makeblastdb.

Writes what the reader (host/blastdb.cpp, hbg_blastdb_*) and a search need:
per volume a .pin index and a .psq sequence file, and a .pal alias listing
the volumes.  Deflines are not written: the .phr file is empty and every
header offset is 0, so these databases search but carry no titles per
sequence.  Layout (integers big-endian unless noted): u32 version 4, u32
type 1 (protein), u32 + bytes title, u32 + bytes date, u32 sequence count N,
8-byte residue total (little-endian, as NCBI writes it), u32 longest
sequence, u32 header offsets[N + 1], u32 sequence offsets[N + 1]; the .psq is
a 0 byte, then each sequence followed by a 0 byte.  H-BLAST parses the same
index fields in ExtractVolumeSequences (NF/functions.cpp:573-609) and the
alias DBLIST in ReadH_BLAST_volinfo (NF/functions.cpp:669-760).
"""
from __future__ import annotations

import os
import struct
from pathlib import Path

import numpy as np

DATE = b"Jan 1, 2026  12:00 AM"


def write_volume(base: str | os.PathLike, residues: np.ndarray, offsets: np.ndarray, title: str = "") -> None:
    """One volume: sequences i = residues[offsets[i]:offsets[i + 1]] (NCBIstdaa 1..27)."""
    base = str(base)
    res = np.ascontiguousarray(residues, dtype=np.uint8)
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    n = len(off) - 1
    lens = np.diff(off)
    if n < 0 or (lens < 0).any():
        raise ValueError("offsets must be non-decreasing")
    seq_off = np.empty(n + 1, dtype=np.int64)
    seq_off[0] = 1
    seq_off[1:] = 1 + np.cumsum(lens + 1)
    if seq_off[-1] >= 2 ** 32:
        raise ValueError("a format-4 volume holds less than 4 GiB; split the database into volumes")
    psq = np.zeros(int(seq_off[-1]), dtype=np.uint8)
    # letters of sequence i go to [seq_off[i], seq_off[i] + len_i); the byte after each stays 0
    dst = np.repeat(seq_off[:-1] - off[:-1], lens) + np.arange(int(off[-1] - off[0])) + off[0] \
        if n else np.zeros(0, dtype=np.int64)
    psq[dst] = res[off[0]:off[-1]]
    Path(base + ".psq").write_bytes(psq.tobytes())
    Path(base + ".phr").write_bytes(b"")
    t = title.encode()
    head = struct.pack(">II", 4, 1) + struct.pack(">I", len(t)) + t + struct.pack(">I", len(DATE)) + DATE
    head += struct.pack(">I", n) + struct.pack("<Q", int(lens.sum())) + struct.pack(">I", int(lens.max()) if n else 0)
    hdr = np.zeros(n + 1, dtype=">u4")
    Path(base + ".pin").write_bytes(head + hdr.tobytes() + seq_off.astype(">u4").tobytes())


def write_alias(path: str | os.PathLike, volumes: list[str], title: str = "") -> None:
    """A .pal naming the volumes (paths relative to the alias file's directory)."""
    lines = ["# alias file", f"TITLE {title}" if title else "TITLE", "DBLIST " + " ".join(volumes)]
    Path(str(path) + ".pal").write_text("\n".join(lines) + "\n")


def write(path: str | os.PathLike, residues: np.ndarray, offsets: np.ndarray, volume_residues: int = 1 << 30,
          title: str = "") -> list[str]:
    """Split a database into volumes of at most volume_residues letters (at least one sequence each),
    write them as path.00, path.01, ... and an alias path.pal; returns the volume names."""
    path = str(path)
    off = np.asarray(offsets, dtype=np.int64)
    n = len(off) - 1
    names, i, v = [], 0, 0
    while i < n or v == 0:
        j = i + 1 if i < n else i
        while j < n and off[j + 1] - off[i] <= volume_residues:
            j += 1
        name = f"{Path(path).name}.{v:02d}"
        write_volume(str(Path(path).parent / name), residues, off[i:j + 1], title)
        names.append(name)
        i, v = j, v + 1
    write_alias(path, names, title)
    return names
