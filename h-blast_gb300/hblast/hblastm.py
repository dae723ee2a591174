"""Command-line front end with H-BLASTM's options (scripts/H-BLASTM:15-39,
options of NCBI blastp/blastx plus -module, -gpu_cards, -screen_out).

H-BLASTM splits the query file across one H-BLAST process per GPU card
(scripts/H-BLASTM:212-305) and each process balances subjects between its
CPU threads and its card (NF/functions.cpp:51-140).  Here every card holds
the whole database resident and runs the continuous-batching server
(hbg_server_*); queries go to the cards round-robin in file order and each
card batches what it has waiting.  The output is the word-hit stage's
product -- ungapped HSPs, one tab-separated line each -- because the gapped
stage that turns them into reports is NCBI code outside this library:

    query_id  subject_oid  context  q_start  s_start  length  score  q_off  s_off

(query_id = the first word of the FASTA title; for blastx, context 0..5 is
the frame in NCBI order +1 +2 +3 -1 -2 -3 and offsets are in that frame's
translation).  Lines come in query order, then in the order the CPU word
finder would create them.

    python -m hblast.hblastm -module blastp -query q.fasta -db nr -out hits.tsv
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

from . import core
from .synth import LETTERS

_AA = np.full(256, 255, dtype=np.uint8)
for _i, _c in enumerate(LETTERS):
    _AA[ord(_c)] = _i
    _AA[ord(_c.lower())] = _i
_AA[ord("-")] = 255                                   # a gap letter in a query is an error
_NT = np.full(256, 255, dtype=np.uint8)
for _c, _v in zip("ACGT", range(4)):
    _NT[ord(_c)] = _v
    _NT[ord(_c.lower())] = _v
for _c in "NnRrYyKkMmSsWwBbDdHhVvUu":
    _NT[ord(_c)] = 4 if _c not in "Uu" else 3         # ambiguity codes translate to X; U reads as T


def read_fasta(path: str | Path) -> list[tuple[str, str]]:
    """(id, letters) per record; the id is the first word of the title line."""
    out, name, seq = [], None, []
    for line in Path(path).read_text().splitlines():
        line = line.strip()
        if not line:
            continue
        if line.startswith(">"):
            if name is not None:
                out.append((name, "".join(seq)))
            words = line[1:].split()
            name, seq = (words[0] if words else f"query_{len(out) + 1}"), []
        elif name is None:
            raise ValueError(f"{path}: sequence data before the first '>' title line")
        else:
            seq.append(line.replace(" ", ""))
    if name is not None:
        out.append((name, "".join(seq)))
    return out


def encode_protein(s: str) -> np.ndarray:
    a = _AA[np.frombuffer(s.encode("latin-1"), dtype=np.uint8)]
    if (a == 255).any() or (a == 0).any():
        bad = s[int(np.flatnonzero((a == 255) | (a == 0))[0])]
        raise ValueError(f"letter {bad!r} is not an amino-acid code")
    return a


def encode_nucleotide(s: str) -> np.ndarray:
    a = _NT[np.frombuffer(s.encode("latin-1"), dtype=np.uint8)]
    if (a == 255).any():
        bad = s[int(np.flatnonzero(a == 255)[0])]
        raise ValueError(f"letter {bad!r} is not a nucleotide code")
    return a


def parse(argv=None):
    p = argparse.ArgumentParser(prog="hblastm", description=__doc__.split("\n\n")[0])
    p.add_argument("-module", default="blastp", choices=["blastp", "blastx"])
    p.add_argument("-query", required=True)
    p.add_argument("-db", required=True, help="BLAST database name (.pal alias or .pin/.psq volume)")
    p.add_argument("-out", default="-")
    p.add_argument("-gpu_cards", type=int, default=1)
    p.add_argument("-num_threads", type=int, default=1, help="accepted for compatibility (host threads)")
    p.add_argument("-screen_out", default=None, help="file for progress and error messages")
    p.add_argument("-gpu", default="T", choices=["T", "F"])
    p.add_argument("-gpu_threads", type=int, default=256)
    p.add_argument("-gpu_blocks", type=int, default=0)
    p.add_argument("-method", type=int, default=0, help="first GPU to use")
    p.add_argument("-threshold", type=int, default=11)
    p.add_argument("-window_size", type=int, default=40)
    p.add_argument("-xdrop_ungap_raw", type=int, default=16, help="ungapped X-drop in raw score units")
    p.add_argument("-cutoff_raw", type=int, default=41, help="ungapped cutoff score in raw units")
    p.add_argument("-max_batch_letters", type=int, default=8192)
    p.add_argument("-seg", default=None, choices=["yes", "no"],
                   help="SEG masking of BLASTX query frames (blastx default: yes; blastp queries are not masked)")
    return p.parse_args(argv)


def main(argv=None) -> int:
    a = parse(argv)
    log = open(a.screen_out, "w") if a.screen_out else sys.stderr
    try:
        if a.gpu == "F":
            print("hblastm: this library has no CPU path; -gpu F is not supported", file=log)
            return 2
        ndev = core.device_count()
        if a.gpu_cards < 1 or a.method < 0 or a.method + a.gpu_cards > ndev:
            print(f"hblastm: -gpu_cards {a.gpu_cards} from -method {a.method} needs more than the {ndev} "
                  "visible GPU(s)", file=log)
            return 2
        records = read_fasta(a.query)
        xd, cu = a.xdrop_ungap_raw, a.cutoff_raw
        queries = []
        for name, s in records:
            if a.module == "blastp":
                queries.append((name, core.ProteinQuery.blastp(encode_protein(s), xd, cu)))
            else:
                queries.append((name, encode_nucleotide(s)))
        cards = []
        for k in range(a.gpu_cards):
            opt = core.default_options(method=a.method + k, num_threadsx=a.gpu_threads, num_blocksx=a.gpu_blocks)
            db = core.Database.from_blastdb(a.db, opt)
            seg = a.module == "blastx" and (a.seg or "yes") == "yes"
            cards.append((db, core.Server(db, a.threshold, a.window_size, opt,
                                          max_batch_letters=a.max_batch_letters, seg_blastx=int(seg))))
        info = cards[0][0].info()
        print(f"hblastm: {a.module}, {len(queries)} queries, database {a.db}: {info[0]} sequences, "
              f"{info[1]} letters, {a.gpu_cards} card(s)", file=log)
        x6, c6 = np.full(6, xd, np.int32), np.full(6, cu, np.int32)
        tickets = []
        for i, (name, q) in enumerate(queries):
            srv = cards[i % len(cards)][1]
            tickets.append(srv.submit(q) if a.module == "blastp" else srv.submit_blastx(q, x6, c6))
        out = sys.stdout if a.out == "-" else open(a.out, "w")
        n_hsps = 0
        try:
            for i, ((name, _), t) in enumerate(zip(queries, tickets)):
                hsps, stats, ms = cards[i % len(cards)][1].take(t)
                for h in hsps:
                    out.write(f"{name}\t{h['subject']}\t{h['context']}\t{h['q_start']}\t{h['s_start']}\t"
                              f"{h['len']}\t{h['score']}\t{h['q_off']}\t{h['s_off']}\n")
                n_hsps += len(hsps)
                print(f"hblastm: {name}: {len(hsps)} HSPs, {stats['lookup_hits']} word hits, "
                      f"{ms:.1f} ms", file=log)
        finally:
            if out is not sys.stdout:
                out.close()
        for db, srv in cards:
            srv.close()
            db.close()
        print(f"hblastm: done, {n_hsps} HSPs", file=log)
        return 0
    except (ValueError, OSError, core.HblastError) as e:
        print(f"hblastm: error: {e}", file=log)
        return 1
    finally:
        if log is not sys.stderr:
            log.close()


if __name__ == "__main__":
    sys.exit(main())
