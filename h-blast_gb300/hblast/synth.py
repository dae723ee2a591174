"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public benchmark dataset is used or stood in for.  Letters are NCBIstdaa
codes of the 20 standard amino acids drawn from background frequencies; the
Robinson & Robinson (1991) table is not available offline, so the background
used here is the one implied by the BLOSUM62 matrix itself: the unique
positive p with sum_j p_j exp(lambda s_ij) = 1 for every i and sum p = 1 (the
implied-frequency construction of Altschul 1991 / Yu & Altschul 2005), solved
numerically from the table in csrc/blosum62.inc.  Planted homologs use
BLOSUM62-conditional substitutions P(b|a) ~ p_b 2^(s(a,b)/2).

Sampling goes through a 65536-entry table (each letter owns round(p * 65536)
slots), so the distribution is the implied background quantised to 1/65536.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

LETTERS = "-ABCDEFGHIKLMNPQRSTVWXYZU*OJ"
STD20 = np.array([LETTERS.index(c) for c in "ARNDCQEGHILKMFPSTWYV"], dtype=np.uint8)
X_DROPOFF = 16      # 7-bit ungapped X-drop in raw BLOSUM62 units (NCBI blastp default)
CUTOFF = 41         # 22-bit gap trigger in raw BLOSUM62 units (NCBI blastp default)


def blosum62() -> np.ndarray:
    """28x28 int matrix parsed from csrc/blosum62.inc (rows = query letter)."""
    src = (Path(__file__).resolve().parent.parent / "csrc" / "blosum62.inc").read_text()
    rows = []
    for line in src.splitlines():
        if line.strip().startswith("/*") and "*/" in line:
            vals = line.split("*/", 1)[1].strip().rstrip(",")
            rows.append([int(v) for v in vals.split(",")][:28])
    m = np.array(rows, dtype=np.int32)
    assert m.shape == (28, 28)
    return m


def implied_background() -> tuple[np.ndarray, float]:
    """Background frequencies (over STD20) and lambda implied by BLOSUM62."""
    s = blosum62()[np.ix_(STD20, STD20)].astype(np.float64)

    def total(lam: float) -> float:
        return float(np.linalg.solve(np.exp(lam * s), np.ones(20)).sum() - 1.0)

    lo, hi = 0.2, 0.5          # total(lo) > 0 > total(hi)
    for _ in range(100):
        mid = 0.5 * (lo + hi)
        if total(mid) > 0:
            lo = mid
        else:
            hi = mid
    lam = 0.5 * (lo + hi)
    p = np.linalg.solve(np.exp(lam * s), np.ones(20))
    p = np.clip(p, 1e-9, None)
    return p / p.sum(), lam


_BG = None


def _tables():
    global _BG
    if _BG is None:
        p, lam = implied_background()
        slots = np.floor(p * 65536).astype(np.int64)
        slots[np.argmax(slots)] += 65536 - slots.sum()
        table = np.repeat(STD20, slots).astype(np.uint8)
        # conditional substitution P(b|a) ~ p_b 2^(s(a,b)/2), b != a
        s = blosum62()[np.ix_(STD20, STD20)].astype(np.float64)
        cond = p[None, :] * np.power(2.0, s / 2.0)
        np.fill_diagonal(cond, 0.0)
        cond /= cond.sum(axis=1, keepdims=True)
        cdf = np.cumsum(cond, axis=1)
        idx = np.full(28, -1, dtype=np.int64)
        idx[STD20] = np.arange(20)
        _BG = (p, lam, table, cdf, idx)
    return _BG


def random_letters(rng: np.random.Generator, n: int) -> np.ndarray:
    table = _tables()[2]
    out = np.empty(n, dtype=np.uint8)
    step = 1 << 26
    for i in range(0, n, step):
        k = min(step, n - i)
        out[i:i + k] = table[rng.integers(0, 65536, size=k, dtype=np.uint16)]
    return out


def mutate(rng: np.random.Generator, seq: np.ndarray, identity: float) -> np.ndarray:
    """Keep each letter with probability `identity`, else substitute b != a by P(b|a)."""
    _, _, _, cdf, idx = _tables()
    seq = np.asarray(seq, dtype=np.uint8)
    out = seq.copy()
    change = rng.random(len(seq)) >= identity
    pos = np.nonzero(change)[0]
    if len(pos):
        a = idx[seq[pos]]
        ok = a >= 0
        pos, a = pos[ok], a[ok]
        u = rng.random(len(pos))
        b = (u[:, None] > cdf[a]).sum(axis=1)
        out[pos] = STD20[np.minimum(b, 19)]
    return out


def lognormal_lengths(rng, n, median, sigma, lo, hi) -> np.ndarray:
    return np.clip(np.rint(np.exp(rng.normal(np.log(median), sigma, n))), lo, hi).astype(np.int64)


@dataclass
class ProteinDB:
    residues: np.ndarray          # uint8, subjects back to back
    offsets: np.ndarray           # int64, n+1
    planted: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))

    @property
    def n(self) -> int:
        return len(self.offsets) - 1

    @property
    def lengths(self) -> np.ndarray:
        return np.diff(self.offsets)

    def subject(self, i: int) -> np.ndarray:
        return self.residues[self.offsets[i]:self.offsets[i + 1]]

    def slice(self, lo: int, hi: int) -> "ProteinDB":
        off = self.offsets[lo:hi + 1]
        res = self.residues[off[0]:off[-1]]
        return ProteinDB(res, off - off[0])


def make_db(rng, n_subjects, median, sigma, lo, hi, planted_frac, donors, seg_len, identity) -> ProteinDB:
    """Subjects of lognormal length; a fraction carry a mutated segment of a donor."""
    lens = lognormal_lengths(rng, n_subjects, median, sigma, lo, hi)
    offsets = np.zeros(n_subjects + 1, dtype=np.int64)
    np.cumsum(lens, out=offsets[1:])
    residues = random_letters(rng, int(offsets[-1]))
    n_plant = int(round(planted_frac * n_subjects)) if planted_frac < 1 else int(planted_frac)
    planted = np.sort(rng.choice(n_subjects, size=min(n_plant, n_subjects), replace=False))
    for j in planted:
        d = donors[rng.integers(len(donors))]
        L = int(seg_len(rng)) if callable(seg_len) else int(seg_len)
        L = min(L, len(d), int(lens[j]))
        if L < 3:
            continue
        a = rng.integers(0, len(d) - L + 1)
        ident = identity(rng) if callable(identity) else identity
        seg = mutate(rng, d[a:a + L], ident)
        b = rng.integers(0, lens[j] - L + 1)
        residues[offsets[j] + b: offsets[j] + b + L] = seg
    return ProteinDB(residues, offsets, planted)


# ---------------------------------------------------------------- workloads

def plain_blastp(seed: int = 0, n_subjects: int = 20000):
    """1 query of 300 aa vs 20,000 lognormal subjects, 50 planted 120-aa segments at 40% identity."""
    rng = np.random.default_rng(seed)
    q = random_letters(rng, 300)
    db = make_db(rng, n_subjects, 300, 0.6, 30, 5000, 50 if n_subjects >= 50 else n_subjects, [q], 120, 0.40)
    return [q], db


def batched_queries(rng, n, lo=50, hi=1500):
    return [random_letters(rng, int(L)) for L in rng.integers(lo, hi + 1, size=n)]


def batched_blastp(seed: int = 0, n_queries: int = 64, n_subjects: int = 2_000_000):
    """64 queries of 50..1500 aa vs 2M lognormal subjects, 1% planted 50..300 aa at 30..60%."""
    rng = np.random.default_rng(seed)
    qs = batched_queries(rng, n_queries)
    db = make_db(rng, n_subjects, 300, 0.6, 30, 5000, 0.01, qs,
                 lambda r: r.integers(50, 301), lambda r: r.uniform(0.30, 0.60))
    return qs, db


_CODONS = None


def _codon_table():
    global _CODONS
    if _CODONS is None:
        code = "FFLLSSSSYY**CC*WLLLLPPPPHHQQRRRRIIIMTTTTNNKKSSRRVVVVAAAADDEEGGGG"
        tcag_to_acgt = {0: 3, 1: 1, 2: 0, 3: 2}   # T C A G -> A=0 C=1 G=2 T=3
        by_aa = {}
        for i, aa in enumerate(code):
            cod = (tcag_to_acgt[i // 16], tcag_to_acgt[(i // 4) % 4], tcag_to_acgt[i % 4])
            by_aa.setdefault(LETTERS.index(aa), []).append(cod)
        _CODONS = by_aa
    return _CODONS


def back_translate(rng, prot: np.ndarray) -> np.ndarray:
    tab = _codon_table()
    out = np.empty(3 * len(prot), dtype=np.uint8)
    for i, a in enumerate(prot):
        choices = tab[int(a)]
        out[3 * i:3 * i + 3] = choices[rng.integers(len(choices))]
    return out


def blastx_queries(seed: int, db: ProteinDB, n_queries: int = 128):
    """Nucleotide queries of 300..3000 nt (GC 0.5), each with a planted ORF of 200..900 nt
    whose translation matches a database protein segment at 40..70% identity."""
    rng = np.random.default_rng(seed + 1)
    out = []
    for _ in range(n_queries):
        L = int(rng.integers(300, 3001))
        nt = rng.integers(0, 4, size=L, dtype=np.uint8)
        orf = int(rng.integers(200, 901)) // 3
        orf = min(orf, (L - 3) // 3)
        for _try in range(100):
            j = int(rng.integers(db.n))
            s = db.subject(j)
            if len(s) >= orf:
                break
        a = int(rng.integers(0, len(s) - orf + 1))
        prot = mutate(rng, s[a:a + orf], rng.uniform(0.40, 0.70))
        cod = back_translate(rng, prot)
        if rng.random() < 0.5:      # plant on the minus strand half of the time
            cod = (3 - cod[::-1]).astype(np.uint8)
        b = int(rng.integers(0, L - len(cod) + 1))
        nt[b:b + len(cod)] = cod
        out.append(nt)
    return out


def heavy_tailed_queries(seed: int, n: int):
    """Queries with lognormal lengths (median 350, sigma 1.0, clipped to 30..35,000)."""
    rng = np.random.default_rng(seed + 7)
    lens = lognormal_lengths(rng, n, 350, 1.0, 30, 35000)
    return [random_letters(rng, int(L)) for L in lens]


def large_db(seed: int = 0, n_subjects: int = 10_000_000, donors=None):
    """The 10,000,000-subject database of the heavy-tailed and served workloads (lognormal
    lengths, median 300, sigma 0.6, 30..5000; 1% carry a 50..300 aa segment of a donor at
    30..60% identity; donors default to one random 400-aa protein)."""
    rng = np.random.default_rng(seed)
    if not donors:
        donors = [random_letters(rng, 400)]
    return make_db(rng, n_subjects, 300, 0.6, 30, 5000, 0.01, list(donors),
                   lambda r: r.integers(50, 301), lambda r: r.uniform(0.3, 0.6))

