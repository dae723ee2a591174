"""The CPU oracle against the reference's tables and hand-derived known answers.

The reference ships no golden vectors for this path, so the oracle is pinned
by (1) the BLOSUM62 table and constants extracted from the H-BLAST sources
(tests/golden/reference_tables.json, made by tests/golden/make_golden.py) and
(2) cases whose expected HSPs are worked out by hand below from the published
NCBI two-hit algorithm (H-BLAST restates it at h_blast_kernel.cu:672-871 and
1069-1540).
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle

GOLD = json.loads((Path(__file__).parent / "golden" / "reference_tables.json").read_text())
L = "-ABCDEFGHIKLMNPQRSTVWXYZU*OJ"


def enc(s: str) -> np.ndarray:
    return np.array([L.index(c) for c in s], dtype=np.uint8)


def hand_lut(cells: dict):
    """CSR lookup table from {word string: [query offsets]}."""
    cs = np.zeros(oracle.NCELLS + 1, dtype=np.int32)
    items = {}
    for w, offs in cells.items():
        a, b, c = enc(w)
        items[(int(a) << 10) | (int(b) << 5) | int(c)] = sorted(offs)
    ent = []
    for i in range(oracle.NCELLS):
        cs[i] = len(ent)
        ent += items.get(i, [])
    cs[oracle.NCELLS] = len(ent)
    return cs, np.array(ent or [0], dtype=np.int32)[:len(ent)]


def run(q: str, s: str, cells: dict, xdrop=16, cutoff=30):
    query = oracle.Query.blastp(enc(q), xdrop, cutoff)
    sub = enc(s)
    off = np.array([0, len(sub)], dtype=np.int64)
    h, subj, cnt = oracle.search(query, sub, off, lut=hand_lut(cells))
    rows = [tuple(int(x) for x in r) for r in h]
    return rows, [int(c) for c in cnt]


def window_case(D):
    """Hits (0,0) and (D,D) on diagonal 0 of W-runs in G/P backgrounds."""
    if D < 3:
        return "W" * (D + 3) + "G" * 10, "W" * (D + 3) + "P" * 10
    return "WWW" + "G" * (D - 3) + "WWW" + "G" * 10, "WWW" + "P" * (D - 3) + "WWW" + "P" * 10


# The hand-derived cases of the tests below as one table, so that the GPU
# tests can run the same cases with the same hand-made lookup tables:
# (name, query, subject, cells, X-drop, cutoff, HSP rows, [lookup hits,
# extensions, kept]); None where the answer is not worked out by hand.
KNOWN_ANSWERS = [
    ("runs", "A" * 10, "A" * 10, {"AAA": [0, 5]}, 16, 30,
     [(0, 0, 5, 5, 10, 40, 0), (0, 1, 5, 6, 9, 36, 0), (0, 2, 5, 7, 8, 32, 0)], [16, 3, 3]),
    ("three_apart", "W" * 6 + "G" * 10, "W" * 6 + "P" * 10, {"WWW": [0, 3]}, 16, 41,
     [(0, 0, 3, 3, 6, 66, 0)], [8, 1, 1]),
    ("flag", "W" * 6 + "G" * 10, "W" * 6 + "PPEHKPQRTP", {"WWW": [0, 3], "EHK": [8], "QRT": [12]}, 16, 41,
     [(0, 0, 3, 3, 6, 66, 0)], [10, 1, 1]),
    ("xdrop_recovers", "WWW" + "G" * 7 + "WWW", "WWW" + "P" * 7 + "WWW", {"WWW": [0, 10]}, 16, 41,
     [(0, 0, 10, 10, 13, 52, 0)], [4, 1, 1]),
    ("xdrop_stops", "WWW" + "G" * 8 + "WWW", "WWW" + "P" * 8 + "WWW", {"WWW": [0, 11]}, 16, 41, [], [4, 1, 0]),
    ("right_walk_zero", "GGGAAA" + "G" * 10, "PPPAAAPPPPKKKRRR",
     {"PPP": [0], "AAA": [3], "KKK": [10], "RRR": [13]}, 16, 10, [(3, 3, 3, 3, 3, 12, 0)], [6, 2, 1]),
] + [("window_%d" % D, *window_case(D), {"WWW": [0, D]}, 16, 41, [] if D == 39 else None,
      [None, int(3 <= D < 40), 0 if D == 39 else None]) for D in (2, 3, 39, 40, 41)]


def test_known_answer_table(built):
    for name, q, s, cells, xdrop, cutoff, rows, cnt in KNOWN_ANSWERS:
        got_rows, got_cnt = run(q, s, cells, xdrop, cutoff)
        if rows is not None:
            assert got_rows == rows, name
        for g, w in zip(got_cnt, cnt):
            assert w is None or g == w, name


def test_matrix_matches_reference(built):
    m = np.array(GOLD["blosum62_ncbistdaa_28x32"])
    for a in range(28):
        for b in range(28):
            assert oracle.score(a, b) == m[a, b], (a, b)
    assert (m[:, 28:] == -128).all()
    assert (m[0] == -128).all() and (m[:, 0] == -128).all()


def test_product_matrix_matches_reference(built):
    from hblast import synth
    m = np.array(GOLD["blosum62_ncbistdaa_28x32"])
    assert np.array_equal(synth.blosum62(), m[:, :28])
    assert (m[:28, :28] == m[:28, :28].T).all()   # symmetric: [q][s] and [s][q] agree


def test_reference_constants():
    assert GOLD["charsize"] == 5            # 5 bits per letter -> 32768 cells
    assert GOLD["aa_hits_per_cell"] == 3    # smallbone cells hold 3 offsets inline


def test_two_hits_on_runs(built):
    # Q = S = A x 10 (A/A = 4); cell AAA = {0, 5}.  Diagonals 0, -1, -2 get a
    # second hit at s = 5, 6, 7 (diff 5).  At s=5: word end q_r = s_r = 8,
    # left walk over 8 letters scores 32 (left_d 8 >= 8-3), right walk 2 more
    # letters -> len 10, score 40.  At s=6: q_r=8, s_r=9, left 8 letters (32),
    # right 1 letter -> s_start 1, len 9, score 36.  At s=7: s_r=10 = end,
    # left 8 letters, no right letters -> s_start 2, len 8, score 32.
    rows, cnt = run("A" * 10, "A" * 10, {"AAA": [0, 5]})
    assert rows == [(0, 0, 5, 5, 10, 40, 0), (0, 1, 5, 6, 9, 36, 0), (0, 2, 5, 7, 8, 32, 0)]
    assert cnt == [16, 3, 3]


@pytest.mark.parametrize("D,extended", [(2, 0), (3, 1), (39, 1), (40, 0), (41, 0)])
def test_window_boundaries(built, D, extended):
    # Hits (0,0) and (D,D) on diagonal 0: extend only when 3 <= D < 40.
    q, s = window_case(D)
    rows, cnt = run(q, s, {"WWW": [0, D]}, cutoff=41)
    assert cnt[1] == extended
    if D == 39:
        # word at 39..41 scores 33 (right_d 3); the left walk keeps only
        # those three letters (G/P = -2 drops 16 after 8 letters), so
        # left_d 3 < 42 - 3: no right walk; score 33 < 41 -> not kept.
        assert rows == [] and cnt[2] == 0


def test_three_apart_extends_and_sets_flag(built):
    # Q = W x 6 + G x 10, S = W x 6 + P x 10, cell WWW = {0, 3}: diagonal 0
    # has hits at s=0 and s=3 (diff 3).  q_r = s_r = 6, left walk 6 W/W = 66,
    # right walk: G/P = -2 per letter, stops after 8 letters (drop 16) with
    # no gain -> HSP (0, 0, len 6, score 66).
    rows, cnt = run("W" * 6 + "G" * 10, "W" * 6 + "P" * 10, {"WWW": [0, 3]}, cutoff=41)
    assert rows == [(0, 0, 3, 3, 6, 66, 0)]
    assert cnt == [8, 1, 1]


@pytest.mark.parametrize("g", [7, 8])
def test_xdrop_recovery_and_stop(built, g):
    # Q = WWW G^g WWW, S = WWW P^g WWW, cell WWW = {0, g+3}: diagonal 0 has
    # hits at s=0 and s=g+3.  Word W/W x 3 = 33, right_d 3, s_r = q_r = g+6.
    # The left walk keeps 33 over the word, then loses 2 per G/P letter.
    # g=7: the drop reaches 14 < 16, the walk goes on and recovers to
    # 33 - 14 + 33 = 52 over all g+6 = 13 letters (it reaches the first hit,
    # and the right walk has no letters left) -> HSP (0, 0, len 13, score 52).
    # g=8: the eighth G/P letter makes the drop 16 (>= X-drop): the walk stops
    # with 33 over 3 letters, short of the first hit, so no right walk; 33 < 41
    # is not kept.
    q = "WWW" + "G" * g + "WWW"
    s = "WWW" + "P" * g + "WWW"
    rows, cnt = run(q, s, {"WWW": [0, g + 3]}, cutoff=41)
    if g == 7:
        assert rows == [(0, 0, 10, 10, 13, 52, 0)] and cnt == [4, 1, 1]
    else:
        assert rows == [] and cnt == [4, 1, 0]


def test_right_walk_stops_at_zero(built):
    # Q = GGG AAA G^10, S = PPP AAA PPPP KKK RRR; the hand table maps PPP->0,
    # AAA->3, KKK->10, RRR->13 (whatever the query holds there).  Diagonal 0:
    # hits at s=0 and s=3 (diff 3): word A/A x 3 = 12, s_r = 6; the left walk
    # keeps those 3 letters (G/P = -2 before them) and reaches the first hit's
    # end (3), so the right walk starts at 12 and loses 2 per letter (P/G, K/G):
    # it stops at score 0 on its sixth letter (s_last_off 11; the X-drop of 16
    # would only stop it two letters later), HSP (3, 3, len 3, score 12), and
    # the diagonal is flagged up to 9.  So KKK at s=10 resets the diagonal and
    # RRR at s=13 (diff 3) tries a second extension (R/G and K/G all -2:
    # score 0, not kept).  With the walk stopped by the X-drop instead, the
    # flag would reach 11, KKK would be skipped and RRR would only reset.
    rows, cnt = run("GGGAAA" + "G" * 10, "PPPAAAPPPPKKKRRR",
                    {"PPP": [0], "AAA": [3], "KKK": [10], "RRR": [13]}, cutoff=10)
    assert rows == [(3, 3, 3, 3, 3, 12, 0)]
    assert cnt == [6, 2, 1]


def test_flag_suppresses_hits_inside_extension(built):
    # Same extension as above (every letter of S[6..15] scores -2 against G),
    # so the right walk ends at s_last_off = 13 and diagonal 0 is flagged with
    # last = 11.  The only other hits are EHK at q=s=8 (inside the extended
    # region: skipped; without the flag it would be a second extension at
    # diff 5) and QRT at q=s=12 (>= 11: resets the diagonal, no extension).
    q = "W" * 6 + "G" * 10
    s = "W" * 6 + "PPEHKPQRTP"
    rows, cnt = run(q, s, {"WWW": [0, 3], "EHK": [8], "QRT": [12]}, cutoff=41)
    assert rows == [(0, 0, 3, 3, 6, 66, 0)]
    assert cnt == [10, 1, 1]


def test_translation_known_codons(built):
    # ATG GCC TAA -> M A *; the reverse complement TTA GGC CAT -> L G H.
    nt = np.array([0, 3, 2, 2, 1, 1, 3, 0, 0], dtype=np.uint8)   # A T G G C C T A A
    prot, off, ln = oracle.translate6(nt)
    frames = [prot[o:o + n] for o, n in zip(off, ln)]
    assert list(ln) == [3, 2, 2, 3, 2, 2]
    assert "".join(L[x] for x in frames[0]) == "MA*"
    assert "".join(L[x] for x in frames[3]) == "LGH"
    assert all(prot[o - 1] == 0 for o in off[1:])   # one sentinel between frames


def test_lookup_table_rule(built):
    rng = np.random.default_rng(3)
    q = rng.integers(1, 23, size=40).astype(np.uint8)
    cs, ent = oracle.lookup_table(oracle.Query.blastp(q), 11)
    m = np.array(GOLD["blosum62_ncbistdaa_28x32"])[:, :28]
    # every stored (word, offset) scores >= 11 and every word >= 11 is stored
    for w in rng.integers(0, 32768, size=3000):
        a, b, c = w >> 10, (w >> 5) & 31, w & 31
        stored = set(ent[cs[w]:cs[w + 1]].tolist())
        assert list(ent[cs[w]:cs[w + 1]]) == sorted(stored)
        for p in range(len(q) - 2):
            ok = a < 28 and b < 28 and c < 28 and m[q[p], a] + m[q[p + 1], b] + m[q[p + 2], c] >= 11
            assert (p in stored) == bool(ok)


def test_threads_do_not_change_results(built):
    from hblast import synth
    rng = np.random.default_rng(5)
    q = synth.random_letters(rng, 200)
    db = synth.make_db(rng, 300, 300, 0.6, 30, 5000, 30, [q], 100, 0.5)
    a = oracle.search(oracle.Query.blastp(q), db.residues, db.offsets, nthreads=1)
    b = oracle.search(oracle.Query.blastp(q), db.residues, db.offsets, nthreads=4)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    assert len(a[0]) > 0


def test_search_many_equals_per_query_search():
    """The multi-query driver (work items of (query, subject block) over a
    thread pool, fresh diagonal table per item) gives the per-query search's
    HSPs and counters: the offset trick makes every subject start from a
    fresh diagonal state, so how subjects are split does not matter."""
    import ctypes as C
    from hblast import synth
    rng = np.random.default_rng(5)
    qs = [synth.random_letters(rng, n) for n in (40, 300, 777)]
    db = synth.make_db(rng, 400, 300, 0.6, 30, 5000, 0.05, qs, lambda r: r.integers(50, 301),
                       lambda r: r.uniform(0.3, 0.6))
    oq = [oracle.Query.blastp(q) for q in qs]
    lens = np.diff(db.offsets).astype(np.int32)
    many = oracle.search_many(oq, db.residues, db.offsets, nthreads=3, block_residues=5000)
    for q, (h, subj, cnt) in zip(oq, many):
        cs, en = oracle.lookup_table(q, 11)
        cs = np.ascontiguousarray(cs, np.int32)
        en = np.ascontiguousarray(en if len(en) else np.zeros(1, np.int32), np.int32)
        cap = 1 << 16
        out = np.zeros(cap, dtype=oracle.HSP_DTYPE)
        osub = np.zeros(cap, dtype=np.int32)
        c0 = np.zeros(3, np.int64)
        cq = q.c()
        n = oracle.lib().orc_search_lut(C.byref(cq), cs.ctypes.data, en.ctypes.data, 40, db.residues.ctypes.data,
                                        db.offsets.ctypes.data, lens.ctypes.data, 0, db.n, 1, out.ctypes.data,
                                        osub.ctypes.data, cap, c0.ctypes.data)
        assert 0 < n < cap
        assert np.array_equal(h, out[:n]) and np.array_equal(subj, osub[:n])
        assert np.array_equal(cnt, c0)
