"""SEG low-complexity masking (host code, no GPU): the library's C++ SEG
against an independent Python restatement of the published method, known
answers (low-complexity stretches masked, random proteins untouched), and the
BLASTX batch built with SEG equal to the tables of frames masked by the
restatement.  Parity with NCBI's own SEG implementation is unpinned: it is not
in the reference tree."""
import numpy as np
import pytest

import hblast
from hblast import synth
from oracle import oracle
from seg_ref import seg as seg_ref

L = "-ABCDEFGHIKLMNPQRSTVWXYZU*OJ"


def enc(s: str) -> np.ndarray:
    return np.array([L.index(c) for c in s], dtype=np.uint8)


def cases():
    rng = np.random.default_rng(3)
    out = []
    for k in range(12):
        q = synth.random_letters(rng, int(rng.integers(20, 160)))
        kind = k % 4
        if kind == 0:
            ins = np.full(int(rng.integers(8, 40)), int(rng.choice([1, 14, 16, 17])), np.uint8)
        elif kind == 1:
            ins = np.tile(enc("PA"), int(rng.integers(5, 20)))
        elif kind == 2:
            ins = rng.choice(enc("SGN"), size=int(rng.integers(12, 50))).astype(np.uint8)
        else:
            ins = synth.random_letters(rng, 30)
        at = int(rng.integers(0, len(q) + 1))
        out.append(np.concatenate([q[:at], ins, q[at:]]))
    out.append(enc("QQQQQQQQQQQQ"))                      # exactly one window
    out.append(enc("QQQQQQQQQQQ"))                       # shorter than a window
    out.append(enc("AAAAAXAAAAAAAAAAAAAAAAAAA"))         # a non-standard letter breaks windows
    out.append(enc("ACDEFGHIKLMNPQRSTVWYKKKKKKKKKKKKKKKKKKKKACDEFGHIK"))
    return out


@pytest.mark.parametrize("k", range(16))
def test_seg_matches_restatement(built, k):
    s = cases()[k]
    assert np.array_equal(hblast.seg_mask(s), seg_ref(s)), k


def test_seg_long_raw_segments(built):
    """Raw segments longer than the trimming bound (100 letters at each end):
    the restatement agrees, and a 35,000-letter low-complexity query is masked
    in well under a second."""
    import time
    rng = np.random.default_rng(8)
    s = np.concatenate([synth.random_letters(rng, 50), rng.choice(enc("QQQQP"), size=260).astype(np.uint8),
                        synth.random_letters(rng, 50)])
    assert np.array_equal(hblast.seg_mask(s), seg_ref(s))
    big = np.full(35000, enc("Q")[0], np.uint8)
    t = time.perf_counter()
    m = hblast.seg_mask(big)
    assert time.perf_counter() - t < 1.0
    assert (m == 21).all()


def test_seg_parameters_matter(built):
    s = np.concatenate([synth.random_letters(np.random.default_rng(9), 60), enc("SGSGSGNSGSGSGGSNSG")])
    for w, lo, hi in ((12, 2.2, 2.5), (8, 1.5, 2.0), (20, 3.0, 3.3)):
        assert np.array_equal(hblast.seg_mask(s, w, lo, hi), seg_ref(s, w, lo, hi)), (w, lo, hi)


def test_seg_idempotent(built):
    """Masking a masked sequence again changes nothing: every window that
    reaches into a masked stretch holds an X and cannot trigger, and the rest
    is scanned as before.  Random proteins with planted stretches of one to
    three letters."""
    rng = np.random.default_rng(5)
    masked = 0
    for _ in range(200):
        n = int(rng.integers(20, 600))
        x = synth.random_letters(rng, n)
        for _ in range(int(rng.integers(0, 4))):
            a, ln = int(rng.integers(0, n)), int(rng.integers(5, 80))
            alph = rng.integers(1, 21, size=int(rng.integers(1, 4)))
            x[a:a + ln] = rng.choice(alph, size=len(x[a:a + ln]))
        m = hblast.seg_mask(x)
        masked += int((m != x).sum())
        assert np.array_equal(hblast.seg_mask(m), m)
    assert masked > 1000


def test_seg_known_answers(built):
    rng = np.random.default_rng(4)
    q = synth.random_letters(rng, 300)
    assert (hblast.seg_mask(q) != q).sum() <= 12           # a random protein is (almost) untouched
    poly = enc("Q" * 30)
    s = np.concatenate([q[:100], poly, q[100:]])
    m = hblast.seg_mask(s)
    assert (m[100:130] == 21).all()                         # the stretch becomes X
    assert np.array_equal(m[:95], s[:95]) and np.array_equal(m[135:], s[135:])
    with pytest.raises(hblast.HblastError):
        hblast.seg_mask(s, 0)


def test_blastx_batch_with_seg(built):
    """Frames masked by the library while it builds the BLASTX tables equal
    frames masked by the restatement, table for table."""
    rng = np.random.default_rng(6)
    nts = [rng.integers(0, 4, size=n).astype(np.uint8) for n in (300, 450)]
    # a low-complexity run in frame +1 of the first query: GCT repeated (Ala)
    nts[0][30:120] = np.tile(np.array([2, 1, 3], np.uint8), 30)
    xd = np.full((2, 6), 16, np.int32)
    cu = np.full((2, 6), 41, np.int32)
    b = hblast.Batch.blastx(nts, xd, cu, max_group_len=1, seg=True)
    plain = hblast.Batch.blastx(nts, xd, cu, max_group_len=1)
    for k, nt in enumerate(nts):
        prot, off, ln = oracle.translate6(nt)
        masked = prot.copy()
        for f in range(6):
            masked[off[f]:off[f] + ln[f]] = seg_ref(prot[off[f]:off[f] + ln[f]])
        cs, oe = oracle.lookup_table(oracle.Query(masked, off, ln, [16] * 6, [41] * 6), 11)
        cells, ent, _, _ = b.lookup_table(k)
        assert np.array_equal(cells.astype(np.int64), cs) and np.array_equal(ent.astype(np.int64), oe)
    assert b.info()["lookup_entries"] < plain.info()["lookup_entries"]
