"""Python restatement of SEG (Wootton and Federhen, Comput. Chem. 17:149-163,
1993; Methods Enzymol. 266:554-571, 1996) used to check the library's C++ SEG
(h-blast_gb300/host/seg.cpp), written independently from the same published
rules: window complexity K2 (bits) over the 20 standard amino acids, trigger
at <= locut, extension over windows <= hicut, trimming to the subsequence
with the least probable complexity state, recursion on the flanks; masked
letters become X.  Small sequences only (cubic time)."""
from __future__ import annotations

import math

import numpy as np

STD = [1, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 22]   # NCBIstdaa of A C D ... W Y
IDX = {c: i for i, c in enumerate(STD)}
N = 20


def k2(win) -> float:
    if any(int(c) not in IDX for c in win):
        return math.inf
    cnt = [0] * N
    for c in win:
        cnt[IDX[int(c)]] += 1
    h = 0.0
    for a in range(N):
        if cnt[a]:
            p = cnt[a] / len(win)
            h -= p * math.log2(p)
    return h


def lfact(k: int) -> float:
    v = 0.0
    for i in range(2, k + 1):
        v += math.log(i)
    return v


def log_p0(cnt, L: int) -> float:
    v = lfact(N) + lfact(L) - L * math.log(N)
    for a in range(N):
        v -= lfact(cnt[a])
    classes = {}
    for a in range(N):
        classes[cnt[a]] = classes.get(cnt[a], 0) + 1
    small = [classes.get(k, 0) for k in range(64)]
    for k in range(64):
        v -= lfact(small[k])
    for k, m in classes.items():
        if k >= 64:
            v -= lfact(m)
    return v


MAX_TRIM = 100    # the library's bound: at most 100 letters trimmed from each end of a raw segment


def optimise(s, a: int, b: int):
    best, bi, bj = math.inf, a, b
    for i in range(a, min(b, a + MAX_TRIM + 1)):
        cnt = [0] * N
        for j in range(i, b):
            cnt[IDX[int(s[j])]] += 1
            if j < b - MAX_TRIM - 1:
                continue
            v = log_p0(cnt, j - i + 1)
            if v < best:
                best, bi, bj = v, i, j + 1
    return bi, bj


def run(s, a: int, b: int, W: int, lo: float, hi: float, mask):
    if b - a < W:
        return
    ks = [k2(s[a + w:a + w + W]) for w in range(b - a - W + 1)]
    w = 0
    while w < len(ks):
        if not ks[w] <= lo:
            w += 1
            continue
        l, h = w, w
        while l > 0 and ks[l - 1] <= hi:
            l -= 1
        while h + 1 < len(ks) and ks[h + 1] <= hi:
            h += 1
        ra, rb = a + l, a + h + W
        i, j = optimise(s, ra, rb)
        mask[i:j] = True
        run(s, ra, i, W, lo, hi, mask)
        run(s, j, rb, W, lo, hi, mask)
        w = h + 1


def seg(seq, window: int = 12, locut: float = 2.2, hicut: float = 2.5) -> np.ndarray:
    s = np.asarray(seq, dtype=np.uint8)
    mask = np.zeros(len(s), dtype=bool)
    run(s, 0, len(s), window, locut, hicut, mask)
    out = s.copy()
    out[mask] = 21
    return out
