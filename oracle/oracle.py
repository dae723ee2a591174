"""ctypes wrapper of the CPU oracle (oracle/hblast_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker for the GPU path and the CPU baseline of
bench.py.  Only tests/, __graft_entry__.smoke() and bench.py may import it.

Build recipe: gcc -O2 -shared -fPIC -pthread on hblast_oracle.c into
oracle/_build/libhblast_oracle.so (see build()).  The H-BLAST sources cannot
be compiled into an oracle/_ref binary: they need the NCBI BLAST+ 2.2.28
headers (algo/blast/core/*.h, h_blast.cu:9-12), which the reference tree does
not contain.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libhblast_oracle.so"
NCELLS = 32768

HSP_FIELDS = ("q_start", "s_start", "q_off", "s_off", "len", "score", "ctx")
HSP_DTYPE = np.dtype([(n, np.int32) for n in HSP_FIELDS])


def build(force: bool = False) -> Path:
    src = HERE / "hblast_oracle.c"
    hdr = HERE / "hblast_oracle.h"
    if (not force and LIB.exists() and LIB.stat().st_mtime >= max(src.stat().st_mtime, hdr.stat().st_mtime)):
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the oracle")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O2", "-std=c11", "-shared", "-fPIC", "-pthread", str(src), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


class _OrcQuery(C.Structure):
    _fields_ = [("seq", C.POINTER(C.c_uint8)), ("len", C.c_int32), ("n_ctx", C.c_int32),
                ("ctx_off", C.POINTER(C.c_int32)), ("ctx_len", C.POINTER(C.c_int32)),
                ("x_dropoff", C.POINTER(C.c_int32)), ("cutoff", C.POINTER(C.c_int32))]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.orc_score.argtypes = [C.c_int32, C.c_int32]
        L.orc_score.restype = C.c_int32
        L.orc_lut_build.argtypes = [C.POINTER(_OrcQuery), C.c_int32, C.c_void_p, C.c_void_p, C.c_int64]
        L.orc_lut_build.restype = C.c_int64
        L.orc_search.argtypes = [C.POINTER(_OrcQuery), C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                 C.c_int64, C.c_void_p]
        L.orc_search.restype = C.c_int64
        L.orc_search_lut.argtypes = [C.POINTER(_OrcQuery), C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                     C.c_void_p, C.c_int64, C.c_void_p]
        L.orc_search_lut.restype = C.c_int64
        L.orc_translate6.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_translate6.restype = C.c_int32
        L.orc_search_many.argtypes = [C.POINTER(_OrcQuery), C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                      C.c_int64]
        L.orc_search_many.restype = C.c_void_p
        L.orc_result_count.argtypes = [C.c_void_p, C.c_int32]
        L.orc_result_count.restype = C.c_int64
        L.orc_result_copy.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_result_copy.restype = C.c_int
        L.orc_result_free.argtypes = [C.c_void_p]
        L.orc_result_free.restype = None
        _lib = L
    return _lib


class Query:
    """One query in NCBI concatenated form for the oracle."""

    def __init__(self, seq, ctx_off, ctx_len, xdrop, cutoff):
        self.seq = np.ascontiguousarray(seq, dtype=np.uint8)
        self.ctx_off = np.ascontiguousarray(ctx_off, dtype=np.int32)
        self.ctx_len = np.ascontiguousarray(ctx_len, dtype=np.int32)
        self.xdrop = np.ascontiguousarray(xdrop, dtype=np.int32)
        self.cutoff = np.ascontiguousarray(cutoff, dtype=np.int32)
        self.length = int(self.ctx_off[-1] + self.ctx_len[-1])

    @classmethod
    def blastp(cls, seq, xdrop=16, cutoff=41):
        return cls(seq, [0], [len(seq)], [xdrop], [cutoff])

    def c(self) -> _OrcQuery:
        i32 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
        return _OrcQuery(self.seq.ctypes.data_as(C.POINTER(C.c_uint8)), self.length, len(self.ctx_off),
                         i32(self.ctx_off), i32(self.ctx_len), i32(self.xdrop), i32(self.cutoff))


def score(a: int, b: int) -> int:
    return lib().orc_score(a, b)


def lookup_table(q: Query, threshold: int = 11):
    """CSR lookup table: (cell_start[32769], entries) with ascending entries per cell."""
    cq = q.c()
    cs = np.zeros(NCELLS + 1, dtype=np.int32)
    n = lib().orc_lut_build(C.byref(cq), threshold, cs.ctypes.data, None, 0)
    ent = np.zeros(max(n, 1), dtype=np.int32)
    lib().orc_lut_build(C.byref(cq), threshold, cs.ctypes.data, ent.ctypes.data, n)
    return cs, ent[:n]


def search(q: Query, residues: np.ndarray, offsets: np.ndarray, threshold: int = 11, window: int = 40,
           nthreads: int = 1, subj_range=None, lut=None):
    """Search one query; returns (hsps structured array, subject index array, counters[3])."""
    return search_many([q], residues, offsets, threshold, window, nthreads, subj_range,
                       None if lut is None else [lut])[0]


def search_many(queries, residues: np.ndarray, offsets: np.ndarray, threshold: int = 11, window: int = 40,
                nthreads: int = 1, subj_range=None, luts=None, block_residues: int = 0):
    """Search several queries in one call: (query, subject block) work items over `nthreads`
    threads.  Returns one (hsps, subject indices, counters[3]) tuple per query; every HSP is
    returned from a single pass (no capacity retries)."""
    residues = np.ascontiguousarray(residues, dtype=np.uint8)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    lens = np.ascontiguousarray(np.diff(offsets), dtype=np.int32)
    n = len(lens)
    lo, hi = subj_range if subj_range is not None else (0, n)
    nq = len(queries)
    if luts is None:
        luts = [lookup_table(q, threshold) for q in queries]
    cs = [np.ascontiguousarray(l[0], dtype=np.int32) for l in luts]
    en = [np.ascontiguousarray(l[1] if len(l[1]) else np.zeros(1, np.int32), dtype=np.int32) for l in luts]
    cq = (_OrcQuery * max(nq, 1))(*[q.c() for q in queries])
    csp = (C.c_void_p * max(nq, 1))(*[a.ctypes.data for a in cs])
    enp = (C.c_void_p * max(nq, 1))(*[a.ctypes.data for a in en])
    r = lib().orc_search_many(cq, nq, csp, enp, window, residues.ctypes.data, offsets.ctypes.data,
                              lens.ctypes.data, lo, hi, nthreads, block_residues)
    if not r:
        raise RuntimeError("oracle search failed")
    try:
        out = []
        for k in range(nq):
            m = lib().orc_result_count(r, k)
            h = np.zeros(m, dtype=HSP_DTYPE)
            subj = np.zeros(m, dtype=np.int32)
            counters = np.zeros(3, dtype=np.int64)
            lib().orc_result_copy(r, k, h.ctypes.data, subj.ctypes.data, counters.ctypes.data)
            out.append((h, subj, counters))
        return out
    finally:
        lib().orc_result_free(r)


def translate6(nt: np.ndarray):
    nt = np.ascontiguousarray(nt, dtype=np.uint8)
    out = np.zeros(2 * len(nt) + 6, dtype=np.uint8)
    off = np.zeros(6, dtype=np.int32)
    ln = np.zeros(6, dtype=np.int32)
    n = lib().orc_translate6(nt.ctypes.data, len(nt), out.ctypes.data, off.ctypes.data, ln.ctypes.data)
    return out[:n], off, ln
