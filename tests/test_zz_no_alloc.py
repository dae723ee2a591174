"""hbg_search_static: the word finder with its scratch in a static device array,
for callers that cannot allocate device memory while they search (real-time
services that cannot afford cudaMalloc's synchronisation, hosts whose device
memory budget is fixed at start-up).

Two calls in a row through the C ABI must give the same HSPs and counters as
hbg_search, bit for bit (tolerance 0: integer work).  The entry point leaves
HSPs unordered, so they are put in reference order before the comparison.
This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

import hblast
from hblast import synth
from hblast.core import HSP_DTYPE, lib

pytestmark = pytest.mark.gpu


def call_static(gdb, batch, d_hsps, cap, d_counts, stream):
    opts = hblast.default_options()
    return lib().hbg_search_static(gdb.handle, batch.handle, C.byref(opts), C.c_void_p(d_hsps.data_ptr()),
                                   cap, C.c_void_p(d_counts.data_ptr()), C.c_void_p(stream.cuda_stream))


def make_batch(kind, rng):
    """(database, batch) for one parity case; every
    group stays within 2008 letters so its diagonal tables live in shared
    memory, which is what the static entry point can serve."""
    if kind == "blastx":
        prot = synth.random_letters(rng, 400)
        db = synth.make_db(rng, 1500, 300, 0.6, 30, 5000, 30, [prot], 150, 0.6)
        nts = synth.blastx_queries(9, db, n_queries=3)
        nts = [nt[:900] for nt in nts]                 # six frames of <= 300 letters: one group each
        xd = np.full((3, 6), 16, dtype=np.int32)
        cu = np.full((3, 6), 41, dtype=np.int32)
        cu[1] = [30, 35, 41, 41, 38, 33]
        return db, hblast.Batch.blastx(nts, xd, cu, max_group_len=2008)
    qs = [synth.random_letters(rng, n) for n in (300, 57, 1200, 800)]
    db = synth.make_db(rng, 3000, 300, 0.6, 30, 5000, 0.05, qs, 150, 0.5)
    batch = hblast.Batch.proteins([hblast.ProteinQuery.blastp(q) for q in qs], max_group_len=2008)
    if kind == "offset_mode":
        batch.set_mode(1)                              # one subject offset at a time, lanes over its cell
    return db, batch


@pytest.mark.parametrize("kind", ["blastp", "blastx", "offset_mode"])
def test_search_static_matches_search(built, kind):
    import torch
    rng = np.random.default_rng(31)
    db, batch = make_batch(kind, rng)
    gdb = hblast.Database(db.residues, db.offsets)
    ref = hblast.search(gdb, batch)          # the set-up search also makes the batch resident
    n, nq = len(ref.hsps), batch.info()["n_queries"]
    assert n > 0
    cap = n + 16
    d_hsps = torch.zeros(cap * 9, dtype=torch.int32, device="cuda")      # 9 int32 fields per record
    d_counts = torch.zeros(1 + 2 * nq, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(2):                       # the array keeps the last call's contents
        d_hsps.fill_(-1)
        torch.cuda.synchronize()
        rc = call_static(gdb, batch, d_hsps, cap, d_counts, stream)
        assert rc == 0, lib().hbg_last_error()
        torch.cuda.synchronize()
        counts = d_counts.cpu().numpy()
        assert counts[0] == n
        got = d_hsps.cpu().numpy().view(HSP_DTYPE)[:n]
        got = got[np.lexsort((got["q_off"], got["s_off"], got["subject"], got["query"]))]
        assert np.array_equal(got, ref.hsps)
        for k in range(nq):
            assert counts[1 + k] == ref.stats[k]["init_extends"]
            assert counts[1 + nq + k] == ref.stats[k]["good_init_extends"]


def test_search_static_rejects_what_needs_global_tables(built):
    import torch
    rng = np.random.default_rng(32)
    q = synth.random_letters(rng, 20000)     # a 32768-entry diagonal table: global memory
    db = synth.make_db(rng, 50, 300, 0.6, 30, 5000, 5, [q], 100, 0.5)
    gdb = hblast.Database(db.residues, db.offsets)
    batch = hblast.Batch.proteins([hblast.ProteinQuery.blastp(q)])
    hblast.search(gdb, batch)
    d_hsps = torch.zeros(9 * 16, dtype=torch.int32, device="cuda")
    d_counts = torch.zeros(3, dtype=torch.int64, device="cuda")
    rc = call_static(gdb, batch, d_hsps, 16, d_counts, torch.cuda.current_stream())
    assert rc == hblast.core.HBG_ERR_TOO_LONG
