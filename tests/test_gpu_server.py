"""The serving loop (hbg_server_*): requests arriving from several threads are
batched as they come, and each request's HSPs and counters must be the same
as a search of that query alone (bit-exact, tolerance 0)."""
import threading
import time

import numpy as np
import pytest

import hblast
from hblast import synth
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def served(built):
    rng = np.random.default_rng(41)
    qs = [synth.random_letters(rng, int(n)) for n in rng.integers(30, 1500, size=24)]
    db = synth.make_db(rng, 4000, 300, 0.6, 30, 5000, 0.05, qs, lambda r: r.integers(50, 301),
                       lambda r: r.uniform(0.3, 0.6))
    nts = synth.blastx_queries(3, db, n_queries=6)
    return qs, nts, db, hblast.Database(db.residues, db.offsets)


def alone(gdb, pq):
    r = hblast.search(gdb, hblast.Batch.proteins([pq]))
    return r.hsps, r.stats[0]


def test_mixed_stream_equals_alone(served):
    qs, nts, db, gdb = served
    xd6, cu6 = np.full(6, 16, np.int32), np.full(6, 41, np.int32)
    srv = hblast.Server(gdb, max_inflight=2, max_batch_queries=8)
    tickets = {}
    lock = threading.Lock()

    def producer(items, seed):
        r = np.random.default_rng(seed)
        for kind, idx in items:
            time.sleep(float(r.exponential(0.003)))
            t = srv.submit(hblast.ProteinQuery.blastp(qs[idx])) if kind == "p" else srv.submit_blastx(nts[idx], xd6, cu6)
            with lock:
                tickets[t] = (kind, idx)

    work = [("p", i) for i in range(len(qs))] + [("x", i) for i in range(len(nts))]
    th = [threading.Thread(target=producer, args=(work[k::3], k)) for k in range(3)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for t, (kind, idx) in tickets.items():
        hsps, stats, lat = srv.take(t)
        if kind == "p":
            pq = hblast.ProteinQuery.blastp(qs[idx])
        else:
            prot, off, ln = oracle.translate6(nts[idx])
            pq = hblast.ProteinQuery(prot, off, ln, xd6, cu6)
        ref, ref_stats = alone(gdb, pq)
        assert np.array_equal(hsps, ref), (kind, idx)
        assert stats == ref_stats, (kind, idx)
        assert lat > 0
    c = srv.counters()
    assert c["queries"] == len(work)
    assert c["largest_batch"] > 1          # requests were batched
    srv.close()


def test_memory_budget_limits_batches(served):
    qs, nts, db, gdb = served
    srv = hblast.Server(gdb, max_inflight=1, max_batch_queries=64, memory_budget=1)   # every request alone
    ts = [srv.submit(hblast.ProteinQuery.blastp(q)) for q in qs[:6]]
    for t, q in zip(ts, qs[:6]):
        hsps, _, _ = srv.take(t)
        assert np.array_equal(hsps, alone(gdb, hblast.ProteinQuery.blastp(q))[0])
    assert srv.counters()["largest_batch"] == 1
    srv.close()


def test_allocation_failures_requeue_requests(served):
    """Device allocations that fail (injected: the library's next allocations
    report out-of-memory) put a batch's requests back in the queue; they are
    searched again and complete with the same HSPs as alone.  The reference's
    counterpart is the CPU fallback when GPU memory falls short
    (NF/functions.cpp:1518-1530)."""
    qs, nts, db, gdb = served
    refs = [alone(gdb, hblast.ProteinQuery.blastp(q)) for q in qs[:8]]
    srv = hblast.Server(gdb, max_inflight=1, max_batch_queries=8)
    hblast.fail_allocations(3)
    try:
        ts = [srv.submit(hblast.ProteinQuery.blastp(q)) for q in qs[:8]]
        got = [srv.take(t) for t in ts]
    finally:
        hblast.fail_allocations(0)
    for (hsps, stats, _), (ref, ref_stats) in zip(got, refs):
        assert np.array_equal(hsps, ref)
        assert stats == ref_stats
    c = srv.counters()
    assert c["requeued"] >= 1 and c["queries"] == 8
    srv.close()


def test_search_out_of_memory_is_recoverable(served):
    """A search whose buffers cannot be allocated returns HBG_ERR_NOMEM and
    leaves nothing broken: the same batch and result search correctly
    afterwards, including a relaunch whose larger HSP buffer fails first."""
    qs, nts, db, gdb = served
    pqs = [hblast.ProteinQuery.blastp(q) for q in qs[:4]]
    ref = hblast.search(gdb, hblast.Batch.proteins(pqs))
    batch = hblast.Batch.proteins(pqs)
    hblast.fail_allocations(1)
    with pytest.raises(hblast.HblastError) as e:
        hblast.search(gdb, batch)
    assert e.value.code == hblast.core.HBG_ERR_NOMEM
    hblast.fail_allocations(0)
    assert np.array_equal(hblast.search(gdb, batch).hsps, ref.hsps)
    # relaunch on HSP-buffer overflow: its allocation fails, then succeeds
    s = hblast.Searcher(gdb, batch, hsp_capacity=1)
    s.launch(None)
    hblast.fail_allocations(1)
    with pytest.raises(hblast.HblastError) as e:
        s.wait()
    assert e.value.code == hblast.core.HBG_ERR_NOMEM
    hblast.fail_allocations(0)
    s.launch(None)
    s.wait()
    assert np.array_equal(s.result().hsps, ref.hsps)
    s.close()


def test_served_blastx_with_seg(served):
    """seg_blastx: served BLASTX requests equal a BLASTX batch built with SEG."""
    qs, nts, db, gdb = served
    xd6, cu6 = np.full(6, 16, np.int32), np.full(6, 41, np.int32)
    srv = hblast.Server(gdb, max_inflight=1, max_batch_queries=4, seg_blastx=1)
    ts = [srv.submit_blastx(nt, xd6, cu6) for nt in nts]
    for t, nt in zip(ts, nts):
        hsps, stats, _ = srv.take(t)
        ref = hblast.search(gdb, hblast.Batch.blastx([nt], xd6[None], cu6[None], seg=True))
        assert np.array_equal(hsps, ref.hsps)
        assert stats == ref.stats[0]
    srv.close()
