#!/usr/bin/env python
"""Benchmark of the BLASTP word-hit stage on the batched workload.

Workload (default, --config batched): 64 protein queries of 50..1500 aa against
2,000,000 lognormal subjects (~720 M uint8 residues resident in HBM), word 3,
T=11, window 40, X-drop 16, cutoff 41, seed 0.  One step = one search of the
whole batch against the whole database (seed scan + two-hit + ungapped
extension + ordering pass).  Metric: query x db residues per second,
sum(query lengths) * sum(subject lengths) / step time.

Arms:
  default            the GB300 path through the C ABI; prints one JSON line.
  --impl reference   the reference's CPU word finder on the host cores: the C
                     restatement in oracle/ (the H-BLAST/NCBI sources cannot be
                     built here), all host threads, on a bounded sample of the
                     same workload.

Multi-GPU (torchrun, N > 1): subjects shard across ranks with no collective on
the data path; each rank searches its own database of the configured size
(weak scaling) and the step time is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "h-blast_gb300"))
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "query x db residues/s"
UNIT = "residues/s"
HSP_BYTES = 36


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="hblast", choices=["hblast", "reference"])
    p.add_argument("--config", default="batched",
                   choices=["batched", "plain", "blastx", "scan", "served", "autotune", "ingest"])
    p.add_argument("--rates", default="50,200,1000,2000", help="served: Poisson arrival rates (queries/s)")
    p.add_argument("--requests", type=int, default=1000, help="served: requests per rate")
    p.add_argument("--forms", default="served,plain", help="served: forms to run (served, served_2, served_fifo, plain)")
    p.add_argument("--batches", default="1,8,64", help="autotune: query batch sizes")
    p.add_argument("--subjects", type=int, default=0, help="override the database size (testing)")
    p.add_argument("--queries", type=int, default=0, help="override the number of queries (testing)")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU-baseline sample time")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-plain", action="store_true", help="skip the one-query-per-launch comparison")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--group-len", type=int, default=0, help="letters per query group (0 = library default)")
    p.add_argument("--mode", type=int, default=-1, help="hit mode of every group (-1 = library default)")
    return p.parse_args()


# --------------------------------------------------------------------------- workload

def frame_letters(nt_len: int) -> int:
    """Letters of the six translated frames of a nucleotide query."""
    return sum(max(nt_len - f % 3, 0) // 3 for f in range(6))


def workload(cfg: str, rank: int, n_subjects: int, n_queries: int):
    from hblast import synth
    if cfg == "blastx":
        _, db = synth.batched_blastp(seed=rank, n_queries=64, n_subjects=n_subjects or 2_000_000)
        nts = synth.blastx_queries(rank, db, n_queries=n_queries or 128)
        desc = dict(workload="batched blastx: 128 nucleotide queries of 300..3000 nt (GC 0.5, planted ORFs matching "
                             "database proteins at 40..70% identity), six frames, vs the 2,000,000-subject database")
        return nts, db, desc
    if cfg == "scan":
        n = n_queries or 1
        qs = synth.heavy_tailed_queries(rank, n)
        db = synth.large_db(rank, n_subjects or 10_000_000, donors=qs)
        desc = dict(workload=f"scan-bound blastp: {n} heavy-tailed quer{'y' if n == 1 else 'ies'} (lognormal median "
                             f"350, sigma 1.0; {sum(len(q) for q in qs)} letters) vs {db.n:,} lognormal subjects "
                             "(median 300, sigma 0.6, 30..5000), 1% planted 50..300 aa at 30..60% identity")
        return qs, db, desc
    if cfg == "plain":
        qs, db = synth.plain_blastp(seed=rank, n_subjects=n_subjects or 20000)
        desc = dict(workload="plain blastp: 1 query of 300 aa vs 20,000 lognormal subjects (median 300, "
                             "sigma 0.6, 30..5000), 50 planted 120-aa segments at 40% identity")
    else:
        qs, db = synth.batched_blastp(seed=rank, n_queries=n_queries or 64, n_subjects=n_subjects or 2_000_000)
        desc = dict(workload="batched blastp: 64 queries of 50..1500 aa vs 2,000,000 lognormal subjects "
                             "(median 300, sigma 0.6, 30..5000), 1% planted 50..300 aa at 30..60% identity")
    return qs, db, desc


# --------------------------------------------------------------------------- clocks

class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons, pw = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                pw.append(float(r[3]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(pw) if pw else None}


# --------------------------------------------------------------------------- CPU sides

CPU_SAMPLE_RESIDUES = 32_000_000


class CpuSample:
    """The CPU word finder (the oracle's C restatement of NCBI's two-hit word
    finder) over a fixed prefix of the workload's database: the first subjects
    holding CPU_SAMPLE_RESIDUES letters, every query, all host threads, one call
    per pass (work items of (query, subject block) over a thread pool).  The
    GPU arm's cpu_baseline and the reference arm both time exactly this, so
    their per-residue rates are one figure."""

    def __init__(self, qs, db, threads: int, blastx: bool = False):
        from oracle import oracle
        self.oracle = oracle
        if blastx:
            self.queries = []
            for nt in qs:
                prot, off, ln = oracle.translate6(nt)
                self.queries.append(oracle.Query(prot, off, ln, [16] * 6, [41] * 6))
        else:
            self.queries = [oracle.Query.blastp(q) for q in qs]
        self.luts = [oracle.lookup_table(q, 11) for q in self.queries]
        self.qsum = float(sum(q.length for q in self.queries))
        self.n = int(min(db.n, np.searchsorted(db.offsets, CPU_SAMPLE_RESIDUES)))
        self.residues = int(db.offsets[self.n] - db.offsets[0])
        self.db = db
        self.threads = threads
        self.sample = (f"{len(self.queries)} queries x first {self.n} subjects ({self.residues} residues) "
                       f"of the workload per pass, {threads} threads")

    def run(self) -> float:
        t0 = time.perf_counter()
        self.oracle.search_many(self.queries, self.db.residues, self.db.offsets, nthreads=self.threads,
                                subj_range=(0, self.n), luts=self.luts)
        return time.perf_counter() - t0

    def rate(self, seconds: float) -> float:
        return self.qsum * self.residues / seconds


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle
    oracle.build()
    qs, db, desc = workload(args.config, 0, args.subjects, args.queries)
    threads = os.cpu_count() or 1
    cs = CpuSample(qs, db, threads, blastx=args.config == "blastx")
    times = []
    for i in range(args.warmup + args.steps):
        t = cs.run()
        if i >= args.warmup:
            times.append(t)
    t = sum(times) / len(times)
    value = cs.rate(t)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": dict(desc, sample=cs.sample),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": cs.sample,
                         "what": "C restatement of the NCBI BLAST+ 2.2.28 two-hit word finder (oracle/)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# --------------------------------------------------------------------------- served and autotune

def served_arm(args):
    """Poisson arrivals of 80% BLASTP (lognormal median 350, sigma 1.0, 30..35,000 aa) and 20% BLASTX
    (300..3000 nt) against a resident database; p50/p99 latency per rate, for the continuous-batching
    server and for the plain form (one query per launch, one at a time)."""
    import threading
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__ as g
    g.build()
    import hblast
    from hblast import synth
    n_sub = args.subjects or 10_000_000
    db = synth.large_db(0, n_sub)
    gdb = hblast.Database(db.residues, db.offsets)
    ssum = int(db.offsets[-1])
    xd6, cu6 = np.full(6, 16, np.int32), np.full(6, 41, np.int32)
    out = {"metric": "served latency", "config": {"workload": f"served mixed stream vs {n_sub} subjects "
                                                               f"({ssum} residues)", "requests_per_rate": args.requests}}
    rates = [float(x) for x in args.rates.split(",")]
    forms = {"served": dict(),
             "served_2": dict(max_inflight=2),
             "served_fifo": dict(max_inflight=2, max_batch_queries=512, max_batch_letters=0, shortest_first_ms=0),
             "plain": dict(max_inflight=1, max_batch_queries=1, max_batch_letters=0, shortest_first_ms=0)}
    out["forms"] = {"served": "library defaults: shortest-first admission (age bound 2 s), <= 8192 query "
                              "letters per batch, 1 batch in flight (the next is chosen when one ends)",
                    "served_2": "as served, 2 batches in flight",
                    "served_fifo": "arrival-order admission, no letter cap, 2 batches in flight",
                    "plain": "one query per launch, one at a time, arrival order"}
    forms = {k: v for k, v in forms.items() if k in args.forms.split(",")}
    for form, so in forms.items():
        res_form = []
        for rate in rates:
            r = np.random.default_rng(int(rate * 1000) + 7)
            kinds = r.random(args.requests) < 0.8
            lens = synth.lognormal_lengths(r, args.requests, 350, 1.0, 30, 35000)
            reqs = []
            for k, L in zip(kinds, lens):
                if k:
                    reqs.append(("p", synth.random_letters(r, int(L))))
                else:
                    reqs.append(("x", r.integers(0, 4, size=int(r.integers(300, 3001))).astype(np.uint8)))
            gaps = r.exponential(1.0 / rate, size=args.requests)
            srv = hblast.Server(gdb, **so)
            tickets = []
            letters = 0
            t_start = time.perf_counter()

            def produce():
                nonlocal letters
                t = time.perf_counter()
                for (kind, seq), gap in zip(reqs, gaps):
                    t += gap
                    d = t - time.perf_counter()
                    if d > 0:
                        time.sleep(d)
                    if kind == "p":
                        tickets.append(srv.submit(hblast.ProteinQuery.blastp(seq)))
                        letters += len(seq)
                    else:
                        tickets.append(srv.submit_blastx(seq, xd6, cu6))
                        letters += frame_letters(len(seq))

            th = threading.Thread(target=produce)
            th.start()
            th.join()
            lat = []
            for t in tickets:
                _, _, ms = srv.take(t)
                lat.append(ms)
            wall = time.perf_counter() - t_start
            c = srv.counters()
            srv.close()
            lat = np.array(lat)
            res_form.append({"rate": rate, "p50_ms": float(np.percentile(lat, 50)),
                             "p99_ms": float(np.percentile(lat, 99)), "wall_s": wall,
                             "queries_per_s": len(lat) / wall, "residues_per_s": letters * ssum / wall,
                             "batches": c["batches"], "largest_batch": c["largest_batch"],
                             "requeued": c["requeued"]})
            print(json.dumps({"form": form, **res_form[-1]}), file=sys.stderr, flush=True)
        out[form] = res_form
    print(json.dumps(out), flush=True)


def autotune_arm(args):
    """Config-4 sweep: batches (default 1, 8 and 64; --batches) of heavy-tailed queries (lognormal
    median 350, sigma 1.0, 30..35,000 aa) against the 10,000,000-subject database (--subjects for a
    sample); per length bucket the tuner's choice and the achieved subject-stream GB/s of every
    candidate."""
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__ as g
    g.build()
    import hblast
    from hblast import autotune, synth
    n_sub = args.subjects or 10_000_000
    db = synth.large_db(0, n_sub)
    gdb = hblast.Database(db.residues, db.offsets)
    ssum = int(db.offsets[-1])
    report = {"metric": "autotune", "config": {"workload": f"heavy-tailed batches vs {n_sub} subjects ({ssum} residues)"}}
    for nb in (int(x) for x in args.batches.split(",")):
        qs = synth.heavy_tailed_queries(nb, nb)
        pqs = [hblast.ProteinQuery.blastp(q) for q in qs]
        table = autotune.tune(gdb, pqs, ssum, reps=1)
        report[f"batch_{nb}"] = [{"bucket": [t.lo, t.hi], "n_queries": t.n_queries,
                                  "best": None if t.best is None else t.best.__dict__,
                                  "rows": t.rows} for t in table]
        print(json.dumps({"batch": nb, "buckets": report[f"batch_{nb}"]}), file=sys.stderr, flush=True)
    print(json.dumps(report), flush=True)


def ingest_arm(args):
    """Opening the batched workload's database from NCBI BLAST files (three format-4 volumes under
    an alias, in the page cache) into device memory, against opening it from host arrays and
    against reading the files into host arrays only."""
    import shutil
    import tempfile
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__ as g
    g.build()
    import hblast
    from hblast import blastdb, synth
    _, db = synth.batched_blastp(seed=0, n_queries=1, n_subjects=args.subjects or 2_000_000)
    tmp = tempfile.mkdtemp(prefix="hbg_ingest_")
    try:
        names = blastdb.write(os.path.join(tmp, "db"), db.residues, db.offsets, volume_residues=256 << 20)
        path = os.path.join(tmp, "db")
        psq_bytes = sum(os.path.getsize(os.path.join(tmp, n + ".psq")) for n in names)

        def timed(fn):
            for _ in range(args.warmup):
                fn()
            ts = []
            for _ in range(args.steps):
                torch.cuda.synchronize()
                t = time.perf_counter()
                fn()
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t)
            return float(np.median(ts))

        t_files = timed(lambda: hblast.Database.from_blastdb(path).close())
        t_arrays = timed(lambda: hblast.Database(db.residues, db.offsets).close())
        t_host = timed(lambda: hblast.blastdb_read(path))
        # the two resident databases search alike
        a, b = hblast.Database(db.residues, db.offsets), hblast.Database.from_blastdb(path)
        same = a.info()[:2] == b.info()[:2]
        a.close(), b.close()
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    gbs = psq_bytes / t_files / 1e9
    print(json.dumps({
        "metric": "database ingest GB/s", "value": gbs, "unit": "GB/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_files * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded; BLOSUM62-implied background)",
        "config": {"workload": f"hbg_db_open_blastdb of {len(names)} format-4 volumes ({psq_bytes} .psq bytes, "
                               f"{db.n} subjects) from the page cache, open + close per step",
                   "same_counts_as_arrays": same},
        "from_arrays_ms": t_arrays * 1e3, "from_arrays_gbs": psq_bytes / t_arrays / 1e9,
        "host_read_only_ms": t_host * 1e3, "host_read_only_gbs": psq_bytes / t_host / 1e9,
    }), flush=True)


# --------------------------------------------------------------------------- GPU arm

def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        reference_arm(args)
        return
    if args.config == "served":
        served_arm(args)
        return
    if args.config == "autotune":
        autotune_arm(args)
        return
    if args.config == "ingest":
        ingest_arm(args)
        return
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)

    import __graft_entry__ as g
    g.build()
    import hblast

    qs, db, desc = workload(args.config, rank, args.subjects, args.queries)
    blastx = args.config == "blastx"
    qsum = int(sum(frame_letters(len(q)) if blastx else len(q) for q in qs))
    ssum = int(db.offsets[-1])
    units_per_step = float(qsum) * float(ssum)
    opts = hblast.default_options(method=0)
    gdb = hblast.Database(db.residues, db.offsets, opts)
    if blastx:
        xd6 = np.full((1, 6), 16, np.int32)
        cu6 = np.full((1, 6), 41, np.int32)
        pqs = list(qs)

        def batch_of(specs, max_group_len=args.group_len):
            n = len(specs)
            b = hblast.Batch.blastx(specs, np.repeat(xd6, n, 0), np.repeat(cu6, n, 0), max_group_len=max_group_len)
            return b.set_mode(args.mode) if args.mode >= 0 else b
    else:
        pqs = [hblast.ProteinQuery.blastp(q) for q in qs]

        def batch_of(specs, max_group_len=args.group_len):
            b = hblast.Batch.proteins(specs, max_group_len=max_group_len)
            return b.set_mode(args.mode) if args.mode >= 0 else b
    batch = batch_of(pqs)
    binfo = batch.info()
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream

    # warm-up (also sizes the HSP buffer so that no timed step relaunches)
    s = hblast.Searcher(gdb, batch, opts)
    for _ in range(max(args.warmup, 1)):
        s.launch(sptr)
        s.sync()
    n_hsps = s.n_hsps()
    s.close()
    s = hblast.Searcher(gdb, batch, opts, hsp_capacity=max(int(n_hsps * 1.1) + 1024, 1 << 20))
    for _ in range(args.warmup):
        s.launch(sptr)
        s.sync()

    # timed region: device-resident inputs, events on the launching stream
    clocks = Clocks(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    wf_ms, ord_ms = [], []
    ev0.record(stream)
    for _ in range(args.steps):
        s.launch(sptr)
        s.sync()
        a, b, launches = s.timing()
        wf_ms.append(a)
        ord_ms.append(b)
    ev1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    elapsed = ev0.elapsed_time(ev1) / 1e3
    if dist:
        t = torch.tensor([elapsed], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
        dist.barrier()
    value = units_per_step * args.steps * world / elapsed
    ms_step = elapsed / args.steps * 1e3
    s.wait()
    res = s.result()
    n_hsps = len(res.hsps)
    stats = res.stats
    hits = sum(st["lookup_hits"] for st in stats)
    ext = sum(st["init_extends"] for st in stats)
    s.close()

    # roofline of the word-finder kernel (HBM-bound subject stream)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    wf_avg = sum(wf_ms) / len(wf_ms) / 1e3
    alg_bytes = ssum + 8 * db.n + HSP_BYTES * n_hsps
    achieved = alg_bytes / wf_avg / 1e9
    traffic = None
    tfile = ROOT / "profiles" / "wordfinder_traffic.json"
    if tfile.exists():
        try:
            tj = json.loads(tfile.read_text())
            if tj.get("config") == args.config:
                traffic = tj.get("dram_bytes_per_launch")
        except ValueError:
            pass

    # one-query-per-launch form (the plain GPU form) on the same database
    plain = None
    if not args.no_plain and args.config in ("batched", "blastx"):
        single = [batch_of([p]) for p in pqs]
        sss = [hblast.Searcher(gdb, b1, opts) for b1 in single]
        for x in sss:
            x.launch(sptr)
            x.sync()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        reps = 2
        for _ in range(reps):
            for x in sss:
                x.launch(sptr)
                x.sync()
        torch.cuda.synchronize()
        tp = (time.perf_counter() - t0) / reps
        plain = {"value": units_per_step * world / tp, "unit": UNIT, "ms_per_step": tp * 1e3,
                 "form": f"{len(pqs)} launches, one query each, same database"}
        for x in sss:
            x.close()
        for b1 in single:
            b1.close()

    # end to end through the public API: host queries in, ordered HSPs out
    e2e = None
    if not args.no_e2e:
        times = []
        h2d = d2h = 0
        for i in range(1 + max(1, args.steps // 3)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b2 = batch_of(pqs)
            r2 = hblast.search(gdb, b2, opts, hsp_capacity=max(int(n_hsps * 1.1) + 1024, 1 << 20), stream=sptr)
            h2d = b2.info()["device_bytes"]
            b2.close()
            torch.cuda.synchronize()
            if i > 0:
                times.append(time.perf_counter() - t0)
            d2h = HSP_BYTES * len(r2.hsps) + 8 * (1 + 4 * len(pqs))
        te = sum(times) / len(times)
        e2e = {"value": units_per_step * world / te, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": te * 1e3,
               "path": "hbg_batch_create (host lookup tables) + hbg_search + hbg_result_wait"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        cs = CpuSample(qs, db, threads, blastx=blastx)
        cs.run()                                   # warm-up pass
        ts = []
        while len(ts) < 3 or (sum(ts) < args.cpu_seconds and len(ts) < 20):
            ts.append(cs.run())
        t = sum(ts) / len(ts)
        cpu = {"value": cs.rate(t), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{cs.sample}; mean of {len(ts)} passes ({sum(ts):.1f} s)",
               "what": "C restatement of the NCBI BLAST+ 2.2.28 two-hit word finder (oracle/)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded; BLOSUM62-implied background)",
            "config": dict(desc, queries=len(qs), query_residues=qsum, subjects=db.n, subject_residues=ssum,
                           groups=binfo["n_groups"], l2="inputs larger than L2 (database > 129 MB)",
                           parallelism=f"replicas x{world}, subjects sharded per rank (no collective)"),
            "gpu_launches": int(launches) * args.steps,
            "clocks": ck,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                         "kernel": "wordfinder_kernel", "kernel_ms": wf_avg * 1e3,
                         "algorithmic_bytes": int(alg_bytes)},
            "lookup_hits_per_s": hits / wf_avg, "extensions_per_s": ext / wf_avg,
            "hsps": n_hsps, "ordering_ms": sum(ord_ms) / len(ord_ms),
            "e2e": e2e, "plain": plain,
            "batched_over_plain": (value / plain["value"]) if plain else None,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
