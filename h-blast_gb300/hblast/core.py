"""ctypes binding of the C ABI in include/hblast_gpu.h.

The library is the compiled CUDA path; there is no Python or CPU fallback.
Loading fails loudly when libhblast_gb300.so is missing.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path
from typing import Sequence

import numpy as np

from ._build import LIB_PATH

HBG_OK = 0
HBG_ERR_INVALID = -1
HBG_ERR_CUDA = -2
HBG_ERR_NOMEM = -3
HBG_ERR_TOO_LONG = -4
HBG_ERR_NO_DEVICE = -5
HBG_ERR_STATE = -6
HBG_ERR_CAPACITY = -7

HSP_DTYPE = np.dtype([(n, np.int32) for n in
                      ("query", "subject", "q_start", "s_start", "q_off", "s_off", "len", "score", "context")])


class HblastError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class _Query(C.Structure):
    _fields_ = [("sequence", C.POINTER(C.c_uint8)), ("length", C.c_int32), ("num_contexts", C.c_int32),
                ("context_offset", C.POINTER(C.c_int32)), ("context_length", C.POINTER(C.c_int32)),
                ("x_dropoff", C.POINTER(C.c_int32)), ("cutoff_score", C.POINTER(C.c_int32))]


class _WordParams(C.Structure):
    _fields_ = [("threshold", C.c_int32), ("window", C.c_int32)]


class GpuOptions(C.Structure):
    """Mirror of BlastGPUOptions: -gpu, -gpu_blocks, -gpu_threads, -method, -num_threads."""
    _fields_ = [("use_gpu", C.c_int32), ("num_blocksx", C.c_int32), ("num_threadsx", C.c_int32),
                ("method", C.c_int32), ("cpu_threads", C.c_int32)]


class SegParams(C.Structure):
    """hbg_seg_params: SEG window and complexity cut-offs (bits)."""
    _fields_ = [("window", C.c_int32), ("pad", C.c_int32), ("locut", C.c_double), ("hicut", C.c_double)]


def seg_params(window: int = 12, locut: float = 2.2, hicut: float = 2.5) -> SegParams:
    return SegParams(window, 0, locut, hicut)


def seg_mask(seq: np.ndarray, window: int = 12, locut: float = 2.2, hicut: float = 2.5) -> np.ndarray:
    """SEG-masked copy of an NCBIstdaa protein sequence (masked letters become X = 21)."""
    out = np.ascontiguousarray(seq, dtype=np.uint8).copy()
    n = C.c_int64()
    p = seg_params(window, locut, hicut)
    _check(lib().hbg_seg_mask(out.ctypes.data, len(out), C.byref(p), C.byref(n)))
    return out


class RuntimeOptions(C.Structure):
    _fields_ = [("gpu_db_used_ratio", C.c_double), ("fixed_ratio", C.c_int32), ("ccr", C.c_double),
                ("avg_hsps_per_sequence", C.c_int32), ("mem_ecc", C.c_int32), ("balancer_method", C.c_int32),
                ("load_factor", C.c_int32), ("chunk_size", C.c_int32), ("base_value", C.c_int32)]


class ServerOptions(C.Structure):
    """hbg_server_options: slots in flight, queries per batch, memory budget, group length, letters per
    batch, shortest-first admission age, SEG masking of BLASTX frames."""
    _fields_ = [("max_inflight", C.c_int32), ("max_batch_queries", C.c_int32), ("memory_budget", C.c_int64),
                ("max_group_len", C.c_int32), ("max_batch_letters", C.c_int32), ("shortest_first_ms", C.c_int32),
                ("seg_blastx", C.c_int32)]


class QueryStats(C.Structure):
    _fields_ = [("lookup_hits", C.c_int64), ("init_extends", C.c_int64), ("good_init_extends", C.c_int64),
                ("subjects_passed", C.c_int64)]


# Entry points and their argument types, exactly as declared in include/hblast_gpu.h.
_P = C.c_void_p
_SIGS = {
    "hbg_last_error": ([], C.c_char_p),
    "hbg_device_count": ([C.POINTER(C.c_int32)], C.c_int),
    "hbg_default_gpu_options": ([C.POINTER(GpuOptions)], C.c_int),
    "hbg_read_runtime_options": ([C.c_char_p, C.POINTER(RuntimeOptions)], C.c_int),
    "hbg_db_open": ([_P, _P, C.c_int32, C.POINTER(GpuOptions), C.POINTER(_P)], C.c_int),
    "hbg_db_close": ([_P], C.c_int),
    "hbg_batch_tune": ([_P, C.c_int32, C.c_int32], C.c_int),
    "hbg_blastdb_info": ([C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                          C.POINTER(C.c_int32)], C.c_int),
    "hbg_blastdb_read": ([C.c_char_p, _P, _P], C.c_int),
    "hbg_db_open_blastdb": ([C.c_char_p, C.POINTER(GpuOptions), C.POINTER(_P)], C.c_int),
    "hbg_db_info": ([_P, C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_int64)], C.c_int),
    "hbg_batch_create": ([C.POINTER(_Query), C.c_int32, C.POINTER(_WordParams), C.c_int32, C.POINTER(_P)], C.c_int),
    "hbg_batch_create_blastx": ([C.POINTER(C.POINTER(C.c_uint8)), C.POINTER(C.c_int32), C.c_int32,
                                 C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(_WordParams), C.c_int32,
                                 C.POINTER(_P)], C.c_int),
    "hbg_batch_create_blastx_masked": ([C.POINTER(C.POINTER(C.c_uint8)), C.POINTER(C.c_int32), C.c_int32,
                                        C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(_WordParams),
                                        C.c_void_p, C.c_int32, C.POINTER(_P)], C.c_int),
    "hbg_seg_default_params": ([C.c_void_p], C.c_int),
    "hbg_seg_mask": ([_P, C.c_int32, C.c_void_p, C.POINTER(C.c_int64)], C.c_int),
    "hbg_batch_create_from_smallbone": ([C.POINTER(_Query), C.POINTER(_WordParams), _P, C.c_int32, _P,
                                         C.c_int64, C.POINTER(_P)], C.c_int),
    "hbg_batch_lookup_table": ([_P, C.c_int32, _P, _P, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                C.POINTER(C.c_int32), _P], C.c_int),
    "hbg_batch_set_mode": ([_P, C.c_int32, C.c_int32], C.c_int),
    "hbg_batch_schedule": ([_P, C.c_int32, C.c_int64], C.c_int),
    "hbg_batch_destroy": ([_P], C.c_int),
    "hbg_batch_info": ([_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                        C.POINTER(C.c_int64), C.POINTER(C.c_int64)], C.c_int),
    "hbg_mem_required": ([_P, _P, C.c_int64, C.POINTER(C.c_int64)], C.c_int),
    "hbg_search": ([_P, _P, C.POINTER(GpuOptions), C.c_int64, _P, C.POINTER(_P)], C.c_int),
    "hbg_result_wait": ([_P], C.c_int),
    "hbg_result_sync": ([_P], C.c_int),
    "hbg_result_timing": ([_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_int32)], C.c_int),
    "hbg_result_counts": ([_P, C.POINTER(C.c_int64), C.POINTER(C.c_int32)], C.c_int),
    "hbg_result_hsps": ([_P, C.c_int64, C.c_int64, _P], C.c_int),
    "hbg_result_query_range": ([_P, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_int64)], C.c_int),
    "hbg_result_stats": ([_P, C.c_int32, C.POINTER(QueryStats)], C.c_int),
    "hbg_result_free": ([_P], C.c_int),
    "hbg_search_sync": ([_P, _P, C.POINTER(GpuOptions), _P, C.c_int64, C.POINTER(C.c_int64),
                         C.POINTER(QueryStats), _P], C.c_int),
    "hbg_search_static": ([_P, _P, C.POINTER(GpuOptions), _P, C.c_int64, _P, _P], C.c_int),
    "hbg_server_default_options": ([C.c_void_p], C.c_int),
    "hbg_server_create": ([_P, C.POINTER(_WordParams), C.POINTER(GpuOptions), C.c_void_p, C.POINTER(_P)], C.c_int),
    "hbg_server_submit": ([_P, C.POINTER(_Query), C.POINTER(C.c_int64)], C.c_int),
    "hbg_server_submit_blastx": ([_P, _P, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                  C.POINTER(C.c_int64)], C.c_int),
    "hbg_server_wait": ([_P, C.c_int64, C.c_int32, C.POINTER(C.c_int64)], C.c_int),
    "hbg_server_take": ([_P, C.c_int64, _P, C.c_int64, C.POINTER(QueryStats), C.POINTER(C.c_double)], C.c_int),
    "hbg_server_counters": ([_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)], C.c_int),
    "hbg_server_requeued": ([_P, C.POINTER(C.c_int64)], C.c_int),
    "hbg_server_destroy": ([_P], C.c_int),
    "hbg_debug_fail_allocations": ([C.c_int32], C.c_int),
}

_lib = None


def library_path() -> Path:
    return LIB_PATH


def lib() -> C.CDLL:
    """Load libhblast_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise HblastError(HBG_ERR_STATE, f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = C.CDLL(str(LIB_PATH))
        for name, (args, res) in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != HBG_OK:
        raise HblastError(rc, lib().hbg_last_error().decode(errors="replace"))


def _i32p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def device_count() -> int:
    n = C.c_int32(0)
    rc = lib().hbg_device_count(C.byref(n))
    return n.value if rc == HBG_OK else 0


def fail_allocations(count: int) -> None:
    """Test hook (hbg_debug_fail_allocations): the library's next `count` device
    allocations fail as if the device were out of memory."""
    _check(lib().hbg_debug_fail_allocations(count))


def default_options(**kw) -> GpuOptions:
    o = GpuOptions()
    _check(lib().hbg_default_gpu_options(C.byref(o)))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def read_runtime_options(path: str | None) -> RuntimeOptions:
    o = RuntimeOptions()
    _check(lib().hbg_read_runtime_options(path.encode() if path else None, C.byref(o)))
    return o


@dataclass
class ProteinQuery:
    """One query as NCBI concatenates it: contexts separated by one sentinel."""
    sequence: np.ndarray                     # uint8 NCBIstdaa
    context_offset: Sequence[int]
    context_length: Sequence[int]
    x_dropoff: Sequence[int]
    cutoff_score: Sequence[int]

    @classmethod
    def blastp(cls, seq: np.ndarray, x_dropoff: int = 16, cutoff: int = 41) -> "ProteinQuery":
        seq = np.ascontiguousarray(seq, dtype=np.uint8)
        return cls(seq, [0], [len(seq)], [x_dropoff], [cutoff])

    @property
    def length(self) -> int:
        return int(self.context_offset[-1] + self.context_length[-1])


def blastdb_info(path) -> dict:
    """Counts of an NCBI BLAST protein database without reading its sequences."""
    n, r, m, v = C.c_int32(), C.c_int64(), C.c_int32(), C.c_int32()
    _check(lib().hbg_blastdb_info(str(path).encode(), C.byref(n), C.byref(r), C.byref(m), C.byref(v)))
    return dict(n_subjects=n.value, n_residues=r.value, max_len=m.value, n_volumes=v.value)


def blastdb_read(path):
    """(residues, offsets) of an NCBI BLAST protein database, in Database's input form."""
    info = blastdb_info(path)
    res = np.zeros(max(info["n_residues"], 1), dtype=np.uint8)
    off = np.zeros(info["n_subjects"] + 1, dtype=np.int64)
    _check(lib().hbg_blastdb_read(str(path).encode(), res.ctypes.data, off.ctypes.data))
    return res[:info["n_residues"]], off


class Database:
    """Subjects resident in device memory (hbg_db_open, or hbg_db_open_blastdb via from_blastdb)."""

    def __init__(self, residues: np.ndarray, offsets: np.ndarray, options: GpuOptions | None = None):
        self.residues = np.ascontiguousarray(residues, dtype=np.uint8)
        self.offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        n = len(self.offsets) - 1
        h = C.c_void_p()
        _check(lib().hbg_db_open(self.residues.ctypes.data, self.offsets.ctypes.data, n,
                                 C.byref(options) if options is not None else None, C.byref(h)))
        self.handle = h
        self.n_subjects = n

    @classmethod
    def from_blastdb(cls, path, options: GpuOptions | None = None) -> "Database":
        """Open an NCBI BLAST protein database (.pal or .pin/.psq) straight into device memory."""
        self = cls.__new__(cls)
        h = C.c_void_p()
        _check(lib().hbg_db_open_blastdb(str(path).encode(), C.byref(options) if options is not None else None,
                                         C.byref(h)))
        self.handle = h
        self.residues = self.offsets = None
        self.n_subjects = self.info()[0]
        return self

    def info(self):
        n, r, b = C.c_int32(), C.c_int64(), C.c_int64()
        _check(lib().hbg_db_info(self.handle, C.byref(n), C.byref(r), C.byref(b)))
        return n.value, r.value, b.value

    def close(self):
        if self.handle:
            _check(lib().hbg_db_close(self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Packed queries and their lookup tables (hbg_batch_create*)."""

    def __init__(self, handle, n_queries: int, keep=None):
        self.handle = handle
        self.n_queries = n_queries
        self._keep = keep

    @classmethod
    def proteins(cls, queries: Sequence[ProteinQuery], threshold: int = 11, window: int = 40,
                 max_group_len: int = 0) -> "Batch":
        n = len(queries)
        arr = (_Query * n)()
        keep = []
        for i, q in enumerate(queries):
            seq = np.ascontiguousarray(q.sequence, dtype=np.uint8)
            co = np.ascontiguousarray(q.context_offset, dtype=np.int32)
            cl = np.ascontiguousarray(q.context_length, dtype=np.int32)
            xd = np.ascontiguousarray(q.x_dropoff, dtype=np.int32)
            cu = np.ascontiguousarray(q.cutoff_score, dtype=np.int32)
            keep += [seq, co, cl, xd, cu]
            arr[i] = _Query(seq.ctypes.data_as(C.POINTER(C.c_uint8)), q.length, len(co), _i32p(co), _i32p(cl),
                            _i32p(xd), _i32p(cu))
        wp = _WordParams(threshold, window)
        h = C.c_void_p()
        _check(lib().hbg_batch_create(arr, n, C.byref(wp), max_group_len, C.byref(h)))
        return cls(h, n)

    @classmethod
    def blastx(cls, nt_queries: Sequence[np.ndarray], x_dropoff: np.ndarray, cutoff: np.ndarray,
               threshold: int = 11, window: int = 40, max_group_len: int = 0, seg=None) -> "Batch":
        """seg: None (no masking), True (SEG 12 2.2 2.5 on every frame) or a SegParams."""
        n = len(nt_queries)
        nts = [np.ascontiguousarray(q, dtype=np.uint8) for q in nt_queries]
        ptrs = (C.POINTER(C.c_uint8) * n)(*[q.ctypes.data_as(C.POINTER(C.c_uint8)) for q in nts])
        lens = np.array([len(q) for q in nts], dtype=np.int32)
        xd = np.ascontiguousarray(x_dropoff, dtype=np.int32).reshape(-1)
        cu = np.ascontiguousarray(cutoff, dtype=np.int32).reshape(-1)
        wp = _WordParams(threshold, window)
        h = C.c_void_p()
        sp = seg_params() if seg is True else seg
        _check(lib().hbg_batch_create_blastx_masked(ptrs, _i32p(lens), n, _i32p(xd), _i32p(cu), C.byref(wp),
                                                    C.byref(sp) if sp is not None else None, max_group_len,
                                                    C.byref(h)))
        return cls(h, n)

    @classmethod
    def from_smallbone(cls, query: ProteinQuery, backbone: np.ndarray, overflow: np.ndarray,
                       threshold: int = 11, window: int = 40) -> "Batch":
        seq = np.ascontiguousarray(query.sequence, dtype=np.uint8)
        co = np.ascontiguousarray(query.context_offset, dtype=np.int32)
        cl = np.ascontiguousarray(query.context_length, dtype=np.int32)
        xd = np.ascontiguousarray(query.x_dropoff, dtype=np.int32)
        cu = np.ascontiguousarray(query.cutoff_score, dtype=np.int32)
        q = _Query(seq.ctypes.data_as(C.POINTER(C.c_uint8)), query.length, len(co), _i32p(co), _i32p(cl),
                   _i32p(xd), _i32p(cu))
        bb = np.ascontiguousarray(backbone)
        ov = np.ascontiguousarray(overflow, dtype=np.uint16)
        wp = _WordParams(threshold, window)
        h = C.c_void_p()
        _check(lib().hbg_batch_create_from_smallbone(C.byref(q), C.byref(wp), bb.ctypes.data,
                                                     len(bb), ov.ctypes.data, len(ov), C.byref(h)))
        return cls(h, 1)

    def info(self):
        nq, ng, ql, ne, db = C.c_int32(), C.c_int32(), C.c_int64(), C.c_int64(), C.c_int64()
        _check(lib().hbg_batch_info(self.handle, C.byref(nq), C.byref(ng), C.byref(ql), C.byref(ne), C.byref(db)))
        return dict(n_queries=nq.value, n_groups=ng.value, total_query_len=ql.value, lookup_entries=ne.value,
                    device_bytes=db.value)

    def lookup_table(self, g: int):
        """(cells[32769] uint32, entries uint16, first_query, query_starts) of group g."""
        n = C.c_int64()
        fq, nq = C.c_int32(), C.c_int32()
        cells = np.zeros(32769, dtype=np.uint32)
        _check(lib().hbg_batch_lookup_table(self.handle, g, cells.ctypes.data, None, 0, C.byref(n), C.byref(fq),
                                            C.byref(nq), None))
        ent = np.zeros(max(n.value, 1), dtype=np.uint16)
        qs = np.zeros(max(nq.value, 1), dtype=np.int32)
        _check(lib().hbg_batch_lookup_table(self.handle, g, cells.ctypes.data, ent.ctypes.data, len(ent),
                                            C.byref(n), C.byref(fq), C.byref(nq), qs.ctypes.data))
        return cells, ent[:n.value], fq.value, qs[:nq.value]

    def tune(self, tile_subjects: int = 0, global_tables: bool = False) -> "Batch":
        """hbg_batch_tune: subjects per work unit (0 = automatic), diagonal tables in global memory."""
        _check(lib().hbg_batch_tune(self.handle, tile_subjects, int(global_tables)))
        return self

    def schedule(self, warps_per_subject: int = 1, tile_bytes: int = 0) -> "Batch":
        """Groups sharing each pass over a subject, and work-unit size in subject letters (before the
        first search)."""
        _check(lib().hbg_batch_schedule(self.handle, warps_per_subject, tile_bytes))
        return self

    def set_mode(self, mode: int, group: int = -1) -> "Batch":
        """0 = chunk mode, 1 = offset mode, for one group or all (before the first search)."""
        _check(lib().hbg_batch_set_mode(self.handle, group, mode))
        return self

    def close(self):
        if self.handle:
            _check(lib().hbg_batch_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class SearchResult:
    hsps: np.ndarray                          # HSP_DTYPE, reference order
    stats: list = field(default_factory=list)  # per query dicts
    wordfinder_ms: float = 0.0
    ordering_ms: float = 0.0

    def for_query(self, q: int) -> np.ndarray:
        return self.hsps[self.hsps["query"] == q]


class Searcher:
    """Repeated searches of one batch against one database, reusing buffers."""

    def __init__(self, db: Database, batch: Batch, options: GpuOptions | None = None, hsp_capacity: int = 0):
        self.db, self.batch = db, batch
        self.options = options if options is not None else default_options()
        self.capacity = hsp_capacity
        self.res = C.c_void_p()

    def launch(self, stream: int | None = None) -> None:
        _check(lib().hbg_search(self.db.handle, self.batch.handle, C.byref(self.options), self.capacity,
                                C.c_void_p(stream) if stream else None, C.byref(self.res)))

    def wait(self) -> None:
        """Wait, order and copy the HSPs to the host."""
        _check(lib().hbg_result_wait(self.res))

    def sync(self) -> None:
        """Wait for the device work only (HSPs stay in device memory)."""
        _check(lib().hbg_result_sync(self.res))

    def n_hsps(self) -> int:
        n, q = C.c_int64(), C.c_int32()
        _check(lib().hbg_result_counts(self.res, C.byref(n), C.byref(q)))
        return n.value

    def timing(self):
        """(word-finder ms, ordering ms, kernels launched per search)."""
        a, b, n = C.c_float(), C.c_float(), C.c_int32()
        _check(lib().hbg_result_timing(self.res, C.byref(a), C.byref(b), C.byref(n)))
        return a.value, b.value, n.value

    def result(self) -> SearchResult:
        n = self.n_hsps()
        out = np.empty(n, dtype=HSP_DTYPE)
        if n:
            _check(lib().hbg_result_hsps(self.res, 0, n, out.ctypes.data))
        stats = []
        for q in range(self.batch.n_queries):
            s = QueryStats()
            _check(lib().hbg_result_stats(self.res, q, C.byref(s)))
            stats.append(dict(lookup_hits=s.lookup_hits, init_extends=s.init_extends,
                              good_init_extends=s.good_init_extends, subjects_passed=s.subjects_passed))
        wf, od, _ = self.timing()
        return SearchResult(out, stats, wf, od)

    def query_range(self, q: int):
        f, c = C.c_int64(), C.c_int64()
        _check(lib().hbg_result_query_range(self.res, q, C.byref(f), C.byref(c)))
        return f.value, c.value

    def close(self):
        if self.res:
            _check(lib().hbg_result_free(self.res))
            self.res = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching request loop over a resident database (hbg_server_*)."""

    def __init__(self, db: Database, threshold: int = 11, window: int = 40, options: GpuOptions | None = None,
                 **server_options):
        so = ServerOptions()
        _check(lib().hbg_server_default_options(C.byref(so)))
        for k, v in server_options.items():
            setattr(so, k, v)
        wp = _WordParams(threshold, window)
        h = C.c_void_p()
        _check(lib().hbg_server_create(db.handle, C.byref(wp), C.byref(options) if options is not None else None,
                                       C.byref(so), C.byref(h)))
        self.handle = h
        self.db = db

    def submit(self, q: ProteinQuery) -> int:
        seq = np.ascontiguousarray(q.sequence, dtype=np.uint8)
        co = np.ascontiguousarray(q.context_offset, dtype=np.int32)
        cl = np.ascontiguousarray(q.context_length, dtype=np.int32)
        xd = np.ascontiguousarray(q.x_dropoff, dtype=np.int32)
        cu = np.ascontiguousarray(q.cutoff_score, dtype=np.int32)
        cq = _Query(seq.ctypes.data_as(C.POINTER(C.c_uint8)), q.length, len(co), _i32p(co), _i32p(cl), _i32p(xd),
                    _i32p(cu))
        t = C.c_int64()
        _check(lib().hbg_server_submit(self.handle, C.byref(cq), C.byref(t)))
        return t.value

    def submit_blastx(self, nt: np.ndarray, x_dropoff, cutoff) -> int:
        nt = np.ascontiguousarray(nt, dtype=np.uint8)
        xd = np.ascontiguousarray(x_dropoff, dtype=np.int32)
        cu = np.ascontiguousarray(cutoff, dtype=np.int32)
        t = C.c_int64()
        _check(lib().hbg_server_submit_blastx(self.handle, nt.ctypes.data, len(nt), _i32p(xd), _i32p(cu),
                                              C.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> int:
        n = C.c_int64()
        _check(lib().hbg_server_wait(self.handle, ticket, timeout_ms, C.byref(n)))
        return n.value

    def take(self, ticket: int):
        """(hsps, stats dict, latency ms) of a finished request."""
        n = self.wait(ticket)
        out = np.zeros(n, dtype=HSP_DTYPE)
        st = QueryStats()
        lat = C.c_double()
        _check(lib().hbg_server_take(self.handle, ticket, out.ctypes.data if n else None, n, C.byref(st),
                                     C.byref(lat)))
        return out, dict(lookup_hits=st.lookup_hits, init_extends=st.init_extends,
                         good_init_extends=st.good_init_extends, subjects_passed=st.subjects_passed), lat.value

    def counters(self):
        b, q, l, rq = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        _check(lib().hbg_server_counters(self.handle, C.byref(b), C.byref(q), C.byref(l)))
        _check(lib().hbg_server_requeued(self.handle, C.byref(rq)))
        return dict(batches=b.value, queries=q.value, largest_batch=l.value, requeued=rq.value)

    def close(self):
        if self.handle:
            _check(lib().hbg_server_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def search(db: Database, batch: Batch, options: GpuOptions | None = None, hsp_capacity: int = 0,
           stream: int | None = None) -> SearchResult:
    s = Searcher(db, batch, options, hsp_capacity)
    try:
        s.launch(stream)
        s.wait()
        return s.result()
    finally:
        s.close()
