// api.cu -- the C ABI (include/hblast_gpu.h): resident database, batches,
// search launch, ordering and result collection.
//
// Replaces H-BLAST's host runtime (h_blast_v1.1/H-BLAST/h_blast.cu): no
// process-static state, no exit() on error, the database uploaded once and
// kept resident, every launch on a caller-chosen stream.
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "../host/batch_builder.h"
#include "../host/blastdb.h"
#include "kernels.h"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

#define CU(call)                                                                  \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess)                                                    \
            return fail(e_ == cudaErrorMemoryAllocation ? HBG_ERR_NOMEM : HBG_ERR_CUDA, \
                        std::string(#call) + ": " + cudaGetErrorString(e_));      \
    } while (0)

int bits_for(int64_t v) {
    int b = 0;
    while (v > 0) {
        ++b;
        v >>= 1;
    }
    return b;
}

// Device allocations of batches and search results go through a small
// per-device cache: blocks freed while idle are kept (up to kPoolBytes per
// device, blocks of up to kPoolBlock) and handed out again for requests of
// at least half their size, so repeated small searches do not pay for
// cudaMalloc / cudaFree each time.  Large blocks (databases) are not kept.
constexpr size_t kPoolBytes = (size_t)2 << 30;
constexpr size_t kPoolBlock = (size_t)512 << 20;

struct DevicePool {
    std::mutex mu;
    std::map<void *, size_t> size_of;                 // every live allocation
    std::map<int, std::multimap<size_t, void *>> idle; // per device, by size
    std::map<int, size_t> idle_bytes;
};
DevicePool &pool() {
    static DevicePool *p = new DevicePool;   // never destroyed: frees may run at exit
    return *p;
}

// Allocation failures injected for tests (hbg_debug_fail_allocations): the
// next this many dalloc calls report cudaErrorMemoryAllocation.
std::atomic<int32_t> g_fail_allocs{0};

template <class T>
cudaError_t dalloc(T **p, size_t n) {
    *p = nullptr;
    for (int32_t k = g_fail_allocs.load(); k > 0;)
        if (g_fail_allocs.compare_exchange_weak(k, k - 1))
            return cudaErrorMemoryAllocation;
    if (n == 0)
        n = 1;
    const size_t bytes = n * sizeof(T);
    int dev = 0;
    cudaGetDevice(&dev);
    DevicePool &P = pool();
    {
        std::lock_guard<std::mutex> lock(P.mu);
        auto &idle = P.idle[dev];
        auto it = idle.lower_bound(bytes);
        if (it != idle.end() && it->first <= 2 * bytes) {
            *p = (T *)it->second;
            P.idle_bytes[dev] -= it->first;
            idle.erase(it);
            return cudaSuccess;
        }
    }
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();   // a failed allocation must not surface at a later launch check
        return e;
    }
    std::lock_guard<std::mutex> lock(P.mu);
    P.size_of[q] = bytes;
    *p = (T *)q;
    return cudaSuccess;
}

// Free now (cudaFree waits for the device).
template <class T>
void dfree(T *&p) {
    if (p) {
        {
            DevicePool &P = pool();
            std::lock_guard<std::mutex> lock(P.mu);
            P.size_of.erase((void *)p);
        }
        cudaFree(p);
    }
    p = nullptr;
}

// Give back a block that no GPU work still uses (the caller has synchronised):
// kept for reuse when it fits the cache, else freed.
template <class T>
void dfree_idle(T *&p) {
    if (!p)
        return;
    int dev = 0;
    cudaGetDevice(&dev);
    DevicePool &P = pool();
    bool keep = false;
    {
        std::lock_guard<std::mutex> lock(P.mu);
        auto it = P.size_of.find((void *)p);
        if (it != P.size_of.end() && it->second <= kPoolBlock && P.idle_bytes[dev] + it->second <= kPoolBytes) {
            P.idle[dev].emplace(it->second, (void *)p);
            P.idle_bytes[dev] += it->second;
            keep = true;
        }
    }
    if (!keep)
        dfree(p);
    p = nullptr;
}

// Device guard: make `dev` current for the scope.
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev)
            cudaSetDevice(dev);
    }
    ~DeviceScope() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev)
            cudaSetDevice(prev);
    }
};

}  // namespace

// Databases and batches carry a process-unique id: a new object can reuse a
// freed one's address, so reuse checks and graph keys compare ids, never
// pointers.
static std::atomic<uint64_t> g_next_object_id{1};

// Groups are searched in launch classes: one hit mode and one shared-table
// size per launch, so a long query's large table does not cut the occupancy
// of every other group in its batch.
struct LaunchClass {
    int mode;        // 0 chunk mode, 1 offset mode; + 2 for groups with global tables
    int smem_diag;   // per-warp 16-bit table entries (small for the global class)
    int first;       // groups [first, first + count) of the batch's group list
    int count;
};
struct LaunchShape {
    int threads;
    int blocks;
    int team;        // groups per tile (warps that share each subject)
};
constexpr int kMaxLaunchClasses = 32;

struct hbg_db {
    uint64_t id = g_next_object_id++;
    int device = 0;
    int32_t n = 0;
    int64_t n_res = 0;
    int64_t letters_len = 0;
    int32_t max_len = 0;
    uint8_t *d_letters = nullptr;
    int64_t *d_off = nullptr;
    int32_t *d_len = nullptr;
    int32_t *d_order = nullptr;
    unsigned long long *d_hist = nullptr;
    int64_t bytes = 0;
};

struct hbg_batch {
    uint64_t id = g_next_object_id++;
    hbg::HostBatch host;
    int device = -1;
    HbgGroup *d_groups = nullptr;
    HbgContext *d_ctx = nullptr;
    HbgQueryDesc *d_queries = nullptr;
    uint8_t *d_letters = nullptr;
    int32_t *d_ctx_of = nullptr;
    uint32_t *d_cells = nullptr;
    uint16_t *d_entries = nullptr;
    uint32_t *d_pv = nullptr;
    uint16_t *d_qcells = nullptr;
    int32_t *d_group_list = nullptr;   // groups ordered by launch class
    std::vector<LaunchClass> classes;
    int64_t device_bytes = 0;
    int32_t tile_subjects = 0;   // 0 = automatic (hbg_batch_tune)
    int64_t tile_bytes = 0;      // > 0: tiles of about this many subject letters (hbg_batch_schedule)
    int32_t team = 1;            // groups searched together per pass over a subject (hbg_batch_schedule)
};

struct hbg_result {
    hbg_db *db = nullptr;
    hbg_batch *batch = nullptr;
    hbg_gpu_options opt{};
    cudaStream_t stream = nullptr;
    int device = 0;
    int64_t cap = 0;
    int blocks = 0, threads = 256;   // the largest grid and CTA over launch classes
    std::vector<LaunchShape> shapes; // one per launch class of the batch
    hbg_gpu_options shape_opt{};     // options the shapes were computed for
    // device
    hbg_hsp *d_raw = nullptr, *d_sorted = nullptr;
    unsigned long long *d_counters = nullptr;  // [0]=hsp count, then per query ext, kept, hits; per group
                                               // hits; per query first, end of its HSPs, subjects passed
    unsigned int *d_tile = nullptr;
    uint32_t *d_gdiag = nullptr;
    int64_t gdiag_entries = 0;
    int32_t gdiag_len = 0;   // entries per (CTA, warp) slice of the global diagonal tables
    uint64_t *d_keys = nullptr;
    uint32_t *d_vals = nullptr;
    uint32_t *d_hist = nullptr;
    int64_t sort_cap = 0;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    // host
    unsigned long long *h_counters = nullptr;  // pinned
    size_t n_counters = 0;
    std::vector<hbg_query_stats> stats;
    std::vector<int64_t> q_first, q_count;
    int64_t n_hsps = 0;
    bool launched = false, synced = false, done = false;
    float wf_ms = 0.f, ord_ms = 0.f;
    int32_t launches = 0;   // kernels per search
    int64_t launch_count = 0;
    cudaGraphExec_t graph_exec = nullptr;
    uint64_t db_id = 0, batch_id = 0;   // what the buffers were last prepared for
    long long graph_key[6] = {0, 0, 0, 0, 0, 0};
};

namespace {

int64_t batch_device_bytes(const hbg::HostBatch &h) {
    return (int64_t)(h.groups.size() * sizeof(HbgGroup) + h.contexts.size() * sizeof(HbgContext) +
                     h.queries.size() * sizeof(HbgQueryDesc) + h.letters.size() + h.ctx_of.size() * 4 +
                     h.cells.size() * 4 + h.entries.size() * 2 + h.pv.size() * 4 + h.query_cells.size() * 2);
}

void free_batch_device(hbg_batch *b) {
    dfree_idle(b->d_groups);
    dfree_idle(b->d_ctx);
    dfree_idle(b->d_queries);
    dfree_idle(b->d_letters);
    dfree_idle(b->d_ctx_of);
    dfree_idle(b->d_cells);
    dfree_idle(b->d_entries);
    dfree_idle(b->d_pv);
    dfree_idle(b->d_qcells);
    dfree_idle(b->d_group_list);
}

int upload_batch_buffers(hbg_batch *b, int device);

// Upload at the first search; a failed upload gives back what it allocated,
// so the batch can be searched again later.
int upload_batch(hbg_batch *b, int device) {
    if (b->device == device)
        return HBG_OK;
    if (b->device >= 0)
        return fail(HBG_ERR_STATE, "batch already resident on another device");
    DeviceScope ds(device);
    const int rc = upload_batch_buffers(b, device);
    if (rc != HBG_OK) {
        cudaDeviceSynchronize();   // copies already issued may still read the host vectors
        free_batch_device(b);
        b->device = -1;
    }
    return rc;
}

int upload_batch_buffers(hbg_batch *b, int device) {
    const hbg::HostBatch &h = b->host;
    CU(dalloc(&b->d_groups, h.groups.size()));
    CU(dalloc(&b->d_ctx, h.contexts.size()));
    CU(dalloc(&b->d_queries, h.queries.size()));
    CU(dalloc(&b->d_letters, h.letters.size() + 64));
    CU(dalloc(&b->d_ctx_of, h.ctx_of.size() + 16));
    CU(dalloc(&b->d_cells, h.cells.size()));
    CU(dalloc(&b->d_entries, h.entries.size() + 8));
    CU(dalloc(&b->d_pv, h.pv.size()));
    CU(dalloc(&b->d_qcells, h.query_cells.size()));
    CU(cudaMemcpy(b->d_groups, h.groups.data(), h.groups.size() * sizeof(HbgGroup), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(b->d_ctx, h.contexts.data(), h.contexts.size() * sizeof(HbgContext), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(b->d_queries, h.queries.data(), h.queries.size() * sizeof(HbgQueryDesc), cudaMemcpyHostToDevice));
    CU(cudaMemset(b->d_letters, 0, h.letters.size() + 64));
    CU(cudaMemcpy(b->d_letters, h.letters.data(), h.letters.size(), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(b->d_ctx_of, h.ctx_of.data(), h.ctx_of.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(b->d_cells, h.cells.data(), h.cells.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    if (!h.entries.empty())
        CU(cudaMemcpy(b->d_entries, h.entries.data(), h.entries.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(b->d_pv, h.pv.data(), h.pv.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(b->d_qcells, h.query_cells.data(), h.query_cells.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    {
        // launch classes: (mode, table size); groups with shared tables are
        // launched by table size, so a short query's warps reserve only the
        // shared memory its table needs (the rest is L1 for cells and entries:
        // one 350-aa query vs 10 M subjects 8 % faster than with 2048-entry
        // tables for every group); global-table groups form their own class
        std::vector<std::pair<std::pair<int, int>, int32_t>> keyed;
        for (int32_t g = 0; g < (int32_t)h.groups.size(); ++g) {
            const HbgGroup &G = h.groups[g];
            const int size = G.placement ? 64 : std::max<int>(64, G.diag_len);
            keyed.push_back({{G.mode, size}, g});
        }
        std::stable_sort(keyed.begin(), keyed.end(),
                         [](const auto &x, const auto &y) { return x.first < y.first; });
        std::vector<int32_t> list;
        b->classes.clear();
        for (size_t i = 0; i < keyed.size(); ++i) {
            const bool global = h.groups[keyed[i].second].placement != 0;
            if (i == 0 || keyed[i].first != keyed[i - 1].first)
                b->classes.push_back(LaunchClass{keyed[i].first.first + (global ? 2 : 0), keyed[i].first.second,
                                                 (int)i, 0});
            b->classes.back().count++;
            list.push_back(keyed[i].second);
        }
        if ((int)b->classes.size() > kMaxLaunchClasses)
            return fail(HBG_ERR_INVALID, "too many launch classes");
        CU(dalloc(&b->d_group_list, list.size()));
        CU(cudaMemcpy(b->d_group_list, list.data(), list.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    }
    b->device_bytes = batch_device_bytes(h);
    b->device = device;
    return HBG_OK;
}

// Length of the per-warp global diagonal table: groups too long for shared
// memory, and subjects whose offsets do not fit the 16-bit shared cells
// (window + length > 32767), use it.
int32_t global_diag_len(const hbg::HostBatch &h, const hbg_db *db) {
    int32_t len = h.max_diag_len;
    if (db->max_len + h.window > 0x7fff)
        len = std::max<int32_t>(len, h.smem_diag_len);
    return len;
}

// Subjects per work tile of one launch class: the batch's tuned value, else
// up to 128, fewer when the class has too little work to give every CTA about
// eight tiles (small databases and single queries would otherwise leave most
// SMs idle).
int32_t class_tile_subjects(const hbg_batch *b, const hbg_db *db, const LaunchClass &lc, int blocks) {
    if (b->tile_subjects > 0)
        return b->tile_subjects;
    if (b->tile_bytes > 0) {                  // subjects of the database's mean length
        const int64_t mean = std::max<int64_t>(1, db->n_res / std::max<int32_t>(1, db->n));
        return (int32_t)std::max<int64_t>(1, std::min<int64_t>(1 << 20, b->tile_bytes / mean));
    }
    const int64_t want = (int64_t)db->n * lc.count / (8 * (int64_t)std::max(blocks, 1));
    return (int32_t)std::max<int64_t>(8, std::min<int64_t>(128, want));
}

// CTA size and grid of each launch class: the CTA is halved until its
// per-warp tables fit the shared-memory carve-out; the grid is one wave at
// the occupancy that leaves (or the caller's num_blocksx).
int plan_launches(const hbg_batch *b, const hbg_gpu_options &o, int device, std::vector<LaunchShape> *out) {
    int optin = 0, sms = 1;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    out->clear();
    for (const LaunchClass &lc : b->classes) {
        // num_threadsx is the largest CTA size: per class take the size (halving
        // down to 64) that keeps the most warps resident per SM -- large diagonal
        // tables fill shared memory, and smaller CTAs pack it better
        // with several groups per pass (team > 1) the CTA keeps at least one
        // warp per group
        int best_t = 0, best_per = 0, best_warps = -1;
        for (int t = o.num_threadsx; t >= 32; t = t > 64 ? ((t / 2) + 31) / 32 * 32 : 0) {
            const int team = std::min(b->team, t / 32);
            if (team < b->team && best_t > 0)
                break;
            if (hbg::wordfinder_smem_bytes(t, lc.smem_diag, team) > (size_t)optin)
                continue;
            int per = 0;
            if (hbg::wordfinder_occupancy(lc.mode, t, lc.smem_diag, team, &per) != cudaSuccess || per < 1)
                per = 1;
            if (per * (t / 32) > best_warps) {
                best_t = t;
                best_per = per;
                best_warps = per * (t / 32);
            }
            if (o.num_blocksx > 0)
                break;                 // a fixed grid keeps the caller's CTA size when it fits
        }
        if (best_t == 0)
            return fail(HBG_ERR_TOO_LONG, "group diagonal tables exceed shared memory");
        const int blocks = o.num_blocksx > 0 ? o.num_blocksx : sms * best_per;
        out->push_back(LaunchShape{best_t, blocks, std::min(b->team, best_t / 32)});
    }
    return HBG_OK;
}

void drop_graph(hbg_result *r) {
    if (r->graph_exec)
        cudaGraphExecDestroy(r->graph_exec);
    r->graph_exec = nullptr;
}

void free_result_device(hbg_result *r) {
    if (r->graph_exec)
        cudaGraphExecDestroy(r->graph_exec);
    r->graph_exec = nullptr;
    if (r->launched && !r->synced)
        cudaStreamSynchronize(r->stream);    // nothing of this search may still run
    dfree_idle(r->d_raw);
    dfree_idle(r->d_sorted);
    dfree_idle(r->d_counters);
    dfree_idle(r->d_tile);
    dfree_idle(r->d_gdiag);
    dfree_idle(r->d_keys);
    dfree_idle(r->d_vals);
    dfree_idle(r->d_hist);
    for (auto &e : r->ev)
        if (e) {
            cudaEventDestroy(e);
            e = nullptr;
        }
    if (r->h_counters) {
        cudaFreeHost(r->h_counters);
        r->h_counters = nullptr;
    }
}

// Allocate (or grow) the result's device buffers for capacity cap.
int prepare_result(hbg_result *r, int64_t cap) {
    const hbg::HostBatch &h = r->batch->host;
    const size_t nq = h.queries.size(), ng = h.groups.size();
    if (!r->d_tile) {
        CU(dalloc(&r->d_tile, kMaxLaunchClasses));
        for (auto &e : r->ev)
            CU(cudaEventCreate(&e));
    }
    // a failed allocation below leaves the recorded size at 0, so the next
    // search allocates again instead of using a missing buffer
    if (r->n_counters < 1 + 6 * nq + ng) {   // first use, or a larger batch
        drop_graph(r);
        dfree(r->d_counters);
        if (r->h_counters)
            cudaFreeHost(r->h_counters);
        r->h_counters = nullptr;
        r->n_counters = 0;
        CU(dalloc(&r->d_counters, 1 + 6 * nq + ng));
        CU(cudaMallocHost((void **)&r->h_counters, (1 + 6 * nq + ng) * sizeof(unsigned long long)));
        r->n_counters = 1 + 6 * nq + ng;
    }
    r->gdiag_len = global_diag_len(h, r->db);
    if (r->gdiag_len > 0) {
        const int64_t need = (int64_t)r->blocks * (r->threads / 32) * r->gdiag_len;
        if (need > r->gdiag_entries) {
            drop_graph(r);
            dfree(r->d_gdiag);
            r->gdiag_entries = 0;
            CU(dalloc(&r->d_gdiag, (size_t)need));
            r->gdiag_entries = need;
        }
    }
    if (cap > r->cap) {
        drop_graph(r);
        r->cap = 0;
        dfree(r->d_raw);
        dfree(r->d_sorted);
        dfree(r->d_keys);
        dfree(r->d_vals);
        dfree(r->d_hist);
        CU(dalloc(&r->d_raw, (size_t)cap));
        CU(dalloc(&r->d_sorted, (size_t)cap));
        CU(dalloc(&r->d_keys, (size_t)cap * 2));
        CU(dalloc(&r->d_vals, (size_t)cap * 2));
        CU(dalloc(&r->d_hist, (size_t)(256 * hbg::order_max_blocks(cap) + 1)));
        r->cap = cap;
    }
    return HBG_OK;
}

// Enqueue one search on r->stream: counter resets, the word finder, the
// ordering pass, the lookup-hit counters and the copy of the counters to
// pinned host memory.  No host synchronisation, so it can be captured.
int enqueue_search(hbg_result *r) {
    hbg_db *db = r->db;
    const hbg::HostBatch &h = r->batch->host;
    const size_t nq = h.queries.size(), ng = h.groups.size();
    cudaStream_t st = r->stream;
    CU(cudaMemsetAsync(r->d_counters, 0, r->n_counters * sizeof(unsigned long long), st));
    CU(cudaMemsetAsync(r->d_tile, 0, kMaxLaunchClasses * sizeof(unsigned int), st));
    if (r->d_gdiag)
        CU(cudaMemsetAsync(r->d_gdiag, 0, (size_t)r->gdiag_entries * sizeof(uint32_t), st));

    hbg::WordFinderArgs a;
    memset(&a, 0, sizeof(a));
    a.db = db->d_letters;
    a.db_off = db->d_off;
    a.db_len = db->d_len;
    a.order = db->d_order;
    a.n_subj = db->n;
    hbg_batch *b = r->batch;
    a.groups = b->d_groups;
    a.n_groups = (int32_t)ng;
    a.group_list = b->d_group_list;
    a.cells = b->d_cells;
    a.entries = b->d_entries;
    a.pv = b->d_pv;
    a.letters = b->d_letters;
    a.ctx_of = b->d_ctx_of;
    a.contexts = b->d_ctx;
    a.queries = b->d_queries;
    a.window = h.window;
    a.tile_subjects = 128;
    a.tiles_per_group = (db->n + a.tile_subjects - 1) / a.tile_subjects;
    a.n_tiles = 0;
    a.tile_counter = r->d_tile;
    a.hsps = r->d_raw;
    a.hsp_count = r->d_counters;
    a.hsp_cap = r->cap;
    a.q_extended = r->d_counters + 1;
    a.q_kept = r->d_counters + 1 + nq;
    a.g_hits = r->d_counters + 1 + 3 * nq;
    a.gdiag = r->d_gdiag;
    a.gdiag_len = r->gdiag_len;
    a.smem_diag = h.smem_diag_len;

    // external records while capturing: they become event-record nodes of
    // the graph (usable for timing), not internal fork/join edges; the flag
    // is only accepted during a capture
    cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
    CU(cudaStreamIsCapturing(st, &cap_status));
    const unsigned ev_flags =
        cap_status == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
    CU(cudaEventRecordWithFlags(r->ev[0], st, ev_flags));
    if (db->n > 0)   // the caller has run wordfinder_configure (not a stream operation)
        for (size_t c = 0; c < b->classes.size(); ++c) {
            const LaunchClass &lc = b->classes[c];
            a.tile_subjects = class_tile_subjects(b, db, lc, r->shapes[c].blocks);
            a.tiles_per_group = (db->n + a.tile_subjects - 1) / a.tile_subjects;
            a.team = r->shapes[c].team;
            a.n_list = lc.count;
            a.group_list = b->d_group_list + lc.first;
            a.n_tiles = (int64_t)a.tiles_per_group * ((lc.count + a.team - 1) / a.team);
            a.tile_counter = r->d_tile + c;
            a.smem_diag = lc.smem_diag;
            CU(hbg::launch_wordfinder(a, lc.mode, r->shapes[c].blocks, r->shapes[c].threads, st));
        }
    CU(cudaEventRecordWithFlags(r->ev[1], st, ev_flags));

    hbg::OrderArgs o;
    memset(&o, 0, sizeof(o));
    o.in = r->d_raw;
    o.out = r->d_sorted;
    o.count = r->d_counters;
    o.cap = r->cap;
    o.keys[0] = r->d_keys;
    o.keys[1] = r->d_keys + r->cap;
    o.vals[0] = r->d_vals;
    o.vals[1] = r->d_vals + r->cap;
    o.hist = r->d_hist;
    o.bits_q = bits_for((int64_t)nq - 1);
    o.bits_s = bits_for((int64_t)db->n - 1);
    o.bits_so = bits_for(db->max_len);
    o.bits_qo = bits_for(h.max_query_len);
    o.q_first = r->d_counters + 1 + 3 * nq + ng;
    o.q_end = o.q_first + nq;
    o.q_passed = o.q_end + nq;
    if (o.bits_q + o.bits_s + o.bits_so + o.bits_qo > 64)
        return fail(HBG_ERR_TOO_LONG, "ordering key exceeds 64 bits for this database and batch");
    CU(hbg::launch_order(o, st));
    {
        const int bits = o.bits_q + o.bits_s + o.bits_so + o.bits_qo;
        r->launches = (db->n > 0 ? (int32_t)b->classes.size() : 0) + (hbg::order_max_blocks(r->cap) > 0 ? 3 + 3 * ((bits + 7) / 8) : 0) +
                      (nq > 0 ? 1 : 0);
    }
    CU(hbg::launch_query_hits(db->d_hist, b->d_qcells, (int32_t)nq, r->d_counters + 1 + 2 * nq, st));
    CU(cudaEventRecordWithFlags(r->ev[2], st, ev_flags));
    CU(cudaMemcpyAsync(r->h_counters, r->d_counters, r->n_counters * sizeof(unsigned long long),
                       cudaMemcpyDeviceToHost, st));
    return HBG_OK;
}

// Launch a search.  A result that is launched again on the same non-default
// stream with the same buffers replays a CUDA graph of the whole sequence
// (captured on its second launch) instead of ~30 separate launches.
int launch_search(hbg_result *r) {
    CU(hbg::wordfinder_configure());
    const bool graphable = r->stream != nullptr && r->launch_count > 0;
    const long long key[6] = {(long long)r->batch_id, (long long)r->cap,
                              ((long long)r->shape_opt.num_blocksx << 32) | (unsigned)r->shape_opt.num_threadsx,
                              r->blocks, (long long)r->gdiag_entries,
                              (long long)(uintptr_t)r->stream};
    if (!graphable) {
        int rc = enqueue_search(r);
        if (rc != HBG_OK)
            return rc;
    } else {
        if (!r->graph_exec || memcmp(key, r->graph_key, sizeof(key)) != 0) {
            drop_graph(r);
            cudaGraph_t graph = nullptr;
            CU(cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal));
            int rc = enqueue_search(r);
            cudaError_t e = cudaStreamEndCapture(r->stream, &graph);
            if (rc != HBG_OK) {
                if (graph)
                    cudaGraphDestroy(graph);
                return rc;
            }
            if (e != cudaSuccess)
                return fail(HBG_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
            e = cudaGraphInstantiate(&r->graph_exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                r->graph_exec = nullptr;
                return fail(HBG_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
            }
            memcpy(r->graph_key, key, sizeof(key));
        }
        CU(cudaGraphLaunch(r->graph_exec, r->stream));
    }
    r->launch_count++;
    r->launched = true;
    r->synced = false;
    r->done = false;
    return HBG_OK;
}

bool valid_opts(const hbg_gpu_options *o) {
    return o && o->num_threadsx >= 32 && o->num_threadsx <= 256 && (o->num_threadsx % 32) == 0 &&
           o->num_blocksx >= 0;
}

}  // namespace

extern "C" {

const char *hbg_last_error(void) { return g_err.c_str(); }

int hbg_device_count(int32_t *count) {
    if (!count)
        return fail(HBG_ERR_INVALID, "null count");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        *count = 0;
        return fail(HBG_ERR_NO_DEVICE, cudaGetErrorString(e));
    }
    *count = n;
    return HBG_OK;
}

int hbg_default_gpu_options(hbg_gpu_options *opt) {
    if (!opt)
        return fail(HBG_ERR_INVALID, "null options");
    opt->use_gpu = 1;
    opt->num_blocksx = 0;
    opt->num_threadsx = 256;
    opt->method = 0;
    opt->cpu_threads = 1;
    return HBG_OK;
}

}  // extern "C"

namespace {

// Checks shared by the database entry points: options, device.
int db_device(const hbg_gpu_options *opt, hbg_gpu_options *o) {
    hbg_default_gpu_options(o);
    if (opt)
        *o = *opt;
    if (!o->use_gpu)
        return fail(HBG_ERR_NO_DEVICE, "use_gpu is 0 and this library has no CPU path");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(HBG_ERR_NO_DEVICE, "no CUDA device");
    if (o->method < 0 || o->method >= ndev)
        return fail(HBG_ERR_INVALID, "method selects a device that does not exist");
    return HBG_OK;
}

// Allocate the resident database for a validated layout (subject i at
// device offset off[i], len[i] letters, sentinels between), let `fill` copy
// the letters (it returns "" or an error), then the offsets, the
// length-descending schedule and the word histogram.
template <typename Fill>
int db_create(int device, int32_t n, const std::vector<int64_t> &off, const std::vector<int32_t> &len,
              int64_t total, int32_t max_len, int64_t letters_len, Fill &&fill, hbg_db **out) {
    std::vector<int32_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t x, int32_t y) { return len[x] > len[y]; });

    hbg_db *db = new (std::nothrow) hbg_db;
    if (!db)
        return fail(HBG_ERR_NOMEM, "host allocation");
    db->device = device;
    DeviceScope ds(db->device);
    auto bail = [&](int code) {
        dfree(db->d_letters);
        dfree(db->d_off);
        dfree(db->d_len);
        dfree(db->d_order);
        dfree(db->d_hist);
        delete db;
        return code;
    };
#define CUB(call)                                                                   \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess)                                                      \
            return bail(fail(e_ == cudaErrorMemoryAllocation ? HBG_ERR_NOMEM : HBG_ERR_CUDA, \
                             std::string(#call) + ": " + cudaGetErrorString(e_)));  \
    } while (0)
    CUB(dalloc(&db->d_letters, (size_t)letters_len));
    CUB(dalloc(&db->d_off, (size_t)n));
    CUB(dalloc(&db->d_len, (size_t)n));
    CUB(dalloc(&db->d_order, (size_t)n));
    CUB(dalloc(&db->d_hist, HBG_NUM_CELLS));
    CUB(cudaMemset(db->d_letters, 0, (size_t)letters_len));
    {
        int code = HBG_OK;
        std::string err = fill(db->d_letters, &code);
        if (!err.empty())
            return bail(fail(code, err));
    }
    if (n > 0) {
        CUB(cudaMemcpy(db->d_off, off.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice));
        CUB(cudaMemcpy(db->d_len, len.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
        CUB(cudaMemcpy(db->d_order, order.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
    }
    CUB(cudaMemset(db->d_hist, 0, sizeof(unsigned long long) * HBG_NUM_CELLS));
    CUB(hbg::launch_db_histogram(db->d_letters, letters_len, db->d_hist, 0));
    CUB(cudaDeviceSynchronize());
#undef CUB
    db->n = n;
    db->n_res = total;
    db->letters_len = letters_len;
    db->max_len = max_len;
    db->bytes = letters_len + (int64_t)n * 16 + HBG_NUM_CELLS * 8;
    *out = db;
    return HBG_OK;
}

std::string cuda_msg(const char *what, cudaError_t e, int *code) {
    *code = e == cudaErrorMemoryAllocation ? HBG_ERR_NOMEM : HBG_ERR_CUDA;
    return std::string(what) + ": " + cudaGetErrorString(e);
}

// Volumes of a BLAST database with their place in the resident layout:
// volume v's .psq byte b lands at device offset base[v] + b (a volume's
// leading 0 is the previous volume's last separator).
struct BlastDbPlan {
    std::vector<hbg::BlastDbVolume> vols;
    std::vector<int64_t> base;
    int64_t n = 0, total = 0, bytes = 0;
    int32_t max_len = 0;
};

int blastdb_plan(const char *path, BlastDbPlan *plan) {
    if (!path)
        return fail(HBG_ERR_INVALID, "null database name");
    std::vector<std::string> names;
    std::string err = hbg::blastdb_volumes(path, &names);
    if (!err.empty())
        return fail(HBG_ERR_INVALID, err);
    plan->vols.resize(names.size());
    int64_t at = 0;
    for (size_t v = 0; v < names.size(); ++v) {
        err = hbg::blastdb_read_index(names[v], &plan->vols[v]);
        if (!err.empty())
            return fail(HBG_ERR_INVALID, err);
        const hbg::BlastDbVolume &V = plan->vols[v];
        if (V.max_len > HBG_MAX_SUBJECT_LEN)
            return fail(HBG_ERR_TOO_LONG, names[v] + ": a sequence longer than the subject limit");
        plan->base.push_back(v == 0 ? 0 : at - 1);
        at = plan->base.back() + V.psq_bytes;
        plan->n += V.n;
        plan->total += V.residues;
        plan->max_len = std::max(plan->max_len, V.max_len);
    }
    if (plan->n > 0x7fffffff)
        return fail(HBG_ERR_TOO_LONG, "more than 2^31 - 1 sequences");
    plan->bytes = at;
    return HBG_OK;
}

}  // namespace

extern "C" {

int hbg_db_open(const uint8_t *residues, const int64_t *offsets, int32_t n,
                const hbg_gpu_options *opt, hbg_db **out) {
    if (!out || !offsets || n < 0 || (n > 0 && !residues))
        return fail(HBG_ERR_INVALID, "hbg_db_open: null argument or negative count");
    *out = nullptr;
    hbg_gpu_options o;
    int rc = db_device(opt, &o);
    if (rc != HBG_OK)
        return rc;
    // validate and lay out: one sentinel before every subject and after the last
    std::vector<int64_t> off(n);
    std::vector<int32_t> len(n);
    int64_t pos = 1, total = 0;
    int32_t max_len = 0;
    for (int32_t i = 0; i < n; ++i) {
        int64_t L = offsets[i + 1] - offsets[i];
        if (L < 0 || L > HBG_MAX_SUBJECT_LEN)
            return fail(L < 0 ? HBG_ERR_INVALID : HBG_ERR_TOO_LONG,
                        "subject " + std::to_string(i) + ": bad length");
        const uint8_t *s = residues + offsets[i];
        for (int64_t k = 0; k < L; ++k)
            if (s[k] == 0 || s[k] >= HBG_ALPHABET)
                return fail(HBG_ERR_INVALID, "subject " + std::to_string(i) +
                                                 ": letter outside NCBIstdaa 1..27");
        off[i] = pos;
        len[i] = (int32_t)L;
        pos += L + 1;
        total += L;
        max_len = std::max<int32_t>(max_len, (int32_t)L);
    }
    const int64_t letters_len = pos + 64;
    // copy subjects with their sentinels through a staging buffer of ~64 MiB
    auto fill = [&](uint8_t *d_letters, int *code) -> std::string {
        int32_t i = 0;
        std::vector<uint8_t> stage;
        while (i < n) {
            const int64_t start_dev = off[i] - 1;
            stage.clear();
            stage.push_back(0);
            while (i < n && (int64_t)stage.size() < (64 << 20)) {
                const uint8_t *s = residues + offsets[i];
                stage.insert(stage.end(), s, s + len[i]);
                stage.push_back(0);
                ++i;
            }
            cudaError_t e = cudaMemcpy(d_letters + start_dev, stage.data(), stage.size(), cudaMemcpyHostToDevice);
            if (e != cudaSuccess)
                return cuda_msg("cudaMemcpy (subjects)", e, code);
        }
        return std::string();
    };
    return db_create(o.method, n, off, len, total, max_len, letters_len, fill, out);
}

int hbg_blastdb_info(const char *path, int32_t *n_subjects, int64_t *n_residues, int32_t *max_len,
                     int32_t *n_volumes) {
    BlastDbPlan plan;
    int rc = blastdb_plan(path, &plan);
    if (rc != HBG_OK)
        return rc;
    if (n_subjects)
        *n_subjects = (int32_t)plan.n;
    if (n_residues)
        *n_residues = plan.total;
    if (max_len)
        *max_len = plan.max_len;
    if (n_volumes)
        *n_volumes = (int32_t)plan.vols.size();
    return HBG_OK;
}

int hbg_blastdb_read(const char *path, uint8_t *residues, int64_t *offsets) {
    if (!offsets)
        return fail(HBG_ERR_INVALID, "hbg_blastdb_read: null offsets");
    BlastDbPlan plan;
    int rc = blastdb_plan(path, &plan);
    if (rc != HBG_OK)
        return rc;
    if (plan.total > 0 && !residues)
        return fail(HBG_ERR_INVALID, "hbg_blastdb_read: null residues");
    int64_t at = 0, k = 0;
    offsets[0] = 0;
    for (const hbg::BlastDbVolume &V : plan.vols) {
        std::unique_ptr<uint8_t[]> buf(new (std::nothrow) uint8_t[(size_t)V.psq_bytes]);   // not zero-filled
        if (!buf)
            return fail(HBG_ERR_NOMEM, "host allocation");
        std::string err = hbg::blastdb_read_psq(V, 0, V.psq_bytes, buf.get());
        if (!err.empty())
            return fail(HBG_ERR_INVALID, err);
        for (int32_t i = 0; i < V.n; ++i) {
            const int64_t L = (int64_t)V.seq_off[i + 1] - V.seq_off[i] - 1;
            memcpy(residues + at, buf.get() + V.seq_off[i], (size_t)L);
            at += L;
            offsets[++k] = at;
        }
    }
    return HBG_OK;
}

int hbg_db_open_blastdb(const char *path, const hbg_gpu_options *opt, hbg_db **out) {
    if (!out)
        return fail(HBG_ERR_INVALID, "hbg_db_open_blastdb: null out");
    *out = nullptr;
    hbg_gpu_options o;
    int rc = db_device(opt, &o);
    if (rc != HBG_OK)
        return rc;
    BlastDbPlan plan;
    rc = blastdb_plan(path, &plan);
    if (rc != HBG_OK)
        return rc;
    const int32_t n = (int32_t)plan.n;
    std::vector<int64_t> off(n);
    std::vector<int32_t> len(n);
    {
        int64_t k = 0;
        for (size_t v = 0; v < plan.vols.size(); ++v) {
            const hbg::BlastDbVolume &V = plan.vols[v];
            for (int32_t i = 0; i < V.n; ++i, ++k) {
                off[k] = plan.base[v] + V.seq_off[i];
                len[k] = (int32_t)(V.seq_off[i + 1] - V.seq_off[i] - 1);
            }
        }
    }
    const int64_t letters_len = plan.bytes + 64;
    // each volume's .psq is already the device layout: read whole sequences
    // in ~64 MiB pieces into two pinned buffers, checking each piece while
    // the previous one is copied
    auto fill = [&](uint8_t *d_letters, int *code) -> std::string {
        const size_t piece = std::max<size_t>(64u << 20, (size_t)plan.max_len + 2);
        uint8_t *pin[2] = {nullptr, nullptr};
        cudaStream_t st = nullptr;
        cudaEvent_t done[2] = {nullptr, nullptr};
        std::string err;
        cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        for (int j = 0; j < 2 && e == cudaSuccess; ++j) {
            e = cudaMallocHost(&pin[j], piece);
            if (e == cudaSuccess)
                e = cudaEventCreateWithFlags(&done[j], cudaEventDisableTiming);
        }
        if (e != cudaSuccess)
            err = cuda_msg("staging buffers", e, code);
        int cur = 0;
        bool used[2] = {false, false};
        for (size_t v = 0; v < plan.vols.size() && err.empty(); ++v) {
            const hbg::BlastDbVolume &V = plan.vols[v];
            int32_t i = 0;
            int64_t from = 0;                      // the leading 0 of volume 0 is copied too
            while (err.empty() && (from == 0 || i < V.n)) {
                // whole sequences (with separators) up to the piece size
                int32_t j = i;
                while (j < V.n && (int64_t)V.seq_off[j + 1] - from <= (int64_t)piece)
                    ++j;
                if (j == i && i < V.n)
                    j = i + 1;                     // piece >= longest + 2, so one always fits
                const int64_t to = i < V.n ? (int64_t)V.seq_off[j] : (int64_t)V.seq_off[0];
                if (used[cur]) {
                    e = cudaEventSynchronize(done[cur]);
                    if (e != cudaSuccess) {
                        err = cuda_msg("cudaEventSynchronize", e, code);
                        break;
                    }
                }
                err = hbg::blastdb_read_psq(V, from, to - from, pin[cur]);
                if (!err.empty()) {
                    *code = HBG_ERR_INVALID;
                    break;
                }
                // volume v > 0: its leading 0 is already in place (the buffer starts zeroed)
                const int64_t skip = (from == 0 && v > 0) ? 1 : 0;
                e = cudaMemcpyAsync(d_letters + plan.base[v] + from + skip, pin[cur] + skip,
                                    (size_t)(to - from - skip), cudaMemcpyHostToDevice, st);
                if (e == cudaSuccess)
                    e = cudaEventRecord(done[cur], st);
                if (e != cudaSuccess) {
                    err = cuda_msg("cudaMemcpyAsync (volume)", e, code);
                    break;
                }
                used[cur] = true;
                cur ^= 1;
                from = to;
                i = j;
            }
        }
        if (st) {
            e = cudaStreamSynchronize(st);
            if (e != cudaSuccess && err.empty())
                err = cuda_msg("cudaStreamSynchronize", e, code);
            cudaStreamDestroy(st);
        }
        for (int j = 0; j < 2; ++j) {
            if (done[j])
                cudaEventDestroy(done[j]);
            if (pin[j])
                cudaFreeHost(pin[j]);
        }
        return err;
    };
    return db_create(o.method, n, off, len, plan.total, plan.max_len, letters_len, fill, out);
}

int hbg_db_close(hbg_db *db) {
    if (!db)
        return fail(HBG_ERR_INVALID, "null db");
    DeviceScope ds(db->device);
    dfree(db->d_letters);
    dfree(db->d_off);
    dfree(db->d_len);
    dfree(db->d_order);
    dfree(db->d_hist);
    delete db;
    return HBG_OK;
}

int hbg_db_info(const hbg_db *db, int32_t *n, int64_t *res, int64_t *bytes) {
    if (!db)
        return fail(HBG_ERR_INVALID, "null db");
    if (n)
        *n = db->n;
    if (res)
        *res = db->n_res;
    if (bytes)
        *bytes = db->bytes;
    return HBG_OK;
}

static int finish_batch(std::vector<hbg::QueryIn> &qs, const hbg_word_params *params,
                        int32_t max_group_len, hbg_batch **out) {
    hbg_batch *b = new (std::nothrow) hbg_batch;
    if (!b)
        return fail(HBG_ERR_NOMEM, "host allocation");
    std::string err = hbg::build_batch(qs, params->threshold, params->window, max_group_len, &b->host);
    if (!err.empty()) {
        delete b;
        return fail(err.find("length") != std::string::npos ? HBG_ERR_TOO_LONG : HBG_ERR_INVALID, err);
    }
    *out = b;
    return HBG_OK;
}

int hbg_batch_create(const hbg_query *queries, int32_t n_queries, const hbg_word_params *params,
                     int32_t max_group_len, hbg_batch **out) {
    if (!out || !params || !queries || n_queries <= 0)
        return fail(HBG_ERR_INVALID, "hbg_batch_create: null argument or empty batch");
    *out = nullptr;
    std::vector<hbg::QueryIn> qs(n_queries);
    for (int32_t k = 0; k < n_queries; ++k) {
        const hbg_query &q = queries[k];
        if (!q.sequence || q.num_contexts <= 0 || !q.context_offset || !q.context_length ||
            !q.x_dropoff || !q.cutoff_score)
            return fail(HBG_ERR_INVALID, "query " + std::to_string(k) + ": null field");
        qs[k].seq = q.sequence;
        qs[k].len = q.length;
        qs[k].ctx_off.assign(q.context_offset, q.context_offset + q.num_contexts);
        qs[k].ctx_len.assign(q.context_length, q.context_length + q.num_contexts);
        qs[k].xdrop.assign(q.x_dropoff, q.x_dropoff + q.num_contexts);
        qs[k].cutoff.assign(q.cutoff_score, q.cutoff_score + q.num_contexts);
    }
    return finish_batch(qs, params, max_group_len, out);
}

int hbg_seg_default_params(hbg_seg_params *p) {
    if (!p)
        return fail(HBG_ERR_INVALID, "hbg_seg_default_params: null argument");
    p->window = 12;
    p->pad = 0;
    p->locut = 2.2;
    p->hicut = 2.5;
    return HBG_OK;
}

static bool valid_seg(const hbg_seg_params *p) {
    return p && p->window >= 1 && p->window <= 1000 && p->locut >= 0 && p->hicut >= p->locut;
}

int hbg_seg_mask(uint8_t *seq, int32_t len, const hbg_seg_params *p, int64_t *n_masked) {
    if (!seq || len < 0 || !valid_seg(p))
        return fail(HBG_ERR_INVALID, "hbg_seg_mask: null sequence, negative length or bad parameters");
    const int64_t n = hbg::seg_mask(seq, len, p->window, p->locut, p->hicut);
    if (n_masked)
        *n_masked = n;
    return HBG_OK;
}

int hbg_batch_create_blastx(const uint8_t *const *nt, const int32_t *nt_len, int32_t n_queries,
                            const int32_t *x_dropoff, const int32_t *cutoff,
                            const hbg_word_params *params, int32_t max_group_len, hbg_batch **out) {
    return hbg_batch_create_blastx_masked(nt, nt_len, n_queries, x_dropoff, cutoff, params, nullptr,
                                          max_group_len, out);
}

int hbg_batch_create_blastx_masked(const uint8_t *const *nt, const int32_t *nt_len, int32_t n_queries,
                                   const int32_t *x_dropoff, const int32_t *cutoff,
                                   const hbg_word_params *params, const hbg_seg_params *seg,
                                   int32_t max_group_len, hbg_batch **out) {
    if (!out || !params || !nt || !nt_len || !x_dropoff || !cutoff || n_queries <= 0)
        return fail(HBG_ERR_INVALID, "hbg_batch_create_blastx: null argument or empty batch");
    if (seg && !valid_seg(seg))
        return fail(HBG_ERR_INVALID, "hbg_batch_create_blastx_masked: bad SEG parameters");
    *out = nullptr;
    std::vector<std::vector<uint8_t>> prot(n_queries);
    std::vector<hbg::QueryIn> qs(n_queries);
    for (int32_t k = 0; k < n_queries; ++k) {
        if (!nt[k] || nt_len[k] < 3)
            return fail(HBG_ERR_INVALID, "query " + std::to_string(k) + ": need >= 3 nucleotides");
        if ((int64_t)nt_len[k] * 2 + 6 > HBG_MAX_QUERY_LEN)
            return fail(HBG_ERR_TOO_LONG, "query " + std::to_string(k) + ": too long");
        prot[k] = hbg::translate_six_frames(nt[k], nt_len[k], &qs[k].ctx_off, &qs[k].ctx_len);
        if (seg)                                  // each frame is masked as a protein of its own
            for (int f = 0; f < 6; ++f)
                hbg::seg_mask(prot[k].data() + qs[k].ctx_off[f], qs[k].ctx_len[f], seg->window, seg->locut,
                              seg->hicut);
        qs[k].seq = prot[k].data();
        qs[k].len = qs[k].ctx_off[5] + qs[k].ctx_len[5];
        qs[k].xdrop.assign(x_dropoff + 6 * k, x_dropoff + 6 * k + 6);
        qs[k].cutoff.assign(cutoff + 6 * k, cutoff + 6 * k + 6);
        // translated letters may include the sentinel-free stop '*' (25): allowed
    }
    return finish_batch(qs, params, max_group_len, out);
}

int hbg_batch_create_from_smallbone(const hbg_query *query, const hbg_word_params *params,
                                    const void *backbone, int32_t backbone_size,
                                    const uint16_t *overflow, int64_t overflow_size,
                                    hbg_batch **out) {
    if (!out || !params || !query || !backbone || backbone_size <= 0 ||
        backbone_size > HBG_NUM_CELLS || overflow_size < 0 || (overflow_size > 0 && !overflow))
        return fail(HBG_ERR_INVALID, "hbg_batch_create_from_smallbone: bad argument");
    int rc = hbg_batch_create(query, 1, params, 1, out);
    if (rc != HBG_OK)
        return rc;
    hbg::HostBatch &h = (*out)->host;
    // NCBI AaLookupSmallboneCell: Int4 num_used; union { Uint2 entries[3]; Int4 cursor; }
    struct Cell {
        int32_t num_used;
        union {
            uint16_t entries[3];
            int32_t cursor;
        } payload;
    };
    const Cell *cells = (const Cell *)backbone;
    std::vector<uint32_t> cs(HBG_CELL_STRIDE, 0);
    std::vector<uint16_t> ents;
    std::vector<uint32_t> pv(HBG_PV_WORDS, 0);
    std::vector<uint16_t> qc(HBG_NUM_CELLS, 0);
    const int32_t qlen = query->length;
    for (int32_t w = 0; w < HBG_NUM_CELLS; ++w) {
        cs[w] = (uint32_t)ents.size();
        if (w >= backbone_size)
            continue;
        const Cell &c = cells[w];
        if (c.num_used < 0)
            goto bad;
        if (c.num_used == 0)
            continue;
        {
            std::vector<uint16_t> v;
            if (c.num_used <= 3) {
                v.assign(c.payload.entries, c.payload.entries + c.num_used);
            } else {
                if (c.payload.cursor < 0 || (int64_t)c.payload.cursor + c.num_used > overflow_size)
                    goto bad;
                v.assign(overflow + c.payload.cursor, overflow + c.payload.cursor + c.num_used);
            }
            std::sort(v.begin(), v.end());
            for (uint16_t x : v)
                if ((int32_t)x + HBG_WORD_SIZE > qlen)
                    goto bad;
            ents.insert(ents.end(), v.begin(), v.end());
            pv[w >> 5] |= 1u << (w & 31);
            qc[w] = (uint16_t)c.num_used;
        }
    }
    cs[HBG_NUM_CELLS] = (uint32_t)ents.size();
    h.cells = cs;
    h.entries = ents;
    h.pv = pv;
    h.query_cells = qc;
    h.groups[0].entry_base = 0;
    return HBG_OK;
bad:
    hbg_batch_destroy(*out);
    *out = nullptr;
    return fail(HBG_ERR_INVALID, "smallbone table: bad cell");
}

int hbg_batch_lookup_table(const hbg_batch *b, int32_t g, uint32_t *cells, uint16_t *entries,
                           int64_t entries_cap, int64_t *n_entries, int32_t *first_query,
                           int32_t *n_queries, int32_t *query_start) {
    if (!b || !n_entries || g < 0 || g >= (int32_t)b->host.groups.size())
        return fail(HBG_ERR_INVALID, "hbg_batch_lookup_table: bad argument");
    const hbg::HostBatch &h = b->host;
    const HbgGroup &G = h.groups[g];
    const uint32_t *cs = h.cells.data() + (size_t)g * HBG_CELL_STRIDE;
    const int64_t n = cs[HBG_NUM_CELLS];
    *n_entries = n;
    if (first_query)
        *first_query = G.first_query;
    if (n_queries)
        *n_queries = G.n_queries;
    if (query_start)
        for (int32_t k = 0; k < G.n_queries; ++k)
            query_start[k] = h.queries[G.first_query + k].start;
    if (cells)
        memcpy(cells, cs, sizeof(uint32_t) * HBG_CELL_STRIDE);
    if (entries) {
        if (entries_cap < n)
            return fail(HBG_ERR_CAPACITY, "entries buffer too small");
        if (n)
            memcpy(entries, h.entries.data() + G.entry_base, sizeof(uint16_t) * (size_t)n);
    }
    return HBG_OK;
}

int hbg_batch_set_mode(hbg_batch *b, int32_t g, int32_t mode) {
    if (!b || (mode != 0 && mode != 1) || g >= (int32_t)b->host.groups.size())
        return fail(HBG_ERR_INVALID, "hbg_batch_set_mode: bad argument");
    if (b->device >= 0)
        return fail(HBG_ERR_STATE, "batch already uploaded: set modes before the first search");
    for (int32_t i = 0; i < (int32_t)b->host.groups.size(); ++i)
        if (g < 0 || i == g)
            b->host.groups[i].mode = mode;
    return HBG_OK;
}

int hbg_batch_tune(hbg_batch *b, int32_t tile_subjects, int32_t global_tables) {
    if (!b || tile_subjects < 0 || (tile_subjects > 0 && (tile_subjects < 8 || tile_subjects > 4096)) ||
        (global_tables != 0 && global_tables != 1))
        return fail(HBG_ERR_INVALID, "hbg_batch_tune: bad argument");
    if (b->device >= 0)
        return fail(HBG_ERR_STATE, "batch already uploaded: tune before the first search");
    b->tile_subjects = tile_subjects;
    if (global_tables) {
        hbg::HostBatch &h = b->host;
        for (HbgGroup &G : h.groups) {
            if (G.placement)
                continue;
            int32_t n = 1;
            while (n < G.glen + h.window)
                n <<= 1;
            G.diag_len = n;                      // global tables are powers of two
            G.placement = 1;
            h.max_diag_len = std::max(h.max_diag_len, G.diag_len);
        }
    }
    return HBG_OK;
}

int hbg_batch_schedule(hbg_batch *b, int32_t warps_per_subject, int64_t tile_bytes) {
    if (!b || warps_per_subject < 1 || warps_per_subject > 8 || tile_bytes < 0 ||
        (tile_bytes > 0 && (tile_bytes < 1024 || tile_bytes > ((int64_t)1 << 24))))
        return fail(HBG_ERR_INVALID, "hbg_batch_schedule: warps_per_subject 1..8, tile_bytes 0 or 1 KiB..16 MiB");
    if (b->device >= 0)
        return fail(HBG_ERR_STATE, "batch already uploaded: schedule before the first search");
    b->team = warps_per_subject;
    b->tile_bytes = tile_bytes;
    return HBG_OK;
}

int hbg_batch_destroy(hbg_batch *b) {
    if (!b)
        return fail(HBG_ERR_INVALID, "null batch");
    if (b->device >= 0) {
        DeviceScope ds(b->device);
        // searches of this batch may run on any stream: wait for the device
        // (as cudaFree would), then keep the buffers for reuse
        cudaDeviceSynchronize();
        free_batch_device(b);
    }
    delete b;
    return HBG_OK;
}

int hbg_batch_info(const hbg_batch *b, int32_t *nq, int32_t *ng, int64_t *qlen, int64_t *entries,
                   int64_t *device_bytes) {
    if (!b)
        return fail(HBG_ERR_INVALID, "null batch");
    if (nq)
        *nq = (int32_t)b->host.queries.size();
    if (ng)
        *ng = (int32_t)b->host.groups.size();
    if (qlen) {
        int64_t t = 0;
        for (auto &q : b->host.queries)
            t += q.len;
        *qlen = t;
    }
    if (entries)
        *entries = (int64_t)b->host.entries.size();
    if (device_bytes)
        *device_bytes = batch_device_bytes(b->host);
    return HBG_OK;
}

int hbg_mem_required(const hbg_db *db, const hbg_batch *b, int64_t cap, int64_t *bytes) {
    if (!db || !b || !bytes || cap < 0)
        return fail(HBG_ERR_INVALID, "hbg_mem_required: bad argument");
    if (cap == 0)
        cap = std::max<int64_t>(1 << 20, (int64_t)db->n);
    const hbg::HostBatch &h = b->host;
    int64_t batch_bytes = (int64_t)(h.letters.size() + h.ctx_of.size() * 4 + h.cells.size() * 4 +
                                    h.entries.size() * 2 + h.pv.size() * 4 + h.query_cells.size() * 2);
    int64_t per_hsp = 2 * (int64_t)sizeof(hbg_hsp) + 2 * 8 + 2 * 4;
    int64_t gdiag = 0;
    if (global_diag_len(h, db) > 0) {
        int sms = 152;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, db->device);
        gdiag = (int64_t)sms * 8 * 8 * global_diag_len(h, db) * 4;
    }
    *bytes = batch_bytes + cap * per_hsp + gdiag + 1024 * 1024;
    return HBG_OK;
}

int hbg_search(hbg_db *db, hbg_batch *batch, const hbg_gpu_options *opt, int64_t cap,
               void *stream, hbg_result **out) {
    if (!db || !batch || !out || cap < 0)
        return fail(HBG_ERR_INVALID, "hbg_search: null argument");
    hbg_gpu_options o;
    hbg_default_gpu_options(&o);
    if (opt)
        o = *opt;
    if (!o.use_gpu)
        return fail(HBG_ERR_NO_DEVICE, "use_gpu is 0 and this library has no CPU path");
    if (!valid_opts(&o))
        return fail(HBG_ERR_INVALID, "num_threadsx must be a multiple of 32 in 32..256");
    DeviceScope ds(db->device);
    int rc = upload_batch(batch, db->device);
    if (rc != HBG_OK)
        return rc;
    hbg_result *r = *out;
    if (r && (r->db != db || r->db_id != db->id))
        return fail(HBG_ERR_STATE, "a reused result must belong to the same database");
    if (r && r->launched && !r->synced)
        return fail(HBG_ERR_STATE, "the result's previous search has not been waited for");
    if (r && (r->batch != batch || r->batch_id != batch->id)) {
        // re-target the buffers to another batch of the same database
        r->batch = batch;
        r->batch_id = batch->id;
        r->graph_exec ? (void)cudaGraphExecDestroy(r->graph_exec) : (void)0;
        r->graph_exec = nullptr;
        r->launch_count = 0;
    }
    if (!r) {
        r = new (std::nothrow) hbg_result;
        if (!r)
            return fail(HBG_ERR_NOMEM, "host allocation");
        r->db = db;
        r->db_id = db->id;
        r->batch = batch;
        r->batch_id = batch->id;
        r->device = db->device;
    }
    r->opt = o;
    r->stream = (cudaStream_t)stream;
    if (hbg::wordfinder_configure() != cudaSuccess) {
        if (!*out)
            delete r;
        return fail(HBG_ERR_CUDA, "cannot configure the word-finder kernel (wrong GPU?)");
    }
    rc = plan_launches(batch, o, db->device, &r->shapes);
    if (rc != HBG_OK) {
        if (!*out)
            delete r;
        return rc;
    }
    r->shape_opt = o;
    r->blocks = 0;
    r->threads = 32;
    for (const LaunchShape &sh : r->shapes) {
        r->blocks = std::max(r->blocks, sh.blocks);
        r->threads = std::max(r->threads, sh.threads);
    }
    if (cap == 0)
        cap = std::max<int64_t>(1 << 20, (int64_t)db->n);
    rc = prepare_result(r, std::max<int64_t>(cap, r->cap));
    if (rc == HBG_OK)
        rc = launch_search(r);
    if (rc != HBG_OK) {
        if (!*out) {
            cudaStreamSynchronize(r->stream);   // a partly enqueued search may still run
            free_result_device(r);
            delete r;
        }
        return rc;
    }
    *out = r;
    return HBG_OK;
}

int hbg_result_sync(hbg_result *r) {
    if (!r || !r->launched)
        return fail(HBG_ERR_STATE, "no search launched on this result");
    if (r->synced)
        return HBG_OK;
    DeviceScope ds(r->device);
    CU(cudaStreamSynchronize(r->stream));
    unsigned long long n = r->h_counters[0];
    if ((int64_t)n > r->cap) {
        // the HSP buffer was too small: relaunch once with the exact size.  If
        // that cannot be set up, nothing of this search runs any more and the
        // result may be relaunched (or reused for another batch) later.
        int rc = prepare_result(r, (int64_t)n);
        if (rc == HBG_OK)
            rc = launch_search(r);
        if (rc != HBG_OK) {
            cudaStreamSynchronize(r->stream);
            r->launched = false;
            return rc;
        }
        CU(cudaStreamSynchronize(r->stream));
        n = r->h_counters[0];
        if ((int64_t)n > r->cap)
            return fail(HBG_ERR_STATE, "HSP count changed between identical launches");
    }
    r->n_hsps = (int64_t)n;
    CU(cudaEventElapsedTime(&r->wf_ms, r->ev[0], r->ev[1]));
    CU(cudaEventElapsedTime(&r->ord_ms, r->ev[1], r->ev[2]));
    r->synced = true;
    return HBG_OK;
}

int hbg_result_wait(hbg_result *r) {
    int rc = hbg_result_sync(r);
    if (rc != HBG_OK)
        return rc;
    if (r->done)
        return HBG_OK;
    // the ordered HSPs stay on the device (read with hbg_result_hsps); the
    // ordering pass left per-query ranges and subject counts beside the counters
    const size_t nq = r->batch->host.queries.size(), ng = r->batch->host.groups.size();
    const unsigned long long *rng = r->h_counters + 1 + 3 * nq + ng;
    r->stats.assign(nq, hbg_query_stats{0, 0, 0, 0});
    r->q_first.assign(nq, 0);
    r->q_count.assign(nq, 0);
    for (size_t q = 0; q < nq; ++q) {
        r->stats[q].init_extends = (int64_t)r->h_counters[1 + q];
        r->stats[q].good_init_extends = (int64_t)r->h_counters[1 + nq + q];
        r->stats[q].lookup_hits = (int64_t)r->h_counters[1 + 2 * nq + q];
        r->stats[q].subjects_passed = (int64_t)rng[2 * nq + q];
        r->q_first[q] = (int64_t)rng[q];
        r->q_count[q] = (int64_t)rng[nq + q] - (int64_t)rng[q];
    }
    r->done = true;
    return HBG_OK;
}

int hbg_result_timing(const hbg_result *r, float *wf, float *ord, int32_t *launches) {
    if (!r || !r->synced)
        return fail(HBG_ERR_STATE, "result not collected");
    if (wf)
        *wf = r->wf_ms;
    if (ord)
        *ord = r->ord_ms;
    if (launches)
        *launches = r->launches;
    return HBG_OK;
}

int hbg_result_counts(const hbg_result *r, int64_t *n_hsps, int32_t *n_queries) {
    if (!r || !r->synced)
        return fail(HBG_ERR_STATE, "result not collected");
    if (n_hsps)
        *n_hsps = r->n_hsps;
    if (n_queries)
        *n_queries = (int32_t)r->batch->host.queries.size();
    return HBG_OK;
}

int hbg_result_hsps(const hbg_result *r, int64_t first, int64_t count, hbg_hsp *out) {
    if (!r || !r->done)
        return fail(HBG_ERR_STATE, "result not collected");
    if (first < 0 || count < 0 || first + count > r->n_hsps || (count > 0 && !out))
        return fail(HBG_ERR_INVALID, "range outside the result");
    if (count) {
        // on the search's own stream, so the copy neither waits for nor races
        // with work on other streams
        DeviceScope ds(r->device);
        CU(cudaMemcpyAsync(out, r->d_sorted + first, (size_t)count * sizeof(hbg_hsp), cudaMemcpyDeviceToHost,
                           r->stream));
        CU(cudaStreamSynchronize(r->stream));
    }
    return HBG_OK;
}

int hbg_result_query_range(const hbg_result *r, int32_t q, int64_t *first, int64_t *count) {
    if (!r || !r->done)
        return fail(HBG_ERR_STATE, "result not collected");
    if (q < 0 || q >= (int32_t)r->q_first.size() || !first || !count)
        return fail(HBG_ERR_INVALID, "query index outside the batch");
    *first = r->q_first[q];
    *count = r->q_count[q];
    return HBG_OK;
}

int hbg_result_stats(const hbg_result *r, int32_t q, hbg_query_stats *out) {
    if (!r || !r->done)
        return fail(HBG_ERR_STATE, "result not collected");
    if (q < 0 || q >= (int32_t)r->stats.size() || !out)
        return fail(HBG_ERR_INVALID, "query index outside the batch");
    *out = r->stats[q];
    return HBG_OK;
}

int hbg_result_free(hbg_result *r) {
    if (!r)
        return fail(HBG_ERR_INVALID, "null result");
    DeviceScope ds(r->device);
    if (r->launched && !r->synced)
        cudaStreamSynchronize(r->stream);
    free_result_device(r);
    delete r;
    return HBG_OK;
}

int hbg_search_sync(hbg_db *db, hbg_batch *batch, const hbg_gpu_options *opt, hbg_hsp *out,
                    int64_t out_cap, int64_t *n_hsps, hbg_query_stats *stats, void *stream) {
    if (!n_hsps || out_cap < 0)
        return fail(HBG_ERR_INVALID, "hbg_search_sync: bad argument");
    hbg_result *r = nullptr;
    int rc = hbg_search(db, batch, opt, 0, stream, &r);
    if (rc != HBG_OK)
        return rc;
    rc = hbg_result_wait(r);
    if (rc == HBG_OK) {
        *n_hsps = r->n_hsps;
        if (stats)
            for (size_t q = 0; q < r->stats.size(); ++q)
                stats[q] = r->stats[q];
        if (out) {
            if (r->n_hsps > out_cap)
                rc = fail(HBG_ERR_CAPACITY, "output buffer too small");
            else if (r->n_hsps) {
                DeviceScope ds(r->device);
                cudaError_t e = cudaMemcpyAsync(out, r->d_sorted, (size_t)r->n_hsps * sizeof(hbg_hsp),
                                                cudaMemcpyDeviceToHost, r->stream);
                if (e == cudaSuccess)
                    e = cudaStreamSynchronize(r->stream);
                if (e != cudaSuccess)
                    rc = fail(HBG_ERR_CUDA, std::string("cudaMemcpy (HSPs): ") + cudaGetErrorString(e));
            }
        }
    }
    hbg_result_free(r);
    return rc;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Search without allocation.
//
// For callers that may not allocate device memory at search time --
// allocator-free real-time services whose latency budget has no room for
// cudaMalloc's implicit synchronisation, and hosts that hand the library a
// fixed memory budget at start-up and own every device byte after that -- this
// entry point launches the word finder with its scratch in a file-scope device
// array instead of cudaMalloc'd buffers.  The array is HBG_STATIC_SCRATCH_BYTES
// on every device that loads the library and stays allocated until exit.

namespace {

constexpr int kStaticMaxDevices = 64;
__device__ __align__(256) unsigned char g_static_scratch[HBG_STATIC_SCRATCH_BYTES];

std::mutex g_static_mu;
void *g_static_ptr[kStaticMaxDevices];   // device address of g_static_scratch, per device

// Device address of the scratch array on `device` (current device on entry).
// The array's name is only a host-side stand-in in host code, so the address
// is looked up once per device with cudaGetSymbolAddress.
int static_scratch(int device, void **out) {
    if (device < 0 || device >= kStaticMaxDevices)
        return fail(HBG_ERR_INVALID, "device index outside the static scratch table");
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_ptr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p)
            return fail(HBG_ERR_CUDA, std::string("cudaGetSymbolAddress(static scratch): ") +
                                          cudaGetErrorString(e));
        g_static_ptr[device] = p;
    }
    *out = g_static_ptr[device];
    return HBG_OK;
}

}  // namespace

extern "C" int hbg_search_static(const hbg_db *db, const hbg_batch *batch, const hbg_gpu_options *opt,
                                 hbg_hsp *d_hsps, int64_t hsp_cap, unsigned long long *d_counts,
                                 void *stream) {
    if (!db || !batch || !d_counts || hsp_cap < 0 || (hsp_cap > 0 && !d_hsps))
        return fail(HBG_ERR_INVALID, "hbg_search_static: null argument or negative capacity");
    if (batch->device != db->device)
        return fail(HBG_ERR_STATE, "hbg_search_static: the batch is not resident on the database's device "
                                   "(run hbg_search on it once during set-up)");
    hbg_gpu_options o;
    hbg_default_gpu_options(&o);
    if (opt)
        o = *opt;
    if (!o.use_gpu)
        return fail(HBG_ERR_NO_DEVICE, "use_gpu is 0 and this library has no CPU path");
    if (!valid_opts(&o))
        return fail(HBG_ERR_INVALID, "num_threadsx must be a multiple of 32 in 32..256");
    const hbg::HostBatch &h = batch->host;
    const int64_t nq = (int64_t)h.queries.size(), ng = (int64_t)h.groups.size();
    // scratch layout: [tile counters (one per launch class) | per-query extensions |
    //                  per-query kept | per-group hits]
    static_assert(kMaxLaunchClasses * sizeof(unsigned int) <= 256,
                  "the tile counters must fit the 256-byte head of the static scratch");
    const int64_t need = 256 + 8 * (2 * nq + ng);
    if (need > HBG_STATIC_SCRATCH_BYTES)
        return fail(HBG_ERR_TOO_LONG, "hbg_search_static: the batch needs " + std::to_string(need) +
                                          " scratch bytes, more than HBG_STATIC_SCRATCH_BYTES");
    if (global_diag_len(h, db) > 0)
        return fail(HBG_ERR_TOO_LONG, "hbg_search_static: groups longer than 2008 letters or subjects "
                                      "longer than 32767 - window need global diagonal tables");
    DeviceScope ds(db->device);
    void *scratch = nullptr;
    int rc = static_scratch(db->device, &scratch);
    if (rc != HBG_OK)
        return rc;
    CU(hbg::wordfinder_configure());
    std::vector<LaunchShape> shapes;   // host-side only; no device allocation
    rc = plan_launches(batch, o, db->device, &shapes);
    if (rc != HBG_OK)
        return rc;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *base = (unsigned char *)scratch;
    unsigned int *tile = (unsigned int *)base;
    unsigned long long *q_ext = (unsigned long long *)(base + 256);
    unsigned long long *q_kept = q_ext + nq;
    unsigned long long *g_hits = q_kept + nq;
    // every call shares the array: clear what the kernel accumulates into
    CU(cudaMemsetAsync(scratch, 0, (size_t)need, st));
    CU(cudaMemsetAsync(d_counts, 0, sizeof(unsigned long long) * (size_t)(1 + 2 * nq), st));

    hbg::WordFinderArgs a;
    memset(&a, 0, sizeof(a));
    a.db = db->d_letters;
    a.db_off = db->d_off;
    a.db_len = db->d_len;
    a.order = db->d_order;
    a.n_subj = db->n;
    a.groups = batch->d_groups;
    a.n_groups = (int32_t)ng;
    a.cells = batch->d_cells;
    a.entries = batch->d_entries;
    a.pv = batch->d_pv;
    a.letters = batch->d_letters;
    a.ctx_of = batch->d_ctx_of;
    a.contexts = batch->d_ctx;
    a.queries = batch->d_queries;
    a.window = h.window;
    a.tile_subjects = 128;
    a.tiles_per_group = (db->n + a.tile_subjects - 1) / a.tile_subjects;
    a.n_tiles = 0;
    a.tile_counter = tile;
    a.hsps = d_hsps;
    a.hsp_count = d_counts;
    a.hsp_cap = hsp_cap;
    a.q_extended = q_ext;
    a.q_kept = q_kept;
    a.g_hits = g_hits;
    a.gdiag = nullptr;
    a.gdiag_len = 0;
    a.smem_diag = h.smem_diag_len;
    if (db->n > 0) {
        for (size_t c = 0; c < batch->classes.size(); ++c) {
            const LaunchClass &lc = batch->classes[c];
            a.tile_subjects = class_tile_subjects(batch, db, lc, shapes[c].blocks);
            a.tiles_per_group = (db->n + a.tile_subjects - 1) / a.tile_subjects;
            a.team = shapes[c].team;
            a.n_list = lc.count;
            a.group_list = batch->d_group_list + lc.first;
            a.n_tiles = (int64_t)a.tiles_per_group * ((lc.count + a.team - 1) / a.team);
            a.tile_counter = tile + c;
            a.smem_diag = lc.smem_diag;
            CU(hbg::launch_wordfinder(a, lc.mode, shapes[c].blocks, shapes[c].threads, st));
        }
    }
    // per-query extension and kept counts follow the HSP count in d_counts
    CU(cudaMemcpyAsync(d_counts + 1, q_ext, sizeof(unsigned long long) * (size_t)(2 * nq),
                       cudaMemcpyDeviceToDevice, st));
    return HBG_OK;
}

extern "C" int hbg_debug_fail_allocations(int32_t count) {
    if (count < 0)
        return fail(HBG_ERR_INVALID, "hbg_debug_fail_allocations: negative count");
    g_fail_allocs.store(count);
    return HBG_OK;
}
