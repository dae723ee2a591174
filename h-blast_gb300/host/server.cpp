// server.cpp -- continuous-batching request loop over a resident database.
//
// A dispatcher thread owns max_inflight slots (a CUDA stream plus a reusable
// search result each).  Whenever a slot is free and requests are waiting it
// admits waiting requests -- as many as fit the memory budget (lookup tables
// + HSP buffers of everything in flight), the batch size cap and the cap on
// query letters per batch -- builds their batch on the host and launches the
// search on the slot's stream, so batches overlap with each other's host work
// and GPU tail.  Admission order is arrival order, or (shortest_first_ms > 0)
// requests that have waited that long first, then the shortest: with query
// lengths spread over three decades, short requests stop queueing behind
// long ones, and no request waits behind newer ones for longer than the age
// bound.  A batch's results come back together, so the letter cap keeps one
// batch from holding its short requests for the time of many long ones.
// A finished slot's HSPs are split per request.  Queries in one batch are
// searched independently (own diagonals, own bounds), so every request's
// result equals a search of it alone.
//
// Memory: requests are chosen by an estimate of their device bytes; once the
// batch is built its exact need (hbg_mem_required: lookup tables, HSP and
// sort buffers, diagonal scratch) is checked against the budget left by the
// batches in flight and against the device's free memory.  A batch that does
// not fit -- or whose search fails with HBG_ERR_NOMEM -- goes back to the
// front of the queue and is retried with half as many requests; a lone
// request that does not fit beside running batches waits for them to end.
// Only a request that fails alone on an otherwise idle device fails.
//
// This takes the place of H-BLAST's CPU/GPU load balancer and its
// one-process-per-GPU query split (NF/functions.cpp:51-140,1221-1827;
// scripts/H-BLASTM:212-305).
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/hblast_gpu.h"
#include "batch_builder.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    std::vector<uint8_t> seq;
    std::vector<int32_t> off, len, xd, cu;
    int64_t est_bytes = 0;
    Clock::time_point t0;
    bool done = false;
    int status = HBG_OK;
    std::vector<hbg_hsp> hsps;
    hbg_query_stats stats{0, 0, 0, 0};
    double latency_ms = 0;
    int32_t lone_failures = 0;   // out-of-memory failures while alone on an otherwise idle device
};

struct Slot {
    cudaStream_t stream = nullptr;
    hbg_result *res = nullptr;
    hbg_batch *batch = nullptr;
    std::vector<int64_t> ids;
    int64_t bytes = 0;
    bool busy = false;
};

}  // namespace

struct hbg_server {
    hbg_db *db = nullptr;
    int device = 0;
    int64_t db_residues = 0;
    hbg_word_params wp{11, 40};
    hbg_gpu_options opt{};
    hbg_server_options so{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<int64_t> pending;
    std::map<int64_t, Request> reqs;
    std::vector<Slot> slots;
    int64_t next_id = 1;
    int64_t inflight_bytes = 0;
    int64_t batches = 0, completed = 0, largest = 0, requeued = 0;
    int32_t admit_cap = 0;   // > 0: the next batch takes at most this many requests
    bool hold = false;       // a lone request waits for a running batch to end
    bool stop = false;
    std::thread th;
};

namespace {

// HSPs a query is expected to produce per database letter and query letter
// (about 1.6e-7 on the benchmark's random background); only sizes the first
// buffer -- an overflow relaunches the search with the exact size.
constexpr double kHspsPerCell = 3e-7;

int64_t estimate_hsps(int64_t qlen, int64_t db_res) {
    return (int64_t)(kHspsPerCell * (double)qlen * (double)db_res) + 1024;
}

int64_t estimate_bytes(int64_t qlen, int64_t db_res) {
    // lookup entries (~20 per letter, 2 B), letters + contexts (5 B), the
    // query's cell counts (64 KiB), its share of group cells (132 KiB per
    // 2000 letters), and HSP buffers (raw + ordered + sort keys, ~100 B each)
    return 65536 + qlen * (40 + 5 + 70) + estimate_hsps(qlen, db_res) * 100;
}

// Device memory left free beside a new batch (the runtime, other streams).
constexpr int64_t kFreeReserve = (int64_t)256 << 20;

bool others_busy(const hbg_server *S, const Slot &me) {
    for (const Slot &sl : S->slots)
        if (&sl != &me && sl.busy)
            return true;
    return false;
}

// A request that runs out of device memory alone on an otherwise idle device
// is tried this many more times (the shortfall may be another process's and
// pass) before it fails.
constexpr int32_t kLoneRetries = 3;

// Requests of a batch that did not fit go back to the front of the queue, in
// their order.  Returns false when they cannot fit at all (alone, with
// nothing else running, after kLoneRetries retries): the caller fails them.
bool back_off(hbg_server *S, const std::vector<int64_t> &ids, bool others) {
    if (ids.size() > 1)
        S->admit_cap = std::max<int32_t>(1, (int32_t)ids.size() / 2);
    else if (others)
        S->hold = true;
    else if (++S->reqs[ids[0]].lone_failures > kLoneRetries)
        return false;
    for (auto it = ids.rbegin(); it != ids.rend(); ++it)
        S->pending.push_front(*it);
    S->requeued += (int64_t)ids.size();
    S->cv_work.notify_one();
    return true;
}

void fail_requests(hbg_server *S, const std::vector<int64_t> &ids, int rc) {
    for (int64_t id : ids) {
        Request &r = S->reqs[id];
        r.status = rc;
        r.done = true;
        r.latency_ms = std::chrono::duration<double, std::milli>(Clock::now() - r.t0).count();
        S->completed++;
    }
    S->cv_done.notify_all();
}

bool valid_query(const hbg_query *q) {
    if (!q || !q->sequence || q->length <= 0 || q->length > HBG_MAX_QUERY_LEN || q->num_contexts <= 0 ||
        !q->context_offset || !q->context_length || !q->x_dropoff || !q->cutoff_score)
        return false;
    for (int32_t c = 0; c < q->num_contexts; ++c) {
        const int32_t o = q->context_offset[c], n = q->context_length[c];
        if (o < 0 || n < 0 || o + n > q->length || (c > 0 && o < q->context_offset[c - 1] + q->context_length[c - 1]))
            return false;
        for (int32_t i = 0; i < n; ++i)
            if (q->sequence[o + i] == 0 || q->sequence[o + i] >= HBG_ALPHABET)
                return false;
    }
    return true;
}

void finish_slot(hbg_server *S, Slot &sl, std::unique_lock<std::mutex> &lk) {
    lk.unlock();
    int rc = hbg_result_wait(sl.res);
    std::vector<std::vector<hbg_hsp>> out(sl.ids.size());
    std::vector<hbg_query_stats> st(sl.ids.size(), hbg_query_stats{0, 0, 0, 0});
    for (size_t k = 0; rc == HBG_OK && k < sl.ids.size(); ++k) {
        int64_t first = 0, count = 0;
        rc = hbg_result_query_range(sl.res, (int32_t)k, &first, &count);
        if (rc == HBG_OK) {
            out[k].resize((size_t)count);
            if (count)
                rc = hbg_result_hsps(sl.res, first, count, out[k].data());
            for (auto &h : out[k])
                h.query = 0;
        }
        if (rc == HBG_OK)
            rc = hbg_result_stats(sl.res, (int32_t)k, &st[k]);
    }
    hbg_batch_destroy(sl.batch);
    sl.batch = nullptr;
    const auto now = Clock::now();
    lk.lock();
    S->inflight_bytes -= sl.bytes;
    sl.bytes = 0;
    sl.busy = false;
    S->hold = false;                   // a waiting lone request may fit now
    if (rc == HBG_ERR_NOMEM && back_off(S, sl.ids, others_busy(S, sl))) {
        sl.ids.clear();
        S->cv_done.notify_all();
        return;
    }
    for (size_t k = 0; k < sl.ids.size(); ++k) {
        Request &r = S->reqs[sl.ids[k]];
        r.status = rc;
        if (rc == HBG_OK) {
            r.hsps.swap(out[k]);
            r.stats = st[k];
        }
        r.latency_ms = std::chrono::duration<double, std::milli>(now - r.t0).count();
        r.done = true;
        S->completed++;
    }
    sl.ids.clear();
    S->cv_done.notify_all();
}

void launch_slot(hbg_server *S, Slot &sl, std::vector<int64_t> ids, int64_t est,
                 std::unique_lock<std::mutex> &lk) {
    std::vector<hbg_query> qs(ids.size());
    int64_t qres = 0;
    for (size_t k = 0; k < ids.size(); ++k) {
        Request &r = S->reqs[ids[k]];   // map nodes are stable while unlocked
        qs[k] = hbg_query{r.seq.data(), (int32_t)r.seq.size(), (int32_t)r.off.size(), r.off.data(),
                          r.len.data(), r.xd.data(), r.cu.data()};
        qres += (int64_t)r.seq.size();
    }
    sl.ids = ids;
    sl.bytes = est;
    sl.busy = true;
    S->inflight_bytes += est;
    lk.unlock();
    const int64_t cap = estimate_hsps(qres, S->db_residues);
    int rc = hbg_batch_create(qs.data(), (int32_t)qs.size(), &S->wp, S->so.max_group_len, &sl.batch);
    int64_t need = 0;
    size_t free_b = 0, total_b = 0;
    if (rc == HBG_OK)
        rc = hbg_mem_required(S->db, sl.batch, cap, &need);
    if (rc == HBG_OK && cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        free_b = (size_t)INT64_MAX;        // unknown: rely on the budget and on allocation failures
    }
    lk.lock();
    const bool others = others_busy(S, sl);
    if (rc == HBG_OK) {
        const bool over = need > S->so.memory_budget - (S->inflight_bytes - est) ||
                          need + kFreeReserve > (int64_t)std::min<size_t>(free_b, (size_t)INT64_MAX);
        if (over && (ids.size() > 1 || others)) {
            S->inflight_bytes -= est;
            sl.busy = false;
            sl.ids.clear();
            sl.bytes = 0;
            hbg_batch *b = sl.batch;
            sl.batch = nullptr;
            back_off(S, ids, others);
            lk.unlock();
            hbg_batch_destroy(b);
            lk.lock();
            return;
        }
        S->inflight_bytes += need - est;    // account the exact size from now on
        sl.bytes = need;
        lk.unlock();
        rc = hbg_search(S->db, sl.batch, &S->opt, cap, sl.stream, &sl.res);
        lk.lock();
    }
    if (rc != HBG_OK) {
        S->inflight_bytes -= sl.bytes;
        sl.busy = false;
        sl.ids.clear();
        sl.bytes = 0;
        hbg_batch *b = sl.batch;
        sl.batch = nullptr;
        if (!(rc == HBG_ERR_NOMEM && back_off(S, ids, others_busy(S, sl))))
            fail_requests(S, ids, rc);
        if (b) {
            lk.unlock();
            hbg_batch_destroy(b);
            lk.lock();
        }
        return;
    }
    S->batches++;
    S->largest = std::max<int64_t>(S->largest, (int64_t)ids.size());
    S->admit_cap = 0;
}

void dispatcher(hbg_server *S) {
    cudaSetDevice(S->device);
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        bool busy = false;
        for (Slot &sl : S->slots) {
            if (!sl.busy)
                continue;
            lk.unlock();
            const cudaError_t q = cudaStreamQuery(sl.stream);
            lk.lock();
            if (q == cudaErrorNotReady) {
                busy = true;
                continue;
            }
            finish_slot(S, sl, lk);
        }
        Slot *free_slot = nullptr;
        for (Slot &sl : S->slots)
            if (!sl.busy) {
                free_slot = &sl;
                break;
            }
        if (free_slot && !S->pending.empty() && !S->hold) {
            std::vector<int64_t> cand(S->pending.begin(), S->pending.end());
            if (S->so.shortest_first_ms > 0) {
                const Clock::time_point now = Clock::now();
                const auto aged = [&](int64_t id) {
                    return std::chrono::duration<double, std::milli>(now - S->reqs[id].t0).count() >=
                           S->so.shortest_first_ms;
                };
                auto mid = std::stable_partition(cand.begin(), cand.end(), aged);
                std::stable_sort(mid, cand.end(), [&](int64_t x, int64_t y) {
                    return S->reqs[x].seq.size() < S->reqs[y].seq.size();
                });
            }
            std::vector<int64_t> ids;
            int64_t bytes = 0, letters = 0;
            const int32_t max_q = S->admit_cap > 0 ? std::min(S->admit_cap, S->so.max_batch_queries)
                                                   : S->so.max_batch_queries;
            for (int64_t id : cand) {
                if ((int32_t)ids.size() >= max_q)
                    break;
                const Request &r = S->reqs[id];
                const int64_t room = S->so.memory_budget - S->inflight_bytes - bytes;
                // admit while the budget and the letter cap hold; an oversized
                // request runs alone
                if (r.est_bytes > room && !(ids.empty() && S->inflight_bytes == 0))
                    break;
                if (S->so.max_batch_letters > 0 && !ids.empty() &&
                    letters + (int64_t)r.seq.size() > S->so.max_batch_letters)
                    break;
                ids.push_back(id);
                bytes += r.est_bytes;
                letters += (int64_t)r.seq.size();
            }
            if (!ids.empty()) {
                std::deque<int64_t> rest;
                for (int64_t id : S->pending)
                    if (std::find(ids.begin(), ids.end(), id) == ids.end())
                        rest.push_back(id);
                S->pending.swap(rest);
                launch_slot(S, *free_slot, ids, bytes, lk);
                continue;
            }
        }
        if (S->stop && S->pending.empty() && !busy)
            break;
        // poll running searches often; otherwise sleep until work arrives
        S->cv_work.wait_for(lk, busy ? std::chrono::microseconds(100) : std::chrono::microseconds(5000));
    }
}

}  // namespace

extern "C" {

int hbg_server_default_options(hbg_server_options *o) {
    if (!o)
        return HBG_ERR_INVALID;
    o->max_inflight = 1;
    o->max_batch_queries = 512;
    o->memory_budget = (int64_t)32 << 30;
    o->max_group_len = 0;
    o->max_batch_letters = 8192;
    o->shortest_first_ms = 2000;
    o->seg_blastx = 0;
    return HBG_OK;
}

int hbg_server_create(hbg_db *db, const hbg_word_params *params, const hbg_gpu_options *opt,
                      const hbg_server_options *sopt, hbg_server **out) {
    if (!db || !params || !out)
        return HBG_ERR_INVALID;
    *out = nullptr;
    hbg_server *S = new hbg_server;
    S->db = db;
    S->wp = *params;
    hbg_default_gpu_options(&S->opt);
    if (opt)
        S->opt = *opt;
    hbg_server_default_options(&S->so);
    if (sopt)
        S->so = *sopt;
    if (S->so.max_inflight < 1 || S->so.max_inflight > 16 || S->so.max_batch_queries < 1 ||
        S->so.memory_budget <= 0 || S->so.max_batch_letters < 0 || S->so.shortest_first_ms < 0 ||
        (S->so.seg_blastx != 0 && S->so.seg_blastx != 1)) {
        delete S;
        return HBG_ERR_INVALID;
    }
    int32_t nsub = 0;
    hbg_db_info(db, &nsub, &S->db_residues, nullptr);
    S->device = S->opt.method;
    cudaSetDevice(S->device);
    S->slots.resize(S->so.max_inflight);
    for (Slot &sl : S->slots)
        if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess) {
            for (Slot &x : S->slots)
                if (x.stream)
                    cudaStreamDestroy(x.stream);
            delete S;
            return HBG_ERR_CUDA;
        }
    S->th = std::thread(dispatcher, S);
    *out = S;
    return HBG_OK;
}

static int submit(hbg_server *S, Request &&r, int64_t *ticket) {
    std::lock_guard<std::mutex> lock(S->mu);
    if (S->stop)
        return HBG_ERR_STATE;
    const int64_t id = S->next_id++;
    r.est_bytes = estimate_bytes((int64_t)r.seq.size(), S->db_residues);
    r.t0 = Clock::now();
    S->reqs.emplace(id, std::move(r));
    S->pending.push_back(id);
    *ticket = id;
    S->cv_work.notify_one();
    return HBG_OK;
}

int hbg_server_submit(hbg_server *S, const hbg_query *q, int64_t *ticket) {
    if (!S || !ticket || !valid_query(q))
        return HBG_ERR_INVALID;
    Request r;
    r.seq.assign(q->sequence, q->sequence + q->length);
    r.off.assign(q->context_offset, q->context_offset + q->num_contexts);
    r.len.assign(q->context_length, q->context_length + q->num_contexts);
    r.xd.assign(q->x_dropoff, q->x_dropoff + q->num_contexts);
    r.cu.assign(q->cutoff_score, q->cutoff_score + q->num_contexts);
    return submit(S, std::move(r), ticket);
}

int hbg_server_submit_blastx(hbg_server *S, const uint8_t *nt, int32_t nt_len, const int32_t *xd,
                             const int32_t *cu, int64_t *ticket) {
    if (!S || !ticket || !nt || nt_len < 3 || (int64_t)nt_len * 2 + 6 > HBG_MAX_QUERY_LEN || !xd || !cu)
        return HBG_ERR_INVALID;
    Request r;
    r.seq = hbg::translate_six_frames(nt, nt_len, &r.off, &r.len);
    if (S->so.seg_blastx)
        for (int f = 0; f < 6; ++f)
            hbg::seg_mask(r.seq.data() + r.off[f], r.len[f], 12, 2.2, 2.5);
    r.xd.assign(xd, xd + 6);
    r.cu.assign(cu, cu + 6);
    return submit(S, std::move(r), ticket);
}

int hbg_server_wait(hbg_server *S, int64_t ticket, int32_t timeout_ms, int64_t *n_hsps) {
    if (!S)
        return HBG_ERR_INVALID;
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end())
        return HBG_ERR_INVALID;
    auto ready = [&] { return it->second.done; };
    if (timeout_ms < 0)
        S->cv_done.wait(lk, ready);
    else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
        return HBG_ERR_STATE;
    if (n_hsps)
        *n_hsps = (int64_t)it->second.hsps.size();
    return it->second.status;
}

int hbg_server_take(hbg_server *S, int64_t ticket, hbg_hsp *out, int64_t cap, hbg_query_stats *stats,
                    double *latency_ms) {
    if (!S)
        return HBG_ERR_INVALID;
    std::lock_guard<std::mutex> lock(S->mu);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end())
        return HBG_ERR_INVALID;
    Request &r = it->second;
    if (!r.done)
        return HBG_ERR_STATE;
    if (r.status != HBG_OK) {
        const int st = r.status;
        S->reqs.erase(it);
        return st;
    }
    if ((int64_t)r.hsps.size() > cap || (!out && !r.hsps.empty()))
        return HBG_ERR_CAPACITY;
    if (!r.hsps.empty())
        memcpy(out, r.hsps.data(), r.hsps.size() * sizeof(hbg_hsp));
    if (stats)
        *stats = r.stats;
    if (latency_ms)
        *latency_ms = r.latency_ms;
    S->reqs.erase(it);
    return HBG_OK;
}

int hbg_server_counters(const hbg_server *S, int64_t *batches, int64_t *queries, int64_t *largest) {
    if (!S)
        return HBG_ERR_INVALID;
    hbg_server *m = const_cast<hbg_server *>(S);
    std::lock_guard<std::mutex> lock(m->mu);
    if (batches)
        *batches = S->batches;
    if (queries)
        *queries = S->completed;
    if (largest)
        *largest = S->largest;
    return HBG_OK;
}

int hbg_server_requeued(const hbg_server *S, int64_t *requeued) {
    if (!S || !requeued)
        return HBG_ERR_INVALID;
    hbg_server *m = const_cast<hbg_server *>(S);
    std::lock_guard<std::mutex> lock(m->mu);
    *requeued = S->requeued;
    return HBG_OK;
}

int hbg_server_destroy(hbg_server *S) {
    if (!S)
        return HBG_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lock(S->mu);
        S->stop = true;
        S->cv_work.notify_all();
    }
    if (S->th.joinable())
        S->th.join();
    cudaSetDevice(S->device);
    for (Slot &sl : S->slots) {
        if (sl.res)
            hbg_result_free(sl.res);
        if (sl.batch)
            hbg_batch_destroy(sl.batch);
        if (sl.stream)
            cudaStreamDestroy(sl.stream);
    }
    delete S;
    return HBG_OK;
}

}  // extern "C"
