// batch_builder.cpp -- query packing, six-frame translation and the
// neighbourhood-word lookup tables of a batch (host side).
//
// Lookup-table rule (NCBI BLAST+ 2.2.28 blast_aalookup.c, the table H-BLAST
// consumes at h_blast_v1.1/H-BLAST/h_blast.cu:940-958): word size 3 over the
// 28-letter NCBIstdaa alphabet, 5 bits per letter (index (a<<10)|(b<<5)|c,
// as the kernel builds it at h_blast_kernel.cu:610-614); query offset p is
// stored in cell w when the three letters at p lie inside one context and
// score(query[p..p+2], w) >= threshold.  Cells hold offsets in ascending
// order, the order lut_sorting enforces (h_blast.cu:165-194).
#include "batch_builder.h"

#include <string.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

namespace hbg {

namespace {

const int8_t kBlosum62[28 * 32] = {
#include "../csrc/blosum62.inc"
};

// Neighbour words of every query word, computed once per distinct word and
// kept for the life of the process (one cache per threshold), so batches
// built one after another -- a serving loop -- reuse the enumerations.
class NeighbourCache {
  public:
    explicit NeighbourCache(int32_t threshold) : threshold_(threshold) {
        for (int x = 0; x < HBG_ALPHABET; ++x) {
            int m = -1000;
            for (int y = 0; y < HBG_ALPHABET; ++y)
                m = std::max<int>(m, kBlosum62[x * 32 + y]);
            row_max_[x] = m;
        }
        done_.assign(HBG_NUM_CELLS, 0);
        lists_.resize(HBG_NUM_CELLS);
    }

    // The neighbours of a word that prepare() has enumerated; read-only, so
    // any number of threads may call it.
    const std::vector<uint16_t> &get(uint8_t a, uint8_t b, uint8_t c) const {
        return lists_[(a << 10) | (b << 5) | c];
    }

    // Enumerate the neighbourhoods of the flagged words not seen before, in
    // parallel.  Builds running at the same time take turns here; a list,
    // once written, never changes.
    template <typename ParallelFor>
    void prepare(const std::vector<uint8_t> &need, ParallelFor &&pfor) {
        std::lock_guard<std::mutex> lock(mu_);
        std::vector<int32_t> keys;
        for (int32_t k = 0; k < HBG_NUM_CELLS; ++k)
            if (need[k] && !done_[k])
                keys.push_back(k);
        pfor((int64_t)keys.size(), [&](int64_t i) {
            const int32_t k = keys[i];
            enumerate((uint8_t)(k >> 10), (uint8_t)((k >> 5) & 31), (uint8_t)(k & 31), &lists_[k]);
        });
        for (int32_t k : keys)
            done_[k] = 1;
    }

  private:
    void enumerate(uint8_t a, uint8_t b, uint8_t c, std::vector<uint16_t> *out) {
        const int8_t *ra = kBlosum62 + a * 32;
        const int8_t *rb = kBlosum62 + b * 32;
        const int8_t *rc = kBlosum62 + c * 32;
        for (int x = 0; x < HBG_ALPHABET; ++x) {
            int s1 = ra[x];
            if (s1 + row_max_[b] + row_max_[c] < threshold_)
                continue;
            for (int y = 0; y < HBG_ALPHABET; ++y) {
                int s2 = s1 + rb[y];
                if (s2 + row_max_[c] < threshold_)
                    continue;
                for (int z = 0; z < HBG_ALPHABET; ++z)
                    if (s2 + rc[z] >= threshold_)
                        out->push_back((uint16_t)((x << 10) | (y << 5) | z));
            }
        }
    }

    int32_t threshold_;
    std::array<int, HBG_ALPHABET> row_max_;
    std::vector<uint8_t> done_;
    std::vector<std::vector<uint16_t>> lists_;
    std::mutex mu_;
};

NeighbourCache &neighbour_cache(int32_t threshold) {
    static std::mutex mu;
    static std::map<int32_t, std::unique_ptr<NeighbourCache>> caches;
    std::lock_guard<std::mutex> lock(mu);
    std::unique_ptr<NeighbourCache> &c = caches[threshold];
    if (!c)
        c.reset(new NeighbourCache(threshold));
    return *c;
}

// Run body(i) for i in [0, n) on up to 16 host threads (items taken from a
// shared counter).
void parallel_for(int64_t n, const std::function<void(int64_t)> &body) {
    const int64_t nt = std::min<int64_t>({n, 16, (int64_t)std::max(1u, std::thread::hardware_concurrency())});
    if (nt <= 1) {
        for (int64_t i = 0; i < n; ++i)
            body(i);
        return;
    }
    std::atomic<int64_t> next{0};
    auto run = [&] {
        for (int64_t i = next++; i < n; i = next++)
            body(i);
    };
    std::vector<std::thread> th;
    for (int64_t t = 1; t < nt; ++t)
        th.emplace_back(run);
    run();
    for (std::thread &x : th)
        x.join();
}

int32_t next_pow2(int32_t v) {
    int32_t n = 1;
    while (n < v)
        n <<= 1;
    return n;
}

}  // namespace

int32_t blosum62(int32_t a, int32_t b) {
    if (a < 0 || a >= HBG_ALPHABET || b < 0 || b >= HBG_ALPHABET)
        return -128;
    return kBlosum62[a * 32 + b];
}

const int8_t *blosum62_table() { return kBlosum62; }

std::string build_batch(const std::vector<QueryIn> &qs, int32_t threshold,
                        int32_t window, int32_t max_group_len, HostBatch *out, double mode_hits) {
    if (window < 1 || window > 100000)
        return "window must be in 1..100000";
    if (qs.empty())
        return "empty batch";
    if (max_group_len <= 0)
        max_group_len = kDefaultGroupLen;
    if (mode_hits < 0)
        mode_hits = kOffsetModeHits;
    HostBatch &b = *out;
    b = HostBatch();
    b.threshold = threshold;
    b.window = window;

    // --- validate and pack queries into groups (in order) ---
    std::vector<int32_t> group_of(qs.size());
    int32_t cur_len = 0, cur_n = 0;
    int32_t n_groups = 0;
    for (size_t k = 0; k < qs.size(); ++k) {
        const QueryIn &q = qs[k];
        if (q.len <= 0 || q.len > HBG_MAX_QUERY_LEN)
            return "query " + std::to_string(k) + ": length must be in 1.." +
                   std::to_string(HBG_MAX_QUERY_LEN);
        size_t nc = q.ctx_off.size();
        if (nc == 0 || q.ctx_len.size() != nc || q.xdrop.size() != nc || q.cutoff.size() != nc)
            return "query " + std::to_string(k) + ": bad context arrays";
        for (size_t c = 0; c < nc; ++c) {
            if (q.ctx_off[c] < 0 || q.ctx_len[c] < 0 ||
                q.ctx_off[c] + q.ctx_len[c] > q.len)
                return "query " + std::to_string(k) + ": context outside the query";
            if (c > 0 && q.ctx_off[c] < q.ctx_off[c - 1] + q.ctx_len[c - 1])
                return "query " + std::to_string(k) + ": contexts overlap or are unordered";
            if (q.xdrop[c] < 0)
                return "query " + std::to_string(k) + ": negative x_dropoff";
            for (int32_t i = 0; i < q.ctx_len[c]; ++i) {
                uint8_t r = q.seq[q.ctx_off[c] + i];
                if (r == 0 || r >= HBG_ALPHABET)
                    return "query " + std::to_string(k) + ": letter outside NCBIstdaa 1..27";
            }
        }
        int32_t need = (cur_n > 0 ? window : 0) + q.len;
        if (cur_n == 0 || cur_len + need > max_group_len || cur_n >= kMaxQueriesPerGroup) {
            if (cur_n > 0)
                ++n_groups;
            cur_len = q.len;
            cur_n = 1;
        } else {
            cur_len += need;
            ++cur_n;
        }
        group_of[k] = n_groups;
        b.max_query_len = std::max(b.max_query_len, q.len);
    }
    ++n_groups;

    // --- lay out letters, queries, contexts ---
    b.groups.resize(n_groups);
    b.queries.resize(qs.size());
    int64_t seq_pos = 0;
    for (int32_t g = 0, k = 0; g < n_groups; ++g) {
        HbgGroup &G = b.groups[g];
        memset(&G, 0, sizeof(G));
        G.seq_base = seq_pos;
        G.first_query = k;
        int32_t glen = 0;
        while (k < (int32_t)qs.size() && group_of[k] == g) {
            const QueryIn &q = qs[k];
            if (glen > 0) {
                b.letters.insert(b.letters.end(), window, 0);
                b.ctx_of.insert(b.ctx_of.end(), window, -1);
                glen += window;
            }
            HbgQueryDesc &Q = b.queries[k];
            memset(&Q, 0, sizeof(Q));
            Q.group = g;
            Q.start = glen;
            Q.len = q.len;
            Q.first_ctx = (int32_t)b.contexts.size();
            Q.n_ctx = (int32_t)q.ctx_off.size();
            size_t at = b.letters.size();
            b.letters.insert(b.letters.end(), q.seq, q.seq + q.len);
            b.ctx_of.insert(b.ctx_of.end(), q.len, -1);
            for (int32_t c = 0; c < Q.n_ctx; ++c) {
                HbgContext C;
                C.query = k;
                C.local = c;
                C.x_dropoff = q.xdrop[c];
                C.cutoff = q.cutoff[c];
                int32_t ci = (int32_t)b.contexts.size();
                b.contexts.push_back(C);
                for (int32_t i = 0; i < q.ctx_len[c]; ++i)
                    b.ctx_of[at + q.ctx_off[c] + i] = ci;
            }
            // letters between contexts are sentinels whatever the caller put there
            for (int32_t i = 0; i < q.len; ++i)
                if (b.ctx_of[at + i] < 0)
                    b.letters[at + i] = 0;
            glen += q.len;
            ++k;
        }
        G.n_queries = k - G.first_query;
        G.glen = glen;
        G.diag_len = next_pow2(glen + window);
        G.placement = G.diag_len <= kSmemDiagMax ? 0 : 1;
        if (G.placement)
            b.max_diag_len = std::max(b.max_diag_len, G.diag_len);
        else
            b.smem_diag_len = std::max(b.smem_diag_len, G.diag_len);
        seq_pos += glen;
    }

    // --- lookup tables: count, then fill ---
    NeighbourCache &nb = neighbour_cache(threshold);
    b.cells.assign((size_t)n_groups * HBG_CELL_STRIDE, 0);
    b.pv.assign((size_t)n_groups * HBG_PV_WORDS, 0);
    b.query_cells.assign(qs.size() * (size_t)HBG_NUM_CELLS, 0);
    // the neighbourhoods of every word in the batch, enumerated in parallel;
    // then per group (in parallel: groups own disjoint cells, queries and
    // entries) count, prefix, and fill
    auto valid = [&](const int32_t *gc, int32_t p) {
        const int32_t c0 = gc[p];
        return c0 >= 0 && gc[p + 1] == c0 && gc[p + 2] == c0;
    };
    {
        std::vector<uint8_t> need(HBG_NUM_CELLS, 0);
        for (int32_t g = 0; g < n_groups; ++g) {
            const HbgGroup &G = b.groups[g];
            const uint8_t *gs = b.letters.data() + G.seq_base;
            const int32_t *gc = b.ctx_of.data() + G.seq_base;
            for (int32_t p = 0; p + HBG_WORD_SIZE <= G.glen; ++p)
                if (valid(gc, p))
                    need[(gs[p] << 10) | (gs[p + 1] << 5) | gs[p + 2]] = 1;
        }
        nb.prepare(need, parallel_for);
    }
    std::vector<uint32_t> group_entries(n_groups, 0);
    parallel_for(n_groups, [&](int64_t gi) {
        const int32_t g = (int32_t)gi;
        HbgGroup &G = b.groups[g];
        const uint8_t *gs = b.letters.data() + G.seq_base;
        const int32_t *gc = b.ctx_of.data() + G.seq_base;
        std::vector<uint32_t> count(HBG_NUM_CELLS, 0);
        for (int32_t p = 0; p + HBG_WORD_SIZE <= G.glen; ++p) {
            if (!valid(gc, p))
                continue;
            const std::vector<uint16_t> &ws = nb.get(gs[p], gs[p + 1], gs[p + 2]);
            uint16_t *qc = b.query_cells.data() + (size_t)b.contexts[gc[p]].query * HBG_NUM_CELLS;
            for (uint16_t w : ws) {
                ++count[w];
                ++qc[w];
            }
        }
        uint32_t *cs = b.cells.data() + (size_t)g * HBG_CELL_STRIDE;
        uint32_t *pv = b.pv.data() + (size_t)g * HBG_PV_WORDS;
        uint32_t acc = 0;
        for (int32_t w = 0; w < HBG_NUM_CELLS; ++w) {
            cs[w] = acc;
            acc += count[w];
            if (count[w])
                pv[w >> 5] |= 1u << (w & 31);
        }
        cs[HBG_NUM_CELLS] = acc;
        group_entries[g] = acc;
        // expected hits per subject offset on typical proteins: entries of
        // words over the 20 standard letters, each such word taken as
        // equally likely (1 / 8000)
        static const uint8_t kStd[20] = {1, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 22};
        uint64_t std_entries = 0;
        for (int x = 0; x < 20; ++x)
            for (int y = 0; y < 20; ++y)
                for (int z = 0; z < 20; ++z)
                    std_entries += count[(kStd[x] << 10) | (kStd[y] << 5) | kStd[z]];
        G.mode = (double)std_entries / 8000.0 >= mode_hits ? 1 : 0;
    });
    int64_t entry_pos = 0;
    for (int32_t g = 0; g < n_groups; ++g) {
        b.groups[g].entry_base = entry_pos;
        entry_pos += group_entries[g];
    }
    b.entries.resize((size_t)entry_pos);
    parallel_for(n_groups, [&](int64_t gi) {
        const int32_t g = (int32_t)gi;
        const HbgGroup &G = b.groups[g];
        const uint8_t *gs = b.letters.data() + G.seq_base;
        const int32_t *gc = b.ctx_of.data() + G.seq_base;
        const uint32_t *cs = b.cells.data() + (size_t)g * HBG_CELL_STRIDE;
        // fill, ascending p inside each cell
        std::vector<uint32_t> cursor(cs, cs + HBG_NUM_CELLS);
        uint16_t *ge = b.entries.data() + G.entry_base;
        for (int32_t p = 0; p + HBG_WORD_SIZE <= G.glen; ++p) {
            if (!valid(gc, p))
                continue;
            const std::vector<uint16_t> &ws = nb.get(gs[p], gs[p + 1], gs[p + 2]);
            for (uint16_t w : ws)
                ge[cursor[w]++] = (uint16_t)p;
        }
    });
    return std::string();
}

// --- six-frame translation ------------------------------------------------

namespace {
// Standard genetic code (NCBI transl_table 1), codons in TCAG order.
const char kStdCode[] = "FFLLSSSSYY**CC*WLLLLPPPPHHQQRRRRIIIMTTTTNNKKSSRRVVVVAAAADDEEGGGG";
const char kStdaa[] = "-ABCDEFGHIKLMNPQRSTVWXYZU*OJ";

struct CodonTable {
    uint8_t aa[64];
    CodonTable() {
        for (int i = 0; i < 64; ++i) {
            const char *p = strchr(kStdaa, kStdCode[i]);
            aa[i] = (uint8_t)(p - kStdaa);
        }
    }
};
const CodonTable kCodons;

// A=0 C=1 G=2 T=3 -> position in TCAG order; -1 for anything else
inline int tcag(uint8_t nt) {
    static const int8_t m[4] = {2, 1, 3, 0};
    return nt < 4 ? m[nt] : -1;
}
inline uint8_t codon(uint8_t a, uint8_t b, uint8_t c) {
    int x = tcag(a), y = tcag(b), z = tcag(c);
    if (x < 0 || y < 0 || z < 0)
        return 21;  // X
    return kCodons.aa[x * 16 + y * 4 + z];
}
inline uint8_t comp(uint8_t nt) { return nt < 4 ? (uint8_t)(3 - nt) : (uint8_t)4; }
}  // namespace

std::vector<uint8_t> translate_six_frames(const uint8_t *nt, int32_t n,
                                          std::vector<int32_t> *ctx_off,
                                          std::vector<int32_t> *ctx_len) {
    std::vector<uint8_t> out;
    out.reserve((size_t)(2 * n + 6));
    ctx_off->assign(6, 0);
    ctx_len->assign(6, 0);
    for (int f = 0; f < 6; ++f) {
        int32_t start = f % 3;
        int32_t len = n > start ? (n - start) / 3 : 0;
        if (f > 0)
            out.push_back(0);
        (*ctx_off)[f] = (int32_t)out.size();
        (*ctx_len)[f] = len;
        for (int32_t i = 0; i < len; ++i) {
            int32_t p = start + 3 * i;
            if (f < 3)
                out.push_back(codon(nt[p], nt[p + 1], nt[p + 2]));
            else
                out.push_back(codon(comp(nt[n - 1 - p]), comp(nt[n - 2 - p]),
                                    comp(nt[n - 3 - p])));
        }
    }
    return out;
}

}  // namespace hbg
