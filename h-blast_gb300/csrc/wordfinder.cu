// wordfinder.cu -- fused seed scan + two-hit diagonal test + ungapped X-drop
// extension for sm_103a.
//
// Work decomposition: a persistent grid of CTAs takes tiles (query group,
// block of subjects) from a global counter; the warps of a CTA take subjects
// of the tile from a shared counter, one warp per (group, subject) item.
//
// Per item the warp scans the subject 32 offsets at a time: lane l computes
// the 15-bit word index of offset s0+l, tests the group's presence vector in
// shared memory and reads the cell bounds.  Hits are then applied in the
// order the CPU word finder visits them (subject offset, then ascending query
// offset) in one of two modes chosen per group: chunk mode (sparse groups) --
// a warp scan compacts the chunk's hits and 32 are applied at a time, hits of
// one batch on the same diagonal ordered with match.any; offset mode (dense
// groups) -- one offset at a time, lane i taking entry i of its cell.
//
// Diagonal state follows NCBI's DiagStruct (last hit + flag) and its offset
// trick: the offset grows by subject length + window per item so stale
// entries read as "no recent hit", and the table is cleared when the offset
// no longer fits (Blast_ExtendWordExit; H-BLAST h_blast_kernel.cu:1023).  Each
// warp owns a 16-bit table in shared memory, or a 32-bit slice of the global
// scratch for groups (or subjects) too long for it.
//
// The per-hit rule is the two-hit state machine of NCBI aa_ungapped.c, which
// H-BLAST restates at h_blast_kernel.cu:672-871; the extension is
// s_BlastAaExtendTwoHit/Left/Right (h_blast_kernel.cu:1069-1540), with the
// left walk also taken when min(s, q) == 0 as NCBI does.
#include <cuda_runtime.h>

#include "kernels.h"

namespace hbg {

namespace {

constexpr int kMaxQ = 64;         // kMaxQueriesPerGroup

__constant__ int8_t c_blosum[28 * 32] = {
#include "blosum62.inc"
};

// Dynamic shared memory of a CTA: a Head, then one Slot per query group the
// CTA searches at a time (the groups that share each pass over a block of
// subjects: "warps per subject"), then the per-warp regions and tables.
// Sizes are multiples of 16 bytes: the per-warp tables after them are
// cleared with 16-byte stores.
extern __shared__ __align__(16) unsigned char g_smem[];

struct __align__(16) Head {
    int8_t matrix[28 * 32];   // BLOSUM62, query letter x 32 + subject letter
    long long tile;
    long long pad;
};

struct __align__(16) Slot {
    uint32_t pv[HBG_PV_WORDS];   // presence vector of the slot's group
    unsigned int q_ext[kMaxQ];   // per query of the group: extensions tried, kept
    unsigned int q_kept[kMaxQ];
    unsigned long long hits;     // lookup hits of the group in this tile
    int next;                    // next subject of the tile for the slot's warps
    int group;                   // group index, -1 when the tile has none for this slot
};

__device__ __forceinline__ const int8_t *score_matrix() { return reinterpret_cast<const Head *>(g_smem)->matrix; }

__device__ __forceinline__ int sc(const int8_t *m, int q, int s) { return m[q * 32 + s]; }

// Four letters from p (any alignment): two aligned 32-bit loads and a funnel
// shift.  Reads up to 7 bytes past p; the database and batch letter buffers
// carry 64 bytes of tail padding, and walks only take blocks that start at or
// after the sequence start.
__device__ __forceinline__ uint32_t load4(const uint8_t *p) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
    return __funnelshift_r(__ldg(w), __ldg(w + 1), (uint32_t)(a & 3) * 8);
}

// X-drop walk to the left from (s_off, q_off) inclusive, at most
// min(s_off, q_off) + 1 letters; returns the best score, *len = letters in
// the best walk.  Letters are read four at a time; every letter is checked.
__device__ int extend_left(const int8_t *m, const uint8_t *s, const uint8_t *q, int s_off,
                           int q_off, int dropoff, int *len) {
    const int n = min(s_off, q_off);
    int best_i = n + 1;
    int score = 0, maxscore = 0;
    int k = 0;             // letters taken: the next is (s_off - k, q_off - k), index i = n - k
    bool stop = false;
    while (!stop && k + 3 <= n) {
        const uint32_t sw = load4(s + s_off - k - 3);
        const uint32_t qw = load4(q + q_off - k - 3);
        // four letters without branches: letters after a stop change nothing
#pragma unroll
        for (int j = 3; j >= 0; --j) {
            const int ns = score + sc(m, (qw >> (8 * j)) & 255u, (sw >> (8 * j)) & 255u);
            const bool better = !stop && ns > maxscore;
            best_i = better ? n - k - (3 - j) : best_i;
            maxscore = better ? ns : maxscore;
            stop = stop || maxscore - ns >= dropoff;
            score = ns;
        }
        k += 4;
    }
    for (; !stop && k <= n; ++k) {
        score += sc(m, q[q_off - k], s[s_off - k]);
        if (score > maxscore) {
            maxscore = score;
            best_i = n - k;
        }
        if (maxscore - score >= dropoff)
            stop = true;
    }
    *len = n - best_i + 1;
    return maxscore;
}

// X-drop walk to the right from (s_off, q_off) that also stops when the
// running score is <= 0; *s_last_off = the last subject offset examined
// (s_off + n when the walk reaches a sequence end).
__device__ int extend_right(const int8_t *m, const uint8_t *s, int s_len, const uint8_t *q,
                            int q_len, int s_off, int q_off, int dropoff, int maxscore,
                            int *len, int *s_last_off) {
    const int n = min(s_len - s_off, q_len - q_off);
    int best_i = -1;
    int score = maxscore;
    int i = 0;
    bool stop = false;
    while (!stop && i + 3 < n) {
        const uint32_t sw = load4(s + s_off + i);
        const uint32_t qw = load4(q + q_off + i);
        int adv = 4;           // letters before the stopping one
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            const int ns = score + sc(m, (qw >> (8 * jj)) & 255u, (sw >> (8 * jj)) & 255u);
            const bool better = !stop && ns > maxscore;
            best_i = better ? i + jj : best_i;
            maxscore = better ? ns : maxscore;
            const bool end = !stop && (ns <= 0 || maxscore - ns >= dropoff);
            adv = end ? jj : adv;
            stop = stop || end;
            score = stop ? score : ns;
        }
        i += adv;
    }
    for (; !stop && i < n; ++i) {
        score += sc(m, q[q_off + i], s[s_off + i]);
        if (score > maxscore) {
            maxscore = score;
            best_i = i;
        }
        if (score <= 0 || maxscore - score >= dropoff)
            break;
    }
    *len = best_i + 1;
    *s_last_off = s_off + i;
    return maxscore;
}

struct Ext {
    int q_start, s_start, len, score, s_last_off;
    bool right;
};

__device__ Ext extend_two_hit(const int8_t *m, const uint8_t *s, int s_len, const uint8_t *q,
                              int q_len, int s_left_off, int s_right_off, int q_right_off,
                              int dropoff) {
    Ext e;
    int right_d = 0, best = 0, acc = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        acc += sc(m, q[q_right_off + i], s[s_right_off + i]);
        if (acc > best) {
            best = acc;
            right_d = i + 1;
        }
    }
    q_right_off += right_d;
    s_right_off += right_d;
    int left_d = 0;
    int left_score = extend_left(m, s, q, s_right_off - 1, q_right_off - 1, dropoff, &left_d);
    int right_score = 0, rlen = 0;
    e.s_last_off = s_right_off;
    e.right = false;
    if (left_d >= s_right_off - s_left_off) {
        e.right = true;
        right_score = extend_right(m, s, s_len, q, q_len, s_right_off, q_right_off, dropoff,
                                   left_score, &rlen, &e.s_last_off);
    }
    e.q_start = q_right_off - left_d;
    e.s_start = s_right_off - left_d;
    e.len = left_d + rlen;
    e.score = max(left_score, right_score);
    return e;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned r;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}
// ---------------------------------------------------------------------------
// Diagonal cells.  NCBI's DiagStruct keeps a 31-bit last hit and a 1-bit flag
// against an offset that grows by subject length + window per subject.  The
// shared-memory tables use 16-bit cells (15-bit last hit): the offset is
// reset and the table cleared whenever offset + subject length would not fit,
// so every stored value stays exact.  Tables in global memory keep 32 bits.

template <typename Cell>
struct CellTraits;
template <>
struct CellTraits<uint16_t> {
    static constexpr uint32_t kFlag = 0x8000u;
    static constexpr uint32_t kLast = 0x7fffu;
    static constexpr int32_t kLimit = 0x7fff;       // offset + subject length must stay <= this
};
template <>
struct CellTraits<uint32_t> {
    static constexpr uint32_t kFlag = 0x80000000u;
    static constexpr uint32_t kLast = 0x7fffffffu;
    static constexpr int32_t kLimit = 0x7fffffff - 1;
};
// 32-bit tables are cleared once the offset passes this (NCBI clears at INT4_MAX/4)
constexpr int32_t kWrap32 = 1 << 29;

// ---------------------------------------------------------------------------
// Per-warp state.  Extensions are queued and run one lane per extension; the
// diagonal of a queued extension holds a "pending" marker (flag bit + the
// current offset - 1, a value no real state of this subject can take, and one
// that reads as a stale, already-passed flag once the offset moves on), and a
// later hit that meets the marker is parked in the blocked list, in order,
// until the extension has written the diagonal's real state.

constexpr int kQueue = 64;
// Subject letters reach the scan through a per-warp ring in shared memory,
// filled by 16-byte asynchronous copies (cp.async) two blocks ahead of the
// scan.  The ring is small so that four 8-warp CTAs with 2048-entry tables
// still fit an SM.
constexpr int kStageBlock = 64;    // letters per block: 16 bytes for each of lanes 0..3
constexpr int kStageRing = 4;      // blocks held: the scan's two, and two in flight

struct WarpQueue {
    uint4 stage[kStageRing * kStageBlock / 16];   // ring of subject letters
    int task_s[kQueue];      // subject offset of the second hit
    int task_q[kQueue];      // group-local query offset
    int task_left[kQueue];   // one past the first hit's word (subject offset)
    int blk_s[2][kQueue];
    int blk_q[2][kQueue];
};
// the 16-bit tables follow the head, the slots and the queues and are cleared 16 bytes at a time
static_assert(sizeof(Head) % 16 == 0 && sizeof(Slot) % 16 == 0 && sizeof(WarpQueue) % 16 == 0,
              "shared-memory regions must keep 16-byte alignment (table lengths are multiples of 8)");

template <typename Cell>
struct Item {
    const uint8_t *s;        // subject letters
    int S;                   // subject length
    int j;                   // subject ordinal id
    Cell *diag;
    int mask;                // table length - 1 (a power of two >= group length + window)
    int dofs;                // diagonal offset for this subject
    int window;
    const uint8_t *gseq;
    const int32_t *gctx;
    int first_query;
};

// One hit on a diagonal whose cell holds `state` (NCBI's two-hit rule, with
// the pending marker): returns the new cell value; when `on`, sets want_task
// (and left, the first hit's end) if the hit starts an extension and
// want_blk if it has to wait behind one.  Branch-free, so that a warp whose
// lanes take different cases runs it once.
template <typename Cell>
__device__ __forceinline__ uint32_t two_hit_step(uint32_t state, int s_h, int dofs, int window,
                                                 uint32_t pend, bool on, bool &want_task,
                                                 bool &want_blk, int &left) {
    using T = CellTraits<Cell>;
    const bool is_pend = state == pend;                  // an extension of this diagonal is queued
    const bool flag = (state & T::kFlag) != 0;           // state = end of the last extension
    const int32_t last = (int32_t)state - dofs;          // else: subject offset of the last hit
    const int32_t diff = s_h - last;
    const bool reset = flag ? (!is_pend && s_h + dofs >= (int32_t)(state & T::kLast)) : diff >= window;
    const bool trig = !flag && diff < window && diff >= 3;
    want_blk = want_blk || (on && is_pend);
    want_task = want_task || (on && trig);
    left = (on && trig) ? last + 3 : left;
    return reset ? (uint32_t)(Cell)(s_h + dofs) : (trig ? pend : state);
}

// Apply one batch of hits (one per active lane, in CPU order by lane) to the
// diagonal table.  Lanes sharing a diagonal form a chain in lane order (rank =
// lanes of the same diagonal below this one); a chain's state moves from lane
// to lane by shuffles, so the table is read and written once per diagonal.
// Warp-collective.
template <typename Cell>
__device__ __forceinline__ void apply_hits(const Item<Cell> &it, bool act, int d, int s_h, int q,
                                           WarpQueue &wq, int &n_tasks, int &n_blk, int blk_out) {
    using T = CellTraits<Cell>;
    const int lane = threadIdx.x & 31;
    const unsigned am = __ballot_sync(0xffffffffu, act);
    unsigned grp = 0;
    int rank = 0, prev = lane, head = lane;
    if (act) {
        grp = __match_any_sync(am, d);
        const unsigned below = grp & lanemask_lt();
        rank = __popc(below);
        if (below)
            prev = 31 - __clz(below);
        head = __ffs(grp) - 1;
    }
    const bool tail = act && (grp >> lane) == 1u;       // last lane of its chain
    const uint32_t pend = T::kFlag | (uint32_t)(it.dofs - 1);
    bool want_task = false, want_blk = false;
    int left = 0;
    uint32_t orig = 0;
    if (act && rank == 0)
        orig = it.diag[d];
    uint32_t state = two_hit_step<Cell>(orig, s_h, it.dofs, it.window, pend, act && rank == 0,
                                        want_task, want_blk, left);
    bool chained = false;
    for (int rr = 1; __any_sync(0xffffffffu, act && rank >= rr); ++rr) {
        const uint32_t ps = __shfl_sync(0xffffffffu, state, prev);
        const bool mine = act && rank == rr;
        const uint32_t nx = two_hit_step<Cell>(ps, s_h, it.dofs, it.window, pend, mine, want_task,
                                               want_blk, left);
        state = mine ? nx : state;
        chained = true;
    }
    if (chained)
        orig = __shfl_sync(0xffffffffu, orig, head);
    if (tail && state != orig)
        it.diag[d] = (Cell)state;
    // queue appends: tasks in any order; blocked hits in lane order, which
    // keeps hits of one diagonal in CPU order
    const unsigned tm = __ballot_sync(0xffffffffu, want_task);
    if (want_task) {
        const int p = n_tasks + __popc(tm & lanemask_lt());
        wq.task_s[p] = s_h;
        wq.task_q[p] = q;
        wq.task_left[p] = left;
    }
    n_tasks += __popc(tm);
    const unsigned bm = __ballot_sync(0xffffffffu, want_blk);
    if (want_blk) {
        const int p = n_blk + __popc(bm & lanemask_lt());
        wq.blk_s[blk_out][p] = s_h;
        wq.blk_q[blk_out][p] = q;
    }
    n_blk += __popc(bm);
    __syncwarp();
}

// One round: run queued extensions (lane per extension; the newest 32 when at
// least 32 wait, else all), then replay the blocked hits once, in order.
// Extensions of distinct diagonals are independent, and a diagonal has at
// most one queued extension, so any subset may run first.  Replayed hits may
// queue new extensions and be blocked again behind them; that is safe
// mid-subject because every later hit on a pending diagonal is blocked after
// them.  Queues hold 64: a replay batch starts only while at most 32 tasks
// wait.  With drain, run everything and repeat until both lists are empty
// (needed before the subject ends).  Warp-collective.
template <typename Cell>
__device__ void flush(const Item<Cell> &it, const WordFinderArgs &a, Slot &sh, WarpQueue &wq,
                      int &n_tasks, int &n_blk, int &blk_cur, bool drain) {
    using T = CellTraits<Cell>;
    const int lane = threadIdx.x & 31;
    do {
        const int first = (!drain && n_tasks >= 32) ? n_tasks - 32 : 0;
        for (int t0 = first; t0 < n_tasks; t0 += 32) {
            const int i = t0 + lane;
            if (i < n_tasks) {
                const int s_h = wq.task_s[i], q = wq.task_q[i];
                const int ci = __ldg(it.gctx + q);
                const HbgContext C = a.contexts[ci];
                const HbgQueryDesc Q = a.queries[C.query];
                const int ql = q - Q.start;
                const Ext e = extend_two_hit(score_matrix(), it.s, it.S, it.gseq + Q.start, Q.len,
                                             wq.task_left[i], s_h, ql, C.x_dropoff);
                atomicAdd(&sh.q_ext[C.query - it.first_query], 1u);
                if (e.score >= C.cutoff) {
                    atomicAdd(&sh.q_kept[C.query - it.first_query], 1u);
                    const unsigned long long o = atomicAdd(a.hsp_count, 1ull);
                    if ((long long)o < a.hsp_cap) {
                        hbg_hsp out;
                        out.query = C.query;
                        out.subject = it.j;
                        out.q_start = e.q_start;
                        out.s_start = e.s_start;
                        out.q_off = ql;
                        out.s_off = s_h;
                        out.len = e.len;
                        out.score = e.score;
                        out.context = C.local;
                        a.hsps[o] = out;
                    }
                }
                const int d = (q - s_h) & it.mask;
                it.diag[d] = e.right ? (Cell)(T::kFlag | (uint32_t)(e.s_last_off - 2 + it.dofs))
                                     : (Cell)(s_h + it.dofs);
            }
        }
        __syncwarp();
        n_tasks = first;
        const int nb = n_blk;
        const int src = blk_cur;
        n_blk = 0;
        blk_cur ^= 1;
        for (int b0 = 0; b0 < nb; b0 += 32) {
            if (n_tasks > 32) {
                // no room for the tasks another batch may queue: the rest of
                // the list follows the re-blocked hits, in order
                for (int i = b0 + lane; i < nb; i += 32) {
                    wq.blk_s[blk_cur][n_blk + i - b0] = wq.blk_s[src][i];
                    wq.blk_q[blk_cur][n_blk + i - b0] = wq.blk_q[src][i];
                }
                n_blk += nb - b0;
                __syncwarp();
                break;
            }
            const int i = b0 + lane;
            const bool act = i < nb;
            int s_h = 0, q = 0, d = 0;
            if (act) {
                s_h = wq.blk_s[src][i];
                q = wq.blk_q[src][i];
                d = (q - s_h) & it.mask;
            }
            apply_hits(it, act, d, s_h, q, wq, n_tasks, n_blk, blk_cur);
        }
    } while (drain && (n_tasks > 0 || n_blk > 0));
}

// Keep every stored value exact: restart the offset (and clear the table)
// when offset + subject length would not fit the cell.  Warp-collective.
template <typename Cell>
__device__ __forceinline__ void restart_offset(Item<Cell> &it, int diag_alloc) {
    using T = CellTraits<Cell>;
    const int lane = threadIdx.x & 31;
    if (sizeof(Cell) == 2 ? (it.dofs + it.S > T::kLimit) : (it.dofs >= kWrap32)) {
        __syncwarp();
        if (sizeof(Cell) == 2 && (diag_alloc & 7) == 0 && (reinterpret_cast<uintptr_t>(it.diag) & 15) == 0) {
            uint4 *p = reinterpret_cast<uint4 *>(it.diag);
            for (int i = lane; i < diag_alloc / 8; i += 32)
                p[i] = make_uint4(0, 0, 0, 0);
        } else {
            for (int i = lane; i < diag_alloc; i += 32)
                it.diag[i] = 0;
        }
        __syncwarp();
        it.dofs = it.window;
    }
}

// Subject letters staged for the scan: blocks of kStageBlock letters counted
// from the 16-byte aligned address at or before the subject's first letter.
// Block k goes to ring slot k % kStageRing.  `next` is the next block the scan
// will need; blocks next and next + 1 have been issued.
struct Stage {
    int next;
};

constexpr int kStageLanes = kStageBlock / 16;

// Issue block k: lanes 0..kStageLanes-1 copy 16 bytes each.  A segment is
// copied only when it holds a letter of the subject (relative position <
// delta + S); it then ends at most 15 bytes past the subject, inside the
// database buffer (a sentinel after every subject, 64 bytes of tail padding).
// Other segments are zero-filled without reading.  Every lane commits one
// copy group per block (empty for lanes that copy nothing).
__device__ __forceinline__ void stage_issue(WarpQueue &wq, const uint8_t *s, int S, int k, int lane) {
    const uintptr_t sa = reinterpret_cast<uintptr_t>(s);
    const int delta = (int)(sa & 15);
    const int r = k * kStageBlock + lane * 16;
    if (lane < kStageLanes) {
        const bool in = r < delta + S;
        const uint8_t *src = reinterpret_cast<const uint8_t *>(sa & ~(uintptr_t)15) + (in ? r : 0);
        const unsigned dst = (unsigned)__cvta_generic_to_shared(&wq.stage[(k & (kStageRing - 1)) * kStageLanes + lane]);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(in ? 16 : 0)
                     : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

__device__ __forceinline__ void stage_begin(Stage &st, WarpQueue &wq, const uint8_t *s, int S, int lane) {
    stage_issue(wq, s, S, 0, lane);
    stage_issue(wq, s, S, 1, lane);
    st.next = 0;
}

// Make blocks up to `blk` resident: for each newly needed block b, wait for
// its copy (all but the newest group, b + 1, complete), then issue b + 2 into
// the slot of b - 2, which no chunk needs any more (a chunk reads at most
// blocks b - 1 and b).  Warp-collective (blk is warp-uniform).
__device__ __forceinline__ void stage_upto(Stage &st, WarpQueue &wq, const uint8_t *s, int S, int blk,
                                           int lane) {
    while (st.next <= blk) {
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        __syncwarp();
        stage_issue(wq, s, S, st.next + 2, lane);
        st.next++;
    }
}

// Before the warp leaves a subject: no copy may still write its ring.
__device__ __forceinline__ void stage_end() {
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncwarp();
}

// Word index of offset s0+lane (three letters from the staged ring),
// presence test and cell bounds: *c = hits of that offset, *base = first
// entry.  Warp-collective.
template <typename Cell>
__device__ __forceinline__ void scan_words(const Item<Cell> &it, Stage &stg, WarpQueue &wq, const Slot &sh,
                                           const uint32_t *cs, int s0, uint32_t *c, uint32_t *base) {
    const int lane = threadIdx.x & 31;
    // the words of this chunk need letters up to delta + s0 + 33
    const int delta = (int)(reinterpret_cast<uintptr_t>(it.s) & 15);
    stage_upto(stg, wq, it.s, it.S, (delta + s0 + 33) / kStageBlock, lane);
    const uint8_t *ring = reinterpret_cast<const uint8_t *>(wq.stage);
    constexpr int kMask = kStageRing * kStageBlock - 1;
    const int sp = s0 + lane;
    const int r = delta + sp;
    *c = 0;
    *base = 0;
    if (sp <= it.S - 3) {
        const uint32_t w = ((uint32_t)ring[r & kMask] << 10) | ((uint32_t)ring[(r + 1) & kMask] << 5) |
                           (uint32_t)ring[(r + 2) & kMask];
        if ((sh.pv[w >> 5] >> (w & 31)) & 1u) {
            *base = __ldg(cs + w);
            *c = __ldg(cs + w + 1) - *base;
        }
    }
}

// Chunk mode: one (group, subject) item scanned 32 offsets at a time, the
// hits of each chunk compacted in CPU order, and the subject's hit stream
// applied 32 at a time across chunk boundaries: a chunk's last, partial batch
// waits in lanes 0..carry-1 and is completed by the next chunk's first hits
// (lane order stays CPU order), so only a subject's last batch runs partly
// empty.  Warp-collective.
template <typename Cell>
__device__ unsigned long long process_item(Item<Cell> &it, const WordFinderArgs &a, Slot &sh,
                                           WarpQueue &wq, const uint32_t *cs, const uint16_t *ents,
                                           int diag_alloc) {
    const int lane = threadIdx.x & 31;
    restart_offset(it, diag_alloc);
    int n_tasks = 0, n_blk = 0, blk_cur = 0;
    unsigned long long item_hits = 0;
    Stage stg;
    stage_begin(stg, wq, it.s, it.S, lane);
    uint32_t carry = 0;        // hits of earlier chunks not applied yet, in lanes 0..carry-1
    int s_n = 0, q_n = 0;      // this lane's next hit: subject and group-local query offset
    // software pipeline: the next chunk's cell bounds are loaded while this
    // chunk's hits are applied, and each batch's query offsets while the
    // previous batch is applied
    uint32_t c_next = 0, base_next = 0;
    if (it.S >= 3)
        scan_words(it, stg, wq, sh, cs, 0, &c_next, &base_next);
    for (int s0 = 0; s0 <= it.S - 3; s0 += 32) {
        const uint32_t c = c_next, base = base_next;
        if (s0 + 32 <= it.S - 3)
            scan_words(it, stg, wq, sh, cs, s0 + 32, &c_next, &base_next);
        uint32_t incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o)
                incl += t;
        }
        const uint32_t T_ = __shfl_sync(0xffffffffu, incl, 31);
        const uint32_t excl = incl - c;
        const uint32_t rel = base - excl;  // entry index of hit h = rel(owner) + h
        item_hits += T_;

        // hit h of the chunk: owner lane (largest lane whose exclusive count
        // is <= h), its subject offset and its query offset
        auto locate = [&](uint32_t h, int *s_h, int *q) {
            int lo = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const uint32_t v = __shfl_sync(0xffffffffu, excl, lo + step);
                if (v <= h)
                    lo += step;
            }
            *s_h = s0 + lo;
            const uint32_t r = __shfl_sync(0xffffffffu, rel, lo);
            *q = h < T_ ? (int)__ldg(ents + (r + h)) : 0;
        };
        // the stream continues: position c = carry + h holds hit h of this chunk
        const uint32_t total = carry + T_;
        if (T_ > 0) {
            int s_c, q_c;
            locate((uint32_t)lane - carry, &s_c, &q_c);
            if ((uint32_t)lane >= carry) {
                s_n = s_c;
                q_n = q_c;
            }
        }
        uint32_t cb = 0;
        for (; cb + 32 <= total; cb += 32) {       // full batches
            const int s_h = s_n, q = q_n;
            if (cb + 32 < total)                   // positions >= 32 are hits of this chunk
                locate(cb + 32 + lane - carry, &s_n, &q_n);
            apply_hits(it, true, (q - s_h) & it.mask, s_h, q, wq, n_tasks, n_blk, blk_cur);
            // queues hold 64: keep room for one more batch of 32
            while (n_tasks >= 32 || n_blk >= 32)
                flush(it, a, sh, wq, n_tasks, n_blk, blk_cur, false);
        }
        carry = total - cb;                        // these wait in (s_n, q_n) of lanes 0..carry-1
    }
    if (carry > 0) {                               // the subject's last batch
        const bool act = (uint32_t)lane < carry;
        apply_hits(it, act, act ? ((q_n - s_n) & it.mask) : 0, s_n, q_n, wq, n_tasks, n_blk, blk_cur);
    }
    flush(it, a, sh, wq, n_tasks, n_blk, blk_cur, true);
    stage_end();
    // advance the diagonal offset past this subject (NCBI Blast_ExtendWordExit)
    it.dofs += it.S + it.window;
    return item_hits;
}

// ---------------------------------------------------------------------------
// Per-offset mode, for groups dense enough that one subject offset has many
// hits: the warp visits the offsets in order and lane i takes entry i of the
// offset's cell (contiguous, so the load is coalesced).  Hits of one offset
// lie on distinct diagonals, so they need no ordering among themselves; the
// next offset's first 32 entries are loaded while this one is applied.

template <typename Cell>
__device__ __forceinline__ void apply_offset(const Item<Cell> &it, bool act, int s_h, int q,
                                             WarpQueue &wq, int &n_tasks, int &n_blk, int blk_out) {
    using T = CellTraits<Cell>;
    const uint32_t pend = T::kFlag | (uint32_t)(it.dofs - 1);
    bool want_task = false, want_blk = false;
    int left = 0;
    if (act) {
        const int d = (q - s_h) & it.mask;
        const uint32_t cell = it.diag[d];
        const uint32_t next = two_hit_step<Cell>(cell, s_h, it.dofs, it.window, pend, true, want_task,
                                                 want_blk, left);
        if (next != cell)
            it.diag[d] = (Cell)next;
    }
    if (__any_sync(0xffffffffu, want_task || want_blk)) {
        const unsigned tm = __ballot_sync(0xffffffffu, want_task);
        if (want_task) {
            const int p = n_tasks + __popc(tm & lanemask_lt());
            wq.task_s[p] = s_h;
            wq.task_q[p] = q;
            wq.task_left[p] = left;
        }
        n_tasks += __popc(tm);
        const unsigned bm = __ballot_sync(0xffffffffu, want_blk);
        if (want_blk) {
            const int p = n_blk + __popc(bm & lanemask_lt());
            wq.blk_s[blk_out][p] = s_h;
            wq.blk_q[blk_out][p] = q;
        }
        n_blk += __popc(bm);
    }
    __syncwarp();
}

template <typename Cell>
__device__ unsigned long long process_item_offsets(Item<Cell> &it, const WordFinderArgs &a, Slot &sh,
                                                   WarpQueue &wq, const uint32_t *cs,
                                                   const uint16_t *ents, int diag_alloc) {
    const int lane = threadIdx.x & 31;
    restart_offset(it, diag_alloc);
    int n_tasks = 0, n_blk = 0, blk_cur = 0;
    unsigned long long item_hits = 0;
    Stage stg;
    stage_begin(stg, wq, it.s, it.S, lane);
    for (int s0 = 0; s0 <= it.S - 3; s0 += 32) {
        uint32_t c, base;
        scan_words(it, stg, wq, sh, cs, s0, &c, &base);
        item_hits += __reduce_add_sync(0xffffffffu, c);
        unsigned m = __ballot_sync(0xffffffffu, c != 0);
        uint32_t nb = 0, nc = 0;
        int q_next = 0;
        if (m) {
            const int p = __ffs(m) - 1;
            nb = __shfl_sync(0xffffffffu, base, p);
            nc = __shfl_sync(0xffffffffu, c, p);
            if ((uint32_t)lane < nc)
                q_next = __ldg(ents + nb + lane);
        }
        while (m) {
            const int p = __ffs(m) - 1;
            m &= m - 1;
            const uint32_t cb = nb, cc = nc;
            const int q_cur = q_next;
            if (m) {
                const int pn = __ffs(m) - 1;
                nb = __shfl_sync(0xffffffffu, base, pn);
                nc = __shfl_sync(0xffffffffu, c, pn);
                q_next = (uint32_t)lane < nc ? __ldg(ents + nb + lane) : 0;
            }
            const int s_h = s0 + p;
            apply_offset(it, (uint32_t)lane < cc, s_h, q_cur, wq, n_tasks, n_blk, blk_cur);
            while (n_tasks >= 32 || n_blk >= 32)
                flush(it, a, sh, wq, n_tasks, n_blk, blk_cur, false);
            for (uint32_t e0 = 32; e0 < cc; e0 += 32) {
                const bool act = e0 + lane < cc;
                const int q = act ? __ldg(ents + cb + e0 + lane) : 0;
                apply_offset(it, act, s_h, q, wq, n_tasks, n_blk, blk_cur);
                while (n_tasks >= 32 || n_blk >= 32)
                    flush(it, a, sh, wq, n_tasks, n_blk, blk_cur, false);
            }
        }
    }
    flush(it, a, sh, wq, n_tasks, n_blk, blk_cur, true);
    stage_end();
    it.dofs += it.S + it.window;
    return item_hits;
}

}  // namespace

// Mode bit 0: offset mode (else chunk mode); bit 1: the launch's groups keep
// their diagonal tables in global memory (same code; that instantiation asks
// for a small shared-memory carve-out so the L1 cache holds more of the
// tables); bit 2: tiles of several groups (warps per subject > 1).  Chunk
// mode is built for four 256-thread CTAs per SM (64 registers a thread),
// offset mode (large tables) for one.
template <int Mode>
__global__ void __launch_bounds__(256, (Mode & 1) == 0 ? 4 : 1) wordfinder_kernel(WordFinderArgs a) {
    constexpr bool kOffsets = (Mode & 1) != 0;
    constexpr bool kTeam = (Mode & 4) != 0;   // several groups per tile (built apart: it needs more registers)
    Head &hd = *reinterpret_cast<Head *>(g_smem);
    Slot *slots = reinterpret_cast<Slot *>(g_smem + sizeof(Head));
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    // a tile covers `team` groups and one block of subjects; warp w serves
    // group slot w % team, and the warps of a slot share its subjects
    const int team = kTeam ? a.team : 1;
    Slot &sh = slots[warp % team];
    unsigned char *per_warp = g_smem + sizeof(Head) + (size_t)team * sizeof(Slot);
    WarpQueue &wq = reinterpret_cast<WarpQueue *>(per_warp)[warp];
    uint16_t *diag_s =
        reinterpret_cast<uint16_t *>(per_warp + nwarps * sizeof(WarpQueue)) + warp * a.smem_diag;
    uint32_t *diag_g =
        a.gdiag ? a.gdiag + ((size_t)blockIdx.x * nwarps + warp) * (size_t)a.gdiag_len : nullptr;

    for (int i = threadIdx.x; i < 28 * 32; i += blockDim.x)
        hd.matrix[i] = c_blosum[i];
    for (int i = threadIdx.x; i < team; i += blockDim.x)
        slots[i].group = -1;
    for (int i = lane; i < a.smem_diag; i += 32)
        diag_s[i] = 0;
    const int window = a.window;
    // the 16-bit shared table starts past its limit so the first item clears it
    // offsets of the three tables a warp may use: its shared 16-bit table,
    // and its global slice seen as 16-bit or as 32-bit cells (switching views
    // forces the other view to clear before its next use)
    int32_t dofs_s = CellTraits<uint16_t>::kLimit + 1, dofs_g = window;
    int32_t dofs_h = CellTraits<uint16_t>::kLimit + 1;

    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0)
            hd.tile = (long long)atomicAdd(a.tile_counter, 1u);
        for (int i = threadIdx.x; i < team * kMaxQ; i += blockDim.x) {
            slots[i / kMaxQ].q_ext[i % kMaxQ] = 0;
            slots[i / kMaxQ].q_kept[i % kMaxQ] = 0;
        }
        for (int i = threadIdx.x; i < team; i += blockDim.x) {
            slots[i].next = 0;
            slots[i].hits = 0;
        }
        __syncthreads();
        const long long tile = hd.tile;
        if (tile >= a.n_tiles)
            break;
        const long long gb = tile / a.tiles_per_group;
        const int blk = (int)(tile % a.tiles_per_group);
        // the presence vectors of this tile's groups (kept when a slot keeps its group)
        for (int t = 0; t < team; ++t) {
            const long long li = gb * team + t;
            const int g = li < a.n_list ? a.group_list[li] : -1;
            if (g >= 0 && g != slots[t].group) {
                const uint32_t *src = a.pv + (size_t)g * HBG_PV_WORDS;
                for (int i = threadIdx.x; i < HBG_PV_WORDS; i += blockDim.x)
                    slots[t].pv[i] = src[i];
            }
        }
        __syncthreads();
        if (threadIdx.x < team) {
            const long long li = gb * team + threadIdx.x;
            slots[threadIdx.x].group = li < a.n_list ? a.group_list[li] : -1;
        }
        __syncthreads();
        const int g = sh.group;
        if (g >= 0) {
            const HbgGroup G = a.groups[g];
            const uint32_t *cs = a.cells + (size_t)g * HBG_CELL_STRIDE;
            const uint16_t *ents = a.entries + G.entry_base;
            for (;;) {
                int k = 0;
                if (lane == 0)
                    k = atomicAdd(&sh.next, 1);
                k = __shfl_sync(0xffffffffu, k, 0);
                const long long idx = (long long)blk * a.tile_subjects + k;
                if (k >= a.tile_subjects || idx >= a.n_subj)
                    break;
                const int j = a.order[idx];
                const int S = a.db_len[j];
                const uint8_t *sp = a.db + a.db_off[j];
                unsigned long long hits;
                // 16-bit cells when window + S fits 15 bits: in shared memory when the
                // group's table fits there, else in this warp's slice of the global
                // scratch (half the footprint of 32-bit cells, so the tables of all
                // resident warps stay in L2); otherwise 32-bit cells in that slice
                if (!G.placement && window + S <= CellTraits<uint16_t>::kLimit) {
                    Item<uint16_t> it{sp, S, j, diag_s, G.diag_len - 1, dofs_s, window,
                                      a.letters + G.seq_base, a.ctx_of + G.seq_base, G.first_query};
                    hits = kOffsets ? process_item_offsets(it, a, sh, wq, cs, ents, a.smem_diag)
                                    : process_item(it, a, sh, wq, cs, ents, a.smem_diag);
                    dofs_s = it.dofs;
                } else if (window + S <= CellTraits<uint16_t>::kLimit) {
                    Item<uint16_t> it{sp, S, j, reinterpret_cast<uint16_t *>(diag_g), G.diag_len - 1, dofs_h,
                                      window, a.letters + G.seq_base, a.ctx_of + G.seq_base, G.first_query};
                    hits = kOffsets ? process_item_offsets(it, a, sh, wq, cs, ents, 2 * a.gdiag_len)
                                    : process_item(it, a, sh, wq, cs, ents, 2 * a.gdiag_len);
                    dofs_h = it.dofs;
                    dofs_g = kWrap32;                  // the 32-bit view clears before its next use
                } else {
                    Item<uint32_t> it{sp, S, j, diag_g, G.diag_len - 1, dofs_g, window,
                                      a.letters + G.seq_base, a.ctx_of + G.seq_base, G.first_query};
                    hits = kOffsets ? process_item_offsets(it, a, sh, wq, cs, ents, a.gdiag_len)
                                    : process_item(it, a, sh, wq, cs, ents, a.gdiag_len);
                    dofs_g = it.dofs;
                    dofs_h = CellTraits<uint16_t>::kLimit + 1;   // the 16-bit view clears before its next use
                }
                if (lane == 0)
                    atomicAdd(&sh.hits, hits);
            }
        }
        __syncthreads();
        for (int t = 0; t < team; ++t) {
            const int gt = slots[t].group;
            if (gt < 0)
                continue;
            const HbgGroup Gt = a.groups[gt];
            for (int i = threadIdx.x; i < Gt.n_queries && i < kMaxQ; i += blockDim.x) {
                if (slots[t].q_ext[i])
                    atomicAdd(a.q_extended + Gt.first_query + i, (unsigned long long)slots[t].q_ext[i]);
                if (slots[t].q_kept[i])
                    atomicAdd(a.q_kept + Gt.first_query + i, (unsigned long long)slots[t].q_kept[i]);
            }
            if (threadIdx.x == 0 && slots[t].hits)
                atomicAdd(a.g_hits + gt, slots[t].hits);
        }
    }
}

size_t wordfinder_smem_bytes(int threads, int smem_diag, int team) {
    return sizeof(Head) + (size_t)team * sizeof(Slot) +
           (size_t)(threads / 32) * (sizeof(WarpQueue) + (size_t)smem_diag * sizeof(uint16_t));
}

namespace {
template <int M>
const void *kernel_ptr() { return (const void *)wordfinder_kernel<M>; }
const void *kernel_of(int mode) {
    switch (mode & 7) {
    case 0: return kernel_ptr<0>();
    case 1: return kernel_ptr<1>();
    case 2: return kernel_ptr<2>();
    case 3: return kernel_ptr<3>();
    case 4: return kernel_ptr<4>();
    case 5: return kernel_ptr<5>();
    case 6: return kernel_ptr<6>();
    default: return kernel_ptr<7>();
    }
}
}  // namespace

cudaError_t wordfinder_configure() {
    // opt in to the largest shared-memory carve-out; launches size their own.
    // The global-table instantiations prefer a carve-out of ~40 % (four CTAs
    // need about 88 KB), leaving the rest of the SM's 256 KB to the L1 cache
    // that holds their diagonal tables (measured 4 % faster than the CUDA
    // driver's default choice); a hint the CUDA driver may round up.
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    for (int m = 0; m < 8; ++m) {
        cudaError_t e = cudaFuncSetAttribute(kernel_of(m), cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        if (e == cudaSuccess && (m & 2))
            e = cudaFuncSetAttribute(kernel_of(m), cudaFuncAttributePreferredSharedMemoryCarveout, 40);
        if (e != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

cudaError_t wordfinder_occupancy(int mode, int threads, int smem_diag, int team, int *blocks_per_sm) {
    const size_t smem = wordfinder_smem_bytes(threads, smem_diag, team);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kernel_of((mode & 3) | (team > 1 ? 4 : 0)),
                                                         threads, smem);
}

cudaError_t launch_wordfinder(const WordFinderArgs &a, int mode, int blocks, int threads,
                              cudaStream_t stream) {
    const size_t smem = wordfinder_smem_bytes(threads, a.smem_diag, a.team);
    switch ((mode & 3) | (a.team > 1 ? 4 : 0)) {
    case 0: wordfinder_kernel<0><<<blocks, threads, smem, stream>>>(a); break;
    case 1: wordfinder_kernel<1><<<blocks, threads, smem, stream>>>(a); break;
    case 2: wordfinder_kernel<2><<<blocks, threads, smem, stream>>>(a); break;
    case 3: wordfinder_kernel<3><<<blocks, threads, smem, stream>>>(a); break;
    case 4: wordfinder_kernel<4><<<blocks, threads, smem, stream>>>(a); break;
    case 5: wordfinder_kernel<5><<<blocks, threads, smem, stream>>>(a); break;
    case 6: wordfinder_kernel<6><<<blocks, threads, smem, stream>>>(a); break;
    default: wordfinder_kernel<7><<<blocks, threads, smem, stream>>>(a); break;
    }
    return cudaGetLastError();
}

}  // namespace hbg
