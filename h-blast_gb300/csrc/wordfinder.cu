// wordfinder.cu -- fused seed scan + two-hit diagonal test + ungapped X-drop
// extension for sm_103a.
//
// Work decomposition: a persistent grid of CTAs takes tiles (query group,
// block of subjects) from a global counter; the warps of a CTA take subjects
// of the tile from a shared counter, one warp per (group, subject) item.
//
// Per item the warp scans the subject 32 offsets at a time: lane l computes
// the 15-bit word index of offset s0+l, tests the group's presence vector in
// shared memory and reads the cell bounds; a warp scan turns the cell sizes
// into a compacted (offset, query offset) hit list in the order the CPU word
// finder visits hits (subject offset, then ascending query offset), which the
// warp then processes 32 hits at a time.  Hits of one batch that fall on the
// same diagonal are found with match.any and applied in order.
//
// Diagonal state follows NCBI's DiagStruct (31-bit last hit + 1-bit flag) and
// its offset trick: the offset grows by subject length + window per item so
// stale entries read as "no recent hit", and the table is cleared when the
// offset passes 2^30 (Blast_ExtendWordExit; H-BLAST h_blast_kernel.cu:1023).
// Each warp owns a table of kSmemDiagLen entries in shared memory, or a slice
// of the global scratch for groups whose table is longer.
//
// The per-hit rule is the two-hit state machine of NCBI aa_ungapped.c, which
// H-BLAST restates at h_blast_kernel.cu:672-871; the extension is
// s_BlastAaExtendTwoHit/Left/Right (h_blast_kernel.cu:1069-1540), with the
// left walk also taken when min(s, q) == 0 as NCBI does.
#include <cuda_runtime.h>

#include "kernels.h"

namespace hbg {

namespace {

constexpr int kSmemDiag = 2048;   // must equal kSmemDiagLen in batch_builder.h
constexpr int kMaxQ = 64;         // kMaxQueriesPerGroup
constexpr uint32_t kFlag = 0x80000000u;
constexpr uint32_t kLast = 0x7fffffffu;
constexpr int32_t kWrap = 1 << 30;

__constant__ int8_t c_blosum[28 * 32] = {
#include "blosum62.inc"
};

struct Smem {
    uint32_t pv[HBG_PV_WORDS];
    int8_t matrix[28 * 32];
    unsigned int q_ext[kMaxQ];
    unsigned int q_kept[kMaxQ];
    unsigned long long hits;
    long long tile;
    int next;
    int pad;
};

__device__ __forceinline__ int sc(const int8_t *m, int q, int s) { return m[q * 32 + s]; }

// X-drop walk to the left from (s_off, q_off) inclusive; returns the best
// score, *len = letters in the best walk.
__device__ int extend_left(const int8_t *m, const uint8_t *s, const uint8_t *q, int s_off,
                           int q_off, int dropoff, int *len) {
    int n = min(s_off, q_off);
    int best_i = n + 1;
    int score = 0, maxscore = 0;
    const uint8_t *sp = s + s_off - n;
    const uint8_t *qp = q + q_off - n;
    for (int i = n; i >= 0; --i) {
        score += sc(m, qp[i], sp[i]);
        if (score > maxscore) {
            maxscore = score;
            best_i = i;
        }
        if (maxscore - score >= dropoff)
            break;
    }
    *len = n - best_i + 1;
    return maxscore;
}

// X-drop walk to the right that also stops when the running score is <= 0.
__device__ int extend_right(const int8_t *m, const uint8_t *s, int s_len, const uint8_t *q,
                            int q_len, int s_off, int q_off, int dropoff, int maxscore,
                            int *len, int *s_last_off) {
    int n = min(s_len - s_off, q_len - q_off);
    int best_i = -1;
    int score = maxscore;
    int i;
    for (i = 0; i < n; ++i) {
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

}  // namespace

__global__ void __launch_bounds__(256) wordfinder_kernel(WordFinderArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem &sh = *reinterpret_cast<Smem *>(smem_raw);
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    uint32_t *diag_s = reinterpret_cast<uint32_t *>(smem_raw + sizeof(Smem)) + warp * kSmemDiag;
    uint32_t *diag_g =
        a.gdiag ? a.gdiag + ((size_t)blockIdx.x * nwarps + warp) * (size_t)a.gdiag_len : nullptr;

    for (int i = threadIdx.x; i < 28 * 32; i += blockDim.x)
        sh.matrix[i] = c_blosum[i];
    for (int i = lane; i < kSmemDiag; i += 32)
        diag_s[i] = 0;
    int32_t dofs_s = a.window, dofs_g = a.window;
    int cur_group = -1;
    const int window = a.window;

    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            sh.tile = (long long)atomicAdd(a.tile_counter, 1u);
            sh.next = 0;
            sh.hits = 0;
        }
        for (int i = threadIdx.x; i < kMaxQ; i += blockDim.x) {
            sh.q_ext[i] = 0;
            sh.q_kept[i] = 0;
        }
        __syncthreads();
        const long long tile = sh.tile;
        if (tile >= a.n_tiles)
            break;
        const int g = (int)(tile / a.tiles_per_group);
        const int blk = (int)(tile % a.tiles_per_group);
        if (g != cur_group) {
            const uint32_t *src = a.pv + (size_t)g * HBG_PV_WORDS;
            for (int i = threadIdx.x; i < HBG_PV_WORDS; i += blockDim.x)
                sh.pv[i] = src[i];
            cur_group = g;
            __syncthreads();
        }
        const HbgGroup G = a.groups[g];
        const uint32_t *cs = a.cells + (size_t)g * HBG_CELL_STRIDE;
        const uint16_t *ents = a.entries + G.entry_base;
        const uint8_t *gseq = a.letters + G.seq_base;
        const int32_t *gctx = a.ctx_of + G.seq_base;
        const int32_t mask = G.diag_len - 1;
        uint32_t *diag = G.placement ? diag_g : diag_s;
        int32_t dofs = G.placement ? dofs_g : dofs_s;
        const int diag_alloc = G.placement ? a.gdiag_len : kSmemDiag;

        for (;;) {
            int k = 0;
            if (lane == 0)
                k = atomicAdd(&sh.next, 1);
            k = __shfl_sync(0xffffffffu, k, 0);
            const long long idx = (long long)blk * a.tile_subjects + k;
            if (k >= a.tile_subjects || idx >= a.n_subj)
                break;
            const int j = a.order[idx];
            const uint8_t *s = a.db + a.db_off[j];
            const int S = a.db_len[j];
            unsigned long long item_hits = 0;

            for (int s0 = 0; s0 <= S - 3; s0 += 32) {
                const int sp = s0 + lane;
                uint32_t c = 0, base = 0;
                if (sp <= S - 3) {
                    const int w = ((int)s[sp] << 10) | ((int)s[sp + 1] << 5) | (int)s[sp + 2];
                    if ((sh.pv[w >> 5] >> (w & 31)) & 1u) {
                        base = __ldg(cs + w);
                        c = __ldg(cs + w + 1) - base;
                    }
                }
                uint32_t incl = c;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o)
                        incl += t;
                }
                const uint32_t T = __shfl_sync(0xffffffffu, incl, 31);
                const uint32_t excl = incl - c;
                const uint32_t rel = base - excl;  // entry index of hit h = rel(owner) + h
                item_hits += T;

                for (uint32_t hb = 0; hb < T; hb += 32) {
                    const uint32_t h = hb + lane;
                    const bool act = h < T;
                    int lo = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        uint32_t v = __shfl_sync(0xffffffffu, excl, lo + step);
                        if (v <= h)
                            lo += step;
                    }
                    const int s_h = s0 + lo;
                    const uint32_t r = __shfl_sync(0xffffffffu, rel, lo);
                    int q = 0, d = 0, rank = 0;
                    const unsigned am = __ballot_sync(0xffffffffu, act);
                    if (act) {
                        q = __ldg(ents + (r + h));
                        d = (q - s_h) & mask;
                        const unsigned grp = __match_any_sync(am, d);
                        rank = __popc(grp & lanemask_lt());
                    }
                    bool pending = act;
                    for (int rr = 0;; ++rr) {
                        if (pending && rank == rr) {
                            pending = false;
                            const uint32_t cell = diag[d];
                            const int32_t last = (int32_t)(cell & kLast);
                            if (cell & kFlag) {
                                if (s_h + dofs >= last)
                                    diag[d] = (uint32_t)(s_h + dofs);
                            } else {
                                const int32_t diff = s_h - (last - dofs);
                                if (diff >= window) {
                                    diag[d] = (uint32_t)(s_h + dofs);
                                } else if (diff >= 3) {
                                    const int ci = __ldg(gctx + q);
                                    const HbgContext C = a.contexts[ci];
                                    const HbgQueryDesc Q = a.queries[C.query];
                                    const int ql = q - Q.start;
                                    const Ext e = extend_two_hit(
                                        sh.matrix, s, S, gseq + Q.start, Q.len,
                                        (last - dofs) + 3, s_h, ql, C.x_dropoff);
                                    atomicAdd(&sh.q_ext[C.query - G.first_query], 1u);
                                    if (e.score >= C.cutoff) {
                                        atomicAdd(&sh.q_kept[C.query - G.first_query], 1u);
                                        const unsigned long long o = atomicAdd(a.hsp_count, 1ull);
                                        if ((long long)o < a.hsp_cap) {
                                            hbg_hsp out;
                                            out.query = C.query;
                                            out.subject = j;
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
                                    diag[d] = e.right ? (kFlag | (uint32_t)(e.s_last_off - 2 + dofs))
                                                      : (uint32_t)(s_h + dofs);
                                }
                            }
                        }
                        __syncwarp();
                        if (!__any_sync(0xffffffffu, pending))
                            break;
                    }
                }
            }
            if (lane == 0)
                atomicAdd(&sh.hits, item_hits);
            // advance the diagonal offset past this subject (NCBI Blast_ExtendWordExit)
            if (dofs >= kWrap) {
                __syncwarp();
                for (int i = lane; i < diag_alloc; i += 32)
                    diag[i] = 0;
                __syncwarp();
                dofs = window;
            } else {
                dofs += S + window;
            }
        }
        if (G.placement)
            dofs_g = dofs;
        else
            dofs_s = dofs;
        __syncthreads();
        for (int i = threadIdx.x; i < G.n_queries && i < kMaxQ; i += blockDim.x) {
            if (sh.q_ext[i])
                atomicAdd(a.q_extended + G.first_query + i, (unsigned long long)sh.q_ext[i]);
            if (sh.q_kept[i])
                atomicAdd(a.q_kept + G.first_query + i, (unsigned long long)sh.q_kept[i]);
        }
        if (threadIdx.x == 0 && sh.hits)
            atomicAdd(a.g_hits + g, sh.hits);
    }
}

size_t wordfinder_smem_bytes(int threads) {
    return sizeof(Smem) + (size_t)(threads / 32) * kSmemDiag * sizeof(uint32_t);
}

cudaError_t wordfinder_configure() {
    return cudaFuncSetAttribute(wordfinder_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)wordfinder_smem_bytes(256));
}

cudaError_t wordfinder_occupancy(int threads, int *blocks_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, wordfinder_kernel, threads,
                                                         wordfinder_smem_bytes(threads));
}

cudaError_t launch_wordfinder(const WordFinderArgs &a, int blocks, int threads,
                              cudaStream_t stream) {
    wordfinder_kernel<<<blocks, threads, wordfinder_smem_bytes(threads), stream>>>(a);
    return cudaGetLastError();
}

}  // namespace hbg
