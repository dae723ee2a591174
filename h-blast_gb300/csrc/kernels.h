// kernels.h -- launch wrappers of the device code (host-callable).
#ifndef HBG_KERNELS_H
#define HBG_KERNELS_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "hbg_internal.h"

namespace hbg {

struct WordFinderArgs {
    // resident database
    const uint8_t *db;            // letters, one sentinel between subjects
    const int64_t *db_off;        // start of subject i
    const int32_t *db_len;        // length of subject i
    const int32_t *order;         // scheduling order of subjects (longest first)
    int32_t n_subj;
    // batch
    const HbgGroup *groups;
    int32_t n_groups;
    const int32_t *group_list;    // groups this launch processes (one hit mode per launch)
    const uint32_t *cells;        // n_groups x HBG_CELL_STRIDE
    const uint16_t *entries;
    const uint32_t *pv;           // n_groups x HBG_PV_WORDS
    const uint8_t *letters;
    const int32_t *ctx_of;
    const HbgContext *contexts;
    const HbgQueryDesc *queries;
    int32_t window;
    // scheduling: tile t covers groups group_list[(t / tiles_per_group) * team
    // .. + team) (those below n_list) and scheduled subjects
    // [(t % tiles_per_group) * tile_subjects, + tile_subjects); warp w of a
    // CTA works on the tile's group w % team
    int32_t tile_subjects;
    int32_t tiles_per_group;
    int64_t n_tiles;
    int32_t team;                 // groups per tile: warps that share each subject, 1..warps per CTA
    int32_t n_list;               // groups in group_list
    unsigned int *tile_counter;   // zeroed before launch
    // outputs
    hbg_hsp *hsps;
    unsigned long long *hsp_count;  // zeroed before launch
    int64_t hsp_cap;
    unsigned long long *q_extended; // per batch query, zeroed
    unsigned long long *q_kept;     // per batch query, zeroed
    unsigned long long *g_hits;     // per group lookup hits, zeroed
    // global-memory diagonal tables (groups with placement 1): one slice of
    // gdiag_len entries per (block, warp), zeroed before launch
    uint32_t *gdiag;
    int32_t gdiag_len;
    // entries per warp of the 16-bit shared-memory tables (a multiple of 8)
    int32_t smem_diag;
};

// Shared memory the word-finder kernel needs for a CTA of `threads` threads.
size_t wordfinder_smem_bytes(int threads, int smem_diag, int team);
cudaError_t wordfinder_configure();
// mode: bit 0 = offset mode (else chunk mode); bit 1 = the groups keep
// their diagonal tables in global memory (kernel built to favour L1); the
// instantiation for tiles of several groups (team > 1) is chosen from
// WordFinderArgs::team / the team argument
cudaError_t wordfinder_occupancy(int mode, int threads, int smem_diag, int team, int *blocks_per_sm);
cudaError_t launch_wordfinder(const WordFinderArgs &a, int mode, int blocks, int threads,
                              cudaStream_t stream);

// Ordering pass: sort HSPs by (query, subject, s_off, q_off).
struct OrderArgs {
    const hbg_hsp *in;
    hbg_hsp *out;
    const unsigned long long *count;  // device count of HSPs (clamped to cap)
    int64_t cap;
    uint64_t *keys[2];
    uint32_t *vals[2];
    uint32_t *hist;                   // 256 x max_blocks
    int bits_q, bits_s, bits_so, bits_qo;
    // optional (null = skip): per-query first / end index in `out` and the
    // number of subjects with HSPs, each n_queries entries, zeroed beforehand
    unsigned long long *q_first, *q_end, *q_passed;
};
int64_t order_max_blocks(int64_t cap);
cudaError_t launch_order(const OrderArgs &a, cudaStream_t stream);

// Database word histogram: hist[w] += positions whose three letters are
// non-sentinel and form word w.
cudaError_t launch_db_histogram(const uint8_t *db, int64_t n, unsigned long long *hist,
                                cudaStream_t stream);

// lookup_hits[q] = sum_w hist[w] * query_cells[q][w]
cudaError_t launch_query_hits(const unsigned long long *hist, const uint16_t *query_cells,
                              int32_t n_queries, unsigned long long *out,
                              cudaStream_t stream);

}  // namespace hbg

#endif
