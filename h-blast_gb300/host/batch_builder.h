// batch_builder.h -- host-side construction of a query batch: query packing
// into groups, six-frame translation for BLASTX, and the neighbourhood-word
// lookup tables.  Pure C++ (no CUDA); the runtime uploads the result.
#ifndef HBG_BATCH_BUILDER_H
#define HBG_BATCH_BUILDER_H

#include <stdint.h>

#include <string>
#include <vector>

#include "../csrc/hbg_internal.h"

namespace hbg {

// Shared-memory diagonal tables (16-bit cells) hold at most this many
// entries per warp; groups whose table is longer use 32-bit tables in the
// global scratch.  Measured on GB300: 2048-entry tables are faster in shared
// memory (four 8-warp CTAs per SM fit); longer shared tables cut resident
// warps to 8-20 per SM, and L2-resident global tables with 32 warps per SM
// beat them by 13-23 % (4096 to 32768 entries, BLASTP and six-frame BLASTX).
constexpr int32_t kSmemDiagMax = 2048;
// Default group length (letters, gaps included): 4056, the longest whose
// table is 4096 entries of 16-bit cells in global memory (8 KB a warp, 40 MB
// for all resident warps, which stay in L2).  On the 64-query batched workload
// (GB300, word-finder ms for 2,000,000 subjects): 4056 letters 936 (16 scans
// of the database); 6000 906, 7000 905, 8152 909 (8192-entry tables: 80 MB,
// which L2 no longer holds -- DRAM writes of evicted table lines rise from
// 6.4 GB to 92 GB per 500,000 subjects, ~15x, for 3 % less time); 10000 942,
// 12000 975, 16344 1159; 2008-letter groups with shared tables are slower
// still (37 scans).  Since each subject's hits are carried across chunks,
// 6000-letter groups are within 0.4 % of 4056 (858 vs 862 ms), so the extra
// traffic buys nothing.
constexpr int32_t kDefaultGroupLen = 4056;
// Groups whose expected hits per subject offset reach this use offset mode
// (off by default: chunk mode at high occupancy measured faster; the autotuner
// and hbg_batch_set_mode choose offset mode explicitly).
constexpr double kOffsetModeHits = 1e30;
// Queries per group are bounded so per-query counters fit in shared memory.
constexpr int32_t kMaxQueriesPerGroup = 64;

struct HostBatch {
    int32_t threshold = 11;
    int32_t window = 40;
    std::vector<HbgGroup> groups;
    std::vector<HbgContext> contexts;
    std::vector<HbgQueryDesc> queries;
    std::vector<uint8_t> letters;        // all groups, gaps included
    std::vector<int32_t> ctx_of;         // per letter, -1 outside contexts
    std::vector<uint32_t> cells;         // groups x HBG_CELL_STRIDE
    std::vector<uint16_t> entries;       // group-local query offsets
    std::vector<uint32_t> pv;            // groups x HBG_PV_WORDS
    std::vector<uint16_t> query_cells;   // queries x HBG_NUM_CELLS cell sizes
    int32_t max_query_len = 0;
    int32_t max_diag_len = 0;            // over groups with global placement
    int32_t smem_diag_len = 64;          // per-warp shared table: max over shared-placed groups
};

// One query already in NCBI concatenated form.
struct QueryIn {
    const uint8_t *seq;
    int32_t len;
    std::vector<int32_t> ctx_off, ctx_len, xdrop, cutoff;
};

// Returns an empty string on success, else the reason.
// max_group_len 0 = default; mode_hits < 0 = default offset-mode threshold,
// 0 = offset mode for every group, a huge value = chunk mode for every group.
std::string build_batch(const std::vector<QueryIn> &queries, int32_t threshold,
                        int32_t window, int32_t max_group_len, HostBatch *out,
                        double mode_hits = -1.0);

// Standard-code six-frame translation (frames +1,+2,+3,-1,-2,-3, one sentinel
// between frames).  Returns the concatenated letters; fills offsets/lengths.
std::vector<uint8_t> translate_six_frames(const uint8_t *nt, int32_t nt_len,
                                          std::vector<int32_t> *ctx_off,
                                          std::vector<int32_t> *ctx_len);

// SEG low-complexity masking of one protein sequence in place (masked
// letters become X); returns the number of letters masked.  seg.cpp.
int64_t seg_mask(uint8_t *seq, int32_t len, int32_t window, double locut, double hicut);

// Substitution score of NCBIstdaa letters (BLOSUM62).
int32_t blosum62(int32_t a, int32_t b);
const int8_t *blosum62_table();   // 28 rows x 32 columns, row = query letter

}  // namespace hbg

#endif
