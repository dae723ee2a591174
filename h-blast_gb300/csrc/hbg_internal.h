// hbg_internal.h -- layouts shared by the host runtime and the kernels.
//
// Device layout of a batch (all arrays in HBM, read through L1/L2):
//   group g concatenates its queries: query k's contexts NCBI-style (one
//   sentinel 0 between contexts), then a gap of `window` zero letters before
//   the next query.  The gap, the query-bounded extensions and a diagonal
//   table of >= group length + window entries make every query's result the
//   same as searching it alone.
//   cells   : (HBG_NUM_CELLS + 1) uint32 per group, CSR starts into entries
//   entries : uint16 group-local query offsets, ascending inside a cell
//   pv      : HBG_NUM_CELLS / 32 uint32 per group, bit w set iff cell w is used
//   ctx_of  : int32 per group letter, the batch-wide context index (-1 in gaps)
#ifndef HBG_INTERNAL_H
#define HBG_INTERNAL_H

#include <stdint.h>

#include "../../include/hblast_gpu.h"

#define HBG_PV_WORDS (HBG_NUM_CELLS / 32)
#define HBG_CELL_STRIDE (HBG_NUM_CELLS + 1)

struct HbgGroup {
    int64_t entry_base;   // first entry of this group in the batch entries array
    int64_t seq_base;     // first letter of this group in the batch letters array
    int32_t glen;         // letters in the group, gaps included
    int32_t diag_len;     // power of two >= glen + window
    int32_t first_query;  // queries [first_query, first_query + n_queries)
    int32_t n_queries;
    int32_t placement;    // 0: diagonal table in shared memory, 1: global scratch
    int32_t mode;         // 0: chunk mode (sparse hits), 1: offset mode (dense hits)
};

struct HbgContext {
    int32_t query;        // batch query index
    int32_t local;        // context index inside its query
    int32_t x_dropoff;
    int32_t cutoff;
};

struct HbgQueryDesc {
    int32_t group;
    int32_t start;        // group-local offset of the query's first letter
    int32_t len;          // NCBI query->length (contexts + inner sentinels)
    int32_t first_ctx;    // batch-wide index of context 0
    int32_t n_ctx;
    int32_t pad;
};

#endif
