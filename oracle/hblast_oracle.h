/*
 * hblast_oracle.h -- CPU restatement of the BLASTP/BLASTX word-hit stage.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the GPU path is compared
 * against; it is never linked into, loaded by, or called from the product
 * library.  Only tests/, __graft_entry__.smoke() and bench.py (its CPU-baseline
 * leg and the reference arm) may load it.
 *
 * What it restates (each function in hblast_oracle.c cites the lines it follows):
 *   - the two-hit diagonal state machine of NCBI BLAST+ 2.2.28
 *     aa_ungapped.c:s_BlastAaWordFinder_TwoHit, which H-BLAST restates on the
 *     GPU in h_blast_v1.1/H-BLAST/h_blast_kernel.cu:672-871;
 *   - the ungapped X-drop extension s_BlastAaExtendTwoHit / ExtendLeft /
 *     ExtendRight (NCBI aa_ungapped.c; H-BLAST h_blast_kernel.cu:1069-1540);
 *   - the diagonal table rules (NCBI blast_extend.c:s_BlastDiagTableNew and
 *     Blast_ExtendWordExit; H-BLAST h_blast.cu:959-966,1080 and
 *     h_blast_kernel.cu:1023);
 *   - the neighbourhood-word lookup table (NCBI blast_aalookup.c, consumed by
 *     H-BLAST at h_blast.cu:940-958, cells sorted ascending by
 *     h_blast.cu:165-194).
 * NCBI BLAST+ 2.2.28 itself is not part of the reference tree, so the NCBI
 * pieces are restatements of its published algorithm.  The reference ships no
 * golden vectors for this path: parity against NCBI is UNPINNED.
 */
#ifndef HBLAST_ORACLE_H
#define HBLAST_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_ALPHABET 28       /* NCBIstdaa letters 0..27 */
#define ORC_CHARSIZE 5        /* bits per letter in a word index */
#define ORC_WORDSIZE 3
#define ORC_NCELLS 32768      /* 1 << (ORC_CHARSIZE * ORC_WORDSIZE) */

typedef struct {
    int32_t q_start;   /* first query residue of the ungapped HSP (query-local) */
    int32_t s_start;   /* first subject residue of the ungapped HSP */
    int32_t q_off;     /* query offset of the second word hit (query-local) */
    int32_t s_off;     /* subject offset of the second word hit */
    int32_t len;       /* HSP length */
    int32_t score;     /* raw ungapped score */
    int32_t ctx;       /* context (frame) index inside the query */
} orc_hsp;

/* One query as NCBI concatenates it: contexts in order, one sentinel (0)
 * between consecutive contexts.  ctx_off[i] is the offset of context i inside
 * seq; len = ctx_off[n_ctx-1] + ctx_len[n_ctx-1]. */
typedef struct {
    const uint8_t *seq;
    int32_t len;
    int32_t n_ctx;
    const int32_t *ctx_off;
    const int32_t *ctx_len;
    const int32_t *x_dropoff;  /* per context, raw score units */
    const int32_t *cutoff;     /* per context, raw score units */
} orc_query;

/* Score of letters a, b (NCBIstdaa) in the BLOSUM62 table the oracle uses. */
int32_t orc_score(int32_t a, int32_t b);

/* Brute-force neighbourhood lookup table of one query, CSR layout:
 * entries[cell_start[w] .. cell_start[w+1]) are the query offsets whose word
 * scores >= threshold against word w, ascending.  cell_start has
 * ORC_NCELLS + 1 entries.  Returns the number of entries (which may exceed
 * entries_cap; then only cell_start is valid and the caller retries). */
int64_t orc_lut_build(const orc_query *q, int32_t threshold,
                      int32_t *cell_start, int32_t *entries, int64_t entries_cap);

/* Search one query against subjects [subj_begin, subj_end) of a database
 * (residues at db + db_off[i], length db_len[i]).  HSPs are written in
 * subject order and, within a subject, in the order the CPU word finder
 * creates them.  out_subject[k] is the subject index of out[k].
 * counters[0..2] += lookup hits, extensions tried, HSPs kept.
 * nthreads > 1 splits the subject range over POSIX threads.
 * Returns the number of HSPs found (may exceed out_cap: only out_cap are
 * written), or -1 on an invalid argument. */
int64_t orc_search(const orc_query *q, int32_t threshold, int32_t window,
                   const uint8_t *db, const int64_t *db_off, const int32_t *db_len,
                   int32_t subj_begin, int32_t subj_end, int32_t nthreads,
                   orc_hsp *out, int32_t *out_subject, int64_t out_cap,
                   int64_t *counters);

/* Same search from a lookup table the caller built (CSR as above). */
int64_t orc_search_lut(const orc_query *q, const int32_t *cell_start,
                       const int32_t *entries, int32_t window,
                       const uint8_t *db, const int64_t *db_off, const int32_t *db_len,
                       int32_t subj_begin, int32_t subj_end, int32_t nthreads,
                       orc_hsp *out, int32_t *out_subject, int64_t out_cap,
                       int64_t *counters);

/* Search nq queries (query k with its CSR table cell_starts[k], entries[k])
 * against subjects [subj_begin, subj_end) with nthreads threads taking
 * (query, block of about block_residues subject letters) items from a shared
 * counter (block_residues <= 0: 262144).  Every HSP is kept in memory owned
 * by the result; results equal orc_search_lut per query.  NULL on an invalid
 * argument or an allocation failure. */
typedef struct orc_result orc_result;
orc_result *orc_search_many(const orc_query *qs, int32_t nq, const int32_t *const *cell_starts,
                            const int32_t *const *entries, int32_t window, const uint8_t *db,
                            const int64_t *db_off, const int32_t *db_len, int32_t subj_begin,
                            int32_t subj_end, int32_t nthreads, int64_t block_residues);
/* HSPs of query q (-1 for a bad q). */
int64_t orc_result_count(const orc_result *r, int32_t q);
/* Copy query q's HSPs (subject order, then the CPU word finder's order) and
 * their subject indices; counters[0..2] += its lookup hits, extensions, kept. */
int orc_result_copy(const orc_result *r, int32_t q, orc_hsp *out, int32_t *out_subject,
                    int64_t *counters);
void orc_result_free(orc_result *r);

/* Standard-code six-frame translation of a nucleotide query (codes
 * A=0 C=1 G=2 T=3, anything else N) into NCBIstdaa contexts in NCBI frame
 * order +1,+2,+3,-1,-2,-3, concatenated with one sentinel between frames.
 * out must hold 2*nt_len + 6 bytes; ctx_off/ctx_len hold 6 entries.
 * Returns the concatenated length. */
int32_t orc_translate6(const uint8_t *nt, int32_t nt_len, uint8_t *out,
                       int32_t *ctx_off, int32_t *ctx_len);

#ifdef __cplusplus
}
#endif
#endif
