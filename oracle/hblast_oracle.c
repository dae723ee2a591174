/*
 * hblast_oracle.c -- CPU restatement of the BLASTP/BLASTX word-hit stage.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Never part of the product path.
 * See hblast_oracle.h for what is restated and from where.  Citations below are
 * paths inside the H-BLAST tree (h_blast_v1.1/H-BLAST/...) and, for the pieces
 * that live in NCBI BLAST+ 2.2.28 (not in the reference tree), the NCBI file
 * and function whose published algorithm is restated.
 */
#include "hblast_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* BLOSUM62 over NCBIstdaa, rows/columns - A B C D E F G H I K L M N P Q R S
 * T V W X Y Z U * O J.  Letter 0 (the sentinel) scores -128 against
 * everything, as in h_blast_v1.1/H-BLAST/h_blast.c:57-86. */
static const signed char kBlosum62[ORC_ALPHABET][ORC_ALPHABET] = {
/*        -    A    B    C    D    E    F    G    H    I    K    L    M    N    P    Q    R    S    T    V    W    X    Y    Z    U    *    O    J */
/* - */ {-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128,-128},
/* A */ {-128,  4, -2,  0, -2, -1, -2,  0, -2, -1, -1, -1, -1, -2, -1, -1, -1,  1,  0,  0, -3, -1, -2, -1, -1, -4, -1, -1},
/* B */ {-128, -2,  4, -3,  4,  1, -3, -1,  0, -3,  0, -4, -3,  4, -2,  0, -1,  0, -1, -3, -4, -1, -3,  0, -1, -4, -1, -3},
/* C */ {-128,  0, -3,  9, -3, -4, -2, -3, -3, -1, -3, -1, -1, -3, -3, -3, -3, -1, -1, -1, -2, -1, -2, -3, -1, -4, -1, -1},
/* D */ {-128, -2,  4, -3,  6,  2, -3, -1, -1, -3, -1, -4, -3,  1, -1,  0, -2,  0, -1, -3, -4, -1, -3,  1, -1, -4, -1, -3},
/* E */ {-128, -1,  1, -4,  2,  5, -3, -2,  0, -3,  1, -3, -2,  0, -1,  2,  0,  0, -1, -2, -3, -1, -2,  4, -1, -4, -1, -3},
/* F */ {-128, -2, -3, -2, -3, -3,  6, -3, -1,  0, -3,  0,  0, -3, -4, -3, -3, -2, -2, -1,  1, -1,  3, -3, -1, -4, -1,  0},
/* G */ {-128,  0, -1, -3, -1, -2, -3,  6, -2, -4, -2, -4, -3,  0, -2, -2, -2,  0, -2, -3, -2, -1, -3, -2, -1, -4, -1, -4},
/* H */ {-128, -2,  0, -3, -1,  0, -1, -2,  8, -3, -1, -3, -2,  1, -2,  0,  0, -1, -2, -3, -2, -1,  2,  0, -1, -4, -1, -3},
/* I */ {-128, -1, -3, -1, -3, -3,  0, -4, -3,  4, -3,  2,  1, -3, -3, -3, -3, -2, -1,  3, -3, -1, -1, -3, -1, -4, -1,  3},
/* K */ {-128, -1,  0, -3, -1,  1, -3, -2, -1, -3,  5, -2, -1,  0, -1,  1,  2,  0, -1, -2, -3, -1, -2,  1, -1, -4, -1, -3},
/* L */ {-128, -1, -4, -1, -4, -3,  0, -4, -3,  2, -2,  4,  2, -3, -3, -2, -2, -2, -1,  1, -2, -1, -1, -3, -1, -4, -1,  3},
/* M */ {-128, -1, -3, -1, -3, -2,  0, -3, -2,  1, -1,  2,  5, -2, -2,  0, -1, -1, -1,  1, -1, -1, -1, -1, -1, -4, -1,  2},
/* N */ {-128, -2,  4, -3,  1,  0, -3,  0,  1, -3,  0, -3, -2,  6, -2,  0,  0,  1,  0, -3, -4, -1, -2,  0, -1, -4, -1, -3},
/* P */ {-128, -1, -2, -3, -1, -1, -4, -2, -2, -3, -1, -3, -2, -2,  7, -1, -2, -1, -1, -2, -4, -1, -3, -1, -1, -4, -1, -3},
/* Q */ {-128, -1,  0, -3,  0,  2, -3, -2,  0, -3,  1, -2,  0,  0, -1,  5,  1,  0, -1, -2, -2, -1, -1,  4, -1, -4, -1, -2},
/* R */ {-128, -1, -1, -3, -2,  0, -3, -2,  0, -3,  2, -2, -1,  0, -2,  1,  5, -1, -1, -3, -3, -1, -2,  0, -1, -4, -1, -2},
/* S */ {-128,  1,  0, -1,  0,  0, -2,  0, -1, -2,  0, -2, -1,  1, -1,  0, -1,  4,  1, -2, -3, -1, -2,  0, -1, -4, -1, -2},
/* T */ {-128,  0, -1, -1, -1, -1, -2, -2, -2, -1, -1, -1, -1,  0, -1, -1, -1,  1,  5,  0, -2, -1, -2, -1, -1, -4, -1, -1},
/* V */ {-128,  0, -3, -1, -3, -2, -1, -3, -3,  3, -2,  1,  1, -3, -2, -2, -3, -2,  0,  4, -3, -1, -1, -2, -1, -4, -1,  2},
/* W */ {-128, -3, -4, -2, -4, -3,  1, -2, -2, -3, -3, -2, -1, -4, -4, -2, -3, -3, -2, -3, 11, -1,  2, -2, -1, -4, -1, -2},
/* X */ {-128, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -4, -1, -1},
/* Y */ {-128, -2, -3, -2, -3, -2,  3, -3,  2, -1, -2, -1, -1, -2, -3, -1, -2, -2, -2, -1,  2, -1,  7, -2, -1, -4, -1, -1},
/* Z */ {-128, -1,  0, -3,  1,  4, -3, -2,  0, -3,  1, -3, -1,  0, -1,  4,  0,  0, -1, -2, -2, -1, -2,  4, -1, -4, -1, -3},
/* U */ {-128, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -4, -1, -1},
/* * */ {-128, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4,  1, -4, -4},
/* O */ {-128, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -4, -1, -1},
/* J */ {-128, -1, -3, -1, -3, -3,  0, -4, -3,  3, -3,  3,  2, -3, -3, -2, -2, -2, -1,  2, -2, -1, -1, -3, -1, -4, -1,  3},
};

int32_t orc_score(int32_t a, int32_t b)
{
    if (a < 0 || a >= ORC_ALPHABET || b < 0 || b >= ORC_ALPHABET)
        return -128;
    return kBlosum62[a][b];
}

#define SC(a, b) ((int32_t)kBlosum62[(a)][(b)])

/* ------------------------------------------------------------------------ */
/* Lookup table.                                                             */
/* Restates NCBI blast_aalookup.c (BlastAaLookupTableNew: 28-letter alphabet,
 * charsize ilog2(28)+1 = 5; s_AddNeighboringWords / s_AddWordHits: every word
 * over the alphabet whose score against the query word reaches the
 * threshold).  Words are taken only inside one context (NCBI indexes each
 * location range separately).  Cell contents are ascending query offsets, the
 * order H-BLAST's lut_sorting (h_blast.cu:165-194) enforces.  The word index
 * is ((a << 5 | b) << 5 | c), as built in h_blast_kernel.cu:610-614,649. */
/* ------------------------------------------------------------------------ */

static void lut_count_or_fill(const orc_query *q, int32_t threshold,
                              int32_t *cursor, int32_t *entries, int fill)
{
    for (int32_t c = 0; c < q->n_ctx; ++c) {
        int32_t from = q->ctx_off[c];
        int32_t to = q->ctx_off[c] + q->ctx_len[c] - ORC_WORDSIZE;
        for (int32_t p = from; p <= to; ++p) {
            const uint8_t *w = q->seq + p;
            for (int a = 0; a < ORC_ALPHABET; ++a) {
                int32_t s1 = SC(w[0], a);
                for (int b = 0; b < ORC_ALPHABET; ++b) {
                    int32_t s2 = s1 + SC(w[1], b);
                    for (int cc = 0; cc < ORC_ALPHABET; ++cc) {
                        int32_t s3 = s2 + SC(w[2], cc);
                        if (s3 >= threshold) {
                            int32_t idx = (a << 10) | (b << 5) | cc;
                            if (fill)
                                entries[cursor[idx]] = p;
                            cursor[idx]++;
                        }
                    }
                }
            }
        }
    }
}

int64_t orc_lut_build(const orc_query *q, int32_t threshold,
                      int32_t *cell_start, int32_t *entries, int64_t entries_cap)
{
    int32_t *count = (int32_t *)calloc(ORC_NCELLS, sizeof(int32_t));
    if (!count)
        return -1;
    lut_count_or_fill(q, threshold, count, NULL, 0);
    int64_t total = 0;
    for (int i = 0; i < ORC_NCELLS; ++i) {
        cell_start[i] = (int32_t)total;
        total += count[i];
    }
    cell_start[ORC_NCELLS] = (int32_t)total;
    if (total <= entries_cap && entries) {
        for (int i = 0; i < ORC_NCELLS; ++i)
            count[i] = cell_start[i];
        lut_count_or_fill(q, threshold, count, entries, 1);
    }
    free(count);
    return total;
}

/* ------------------------------------------------------------------------ */
/* Ungapped extension.                                                       */
/* ------------------------------------------------------------------------ */

/* NCBI aa_ungapped.c:s_BlastAaExtendLeft; H-BLAST h_blast_kernel.cu:1329-1540.
 * Walks left from (s_off, q_off) inclusive while the drop from the best score
 * stays below dropoff, at most min(s_off, q_off)+1 letters.  Note: the
 * H-BLAST kernel skips the walk entirely when min(s_off, q_off) == 0
 * (h_blast_kernel.cu:1368); the NCBI loop scores that single letter, and the
 * oracle follows NCBI. */
static int32_t extend_left(const uint8_t *s, const uint8_t *q, int32_t s_off,
                           int32_t q_off, int32_t dropoff, int32_t *length,
                           int32_t maxscore)
{
    int32_t n = s_off < q_off ? s_off : q_off;
    int32_t best_i = n + 1;
    int32_t score = maxscore;
    const uint8_t *sp = s + s_off - n;
    const uint8_t *qp = q + q_off - n;
    for (int32_t i = n; i >= 0; --i) {
        score += SC(qp[i], sp[i]);
        if (score > maxscore) {
            maxscore = score;
            best_i = i;
        }
        if (maxscore - score >= dropoff)
            break;
    }
    *length = n - best_i + 1;
    return maxscore;
}

/* NCBI aa_ungapped.c:s_BlastAaExtendRight; H-BLAST h_blast_kernel.cu:1133-1326.
 * Walks right from (s_off, q_off) while the running score stays positive and
 * the drop stays below dropoff; reports the last subject offset examined. */
static int32_t extend_right(const uint8_t *s, int32_t s_len, const uint8_t *q,
                            int32_t q_len, int32_t s_off, int32_t q_off,
                            int32_t dropoff, int32_t *length, int32_t maxscore,
                            int32_t *s_last_off)
{
    int32_t n = (s_len - s_off) < (q_len - q_off) ? (s_len - s_off) : (q_len - q_off);
    int32_t best_i = -1;
    int32_t score = maxscore;
    int32_t i;
    for (i = 0; i < n; ++i) {
        score += SC(q[q_off + i], s[s_off + i]);
        if (score > maxscore) {
            maxscore = score;
            best_i = i;
        }
        if (score <= 0 || maxscore - score >= dropoff)
            break;
    }
    *length = best_i + 1;
    *s_last_off = s_off + i;
    return maxscore;
}

/* NCBI aa_ungapped.c:s_BlastAaExtendTwoHit; H-BLAST h_blast_kernel.cu:1069-1130.
 * s_left_off is one past the end of the first hit's word.  The left walk
 * restarts from score 0 at the end of the best-scoring prefix of the second
 * word; the right walk runs only when the left walk reached the first hit. */
static int32_t extend_two_hit(const uint8_t *s, int32_t s_len, const uint8_t *q,
                              int32_t q_len, int32_t s_left_off, int32_t s_right_off,
                              int32_t q_right_off, int32_t dropoff,
                              int32_t *hsp_q, int32_t *hsp_s, int32_t *hsp_len,
                              int *right_extend, int32_t *s_last_off)
{
    int32_t left_d = 0, right_d = 0;
    int32_t left_score = 0, right_score = 0;
    int32_t score = 0;
    for (int32_t i = 0; i < ORC_WORDSIZE; ++i) {
        score += SC(q[q_right_off + i], s[s_right_off + i]);
        if (score > left_score) {
            left_score = score;
            right_d = i + 1;
        }
    }
    q_right_off += right_d;
    s_right_off += right_d;
    right_d = 0;
    *right_extend = 0;
    *s_last_off = s_right_off;

    left_score = extend_left(s, q, s_right_off - 1, q_right_off - 1, dropoff,
                             &left_d, 0);
    if (left_d >= s_right_off - s_left_off) {
        *right_extend = 1;
        right_score = extend_right(s, s_len, q, q_len, s_right_off, q_right_off,
                                   dropoff, &right_d, left_score, s_last_off);
    }
    *hsp_q = q_right_off - left_d;
    *hsp_s = s_right_off - left_d;
    *hsp_len = left_d + right_d;
    return left_score > right_score ? left_score : right_score;
}

/* ------------------------------------------------------------------------ */
/* Diagonal table.                                                           */
/* NCBI blast_extend.c:s_BlastDiagTableNew: the array length is the smallest
 * power of two >= query length + window, the mask is length-1, the offset
 * starts at window; NCBI DiagStruct packs last_hit in 31 bits with a 1-bit
 * flag.  Blast_ExtendWordExit advances the offset by subject length + window
 * after each subject and clears the table once the offset passes INT4_MAX/4.
 * H-BLAST: h_blast.cu:959-966,1080; h_blast_kernel.cu:1023. */
/* ------------------------------------------------------------------------ */

typedef struct {
    uint32_t *cell;    /* bit 31 = flag, bits 0..30 = last_hit */
    int32_t length;
    int32_t mask;
    int32_t offset;
    int32_t window;
} diag_table;

static int diag_init(diag_table *d, int32_t qlen, int32_t window)
{
    int32_t n = 1;
    while (n < qlen + window)
        n <<= 1;
    d->cell = (uint32_t *)calloc((size_t)n, sizeof(uint32_t));
    d->length = n;
    d->mask = n - 1;
    d->offset = window;
    d->window = window;
    return d->cell ? 0 : -1;
}

static void diag_exit_subject(diag_table *d, int32_t s_len)
{
    if (d->offset >= INT32_MAX / 4) {
        d->offset = d->window;
        memset(d->cell, 0, sizeof(uint32_t) * (size_t)d->length);
    } else {
        d->offset += s_len + d->window;
    }
}

#define DG_FLAG 0x80000000u
#define DG_LAST 0x7fffffffu

/* ------------------------------------------------------------------------ */
/* Two-hit word finder for one subject.                                      */
/* NCBI aa_ungapped.c:s_BlastAaWordFinder_TwoHit (scan every subject offset
 * 0..len-3 in order, every cell entry in order); H-BLAST restates the per-hit
 * state machine at h_blast_kernel.cu:672-871, the context search at :707-719
 * and the cutoff test at :740.  HSP offsets follow NF/blast_engine.c:567-576. */
/* ------------------------------------------------------------------------ */

typedef struct {
    orc_hsp *v;
    int64_t n, cap;
} hsp_vec;

static int hsp_push(hsp_vec *h, const orc_hsp *x)
{
    if (h->n == h->cap) {
        int64_t nc = h->cap ? h->cap * 2 : 64;
        orc_hsp *nv = (orc_hsp *)realloc(h->v, (size_t)nc * sizeof(orc_hsp));
        if (!nv)
            return -1;
        h->v = nv;
        h->cap = nc;
    }
    h->v[h->n++] = *x;
    return 0;
}

static int32_t context_of(const orc_query *q, int32_t q_off)
{
    /* last context whose start is <= q_off (h_blast_kernel.cu:707-719) */
    int32_t lo = 0, hi = q->n_ctx;
    while (hi - lo > 1) {
        int32_t mid = (lo + hi) >> 1;
        if (q->ctx_off[mid] <= q_off)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

static int word_finder_subject(const orc_query *q, const int32_t *cell_start,
                               const int32_t *entries, diag_table *dg,
                               const uint8_t *s, int32_t s_len,
                               hsp_vec *out, int64_t *counters)
{
    const int32_t W = ORC_WORDSIZE;
    const int32_t window = dg->window;
    const int32_t off = dg->offset;
    int64_t hits = 0, extended = 0, kept = 0;

    for (int32_t s_off = 0; s_off <= s_len - W; ++s_off) {
        int32_t idx = ((s[s_off] << 10) | (s[s_off + 1] << 5) | s[s_off + 2]) &
                      (ORC_NCELLS - 1);
        int32_t b = cell_start[idx], e = cell_start[idx + 1];
        hits += e - b;
        for (int32_t k = b; k < e; ++k) {
            int32_t q_off = entries[k];
            int32_t dc = (q_off - s_off) & dg->mask;
            uint32_t cell = dg->cell[dc];
            int32_t last_hit = (int32_t)(cell & DG_LAST);
            if (cell & DG_FLAG) {
                if (s_off + off < last_hit)
                    continue;
                dg->cell[dc] = (uint32_t)(s_off + off);
                continue;
            }
            int32_t diff = s_off - (last_hit - off);
            if (diff >= window) {
                dg->cell[dc] = (uint32_t)(s_off + off);
                continue;
            }
            if (diff < W)
                continue;
            int32_t ctx = context_of(q, q_off);
            int32_t hq, hs, hl, s_last_off;
            int rext;
            int32_t score = extend_two_hit(s, s_len, q->seq, q->len,
                                           (last_hit - off) + W, s_off, q_off,
                                           q->x_dropoff[ctx], &hq, &hs, &hl,
                                           &rext, &s_last_off);
            ++extended;
            if (score >= q->cutoff[ctx]) {
                orc_hsp h = {hq, hs, q_off, s_off, hl, score, ctx};
                if (hsp_push(out, &h))
                    return -1;
                ++kept;
            }
            if (rext)
                dg->cell[dc] = DG_FLAG | (uint32_t)(s_last_off - (W - 1) + off);
            else
                dg->cell[dc] = (uint32_t)(s_off + off);
        }
    }
    counters[0] += hits;
    counters[1] += extended;
    counters[2] += kept;
    diag_exit_subject(dg, s_len);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Search driver (threads over contiguous subject ranges).                   */
/* ------------------------------------------------------------------------ */

typedef struct {
    const orc_query *q;
    const int32_t *cell_start, *entries;
    int32_t window;
    const uint8_t *db;
    const int64_t *db_off;
    const int32_t *db_len;
    int32_t begin, end;
    hsp_vec hsps;
    int32_t *subj;        /* subject of each HSP */
    int64_t subj_cap;
    int64_t counters[3];
    int status;
} worker;

static void *worker_run(void *arg)
{
    worker *w = (worker *)arg;
    diag_table dg;
    if (diag_init(&dg, w->q->len, w->window)) {
        w->status = -1;
        return NULL;
    }
    for (int32_t j = w->begin; j < w->end; ++j) {
        int64_t before = w->hsps.n;
        if (word_finder_subject(w->q, w->cell_start, w->entries, &dg,
                                w->db + w->db_off[j], w->db_len[j], &w->hsps,
                                w->counters)) {
            w->status = -1;
            break;
        }
        if (w->hsps.n > before) {
            if (w->hsps.n > w->subj_cap) {
                int64_t nc = w->hsps.cap;
                int32_t *ns = (int32_t *)realloc(w->subj, (size_t)nc * sizeof(int32_t));
                if (!ns) {
                    w->status = -1;
                    break;
                }
                w->subj = ns;
                w->subj_cap = nc;
            }
            for (int64_t k = before; k < w->hsps.n; ++k)
                w->subj[k] = j;
        }
    }
    free(dg.cell);
    return NULL;
}

int64_t orc_search_lut(const orc_query *q, const int32_t *cell_start,
                       const int32_t *entries, int32_t window,
                       const uint8_t *db, const int64_t *db_off, const int32_t *db_len,
                       int32_t subj_begin, int32_t subj_end, int32_t nthreads,
                       orc_hsp *out, int32_t *out_subject, int64_t out_cap,
                       int64_t *counters)
{
    if (!q || !cell_start || subj_end < subj_begin || window <= 0)
        return -1;
    if (nthreads < 1)
        nthreads = 1;
    int32_t n = subj_end - subj_begin;
    if (nthreads > n && n > 0)
        nthreads = n;
    if (n == 0)
        return 0;
    worker *ws = (worker *)calloc((size_t)nthreads, sizeof(worker));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!ws || !th) {
        free(ws);
        free(th);
        return -1;
    }
    /* balance by residues */
    int64_t total = 0;
    for (int32_t j = subj_begin; j < subj_end; ++j)
        total += db_len[j];
    int32_t j = subj_begin;
    for (int t = 0; t < nthreads; ++t) {
        ws[t].q = q;
        ws[t].cell_start = cell_start;
        ws[t].entries = entries;
        ws[t].window = window;
        ws[t].db = db;
        ws[t].db_off = db_off;
        ws[t].db_len = db_len;
        ws[t].begin = j;
        int64_t target = total * (t + 1) / nthreads, acc = 0;
        for (int32_t k = subj_begin; k < j; ++k)
            acc += db_len[k];
        while (j < subj_end && (acc < target || t == nthreads - 1)) {
            acc += db_len[j];
            ++j;
        }
        ws[t].end = j;
    }
    for (int t = 0; t < nthreads; ++t)
        pthread_create(&th[t], NULL, worker_run, &ws[t]);
    for (int t = 0; t < nthreads; ++t)
        pthread_join(th[t], NULL);

    int64_t found = 0;
    int status = 0;
    for (int t = 0; t < nthreads; ++t) {
        status |= ws[t].status;
        for (int c = 0; c < 3; ++c)
            counters[c] += ws[t].counters[c];
        for (int64_t k = 0; k < ws[t].hsps.n; ++k, ++found) {
            if (found < out_cap) {
                if (out)
                    out[found] = ws[t].hsps.v[k];
                if (out_subject)
                    out_subject[found] = ws[t].subj[k];
            }
        }
        free(ws[t].hsps.v);
        free(ws[t].subj);
    }
    free(ws);
    free(th);
    return status ? -1 : found;
}

int64_t orc_search(const orc_query *q, int32_t threshold, int32_t window,
                   const uint8_t *db, const int64_t *db_off, const int32_t *db_len,
                   int32_t subj_begin, int32_t subj_end, int32_t nthreads,
                   orc_hsp *out, int32_t *out_subject, int64_t out_cap,
                   int64_t *counters)
{
    int32_t *cell_start = (int32_t *)malloc(sizeof(int32_t) * (ORC_NCELLS + 1));
    if (!cell_start)
        return -1;
    int64_t n = orc_lut_build(q, threshold, cell_start, NULL, 0);
    int32_t *entries = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    if (n < 0 || !entries) {
        free(cell_start);
        free(entries);
        return -1;
    }
    orc_lut_build(q, threshold, cell_start, entries, n);
    int64_t r = orc_search_lut(q, cell_start, entries, window, db, db_off, db_len,
                               subj_begin, subj_end, nthreads, out, out_subject,
                               out_cap, counters);
    free(cell_start);
    free(entries);
    return r;
}

/* ------------------------------------------------------------------------ */
/* Many queries in one call.                                                 */
/* Work items are (query, block of subjects), taken in order by a pool of    */
/* threads from a shared counter; each item starts a fresh diagonal table,   */
/* which changes no result (the offset trick makes the table's state fresh   */
/* for every subject, Blast_ExtendWordExit).  Every HSP is kept: there is no */
/* caller-sized buffer to overflow and no search is repeated.                */
/* ------------------------------------------------------------------------ */

typedef struct {
    int32_t q, begin, end;
    hsp_vec hsps;
    int32_t *subj;
    int64_t subj_cap;
    int64_t counters[3];
} many_item;

struct orc_result {
    int32_t nq;
    int64_t n_items;
    int64_t *item_first;     /* per query: first item; items of a query are contiguous */
    many_item *items;
    const orc_query *qs;
    const int32_t *const *cell_starts;
    const int32_t *const *entries;
    int32_t window;
    const uint8_t *db;
    const int64_t *db_off;
    const int32_t *db_len;
    int64_t next;            /* next item to take */
    pthread_mutex_t lock;
    int status;
};

static int run_item(orc_result *r, many_item *it)
{
    const orc_query *q = &r->qs[it->q];
    diag_table dg;
    if (diag_init(&dg, q->len, r->window))
        return -1;
    int rc = 0;
    for (int32_t j = it->begin; j < it->end && rc == 0; ++j) {
        int64_t before = it->hsps.n;
        rc = word_finder_subject(q, r->cell_starts[it->q], r->entries[it->q], &dg,
                                 r->db + r->db_off[j], r->db_len[j], &it->hsps, it->counters);
        if (rc == 0 && it->hsps.n > before) {
            if (it->hsps.n > it->subj_cap) {
                int32_t *ns = (int32_t *)realloc(it->subj, (size_t)it->hsps.cap * sizeof(int32_t));
                if (!ns) {
                    rc = -1;
                    break;
                }
                it->subj = ns;
                it->subj_cap = it->hsps.cap;
            }
            for (int64_t k = before; k < it->hsps.n; ++k)
                it->subj[k] = j;
        }
    }
    free(dg.cell);
    return rc;
}

static void *many_worker(void *arg)
{
    orc_result *r = (orc_result *)arg;
    for (;;) {
        pthread_mutex_lock(&r->lock);
        int64_t i = r->next++;
        pthread_mutex_unlock(&r->lock);
        if (i >= r->n_items)
            break;
        if (run_item(r, &r->items[i])) {
            pthread_mutex_lock(&r->lock);
            r->status = -1;
            pthread_mutex_unlock(&r->lock);
        }
    }
    return NULL;
}

void orc_result_free(orc_result *r)
{
    if (!r)
        return;
    for (int64_t i = 0; i < r->n_items; ++i) {
        free(r->items[i].hsps.v);
        free(r->items[i].subj);
    }
    free(r->items);
    free(r->item_first);
    pthread_mutex_destroy(&r->lock);
    free(r);
}

orc_result *orc_search_many(const orc_query *qs, int32_t nq, const int32_t *const *cell_starts,
                            const int32_t *const *entries, int32_t window, const uint8_t *db,
                            const int64_t *db_off, const int32_t *db_len, int32_t subj_begin,
                            int32_t subj_end, int32_t nthreads, int64_t block_residues)
{
    if (!qs || nq < 0 || !cell_starts || !entries || window <= 0 || subj_end < subj_begin)
        return NULL;
    if (block_residues <= 0)
        block_residues = 1 << 18;
    orc_result *r = (orc_result *)calloc(1, sizeof(orc_result));
    if (!r)
        return NULL;
    pthread_mutex_init(&r->lock, NULL);
    r->nq = nq;
    r->qs = qs;
    r->cell_starts = cell_starts;
    r->entries = entries;
    r->window = window;
    r->db = db;
    r->db_off = db_off;
    r->db_len = db_len;
    /* subject blocks of about block_residues letters */
    int64_t n_blocks = 0;
    int32_t *bstart = (int32_t *)malloc(sizeof(int32_t) * ((size_t)(subj_end - subj_begin) + 2));
    r->item_first = (int64_t *)calloc((size_t)nq + 1, sizeof(int64_t));
    if (!bstart || !r->item_first) {
        free(bstart);
        orc_result_free(r);
        return NULL;
    }
    for (int32_t j = subj_begin; j < subj_end;) {
        bstart[n_blocks++] = j;
        int64_t acc = 0;
        while (j < subj_end && (acc == 0 || acc + db_len[j] <= block_residues))
            acc += db_len[j++] + 1;
    }
    bstart[n_blocks] = subj_end;
    r->n_items = n_blocks * nq;
    r->items = (many_item *)calloc((size_t)(r->n_items > 0 ? r->n_items : 1), sizeof(many_item));
    if (!r->items) {
        free(bstart);
        orc_result_free(r);
        return NULL;
    }
    for (int32_t q = 0; q < nq; ++q) {
        r->item_first[q] = (int64_t)q * n_blocks;
        for (int64_t b = 0; b < n_blocks; ++b) {
            many_item *it = &r->items[(int64_t)q * n_blocks + b];
            it->q = q;
            it->begin = bstart[b];
            it->end = bstart[b + 1];
        }
    }
    r->item_first[nq] = r->n_items;
    free(bstart);
    if (nthreads < 1)
        nthreads = 1;
    if (nthreads > r->n_items)
        nthreads = (int32_t)(r->n_items > 0 ? r->n_items : 1);
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!th) {
        orc_result_free(r);
        return NULL;
    }
    int started = 0;
    for (int t = 0; t < nthreads; ++t)
        if (pthread_create(&th[t], NULL, many_worker, r) == 0)
            ++started;
    if (started == 0)
        many_worker(r);
    for (int t = 0; t < started; ++t)
        pthread_join(th[t], NULL);
    free(th);
    if (r->status) {
        orc_result_free(r);
        return NULL;
    }
    return r;
}

int64_t orc_result_count(const orc_result *r, int32_t q)
{
    if (!r || q < 0 || q >= r->nq)
        return -1;
    int64_t n = 0;
    for (int64_t i = r->item_first[q]; i < r->item_first[q + 1]; ++i)
        n += r->items[i].hsps.n;
    return n;
}

int orc_result_copy(const orc_result *r, int32_t q, orc_hsp *out, int32_t *out_subject,
                    int64_t *counters)
{
    if (!r || q < 0 || q >= r->nq)
        return -1;
    int64_t k = 0;
    for (int64_t i = r->item_first[q]; i < r->item_first[q + 1]; ++i) {
        const many_item *it = &r->items[i];
        if (out)
            memcpy(out + k, it->hsps.v, (size_t)it->hsps.n * sizeof(orc_hsp));
        if (out_subject)
            memcpy(out_subject + k, it->subj, (size_t)it->hsps.n * sizeof(int32_t));
        k += it->hsps.n;
        if (counters)
            for (int c = 0; c < 3; ++c)
                counters[c] += it->counters[c];
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Six-frame translation (standard genetic code, NCBI transl_table 1).       */
/* NCBI concatenates the six frames of a blastx query as contexts 0..5 =
 * frames +1,+2,+3,-1,-2,-3 (H-BLAST bins them by context at
 * h_blast_kernel.cu:369-380 and reads the per-frame cutoffs from
 * h_blast.cu:977-983). */
/* ------------------------------------------------------------------------ */

/* amino acid of codon (b1,b2,b3) in TCAG order, as one-letter codes */
static const char kStdCode[65] =
    "FFLLSSSSYY**CC*WLLLLPPPPHHQQRRRRIIIMTTTTNNKKSSRRVVVVAAAADDEEGGGG";

static uint8_t aa_code(char c)
{
    static const char letters[] = "-ABCDEFGHIKLMNPQRSTVWXYZU*OJ";
    for (int i = 0; i < ORC_ALPHABET; ++i)
        if (letters[i] == c)
            return (uint8_t)i;
    return 21; /* X */
}

static int tcag(uint8_t nt)
{
    /* input codes A=0 C=1 G=2 T=3 -> TCAG index T=0 C=1 A=2 G=3 */
    switch (nt) {
    case 0: return 2;
    case 1: return 1;
    case 2: return 3;
    case 3: return 0;
    default: return -1;
    }
}

static uint8_t translate_codon(uint8_t a, uint8_t b, uint8_t c)
{
    int x = tcag(a), y = tcag(b), z = tcag(c);
    if (x < 0 || y < 0 || z < 0)
        return 21;
    return aa_code(kStdCode[x * 16 + y * 4 + z]);
}

int32_t orc_translate6(const uint8_t *nt, int32_t nt_len, uint8_t *out,
                       int32_t *ctx_off, int32_t *ctx_len)
{
    int32_t pos = 0;
    for (int f = 0; f < 6; ++f) {
        int32_t start = f % 3;
        int32_t n = nt_len > start ? (nt_len - start) / 3 : 0;
        if (f > 0)
            out[pos++] = 0;
        ctx_off[f] = pos;
        ctx_len[f] = n;
        for (int32_t i = 0; i < n; ++i) {
            uint8_t a, b, c;
            int32_t p = start + 3 * i;
            if (f < 3) {
                a = nt[p];
                b = nt[p + 1];
                c = nt[p + 2];
            } else {
                /* reverse complement position r maps to nt[nt_len-1-r] */
                a = nt[nt_len - 1 - p] < 4 ? 3 - nt[nt_len - 1 - p] : 4;
                b = nt[nt_len - 2 - p] < 4 ? 3 - nt[nt_len - 2 - p] : 4;
                c = nt[nt_len - 3 - p] < 4 ? 3 - nt[nt_len - 3 - p] : 4;
            }
            out[pos++] = translate_codon(a, b, c);
        }
    }
    return pos;
}
