/*
 * hblast_gpu.h -- C ABI of the GB300 word-hit stage (BLASTP/BLASTX lookup,
 * two-hit diagonal detection, ungapped X-drop extension).
 *
 * Plain C types only: pointers, sizes, int32/int64.  Every call returns an
 * int status (HBG_OK or a negative HBG_ERR_* code); nothing here exits the
 * process or resets a device.  Handles are independent: a process may hold
 * several databases and batches, and calls on different handles may run from
 * different host threads.
 *
 * Each entry point names the H-BLAST interface it replaces.  H-BLAST paths are
 * inside h_blast_v1.1/H-BLAST/ (NF = ncbi_blast_files/).
 */
#ifndef HBLAST_GPU_H
#define HBLAST_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define HBG_OK 0
#define HBG_ERR_INVALID -1      /* bad argument (null pointer, bad size, bad residue) */
#define HBG_ERR_CUDA -2         /* a CUDA runtime call failed; see hbg_last_error() */
#define HBG_ERR_NOMEM -3        /* host or device allocation failed */
#define HBG_ERR_TOO_LONG -4     /* a query or subject exceeds a documented limit */
#define HBG_ERR_NO_DEVICE -5    /* no CUDA device, or the library was built for another GPU */
#define HBG_ERR_STATE -6        /* call out of order (e.g. collect before search) */
#define HBG_ERR_CAPACITY -7     /* a caller-sized buffer is too small; the needed size is reported */

/* ---- limits ------------------------------------------------------------- */
#define HBG_WORD_SIZE 3
#define HBG_NUM_CELLS 32768            /* 1 << (5 bits x 3 letters) */
#define HBG_ALPHABET 28                /* NCBIstdaa letters 0..27 */
#define HBG_MAX_QUERY_LEN 65000        /* concatenated contexts of one query */
#define HBG_MAX_SUBJECT_LEN 1000000000 /* subjects are int32-indexed */

/* ---- records ------------------------------------------------------------ */

/* One ungapped HSP.  Offsets are local to the query (its contexts
 * concatenated NCBI-style, one sentinel between contexts) and to the subject.
 * Replaces GPUBlastInitHitList (NF/gpu_cpu_common.h:31-40): int32 fields
 * instead of uint16, the hit offset stored directly instead of
 * offset_from_first_position, and the query/subject/context written out.
 * BlastSaveInitHsp(list, q_start, s_start, q_off, s_off, len, score) takes
 * these fields as they are (NF/blast_engine.c:567-576). */
typedef struct hbg_hsp {
    int32_t query;     /* index of the query in its batch */
    int32_t subject;   /* ordinal id of the subject in the database */
    int32_t q_start;   /* first query residue of the HSP */
    int32_t s_start;   /* first subject residue of the HSP */
    int32_t q_off;     /* query offset of the word hit that triggered it */
    int32_t s_off;     /* subject offset of that word hit */
    int32_t len;       /* HSP length */
    int32_t score;     /* raw ungapped score */
    int32_t context;   /* context of the query (0 for blastp, frame 0..5 for blastx) */
} hbg_hsp;

/* Per-query diagnostics, the numbers NCBI feeds to Blast_UngappedStatsUpdate
 * (NF/blast_engine.c:579-582) summed over the database. */
typedef struct hbg_query_stats {
    int64_t lookup_hits;       /* word hits found by the scan */
    int64_t init_extends;      /* ungapped extensions tried */
    int64_t good_init_extends; /* extensions that reached the cutoff */
    int64_t subjects_passed;   /* subjects with at least one HSP */
} hbg_query_stats;

/* One query as NCBI concatenates it (BLAST_SequenceBlk + BlastQueryInfo,
 * read by H-BLAST at h_blast.cu:968-983): residues in NCBIstdaa, contexts in
 * order, one sentinel (0) between consecutive contexts; length =
 * context_offset[last] + context_length[last].  x_dropoff and cutoff_score
 * are per context in raw score units (word_params->cutoffs[ctx], read at
 * h_blast.cu:977-983). */
typedef struct hbg_query {
    const uint8_t *sequence;
    int32_t length;
    int32_t num_contexts;
    const int32_t *context_offset;
    const int32_t *context_length;
    const int32_t *x_dropoff;
    const int32_t *cutoff_score;
} hbg_query;

/* Word-finder parameters (LookupTableOptions + the diagonal window). */
typedef struct hbg_word_params {
    int32_t threshold;   /* neighbourhood threshold T (11 for blastp/blastx) */
    int32_t window;      /* two-hit window A (40) */
} hbg_word_params;

/* Mirror of BlastGPUOptions (NF/blast_options.h:503-514), the values of the
 * -gpu, -gpu_threads, -gpu_blocks, -method and -num_threads flags
 * (NF/blast_args.cpp:2705-2778).  num_threadsx is the largest CTA size (a
 * multiple of 32, 32..1024): with num_blocksx 0 (one persistent wave sized
 * from the SM count) each launch uses the size, halving down to 64, that
 * keeps the most warps resident (large diagonal tables fill shared memory);
 * with num_blocksx > 0 both are used as given when they fit.  method selects
 * the device among the visible ones (0 = first);
 * use_gpu 0 makes hbg_search return HBG_ERR_NO_DEVICE (this library has no
 * CPU path). */
typedef struct hbg_gpu_options {
    int32_t use_gpu;
    int32_t num_blocksx;
    int32_t num_threadsx;
    int32_t method;
    int32_t cpu_threads;
} hbg_gpu_options;

/* Values of the H-BLAST_runtime_options text file
 * (runtime_setting_files/H-BLAST_runtime_options:1-18, parsed by
 * NF/functions.cpp:142-202).  avg_hsps_per_sequence sizes the HSP buffer;
 * the other values drive H-BLAST's CPU/GPU balancer and are kept readable
 * for compatibility. */
typedef struct hbg_runtime_options {
    double gpu_db_used_ratio;
    int32_t fixed_ratio;
    double ccr;
    int32_t avg_hsps_per_sequence;
    int32_t mem_ecc;
    int32_t balancer_method;
    int32_t load_factor;
    int32_t chunk_size;
    int32_t base_value;
} hbg_runtime_options;

typedef struct hbg_db hbg_db;         /* device-resident subject database */
typedef struct hbg_batch hbg_batch;   /* packed queries + lookup tables */
typedef struct hbg_result hbg_result; /* one search: device buffers + host copy */

/* ---- library ------------------------------------------------------------ */

/* Text of the last error on the calling thread ("" if none). */
const char *hbg_last_error(void);

/* Number of usable devices (replaces GPU_BLAST_check_availability,
 * NF/gpu_cpu_common.h:103, and gpu_get_device_count). */
int hbg_device_count(int32_t *count);

/* Defaults: use_gpu 1, num_blocksx 0, num_threadsx 256, method 0,
 * cpu_threads 1 (cf. NF/cmdline_flags.cpp:215-228). */
int hbg_default_gpu_options(hbg_gpu_options *opt);

/* Parse an H-BLAST_runtime_options file: comment/value line pairs in the
 * order of runtime_setting_files/H-BLAST_runtime_options, with the same
 * range fix-ups as Read_H_BLAST_runtime_options (NF/functions.cpp:142-202).
 * A missing file gives the defaults and HBG_OK (the reference prints a
 * warning and keeps its defaults). */
int hbg_read_runtime_options(const char *path, hbg_runtime_options *out);

/* ---- database ----------------------------------------------------------- */

/* Copy n_subjects protein sequences to device memory and keep them resident.
 * Subject i is residues[offsets[i] .. offsets[i+1]) (offsets has n_subjects+1
 * entries), NCBIstdaa letters 1..27.  Replaces the per-volume .hDb staging
 * of Read_H_BLAST_GPU_DB + H_BLAST's database copy (h_blast.cu:587-653,
 * 993, 1094-1096): the database is packed uint8 with one sentinel between
 * subjects plus an int64 offset array, uploaded once. */
int hbg_db_open(const uint8_t *residues, const int64_t *offsets, int32_t n_subjects,
                const hbg_gpu_options *opt, hbg_db **out);
int hbg_db_close(hbg_db *db);
int hbg_db_info(const hbg_db *db, int32_t *n_subjects, int64_t *n_residues,
                int64_t *device_bytes);

/* ---- NCBI BLAST databases on disk ------------------------------------------ */

/* `path` names a protein BLAST database as blastp's -db does: `path`.pal (an
 * alias whose DBLIST names the volumes, relative to the alias file) or a
 * single volume `path`.pin + `path`.psq, NCBI format version 4 (what
 * makeblastdb 2.2.28 writes).  H-BLAST reads the same files only to count
 * each volume's sequences (ExtractVolumeSequences / ReadH_BLAST_volinfo,
 * NF/functions.cpp:573-760) and searches its own length-sorted .hDb copy
 * (Read_H_BLAST_GPU_DB, NF/functions.cpp:1058-1165, written by makeblastdb
 * -sort_volumes, NF/writedb_volume.cpp:255-513); these calls read the .psq
 * directly, so no .hDb and no re-sorted volumes are needed.  Every file is
 * checked (version, protein type, offset table against the .psq size,
 * residue total, longest sequence, letters 1..27, 0 bytes exactly between
 * sequences); a bad file gives HBG_ERR_INVALID and a message naming it.
 * Subjects are numbered across volumes in DBLIST order. */

/* Counts of a database without reading its sequences (host only). */
int hbg_blastdb_info(const char *path, int32_t *n_subjects, int64_t *n_residues,
                     int32_t *max_len, int32_t *n_volumes);

/* Read the sequences into host arrays in hbg_db_open's input form:
 * residues[n_residues] packed without separators, offsets[n_subjects + 1]. */
int hbg_blastdb_read(const char *path, uint8_t *residues, int64_t *offsets);

/* Open a resident database straight from the files: each volume's .psq is
 * streamed to the device through two pinned staging buffers (it already has
 * the resident layout: a 0 byte, then every sequence followed by a 0 byte).
 * The result is the same as hbg_db_open on the arrays hbg_blastdb_read
 * returns. */
int hbg_db_open_blastdb(const char *path, const hbg_gpu_options *opt, hbg_db **out);

/* ---- query batches -------------------------------------------------------- */

/* Build the neighbourhood lookup tables of a batch of protein queries on the
 * host (the work NCBI's BlastAaLookupTableNew/BlastAaLookupIndexQuery do
 * before H-BLAST reads the table at h_blast.cu:940-958, with cells sorted as
 * lut_sorting does at h_blast.cu:165-194).  Queries are packed into groups
 * that share one scan of the database; results are identical to searching
 * each query alone.  max_group_len 0 = library default; 1 packs one query
 * per group (the plain one-query-per-launch form). */
int hbg_batch_create(const hbg_query *queries, int32_t n_queries,
                     const hbg_word_params *params, int32_t max_group_len,
                     hbg_batch **out);

/* BLASTX batch: nucleotide queries (A=0 C=1 G=2 T=3, other = N) are
 * translated in six frames with the standard genetic code while the lookup
 * tables are built; contexts are frames +1,+2,+3,-1,-2,-3.  x_dropoff and
 * cutoff_score hold 6 values per query. */
int hbg_batch_create_blastx(const uint8_t *const *nt_sequences, const int32_t *nt_lengths,
                            int32_t n_queries, const int32_t *x_dropoff,
                            const int32_t *cutoff_score, const hbg_word_params *params,
                            int32_t max_group_len, hbg_batch **out);

/* SEG low-complexity masking (NCBI's -seg option; blastx masks its
 * translated query frames with the default "12 2.2 2.5" before the word
 * finder runs: NF/blastx_args.cpp:133-134, query set-up at
 * NF/blast_engine.c:367-433).  The algorithm is Wootton and Federhen's
 * published SEG: windows of `window` letters whose compositional complexity
 * (bits) is <= locut trigger a segment, which extends over windows <= hicut
 * and is trimmed to its least probable subsequence; masked letters become X
 * (hard masking). */
typedef struct hbg_seg_params {
    int32_t window;   /* 12 */
    int32_t pad;
    double locut;     /* 2.2 */
    double hicut;     /* 2.5 */
} hbg_seg_params;

int hbg_seg_default_params(hbg_seg_params *p);

/* Mask one NCBIstdaa protein sequence in place; *n_masked (may be NULL)
 * receives the number of letters set to X. */
int hbg_seg_mask(uint8_t *seq, int32_t len, const hbg_seg_params *p, int64_t *n_masked);

/* hbg_batch_create_blastx with each translated frame SEG-masked first (seg
 * NULL: no masking, the same as hbg_batch_create_blastx). */
int hbg_batch_create_blastx_masked(const uint8_t *const *nt_sequences, const int32_t *nt_lengths,
                                   int32_t n_queries, const int32_t *x_dropoff,
                                   const int32_t *cutoff_score, const hbg_word_params *params,
                                   const hbg_seg_params *seg, int32_t max_group_len, hbg_batch **out);

/* Use a lookup table the caller already has in NCBI's small-backbone layout
 * for one query (the table H_BLAST copies at h_blast.cu:953-958):
 * backbone[i] = {num_used, payload} cells of 8 bytes (payload = 3 uint16
 * offsets when num_used <= 3, else an int32 cursor into overflow),
 * backbone_size cells.  Cells are used in ascending order of offset, the order
 * lut_sorting produces. */
int hbg_batch_create_from_smallbone(const hbg_query *query, const hbg_word_params *params,
                                    const void *backbone, int32_t backbone_size,
                                    const uint16_t *overflow, int64_t overflow_size,
                                    hbg_batch **out);

/* Export group g's lookup table in CSR form: cells[w] .. cells[w+1] index
 * entries (group-local query offsets, ascending).  cells holds
 * HBG_NUM_CELLS + 1 values; *n_entries receives the entry count, and
 * HBG_ERR_CAPACITY is returned when entries_cap is smaller.  Also reports the
 * group's first query and each of its queries' start inside the group via
 * query_start (n_queries values, may be NULL).  The NCBI table H-BLAST reads
 * (h_blast.cu:940-958) carries the same cells. */
int hbg_batch_lookup_table(const hbg_batch *batch, int32_t g, uint32_t *cells,
                           uint16_t *entries, int64_t entries_cap, int64_t *n_entries,
                           int32_t *first_query, int32_t *n_queries, int32_t *query_start);

/* Choose how group g (all groups when g < 0) applies its hits: mode 0 =
 * chunk mode (32 offsets compacted at a time; best for sparse groups), 1 =
 * offset mode (one subject offset at a time, lanes over its cell; best for
 * dense groups).  The builder picks by expected hits per offset; results do
 * not depend on the choice.  Call before the batch's first search. */
int hbg_batch_set_mode(hbg_batch *batch, int32_t g, int32_t mode);

/* Work-unit and table placement knobs for tuning (results do not depend on
 * them).  tile_subjects: subjects per work unit a CTA takes (8..4096; 0 =
 * automatic: 128, fewer when the work is small); with the benchmark's length
 * law a tile of 128 subjects is about 46 KB of subject letters.
 * global_tables 1: every group keeps its diagonal table (32-bit cells) in
 * global memory instead of shared memory.  Call before the batch's first
 * search.  (H-BLAST fixes these at compile time: its per-thread diagonal
 * arrays are global, h_blast_kernel.cu:603-630.) */
int hbg_batch_tune(hbg_batch *batch, int32_t tile_subjects, int32_t global_tables);

/* Scheduling knobs for tuning (results do not depend on them).
 * warps_per_subject (1..8): how many query groups share each pass over a
 * block of subjects.  1 (default): the warps of a CTA take different subjects
 * of one group.  W > 1: a CTA searches W groups at a time, warp w serving
 * group w mod W, so W warps (up to the whole CTA) read each subject and its
 * letters come from the SM's caches after the first.  tile_bytes (0 =
 * automatic, else 1 KiB..16 MiB): subjects per work unit sized by letters,
 * about tile_bytes / mean subject length (hbg_batch_tune's tile_subjects,
 * when set, wins).  H-BLAST fixes the corresponding choices at compile time
 * or by query length: one thread per subject (kernel K-A,
 * h_blast_kernel.cu:504) or four (K-B, :21), chosen at
 * NF/functions.cpp:1400-1406.  Call before the batch's first search. */
int hbg_batch_schedule(hbg_batch *batch, int32_t warps_per_subject, int64_t tile_bytes);

int hbg_batch_destroy(hbg_batch *batch);
/* Sizes of a batch; device_bytes is what its upload copies host-to-device. */
int hbg_batch_info(const hbg_batch *batch, int32_t *n_queries, int32_t *n_groups,
                   int64_t *total_query_len, int64_t *lookup_entries, int64_t *device_bytes);

/* Estimate of the device bytes one search of batch against db needs beyond
 * the resident database (replaces H_BLAST_check_memory, h_blast.cu:1280-1349).
 * hsp_capacity 0 = default sizing. */
int hbg_mem_required(const hbg_db *db, const hbg_batch *batch, int64_t hsp_capacity,
                     int64_t *bytes);

/* ---- search --------------------------------------------------------------- */

/* Launch the word-hit stage of batch against db on stream (a cudaStream_t,
 * NULL = the legacy default stream) and return at once.  Replaces H_BLAST_pre
 * + H_BLAST (h_blast.cu:873-1157).  hsp_capacity bounds the HSP buffer (0 =
 * one slot per subject, at least 1 Mi; H-BLAST sizes it as AVG_HSPS_PER_SEQUENCE
 * slots per subject, NF/functions.cpp:1513-1516);
 * if a search finds more, hbg_result_wait relaunches it once with a buffer of
 * the exact size, so results never depend on the capacity.  *out == NULL
 * creates a result; a result from an earlier search of the same database may
 * be passed back (after it was waited for) to reuse its buffers, with the
 * same or another batch. */
int hbg_search(hbg_db *db, hbg_batch *batch, const hbg_gpu_options *opt,
               int64_t hsp_capacity, void *stream, hbg_result **out);

/* Wait for the search and collect it: HSPs in reference order -- by query,
 * then subject, then the order the CPU word finder creates them (subject
 * offset, then query offset) -- with per-query ranges, counters and subjects
 * passed (all computed on the device).  The ordered HSPs stay in device
 * memory until the result is relaunched or freed; hbg_result_hsps copies any
 * range of them to the host.  Replaces H_BLAST_get_data + memory_defrag
 * (h_blast.cu:1160-1252). */
int hbg_result_wait(hbg_result *res);

/* Wait for the search and read its HSP count and timings only; relaunches on
 * HSP-buffer overflow like hbg_result_wait. */
int hbg_result_sync(hbg_result *res);

/* Device time of the word-finder kernel and of the ordering pass, in ms,
 * and the number of kernels one search launches. */
int hbg_result_timing(const hbg_result *res, float *wordfinder_ms, float *ordering_ms,
                      int32_t *kernel_launches);

int hbg_result_counts(const hbg_result *res, int64_t *n_hsps, int32_t *n_queries);

/* Copy HSPs [first, first+count) of the ordered list from device memory to
 * `out` (host), on the search's stream. */
int hbg_result_hsps(const hbg_result *res, int64_t first, int64_t count, hbg_hsp *out);

/* Range of query q in the ordered list: HSPs [*first, *first + *count). */
int hbg_result_query_range(const hbg_result *res, int32_t q, int64_t *first, int64_t *count);

int hbg_result_stats(const hbg_result *res, int32_t q, hbg_query_stats *out);

/* Release device and host buffers (replaces H_BLAST_free_memory,
 * h_blast.cu:1254-1278). */
int hbg_result_free(hbg_result *res);

/* ---- serving ---------------------------------------------------------------- */

/* A request loop over a resident database: queries submitted from any thread
 * are admitted in arrival order while device memory for their lookup tables
 * and HSP buffers stays within memory_budget, packed into batches as they
 * arrive, and searched with up to max_inflight searches on the GPU at once
 * (continuous batching: a batch is formed whenever a slot frees).  Each
 * query's HSPs are the same as searching it alone.  Replaces the CPU/GPU load
 * balancer and the multi-process query split of H-BLAST
 * (NF/functions.cpp:51-140,1221-1827; scripts/H-BLASTM:212-305). */
typedef struct hbg_server hbg_server;

typedef struct hbg_server_options {
    int32_t max_inflight;        /* searches in flight (default 1: the next batch is chosen
                                    when one ends, from everything then waiting) */
    int32_t max_batch_queries;   /* queries per batch (default 512) */
    int64_t memory_budget;       /* device bytes for in-flight batches (default 32 GiB) */
    int32_t max_group_len;       /* 0 = library default */
    int32_t max_batch_letters;   /* query letters per batch, 0 = no cap (default 8192); a
                                    longer request runs alone */
    int32_t shortest_first_ms;   /* 0: admit in arrival order.  > 0 (default 2000): requests
                                    waiting at least this long go first, in arrival order,
                                    then the shortest waiting requests */
    int32_t seg_blastx;          /* 1: BLASTX requests' frames are SEG-masked with the
                                    default parameters (blastx's own default); default 0 */
} hbg_server_options;

int hbg_server_default_options(hbg_server_options *opt);
int hbg_server_create(hbg_db *db, const hbg_word_params *params, const hbg_gpu_options *opt,
                      const hbg_server_options *sopt, hbg_server **out);

/* Submit one protein query (any number of contexts); *ticket identifies it. */
int hbg_server_submit(hbg_server *s, const hbg_query *query, int64_t *ticket);

/* Submit one nucleotide query for BLASTX (six frames, per-frame x_dropoff and
 * cutoff_score, 6 values each). */
int hbg_server_submit_blastx(hbg_server *s, const uint8_t *nt, int32_t nt_len,
                             const int32_t *x_dropoff, const int32_t *cutoff_score,
                             int64_t *ticket);

/* Wait up to timeout_ms (< 0 = forever) for a request; HBG_ERR_STATE if it is
 * not done in time.  *n_hsps receives its HSP count. */
int hbg_server_wait(hbg_server *s, int64_t ticket, int32_t timeout_ms, int64_t *n_hsps);

/* Copy a finished request's HSPs (query field 0; reference order) and stats,
 * its latency from submission to completion, then forget the request. */
int hbg_server_take(hbg_server *s, int64_t ticket, hbg_hsp *out, int64_t cap,
                    hbg_query_stats *stats, double *latency_ms);

/* Totals since creation: batches launched, queries completed, largest batch. */
int hbg_server_counters(const hbg_server *s, int64_t *batches, int64_t *queries,
                        int64_t *largest_batch);

/* Requests put back in the queue since creation because their batch did not
 * fit (the budget, the device's free memory, or an allocation that failed);
 * each was searched again later.  No counterpart in the reference: H-BLAST
 * checks memory before it launches (H_BLAST_check_memory, h_blast.cu:1280-1349)
 * and sends a search that does not fit to the CPU (NF/functions.cpp:1518-1530). */
int hbg_server_requeued(const hbg_server *s, int64_t *requeued);

/* Finish every admitted request, then stop. */
int hbg_server_destroy(hbg_server *s);

/* ---- search without allocation -------------------------------------------- */

/* Size of the device array that hbg_search_static uses for its scratch.  The
 * array is a file-scope __device__ variable: every GPU that loads the library
 * holds it until the process exits. */
#define HBG_STATIC_SCRATCH_BYTES 262144

/* Run the word finder without allocating anything.  No counterpart in the
 * reference: H-BLAST allocates its buffers on every call.
 *
 * For callers that cannot call cudaMalloc at search time: allocator-free
 * real-time services (cudaMalloc and cudaFree may synchronise the device and
 * take unbounded time), and hosts that give the library a fixed memory budget
 * at start-up and account for every device byte after that.  It calls no
 * cudaMalloc, cudaFree or allocating library routine; its scratch (a tile
 * counter and per-query / per-group counters, 256 + 8 x (2 x queries + groups)
 * bytes) lives in a static device array of HBG_STATIC_SCRATCH_BYTES.
 *
 * Inputs: a resident database and a batch that is already resident on the
 * same device (search it once with hbg_search during set-up).  Outputs, in
 * caller-owned device memory: d_hsps (hsp_cap records, in no particular order;
 * hbg_search returns the same records in reference order) and d_counts
 * (1 + 2 x queries values: the number of HSPs found -- which may exceed
 * hsp_cap, in which case only hsp_cap were written -- then the extensions
 * tried per query, then the extensions kept per query).  Work is queued on
 * stream; the call returns at once.
 *
 * Limits: batches whose scratch would exceed HBG_STATIC_SCRATCH_BYTES, groups
 * longer than 2008 letters and subjects longer than 32767 - window (both need
 * global diagonal tables) are rejected with HBG_ERR_TOO_LONG.
 *
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * Every call uses the same array and clears it first, so calls whose work
 * overlaps on the GPU (other streams, other threads) race: serialise them. */
int hbg_search_static(const hbg_db *db, const hbg_batch *batch, const hbg_gpu_options *opt,
                      hbg_hsp *d_hsps, int64_t hsp_cap, unsigned long long *d_counts,
                      void *stream);

/* ---- testing --------------------------------------------------------------- */

/* Make the library's next `count` device allocations fail as if the device
 * were out of memory (HBG_ERR_NOMEM from the call that needed them); 0 stops
 * it.  For tests of the out-of-memory paths without exhausting a shared GPU.
 * No counterpart in the reference. */
int hbg_debug_fail_allocations(int32_t count);

/* ---- one-call helper ------------------------------------------------------ */

/* Host-to-host search: upload nothing that is already resident, run, wait and
 * copy out.  out may be NULL to only count.  Returns HBG_ERR_CAPACITY with
 * *n_hsps set when out_cap is too small. */
int hbg_search_sync(hbg_db *db, hbg_batch *batch, const hbg_gpu_options *opt,
                    hbg_hsp *out, int64_t out_cap, int64_t *n_hsps,
                    hbg_query_stats *stats, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* HBLAST_GPU_H */
