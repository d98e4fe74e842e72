/*
 * swift_gb300.h — C ABI of the GB300 (sm_103a) implementation of the SWIFT
 * two-phase short-read aligner hot path: SSAHA seeding (Phase 1) and
 * Smith-Waterman with traceback (Phase 2), then best-per-read selection and
 * the default text record.
 *
 * All functions return 0 on success and a negative SWIFT_E_* code on
 * failure; they never exit the process.  swift_last_error() gives a message
 * for the last failure on a context.  A context is used by one host thread
 * at a time.
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   swift_index_build  <- lookupTable5Create           src/lookupTable5.h:28
 *                         + refMapCreate               src/refMap.h (src/refMap.cu:59)
 *   swift_seed         <- searchQueries3               src/search.h:33
 *                         (lookupTable5MapQry          src/lookupTable5.h:42,
 *                          mapHits6GetBestHits         src/mapHits6.h:34)
 *   swift_sw_batch     <- alignSequences               src/align.cu:2904-2921
 *                         (kernel smithWaterman        src/smithWaterman.h)
 *   swift_align        <- searchQueries3 + alignQueries3 (src/align.h:33)
 *                         with chooseBestAlignment and printOutput
 *   swift_align_files  <- the swift CLI, src/main.cu:42-223
 */
#ifndef SWIFT_GB300_H_
#define SWIFT_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWIFT_OK 0
#define SWIFT_E_ARG (-1)     /* invalid argument                          */
#define SWIFT_E_INPUT (-2)   /* malformed or unsupported FASTA input      */
#define SWIFT_E_CUDA (-3)    /* CUDA runtime error                        */
#define SWIFT_E_NOMEM (-4)   /* device or host allocation failed          */
#define SWIFT_E_LIMIT (-5)   /* size beyond a documented maximum          */
#define SWIFT_E_DEVICE (-6)  /* a kernel reported an internal error       */
#define SWIFT_E_CANCELLED (-7) /* serving: the request was cancelled       */

typedef struct swift_ctx swift_ctx;
typedef struct swift_index swift_index;

/* Parameters of one alignment run; defaults from swift_params_default() are
 * the reference's (src/common.h:29-75, src/main.cu:52-62). */
typedef struct {
  int32_t seed_len;      /* -l  (12)                                       */
  int32_t ignore_thres;  /* -t  (1000)                                     */
  int32_t max_hits;      /* hits per read strand (3)                       */
  int32_t match;         /* -m  (2)                                        */
  int32_t mismatch;      /* -M  (-1)                                       */
  int32_t gap_open;      /* -O  (-10)                                      */
  int32_t gap_ext;       /* -E  (-1)                                       */
  int32_t qry_len;       /* -s; <= 0: length of the first read             */
  int64_t device_mem;    /* bytes used to size Phase-2 batches the way the
                            reference does from its device; 0: this GPU's  */
  int32_t out_format;    /* -f: 1 SAM records of every alignment
                            (printOutputSam, src/output.cu:98-130); any
                            other value the default record of the best one
                            per read (printOutput, src/output.cu:154-201)  */
  int32_t seeder;        /* Phase 1: 0 SSAHA seeding (searchQueries3,
                            src/search.cu:275-382); 1 lt13 seed-and-extend
                            (search2Queries, src/search2.cu:48-259), the
                            GPU default of the reference CLI               */
  int32_t max_read_len;  /* longest read taken, up to 300; 0: the
                            reference's 199 (its query buffer,
                            src/common.h:40).  Longer reads are aligned the
                            same way (query = first qry_len bases, 300-base
                            windows); SSAHA seeding only                   */
} swift_params;

/* One Phase-1 record (one line of the reference's match file,
 * src/search.cu:2230-2240). */
typedef struct {
  int32_t read;      /* read index in file order                          */
  int32_t strand;    /* 0 forward, 1 reverse complement                   */
  int32_t ref_idx;   /* reference sequence index                          */
  int32_t shift;     /* reference position - query offset                 */
  int32_t ref_pos;   /* first reference position of the cluster           */
} swift_match;

/* Timings of the last swift_align call, in milliseconds of device time
 * (CUDA events on the context stream). */
typedef struct {
  double seed_ms, pairs_ms, sw_ms, select_ms, traceback_ms, format_ms, total_ms;
  int64_t reads, records, printed, cells, out_bytes;
  int64_t seed_overflow_strands, sw_generic_pairs;
  int64_t launches;   /* kernels this library launched for the call       */
  double host_parse_ms, h2d_ms, d2h_ms;  /* swift_align only: host side    */
  int64_t traced_pairs;  /* pairs that went through the traceback pass       */
  int64_t bound_pruned;  /* pairs whose score bound ruled them out, so they
                            needed no exact score                            */
  int64_t retraced_pairs;/* printed pairs traced after selection (bounded
                            selection: the read's candidate was not best)    */
  double first_pass_ms;  /* the packed path's first kernel alone: the LCS
                            bound (default) or the exact score pass; 0 with
                            SAM output (every pair traced)                   */
  int64_t first_pass_cells; /* DP cells that kernel covered               */
  int64_t first_pass_kind;  /* 1 exact score, 3 LCS bound                 */
  double trace_ms;       /* trace-pass launches: the candidates (default;
                            they stop early on suffix LCS values) or every
                            packed pair over whole windows (SAM)            */
  int64_t trace_cells;   /* DP cells those launches computed (the columns
                            every lane of a warp finished)                  */
  int64_t lcs_kept;      /* pairs the LCS bound could not rule out (they get
                            the exact score pass)                            */
  double seed_kernel_ms; /* SSAHA seeding's warp kernels alone (CUDA events) */
  int64_t seed_model_bytes; /* their bytes under the seeding roofline's sector
                            model: per read strand ceil(L/4) + 32 per k-mer
                            lookup + 32 * ceil(5 n / 32) per occupied bucket
                            of n postings + 12 per hit written             */
  int64_t sw_cells_computed; /* DP cells the Smith-Waterman kernels computed:
                            trace and exact score passes (up to their early
                            stop), generic kernel; the LCS bound's
                            bit-parallel columns not counted                */
} swift_stats;

void swift_params_default(swift_params *p);

/* device: CUDA ordinal; stream: a cudaStream_t to run on, or NULL to make
 * one owned by the context. */
int swift_ctx_create(int device, void *stream, swift_ctx **out);
int swift_ctx_destroy(swift_ctx *ctx);
const char *swift_last_error(const swift_ctx *ctx);
/* Device facts the pipeline depends on: total device memory (it sizes the
 * Phase-2 batches, as in the reference) and the SM count. */
int swift_ctx_info(const swift_ctx *ctx, int64_t *total_mem, int32_t *sm_count);
/* Phase-2 kernel choice; all give identical output.
 *   0 (default) bounded selection: an upper bound of every packed-path
 *     pair's score, the exact score and traceback of each read's most
 *     promising pair, exact scores only for the pairs the bound cannot rule
 *     out, then traceback of any printed pair not traced yet;
 *   1 the generic kernel for every pair;
 *   2 the exact score of every packed-path pair, then traceback of the
 *     printed ones. */
int swift_ctx_set_sw_path(swift_ctx *ctx, int32_t path);

/* Builds the device-resident reference (file bytes, 2-bit codes) and SSAHA
 * index from a reference FASTA held in host memory. */
int swift_index_build(swift_ctx *ctx, const char *ref_fasta, size_t len,
                      int32_t seed_len, int32_t ignore_thres,
                      swift_index **out);
int swift_index_destroy(swift_index *idx);

/* Index persistence for warm starts.  swift_index_save writes the index to
 * one binary file: what lookupTable13Create2 reads back in the reference
 * (bucket starts and counts, composite values, refPosHashMap;
 * src/lookupTable13.cu:257-322, there three text files) together with the
 * reference bytes, sequence records, SSAHA postings, bucket directory and
 * packed sequence, so swift_index_load rebuilds the index on the context's
 * device without parsing or hashing the reference again.  The lt13 tables
 * are included when they were built.  Loading refuses (SWIFT_E_INPUT) a
 * file whose magic, version, section sizes or checksum do not match;
 * SWIFT_E_ARG when the file cannot be opened. */
int swift_index_save(swift_ctx *ctx, const swift_index *idx, const char *path);
int swift_index_load(swift_ctx *ctx, const char *path, swift_index **out);
/* The seed length and ignore threshold an index was built with. */
int swift_index_params(swift_ctx *ctx, const swift_index *idx, int32_t *seed_len,
                       int32_t *ignore_thres);
/* Index contents in the reference layout (src/lookupTable5.cu:199-231):
 * lookup[h] is the 1-based start of bucket h or 0; ref_idx/ref_pos have
 * total+1 entries with slot 0 = -1.  Any pointer may be NULL. */
int swift_index_info(swift_ctx *ctx, const swift_index *idx, int32_t *n_refs,
                     int64_t *total_tuples, int64_t *n_buckets);
int swift_index_export(swift_ctx *ctx, const swift_index *idx, int32_t *lookup,
                       int32_t *repeats, int8_t *ref_idx, int32_t *ref_pos);

/* Phase 1: SSAHA seeding of every read (and its reverse complement) of a
 * reads FASTA in host memory.  Writes up to cap records in match-file order
 * and the total count to *n (records beyond cap are counted, not written). */
int swift_seed(swift_ctx *ctx, const swift_index *idx, const char *reads_fasta,
               size_t len, int32_t max_hits, swift_match *out, int64_t cap,
               int64_t *n);

/* Phase 1 of the reference CLI's GPU default: lt13 seed-and-extend
 * (replaces search2Queries, src/search2.cu:48-259, with
 * lookupTable13Create and lookupTable13MapQry2_gpu,
 * src/lookupTable13.cu:64-242,646-868).  Up to 3 records per read strand,
 * every read once in file order (forward, then reverse complement), shift 0.
 * The index's extra tables are built on first use.  SWIFT_E_LIMIT for more
 * than 64 reference sequences, an ignore threshold above 1176 or a
 * sequence of 2^25 - 64 tuples or more.  Output as swift_seed. */
int swift_seed_lt13(swift_ctx *ctx, const swift_index *idx, const char *reads_fasta,
                    size_t len, swift_match *out, int64_t cap, int64_t *n);

/* Phase 2 on explicit pairs, the alignSequences contract: n pairs, query i
 * at qry + i*(Q+1) (Q bytes used), window i at ref + i*(R+1) (R bytes
 * used), outputs per pair: score, start, end, length and the reversed
 * consensus strings at qcons/rcons + i*(Q+R+2).  Pointers may be host or
 * device memory (device memory of the context's device; SWIFT_E_ARG for
 * another device's).  1 <= Q <= 320, 1 <= R <= 1024, every shape in that
 * range.  The scores are float, as alignSequences takes them; they must be
 * whole numbers within +-32767 (the reference CLI reads them with atoi),
 * SWIFT_E_ARG otherwise. */
int swift_sw_batch(swift_ctx *ctx, const char *qry, const char *ref, int32_t Q,
                   int32_t R, int64_t n_pairs, float match, float mismatch,
                   float gap_open, float gap_ext, float *score,
                   int32_t *start, int32_t *end, int32_t *len, char *qcons,
                   char *rcons);

/* swift_sw_batch for device buffers that allocates no memory: no
 * cudaMalloc, no pool allocation, no library routine that allocates.  For
 * callers that cannot allocate at call time, such as a serving loop that has
 * reserved the rest of device memory for its own pools up front and must not
 * have a request fail or stall in the allocator.  No counterpart in the
 * reference (its alignSequences works on buffers alignQueries3 allocates for
 * every batch).
 *   - every pointer must be device memory of the context's device
 *     (SWIFT_E_ARG otherwise); scores as for swift_sw_batch;
 *   - n_pairs <= SWIFT_SW_NOALLOC_MAX_PAIRS (SWIFT_E_LIMIT otherwise): the
 *     per-pair intermediate results live in a fixed array in the library's
 *     module memory (16 bytes per pair, 1 MiB);
 *   - the call only enqueues work on the context's stream and returns;
 *     outputs are ready when that stream is synchronised;
 *   - the first call on a device looks up the array's address (a runtime
 *     call, no allocation): make it once before any stream capture;
 *   - all callers on a device share the array, so calls that can run at the
 *     same time (other streams or contexts on that device) race; calls on one
 *     stream are ordered and safe. */
#define SWIFT_SW_NOALLOC_MAX_PAIRS 65536
int swift_sw_batch_noalloc(swift_ctx *ctx, const char *qry, const char *ref, int32_t Q,
                           int32_t R, int64_t n_pairs, float match, float mismatch,
                           float gap_open, float gap_ext, float *score,
                           int32_t *start, int32_t *end, int32_t *len, char *qcons,
                           char *rcons);

/* Statistics of one swift_sw_pairs call. */
typedef struct {
  double ms;               /* device time of the call (CUDA events)           */
  int64_t pairs, cells;    /* cells = sum over pairs of q_len * r_len         */
  int64_t segments;        /* groups of one shape, one launch set each        */
  int64_t generic_pairs;   /* pairs on the int32 kernel                       */
  int64_t launches;        /* kernels this library launched                   */
  /* the packed shape (lanes, rows per lane) each query class ran with
   * (classes: queries up to 32, 64, 104, 128, 208, 256, 320 bases; 0: the
   * class had no packed pairs), the last window bin's; and the device time
   * this call spent timing candidate shapes                                 */
  int32_t shape_lanes[8], shape_rows[8];
  double tune_ms;
} swift_pairs_stats;

/* Packed-shape choice of swift_sw_pairs: 1 (default) times the candidate
 * (lanes, rows per lane) shapes of each row class and window bin (with at
 * least 1,024 pairs) on a sample of the call's pairs the first time the
 * context meets them, and
 * keeps the fastest for the context; 0 uses the fixed default shapes;
 * k >= 2 runs the (k - 2)-th candidate of every class (the default when it
 * has fewer).  All give identical results. */
int swift_ctx_set_tuning(swift_ctx *ctx, int32_t mode);

/* Phase 2 on explicit pairs of varying lengths: the batched form of
 * alignSequences (src/align.cu:2904-2921, whose pairs all share one query
 * and window length).  Pair i aligns qry[q_off[i], q_off[i] + q_len[i])
 * against ref[r_off[i], r_off[i] + r_len[i]) with the reference kernel's
 * recurrence, tie rules and traceback.  Outputs per pair: score, start,
 * end, length and, when qcons/rcons are not NULL, the reversed consensus
 * strings at qcons/rcons + i * cons_stride (cons_stride >= q_len + r_len + 2
 * for every pair, a multiple of 4).  1 <= q_len <= 4096, 1 <= r_len <= 8192;
 * pairs beyond 256 x 1024 (or q_len > 128 with r_len > 768) run on the long
 * kernel, one CTA each, which needs negative mismatch and gap penalties.
 * Inputs all host or all device memory; outputs likewise.
 *   mode 0 (batched): pairs sorted on the device by row class (q_len rounded
 *          up to 8 rows up to 128, 16 up to 256) and r_len, one set of
 *          launches per class: packed 16-bit passes for pairs of ACGT bytes,
 *          the int32 kernel for the rest;
 *   mode 1 (plain): every pair padded to the largest shape, one launch of
 *          the int32 kernel, as the reference runs a batch (pairs up to
 *          256 x 1024 only).  Padding leaves
 *          results unchanged when mismatch and both gap penalties are
 *          negative (otherwise mode 1 is refused, SWIFT_E_ARG); bytes 0x00
 *          and 0x01 are the padding and are refused in pairs (SWIFT_E_INPUT). */
int swift_sw_pairs(swift_ctx *ctx, const char *qry, const int64_t *q_off, const int32_t *q_len,
                   const char *ref, const int64_t *r_off, const int32_t *r_len, int64_t n_pairs,
                   int32_t match, int32_t mismatch, int32_t gap_open, int32_t gap_ext,
                   int32_t *score, int32_t *start, int32_t *end, int32_t *len, char *qcons,
                   char *rcons, int64_t cons_stride, int32_t mode, swift_pairs_stats *stats);

/* The whole pipeline on a reads FASTA in host memory: seeding, windows,
 * Smith-Waterman, best alignment per read, default records.  *out receives
 * a buffer owned by the library (free with swift_free). */
int swift_align(swift_ctx *ctx, const swift_index *idx, const char *reads_fasta,
                size_t len, const swift_params *p, char **out, size_t *out_len,
                swift_stats *stats);

/* swift_align writing the text into a caller buffer (for example pinned
 * host memory, for the fastest copy).  If cap is too small nothing is
 * copied, *out_len receives the size needed and SWIFT_E_LIMIT is returned. */
int swift_align_into(swift_ctx *ctx, const swift_index *idx, const char *reads_fasta,
                     size_t len, const swift_params *p, char *out, size_t cap,
                     size_t *out_len, swift_stats *stats);

/* Resident form for serving and benchmarking: reads parsed and kept on the
 * device; the output text stays on the device until fetched. */
typedef struct swift_reads swift_reads;
int swift_reads_upload(swift_ctx *ctx, const char *reads_fasta, size_t len,
                       swift_reads **out);
int swift_reads_destroy(swift_reads *r);
int swift_align_resident(swift_ctx *ctx, const swift_index *idx,
                         const swift_reads *reads, const swift_params *p,
                         size_t *out_len, swift_stats *stats);
/* Copies the text of the last swift_align_resident call into dst (at most
 * cap bytes). */
int swift_fetch_output(swift_ctx *ctx, char *dst, size_t cap);

/* Paired-end alignment (-q / -q2), the GPU branch of src/main.cu:172-212:
 * replaces searchQueries_paired2 (src/search.cu:2084-2200, lookupTable2
 * seeding of both mates and their reverse complements, 3 hits each) and
 * alignQueries_paired2 (src/align.cu:1879-2110: windows of 3Q bases from
 * getSeq, chooseBestAlignment_paired3 keeping the best mate pair whose
 * fragment length lies in [min_frag, max_frag] on one reference,
 * printOutput_paired2 records; out_format 1: SAM records of every hit).
 * The reference's MIN/MAX_FRAG_SIZE are 99 and 600 (src/common.h:66-68).
 * Both reads buffers hold the same number of reads, every read at least
 * the query length (first read of reads1, or qry_len), names ending in 1
 * or 2 (SWIFT_E_INPUT otherwise).  The lookupTable2 positions are built on
 * the index at first use (with the reference's fixed 1000-repeat threshold).
 * The output is malloc'ed (swift_free).  Of the stats, seed_ms (both
 * files), pairs_ms, sw_ms, select_ms (mate pairing), format_ms and
 * total_ms, reads (both mates), records, printed and cells are set. */
int swift_align_paired(swift_ctx *ctx, const swift_index *idx, const char *reads1,
                       size_t len1, const char *reads2, size_t len2, const swift_params *p,
                       uint32_t min_frag, uint32_t max_frag, char **out, size_t *out_len,
                       swift_stats *stats);
/* swift_align_paired into the caller's buffer out (cap bytes; pinned host
 * memory lets the copies overlap the writing of the text): *out_len is the
 * text length, SWIFT_E_LIMIT when it exceeds cap. */
int swift_align_paired_into(swift_ctx *ctx, const swift_index *idx, const char *reads1,
                            size_t len1, const char *reads2, size_t len2,
                            const swift_params *p, uint32_t min_frag, uint32_t max_frag,
                            char *out, size_t cap, size_t *out_len, swift_stats *stats);

/* File-to-file pipeline, the CLI: reads the two FASTA files and writes the
 * default output records to out_path. */
int swift_align_files(swift_ctx *ctx, const char *qry_path, const char *ref_path,
                      const char *out_path, const swift_params *p);

/* Serving loop.  No counterpart in the reference (a one-shot CLI).  The
 * index stays resident while requests, one reads FASTA each, queue up.
 * Continuous batching: each of `workers` pipelines (a context and stream
 * each, on the given device) takes every queued request of one query-length
 * class, oldest first, and runs them as one merged wave (one seeding
 * launch over all their reads, shared Smith-Waterman launches over all
 * their pairs); requests that arrive meanwhile join the next wave.  A wave
 * starts when its estimated device memory fits within mem_budget bytes
 * beside the waves in flight (0: half of the free memory at creation); a
 * request larger than the budget runs alone.  A request is parsed and
 * checked by the worker that takes it (reads up to p->max_read_len bases);
 * one that fails finishes at once with swift_align's error; each result is
 * byte-identical to swift_align on that request alone. */
typedef struct swift_server swift_server;
typedef struct {
  double queue_ms;   /* submit to the start of its wave (host clock)          */
  double run_ms;     /* start to result                                       */
  double total_ms;   /* submit to result: the request's latency               */
  double device_ms;  /* its wave's device time (CUDA events)                  */
  int64_t reads, out_bytes;
  int64_t wave_requests;  /* requests of its wave                             */
  int64_t wave_reads;     /* reads of its wave                                */
  double parse_ms;        /* host time parsing and checking its reads         */
  double wave_ms;         /* host time of its wave's pipeline call, from the
                             upload of the reads to the text on the host      */
} swift_request_stats;
int swift_server_create(int device, const swift_index *idx, const swift_params *p,
                        int32_t workers, int64_t mem_budget, swift_server **out);
/* Queues a copy of the reads; *ticket identifies the request. */
int swift_server_submit(swift_server *s, const char *reads_fasta, size_t len, int64_t *ticket);
/* Non-blocking state of a request: SWIFT_SERVE_QUEUED, _RUNNING, _DONE (its
 * result waits for swift_server_wait) or _CANCELLED; SWIFT_E_ARG for an
 * unknown ticket. */
#define SWIFT_SERVE_QUEUED 0
#define SWIFT_SERVE_RUNNING 1
#define SWIFT_SERVE_DONE 2
#define SWIFT_SERVE_CANCELLED 3
int swift_server_poll(swift_server *s, int64_t ticket, int32_t *state);
/* Cancels a request that has not started: it leaves the queue and
 * swift_server_wait returns SWIFT_E_CANCELLED for it.  SWIFT_E_LIMIT once it
 * runs or is done (its result stands), SWIFT_E_ARG for an unknown ticket. */
int swift_server_cancel(swift_server *s, int64_t ticket);
/* Blocks until the request is done and returns its status; *out (free with
 * swift_free) holds the records; err receives the message of a failure.
 * The ticket is released. */
int swift_server_wait(swift_server *s, int64_t ticket, char **out, size_t *out_len,
                      swift_request_stats *stats, char *err, size_t err_cap);
/* Runs the queued requests to completion, then frees everything. */
int swift_server_destroy(swift_server *s);

/* Measured peak cell-update rate of the packed-int16 max-plus instruction
 * on this GPU (2 cells per __vimax3_s16x2_relu lane instruction): the
 * denominator of the Smith-Waterman roofline. */
int swift_peak_dpx(swift_ctx *ctx, double *cells_per_s);

void swift_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
