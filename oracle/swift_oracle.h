/*
 * swift_oracle.h — CPU restatement of the reference aligner's hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path
 * is compared against (and, multithreaded, the timed CPU baseline of the
 * benchmark).  Nothing in the product links, loads or calls it.
 *
 * Every function restates the behaviour of a reference function; the
 * citation next to each declaration names it (paths are relative to the
 * reference project root).
 */
#ifndef SWIFT_ORACLE_H_
#define SWIFT_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Direction codes of one DP cell (the reference keeps the same information
 * in three bit planes topLeft/top/left, src/smithWaterman.cu:575-611). */
enum { SO_NONE = 0, SO_DIAG = 1, SO_UP = 2, SO_LEFT = 3 };

typedef struct {
  int seed_len;      /* -l, default 12 (src/common.h:29)                     */
  int ignore_thres;  /* -t, default 1000 (src/common.h:75, src/main.cu:61)   */
  int max_hits;      /* 3 (MAX_NUM_HITS_SINGLE_END, src/common.h:59)         */
  int match, mismatch, gap_open, gap_ext; /* 2 -1 -10 -1 (src/common.h:45-48) */
  int qry_len;       /* -s; <= 0 means "length of the first read"            */
  long long device_mem;/* device bytes that size the Phase-2 batches the way
                        getNumQueriesPerIteration does; <= 0: one batch */
  int threads;       /* worker threads (>= 1)                                */
  int out_format;    /* -f: 1 SAM (printOutputSam, src/output.cu:98-130,
                        every record); other values printOutput           */
  int seeder;        /* 0 SSAHA (searchQueries3); 1 lt13 seed-and-extend
                        (search2Queries, the GPU default of src/main.cu)   */
  int max_read_len;  /* longest read taken, up to 300; <= 0: the reference's
                        199 (MAX_QRY_SEQ_LENGTH - 1, src/common.h:40)       */
} so_params;

typedef struct {
  int32_t slot_read;   /* index into the query-record stream              */
  int32_t strand;      /* 0 forward, 1 reverse complement                 */
  int32_t ref_idx;
  int32_t shift;
  int32_t ref_pos;
} so_match;

typedef struct {
  float score;
  int32_t start, end, len, cell_max;
} so_aln;

/* getHash (src/preprocess.cu:70-91) with the code table of
 * preprocessCreate (src/preprocess.cu:30-48). */
int so_hash(const char *s, int k);

/* ---- SSAHA index (lookupTable5Create, src/lookupTable5.cu:101-252) ---- */
typedef struct so_index so_index;
int so_index_build(const char *fasta, size_t len, int k, int thres,
                   so_index **out, char *err, size_t errlen);
void so_index_free(so_index *);
int so_index_num_buckets(const so_index *);
int so_index_total(const so_index *);             /* numTotalTuples        */
int so_index_start(const so_index *, int h);      /* lookupTable[h]        */
int so_index_repeats(const so_index *, int h);    /* numRepeatsPerTuple[h] */
int so_index_actual(const so_index *, int h);     /* numActualRepeats[h]   */
/* refIdx[] and refPos[] of the reference layout: total+1 entries, slot 0 is
 * -1, each bucket in reverse order of occurrence. */
void so_index_postings(const so_index *, int8_t *ref_idx, int32_t *ref_pos);
/* lookupTable[] and numRepeatsPerTuple[] of every bucket at once. */
void so_index_buckets(const so_index *, int32_t *lookup, int32_t *repeats);
int so_index_num_refs(const so_index *);

/* mapHits6GetBestHits (src/mapHits6.cu:40-70) with the deterministic tie
 * rule: the first min(max_hits, n_biggest) biggest clusters in sort order. */
int so_best_hits(int max_hits, const int8_t *ref_idx, const int32_t *shift,
                 const int32_t *ref_pos, int n, int8_t *o_ri, int32_t *o_sh,
                 int32_t *o_rp);

/* lookupTable5MapQry (src/lookupTable5.cu:557-603) on an explicit strand
 * sequence of length len. */
int so_map_query(const so_index *, const char *seq, int len, int max_hits,
                 int8_t *o_ri, int32_t *o_sh, int32_t *o_rp);

/* qryGetReverseComplement (src/query.cu:265-282). */
void so_revcomp(const char *seq, int len, char *out);

/* GPU Smith-Waterman kernel semantics (src/smithWaterman.cu:360-395,
 * 510-645, 911-1026).  q has Q bytes, r has R bytes (NUL padded).  qcons and
 * rcons receive the reversed consensus strings (Q+R+2 bytes each).  dirs, if
 * not NULL, receives (Q+1)*(R+1) direction codes. */
void so_sw(const char *q, int Q, const char *r, int R, int m, int x, int o,
           int e, so_aln *out, char *qcons, char *rcons, uint8_t *dirs);
/* so_sw over n pairs on `threads` host threads (the CPU baseline). */
int so_sw_batch(const char *q, int Q, int qs, const char *r, int R, int rs, long n, int m,
                int x, int o, int e, int threads, so_aln *out);

/* The whole spec pipeline: SSAHA seeding (searchQueries3,
 * src/search.cu:275-382) -> GPU-kernel Smith-Waterman over 300-base windows
 * (alignQueries3, src/align.cu:574-808) -> chooseBestAlignment
 * (src/align.cu:844-905) -> printOutput (src/output.cu:154-201).
 * *out is malloc'ed; free with so_free. */
int so_align(const char *ref, size_t ref_len, const char *reads,
             size_t reads_len, const so_params *p, char **out,
             size_t *out_len, char *err, size_t errlen);

/* The same pipeline with the reference parsed and indexed once (the index
 * build is then outside the timed alignment). */
typedef struct so_session so_session;
int so_session_create(const char *ref, size_t ref_len, const so_params *p,
                      so_session **out, char *err, size_t errlen);
int so_session_align(so_session *s, const char *reads, size_t reads_len,
                     char **out, size_t *out_len, char *err, size_t errlen);
void so_session_free(so_session *s);

/* Phase 1 only: the match-file records in file order (including the
 * trailing-batch repeats of searchQueries3).  *out is malloc'ed. */
/* lt13 seed-and-extend mapping of one query strand (lookupTable13MapQry2_gpu,
 * src/lookupTable13.cu:646-868) on the index built from fasta with seed
 * length k and threshold thres: up to 3 (ref_idx, ref_pos) hits in the
 * printed order.  Returns the count, or < 0 with err set. */
int so_lt13_map(const char *fasta, size_t len, int k, int thres, const char *seq,
                int seq_len, int32_t *ri, int32_t *rp, char *err, size_t errlen);

int so_phase1(const char *ref, size_t ref_len, const char *reads,
              size_t reads_len, const so_params *p, so_match **out,
              int *n_out, char *err, size_t errlen);

void so_free(void *);

/* Paired-end pipeline (-q2, src/main.cu:172-212): Phase-1 records as 7
 * ints each (id, rev, mate, ref_idx, shift, offset, read index), and the
 * whole output (out_format 1: SAM).  Reads files must hold the same number
 * of reads. */
int so_phase1_paired(const char *ref, size_t ref_len, const char *reads1, size_t len1,
                     const char *reads2, size_t len2, const so_params *p, int32_t **out,
                     long *n_out, char *err, size_t errlen);
int so_align_paired(const char *ref, size_t ref_len, const char *reads1, size_t len1,
                    const char *reads2, size_t len2, const so_params *p, unsigned min_frag,
                    unsigned max_frag, char **out, size_t *out_len, char *err, size_t errlen);

#ifdef __cplusplus
}
#endif
#endif
