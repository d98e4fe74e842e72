/*
 * swift_oracle.c — CPU restatement of the reference aligner's hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
 * baseline ("port") of the benchmark.  The product never links or calls it.
 *
 * Pipeline restated (paths relative to the reference project root):
 *   reference FASTA parse ............ refMapCreate      src/refMap.cu:59-117
 *   k-mer code + hash ................ getHash           src/preprocess.cu:30-48,70-91
 *   SSAHA index ...................... lookupTable5Create src/lookupTable5.cu:101-252
 *   query stream ..................... qryGetNext2       src/query.cu:174-213
 *   reverse complement ............... qryGetReverseComplement src/query.cu:265-282
 *   hit emission ..................... lookupTable5MapQry src/lookupTable5.cu:557-603
 *   best clusters .................... mapHits6GetBestHits src/mapHits6.cu:40-318
 *   Phase-1 driver ................... searchQueries3    src/search.cu:275-382
 *   Phase-2 driver ................... alignQueries3     src/align.cu:574-808
 *   window fetch ..................... refMapGetOffsets  src/refMap.cu:148-155
 *                                      getRefSeq2        src/input.cu:348-403
 *   query fetch ...................... getSeq2           src/input.cu:216-258
 *   batch sizing ..................... getNumQueriesPerIteration src/align.cu:2767-2793
 *   Smith-Waterman (GPU semantics) ... smithWaterman     src/smithWaterman.cu:360-395,510-645,911-1026
 *   best per read .................... chooseBestAlignment src/align.cu:844-905
 *   record writer .................... printOutput       src/output.cu:154-201
 *
 * Tie rules that are random in the reference are pinned: mapHits6 keeps the
 * first biggest clusters in sort order (src/mapHits6.cu:152-155) and
 * chooseBestAlignment keeps the first maximum (src/align.cu:891).
 */
#include "swift_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define SO_LINE_MAX 100000  /* MAX_LINE_LENGTH, src/common.h:41       */
#define SO_NAME_MAX 50      /* MAX_QRY_NAME_LENGTH, src/common.h:37    */
#define SO_QSEQ_MAX 200     /* MAX_QRY_SEQ_LENGTH, src/common.h:40     */
#define SO_READ_LONGEST 300 /* longest read with so_params.max_read_len */
#define SO_QMAX 320         /* longest query the restatement takes      */
#define SO_WIN 300          /* REF_LENGTH, src/common.h:57             */
#define SO_SHIFT_BASES 100  /* refSeqLength / 3, src/align.cu:668      */
#define SO_MEM_MARGIN 100000000LL /* GLOBAL_MEM_MARGIN, src/common.h:43 */

static void so_err(char *err, size_t n, const char *fmt, ...) {
  if (!err || !n) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(err, n, fmt, ap);
  va_end(ap);
}

void so_free(void *p) { free(p); }

/* ------------------------------------------------------------------ */
/* codes and hash                                                      */

static inline int so_code(unsigned char c) {
  switch (c) {
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 0; /* A, a, N, n and every other byte */
  }
}

int so_hash(const char *s, int k) {
  int h = 0, p = 1;
  for (int i = 0; i < k; ++i) {
    h += p * so_code((unsigned char)s[i]);
    p *= 4;
  }
  return h;
}

void so_revcomp(const char *seq, int len, char *out) {
  for (int i = 0; i < len; ++i) {
    char c = seq[len - 1 - i];
    out[i] = c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : 'A';
  }
  out[len] = '\0';
}

/* fgets(line, MAX_LINE_LENGTH, f) starting at byte pos: chunk length. */
static size_t so_chunk(const char *b, size_t n, size_t pos) {
  if (pos >= n) return 0;
  size_t lim = n - pos;
  if (lim > SO_LINE_MAX - 1) lim = SO_LINE_MAX - 1;
  const char *nl = (const char *)memchr(b + pos, '\n', lim);
  return nl ? (size_t)(nl - (b + pos)) + 1 : lim;
}

static int so_check_bytes(const char *b, size_t n, const char *what, char *err,
                          size_t errlen) {
  for (size_t i = 0; i < n; ++i) {
    unsigned char c = (unsigned char)b[i];
    if (c == 0 || c >= 128) {
      so_err(err, errlen, "%s: byte %u at offset %zu is not 7-bit text", what,
             c, i);
      return -1;
    }
    if (c == '>' && i > 0 && b[i - 1] != '\n') {
      so_err(err, errlen, "%s: '>' inside a line at offset %zu", what, i);
      return -1;
    }
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* reference FASTA                                                     */

typedef struct {
  size_t name_off, seq_off;
  unsigned bpl;           /* _numBasesPerLine (refMap)                */
  char name[SO_NAME_MAX];
  size_t cat_start, cat_len;
} so_rec;

typedef struct {
  const char *file;
  size_t file_len;
  so_rec *recs;
  int n;
  char *cat;               /* concatenated sequence lines of each record */
  size_t cat_len;
} so_ref;

static void so_ref_free(so_ref *r) {
  free(r->recs);
  free(r->cat);
  memset(r, 0, sizeof(*r));
}

static int so_ref_parse(const char *b, size_t n, so_ref *r, char *err,
                        size_t errlen) {
  memset(r, 0, sizeof(*r));
  if (so_check_bytes(b, n, "reference", err, errlen)) return -1;
  r->file = b;
  r->file_len = n;
  r->cat = (char *)malloc(n + 1);
  int cap = 16;
  r->recs = (so_rec *)calloc(cap, sizeof(so_rec));
  if (!r->cat || !r->recs) return -2;
  /* refMapCreate state (src/refMap.cu:61-116) */
  long prev_ll = 0, old_ll = 0;
  unsigned pos_count = 0;
  int num_lines = 0;
  size_t pos = 0, c;
  while ((c = so_chunk(b, n, pos)) > 0) {
    long ll = (long)c - (b[pos + c - 1] == '\n');
    if (prev_ll > 0) old_ll = prev_ll;
    prev_ll = ll;
    if (ll == 0) { pos += c; continue; }
    if (b[pos] == '>') {
      if (r->n >= 1) {
        so_rec *p = &r->recs[r->n - 1];
        p->bpl = num_lines > 1
                     ? (unsigned)(pos_count - (unsigned)old_ll) / (unsigned)(num_lines - 1)
                     : 0;
      }
      if (r->n == 127) {
        so_err(err, errlen, "reference: more than 127 sequences (the "
               "reference keeps the sequence index in a char)");
        return -1;
      }
      if (r->n == cap) {
        cap *= 2;
        r->recs = (so_rec *)realloc(r->recs, cap * sizeof(so_rec));
      }
      so_rec *q = &r->recs[r->n++];
      memset(q, 0, sizeof(*q));
      q->name_off = pos + c - (size_t)ll - 1;
      q->seq_off = pos + c;
      if (ll - 1 >= SO_NAME_MAX) {
        so_err(err, errlen, "reference: name longer than %d characters",
               SO_NAME_MAX - 1);
        return -1;
      }
      memcpy(q->name, b + pos + 1, (size_t)(ll - 1));
      q->name[ll - 1] = '\0';
      q->cat_start = r->cat_len;
      pos_count = 0;
      num_lines = 0;
    } else {
      if (r->n == 0) {
        so_err(err, errlen, "reference: sequence before the first header");
        return -1;
      }
      ++num_lines;
      pos_count += (unsigned)ll;
      memcpy(r->cat + r->cat_len, b + pos, (size_t)ll);
      r->cat_len += (size_t)ll;
      r->recs[r->n - 1].cat_len += (size_t)ll;
    }
    pos += c;
  }
  if (prev_ll > 0) old_ll = prev_ll;
  if (r->n >= 1) {
    so_rec *p = &r->recs[r->n - 1];
    p->bpl = num_lines > 1
                 ? (unsigned)(pos_count - (unsigned)old_ll) / (unsigned)(num_lines - 1)
                 : 0;
  }
  if (r->n == 0) {
    so_err(err, errlen, "reference: no sequence header");
    return -1;
  }
  return 0;
}

/* getRefSeq2 from file offset (src/input.cu:348-403) into out[SO_WIN+1]
 * (NUL padded).  Returns the window length. */
static int so_fetch_window(const char *b, size_t n, size_t off, char *out) {
  char tmp[SO_WIN + 1];
  int cnt = 0, got = 0;
  size_t pos = off, c;
  memset(out, 0, SO_WIN + 1);
  while ((c = so_chunk(b, n, pos)) > 0) {
    const char *line = b + pos;
    pos += c;
    if (line[0] == '>') break;
    int ll = (int)c - (line[c - 1] == '\n');
    cnt += ll;
    if (cnt > SO_WIN) ll -= cnt - SO_WIN;
    if (ll > 0) {
      memcpy(tmp + got, line, (size_t)ll);
      got += ll;
    }
    if (cnt >= SO_WIN) break;
  }
  tmp[got] = '\0';
  /* N trimming, including the reference's indexing of the trailing loop
   * through the shifted pointer (src/input.cu:394-402): with one leading N
   * the trailing loop reads the terminator and trims nothing; with more it
   * reads bytes past the string, which this restatement treats as not N. */
  int lead = 0;
  while (lead < got && (tmp[lead] == 'n' || tmp[lead] == 'N')) ++lead;
  int len = got;
  if (lead == 0) {
    while (len > 0 && (tmp[len - 1] == 'n' || tmp[len - 1] == 'N')) --len;
  }
  int w = len - lead;
  if (w < 0) w = 0;
  memcpy(out, tmp + lead, (size_t)w);
  return w;
}

/* ------------------------------------------------------------------ */
/* SSAHA index                                                         */

struct so_index {
  int k, thres, nb, total;
  int *lookup;      /* _lookupTable                 */
  int *repeats;     /* _numRepeatsPerTuple          */
  int *actual;      /* _numActualRepeatsPerTuple    */
  int8_t *ref_idx;  /* total + 1                    */
  int32_t *ref_pos; /* total + 1                    */
  int nrefs;
};

static int so_index_from_ref(const so_ref *r, int k, int thres, so_index **out,
                             char *err, size_t errlen) {
  if (k < 1 || k > 15) {
    so_err(err, errlen, "seed length %d outside 1..15", k);
    return -1;
  }
  so_index *ix = (so_index *)calloc(1, sizeof(so_index));
  ix->k = k;
  ix->thres = thres;
  ix->nb = 1 << (2 * k);
  ix->nrefs = r->n;
  ix->lookup = (int *)calloc((size_t)ix->nb, sizeof(int));
  ix->repeats = (int *)calloc((size_t)ix->nb, sizeof(int));
  ix->actual = (int *)calloc((size_t)ix->nb, sizeof(int));
  int *nrep = (int *)calloc((size_t)ix->nb, sizeof(int));
  size_t ntup = 0;
  for (int i = 0; i < r->n; ++i) ntup += r->recs[i].cat_len / (size_t)k;
  int32_t *th = (int32_t *)malloc((ntup + 1) * sizeof(int32_t));
  int32_t *tr = (int32_t *)malloc((ntup + 1) * sizeof(int32_t));
  int32_t *tp = (int32_t *)malloc((ntup + 1) * sizeof(int32_t));
  size_t nt = 0;
  long total = 0;
  /* pass 1 (src/lookupTable5.cu:127-187) */
  for (int ri = 0; ri < r->n; ++ri) {
    const char *s = r->cat + r->recs[ri].cat_start;
    size_t len = r->recs[ri].cat_len;
    for (size_t p = 0; p + (size_t)k <= len; p += (size_t)k) {
      int h = so_hash(s + p, k);
      ++ix->repeats[h];
      if (ix->repeats[h] <= thres) {
        ++ix->actual[h];
        ++nrep[h];
        ++total;
        th[nt] = h;
        tr[nt] = ri;
        tp[nt] = (int32_t)p;
        ++nt;
      } else if (ix->repeats[h] == ix->actual[h] + 1) {
        ix->actual[h] = 0;
        nrep[h] = 0;
        total -= thres;
      }
    }
  }
  ix->total = (int)total;
  ix->ref_idx = (int8_t *)calloc((size_t)total + 1, 1);
  ix->ref_pos = (int32_t *)calloc((size_t)total + 1, sizeof(int32_t));
  ix->ref_idx[0] = -1;
  ix->ref_pos[0] = -1;
  /* bucket starts (src/lookupTable5.cu:201-211) */
  int start = 1;
  for (int h = 0; h < ix->nb; ++h)
    if (ix->repeats[h] > 0 && ix->repeats[h] <= thres) {
      ix->lookup[h] = start;
      start += ix->repeats[h];
    }
  /* pass 2 (src/lookupTable5.cu:219-231) */
  for (size_t t = 0; t < nt; ++t) {
    int h = th[t];
    if (ix->repeats[h] <= thres) {
      int idx = ix->lookup[h] + nrep[h] - 1;
      ix->ref_idx[idx] = (int8_t)tr[t];
      ix->ref_pos[idx] = tp[t];
      --nrep[h];
    }
  }
  free(th);
  free(tr);
  free(tp);
  free(nrep);
  *out = ix;
  return 0;
}

int so_index_build(const char *fasta, size_t len, int k, int thres,
                   so_index **out, char *err, size_t errlen) {
  so_ref r;
  int rc = so_ref_parse(fasta, len, &r, err, errlen);
  if (rc == 0) rc = so_index_from_ref(&r, k, thres, out, err, errlen);
  so_ref_free(&r);
  return rc;
}

void so_index_free(so_index *ix) {
  if (!ix) return;
  free(ix->lookup);
  free(ix->repeats);
  free(ix->actual);
  free(ix->ref_idx);
  free(ix->ref_pos);
  free(ix);
}
int so_index_num_buckets(const so_index *ix) { return ix->nb; }
int so_index_total(const so_index *ix) { return ix->total; }
int so_index_start(const so_index *ix, int h) { return ix->lookup[h]; }
int so_index_repeats(const so_index *ix, int h) { return ix->repeats[h]; }
int so_index_actual(const so_index *ix, int h) { return ix->actual[h]; }
int so_index_num_refs(const so_index *ix) { return ix->nrefs; }
void so_index_postings(const so_index *ix, int8_t *ri, int32_t *rp) {
  memcpy(ri, ix->ref_idx, (size_t)ix->total + 1);
  memcpy(rp, ix->ref_pos, ((size_t)ix->total + 1) * sizeof(int32_t));
}
void so_index_buckets(const so_index *ix, int32_t *lookup, int32_t *repeats) {
  memcpy(lookup, ix->lookup, (size_t)ix->nb * sizeof(int32_t));
  memcpy(repeats, ix->repeats, (size_t)ix->nb * sizeof(int32_t));
}

/* ------------------------------------------------------------------ */
/* hits and best clusters                                              */

typedef struct { int8_t ri; int32_t sh, rp; } so_hit;

static int so_hit_cmp(const void *a, const void *b) {
  const so_hit *x = (const so_hit *)a, *y = (const so_hit *)b;
  if (x->ri != y->ri) return x->ri < y->ri ? -1 : 1;
  if (x->sh != y->sh) return x->sh < y->sh ? -1 : 1;
  if (x->rp != y->rp) return x->rp < y->rp ? -1 : 1;
  return 0;
}

static int so_best_of_sorted(int max_hits, const so_hit *h, int n,
                             int8_t *o_ri, int32_t *o_sh, int32_t *o_rp) {
  if (n == 0) return 0;
  /* createClusters / findBiggestClusterSize (src/mapHits6.cu:202-272) */
  int biggest = 0;
  for (int i = 0; i < n;) {
    int j = i + 1;
    while (j < n && h[j].ri == h[i].ri && h[j].sh == h[i].sh) ++j;
    if (j - i > biggest) biggest = j - i;
    i = j;
  }
  /* findBiggestClusters (src/mapHits6.cu:132-167), first clusters kept */
  int got = 0;
  for (int i = 0; i < n && got < max_hits;) {
    int j = i + 1;
    while (j < n && h[j].ri == h[i].ri && h[j].sh == h[i].sh) ++j;
    if (j - i == biggest) {
      o_ri[got] = h[i].ri;
      o_sh[got] = h[i].sh;
      o_rp[got] = h[i].rp;
      ++got;
    }
    i = j;
  }
  return got;
}

int so_best_hits(int max_hits, const int8_t *ri, const int32_t *sh,
                 const int32_t *rp, int n, int8_t *o_ri, int32_t *o_sh,
                 int32_t *o_rp) {
  if (n <= 0) return 0;
  so_hit *h = (so_hit *)malloc((size_t)n * sizeof(so_hit));
  for (int i = 0; i < n; ++i) {
    h[i].ri = ri[i];
    h[i].sh = sh[i];
    h[i].rp = rp[i];
  }
  qsort(h, (size_t)n, sizeof(so_hit), so_hit_cmp);
  int got = so_best_of_sorted(max_hits, h, n, o_ri, o_sh, o_rp);
  free(h);
  return got;
}

int so_map_query(const so_index *ix, const char *seq, int len, int max_hits,
                 int8_t *o_ri, int32_t *o_sh, int32_t *o_rp) {
  int nq = len - ix->k + 1;
  if (nq <= 0) return 0;
  size_t n = 0;
  for (int i = 0; i < nq; ++i) {
    int h = so_hash(seq + i, ix->k);
    n += (size_t)ix->actual[h];
  }
  if (n == 0) return 0;
  so_hit *hits = (so_hit *)malloc(n * sizeof(so_hit));
  size_t m = 0;
  for (int i = 0; i < nq; ++i) {
    int h = so_hash(seq + i, ix->k);
    if (ix->actual[h] == 0) continue;
    int s = ix->lookup[h], e = s + ix->actual[h] - 1;
    for (int j = s; j <= e; ++j) {
      hits[m].ri = ix->ref_idx[j];
      hits[m].sh = ix->ref_pos[j] - i;
      hits[m].rp = ix->ref_pos[j];
      ++m;
    }
  }
  qsort(hits, m, sizeof(so_hit), so_hit_cmp);
  int got = so_best_of_sorted(max_hits, hits, (int)m, o_ri, o_sh, o_rp);
  free(hits);
  return got;
}

/* ------------------------------------------------------------------ */
/* Smith-Waterman with the GPU kernel's semantics                      */

static inline unsigned char so_up(unsigned char c) {
  return (unsigned)(c - 'a') < 26u ? (unsigned char)(c - 'a' + 'A') : c;
}

void so_sw(const char *q, int Q, const char *r, int R, int m, int x, int o,
           int e, so_aln *out, char *qcons, char *rcons, uint8_t *dirs) {
  const int W = R + 1;
  uint8_t *dir = dirs ? dirs : (uint8_t *)malloc((size_t)(Q + 1) * W);
  memset(dir, 0, (size_t)(Q + 1) * W);
  int *hp = (int *)calloc((size_t)W, sizeof(int));
  int *hc = (int *)calloc((size_t)W, sizeof(int));
  int best = 0, best_cell = 0;
  for (int i = 1; i <= Q; ++i) {
    unsigned char qc = so_up((unsigned char)q[i - 1]);
    int row_best = 0, row_cell = 0;
    hc[0] = 0;
    for (int j = 1; j <= R; ++j) {
      unsigned char rc = so_up((unsigned char)r[j - 1]);
      int s = (qc == rc || qc == 'N' || rc == 'N') ? m : x;
      int d = hp[j - 1] + s;
      int t = hp[j] + (dir[(i - 1) * W + j] == SO_UP ? e : o);
      int l = hc[j - 1] + (dir[i * W + j - 1] == SO_LEFT ? e : o);
      int v = 0;
      uint8_t dd = SO_NONE;
      if (v < d) { v = d; dd = SO_DIAG; }
      if (v < t) { v = t; dd = SO_UP; }
      if (v < l) { v = l; dd = SO_LEFT; }
      hc[j] = v;
      dir[i * W + j] = dd;
      if (row_best < v) { row_best = v; row_cell = i * W + j; }
    }
    if (best < row_best) { best = row_best; best_cell = row_cell; }
    int *t = hp; hp = hc; hc = t;
  }
  free(hp);
  free(hc);
  /* backtrack (src/smithWaterman.cu:911-1026) */
  int cur = best_cell, cr = cur / W, cc = cur % W, nxt;
  uint8_t d0 = dir[cur];
  if (d0 == SO_UP) nxt = cur - W;
  else if (d0 == SO_LEFT) nxt = cur - 1;
  else if (d0 == SO_DIAG) nxt = cur - W - 1;
  else nxt = cur; /* the reference leaves nextCell unset here (score 0) */
  int nr = nxt / W, nc = nxt % W;
  int tick = -1, nref = -1, start = 0;
  while ((cr != nr || cc != nc) && nc != 0 && nr != 0) {
    ++tick;
    if (nc == cc) rcons[tick] = '-';
    else { rcons[tick] = r[cc - 1]; ++nref; }
    qcons[tick] = (nr == cr) ? '-' : q[cr - 1];
    start = cc;
    cur = nxt; cr = nr; cc = nc;
    uint8_t dd = dir[cur];
    if (dd == SO_UP) nxt = cur - W;
    else if (dd == SO_LEFT) nxt = cur - 1;
    else if (dd == SO_DIAG) nxt = cur - W - 1;
    else break;
    nr = nxt / W; nc = nxt % W;
  }
  if ((cr != nr || cc != nc) && (nc == 0 || nr == 0)) {
    ++tick;
    if (nc == cc) rcons[tick] = '-';
    else { rcons[tick] = r[cc - 1]; ++nref; }
    qcons[tick] = (nr == cr) ? '-' : q[cr - 1];
    start = cc;
  }
  out->score = (float)best;
  out->cell_max = best_cell;
  out->start = start;
  out->end = start + nref;
  out->len = tick + 1;
  if (!dirs) free(dir);
}

/* so_sw over n pairs (query i at q + i * qs, window i at r + i * rs) on
 * `threads` host threads, each with its own direction matrix: the CPU
 * Smith-Waterman baseline, threaded the way the reference's CPU path hands
 * pairs to threads with one matrix set each (src/align.cu:2395-2422). */
typedef struct {
  const char *q, *r;
  int Q, R, qs, rs, m, x, o, e, T, t;
  long n;
  so_aln *out;
} so_swb;

static void *so_swb_run(void *p) {
  so_swb *a = (so_swb *)p;
  uint8_t *dirs = (uint8_t *)malloc((size_t)(a->Q + 1) * (a->R + 1));
  char *qc = (char *)malloc((size_t)a->Q + a->R + 2);
  char *rc = (char *)malloc((size_t)a->Q + a->R + 2);
  for (long i = a->t; i < a->n; i += a->T)
    so_sw(a->q + i * (long)a->qs, a->Q, a->r + i * (long)a->rs, a->R, a->m, a->x, a->o, a->e,
          &a->out[i], qc, rc, dirs);
  free(dirs);
  free(qc);
  free(rc);
  return NULL;
}

int so_sw_batch(const char *q, int Q, int qs, const char *r, int R, int rs, long n, int m,
                int x, int o, int e, int threads, so_aln *out) {
  if (threads < 1) threads = 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
  so_swb *args = (so_swb *)malloc(sizeof(so_swb) * (size_t)threads);
  for (int t = 0; t < threads; ++t) {
    so_swb a = {q, r, Q, R, qs, rs, m, x, o, e, threads, t, n, out};
    args[t] = a;
    pthread_create(&th[t], NULL, so_swb_run, &args[t]);
  }
  for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
  free(th);
  free(args);
  return 0;
}

/* ------------------------------------------------------------------ */
/* reads (qryGetNext2 stream) and Phase 1                              */

typedef struct {
  size_t name_off, seq_off;
  const char *seq;
  int len;
  char name[SO_NAME_MAX];
} so_read;

typedef struct {
  so_read *r;
  int n;
  long n_gt;      /* getSeqCount: '>' bytes in the file (src/input.cu:505-524) */
  int first_len;  /* getSeqSize (src/input.cu:475-496)                         */
} so_reads;

/* the longest read a run takes: the reference's 199 unless max_read_len
 * allows more (up to SO_READ_LONGEST) */
static int so_read_limit(const so_params *p) {
  if (p->max_read_len <= 0) return SO_QSEQ_MAX - 1;
  return p->max_read_len < SO_READ_LONGEST ? p->max_read_len : SO_READ_LONGEST;
}

static int so_reads_parse(const char *b, size_t n, so_reads *rd, char *err,
                          size_t errlen, int max_read) {
  memset(rd, 0, sizeof(*rd));
  if (so_check_bytes(b, n, "reads", err, errlen)) return -1;
  int cap = 1024;
  rd->r = (so_read *)malloc((size_t)cap * sizeof(so_read));
  size_t pos = 0, c;
  int have_header = 0, nheaders = 0;
  so_read cur;
  memset(&cur, 0, sizeof(cur));
  for (size_t i = 0; i < n; ++i) rd->n_gt += b[i] == '>';
  while ((c = so_chunk(b, n, pos)) > 0) {
    const char *line = b + pos;
    int ll = (int)c - (line[c - 1] == '\n');
    if (ll == 0) {
      so_err(err, errlen, "reads: empty line at offset %zu (the reference "
             "reader loops forever on it)", pos);
      return -1;
    }
    if (line[0] == '>') {
      if (have_header) {
        so_err(err, errlen, "reads: header without a sequence line at "
               "offset %zu", cur.name_off);
        return -1;
      }
      if (ll - 1 > SO_NAME_MAX - 2) {
        so_err(err, errlen, "reads: name longer than %d characters",
               SO_NAME_MAX - 2);
        return -1;
      }
      memcpy(cur.name, line + 1, (size_t)(ll - 1));
      cur.name[ll - 1] = '\0';
      cur.name_off = pos + c - (size_t)ll - 1;
      cur.seq_off = pos + c;
      have_header = 1;
      ++nheaders;
    } else {
      if (!have_header) {
        so_err(err, errlen, "reads: sequence line without a header at "
               "offset %zu (multi-line reads are not supported)", pos);
        return -1;
      }
      if (ll > max_read) {
        so_err(err, errlen, "reads: read longer than %d bases", max_read);
        return -1;
      }
      cur.seq = line;
      cur.len = ll;
      if (rd->n == 0) rd->first_len = (int)c - 1; /* strlen(line) - 1 */
      if (rd->n == cap) {
        cap *= 2;
        rd->r = (so_read *)realloc(rd->r, (size_t)cap * sizeof(so_read));
      }
      rd->r[rd->n++] = cur;
      have_header = 0;
    }
    pos += c;
  }
  if (have_header) {
    so_err(err, errlen, "reads: trailing header without a sequence line");
    return -1;
  }
  return 0;
}

/* Phase-1 slot schedule of searchQueries3 (src/search.cu:325-357): batches
 * of 16 calls to qryGetNext2 while i < numQrs; a call past the end of the
 * file leaves its slot holding the read it last held.  Fills order[] with
 * read indices (-1: slot never filled) and returns the count. */
#define SO_P1_THREADS 16 /* NUM_THREADS, src/common.h:97 */
static long so_p1_schedule(const so_reads *rd, int **order) {
  long nb = (rd->n_gt + SO_P1_THREADS - 1) / SO_P1_THREADS;
  if (rd->n_gt <= 0) nb = 0;
  long tot = nb * SO_P1_THREADS;
  int *o = (int *)malloc((size_t)(tot > 0 ? tot : 1) * sizeof(int));
  int slot[SO_P1_THREADS];
  for (int j = 0; j < SO_P1_THREADS; ++j) slot[j] = -1;
  long next = 0;
  for (long bi = 0; bi < nb; ++bi)
    for (int j = 0; j < SO_P1_THREADS; ++j) {
      if (next < rd->n) slot[j] = (int)next++;
      o[bi * SO_P1_THREADS + j] = slot[j];
    }
  *order = o;
  return tot;
}

typedef struct {
  const so_index *ix;
  const so_reads *rd;
  int max_hits;
  int8_t *ri;   /* per read: 2*max_hits entries */
  int32_t *sh, *rp;
  int *cnt;     /* per read: [fwd, rev] */
  long next;
  pthread_mutex_t mu;
} so_p1_job;

static void *so_p1_worker(void *arg) {
  so_p1_job *jb = (so_p1_job *)arg;
  char rev[SO_READ_LONGEST + 1];
  for (;;) {
    pthread_mutex_lock(&jb->mu);
    long i = jb->next;
    jb->next += 64;
    pthread_mutex_unlock(&jb->mu);
    if (i >= jb->rd->n) break;
    long e = i + 64 < jb->rd->n ? i + 64 : jb->rd->n;
    for (; i < e; ++i) {
      const so_read *r = &jb->rd->r[i];
      int mh = jb->max_hits;
      size_t b0 = (size_t)i * 2 * (size_t)mh;
      jb->cnt[2 * i] = so_map_query(jb->ix, r->seq, r->len, mh, jb->ri + b0,
                                    jb->sh + b0, jb->rp + b0);
      so_revcomp(r->seq, r->len, rev);
      jb->cnt[2 * i + 1] =
          so_map_query(jb->ix, rev, r->len, mh, jb->ri + b0 + mh,
                       jb->sh + b0 + mh, jb->rp + b0 + mh);
    }
  }
  return NULL;
}

static int so_run_phase1(const so_index *ix, const so_reads *rd, int max_hits,
                         int threads, so_match **out, int *n_out) {
  so_p1_job jb;
  memset(&jb, 0, sizeof(jb));
  jb.ix = ix;
  jb.rd = rd;
  jb.max_hits = max_hits;
  size_t per = (size_t)2 * (size_t)max_hits;
  size_t nr = (size_t)(rd->n > 0 ? rd->n : 1);
  jb.ri = (int8_t *)malloc(nr * per);
  jb.sh = (int32_t *)malloc(nr * per * sizeof(int32_t));
  jb.rp = (int32_t *)malloc(nr * per * sizeof(int32_t));
  jb.cnt = (int *)calloc(nr * 2, sizeof(int));
  pthread_mutex_init(&jb.mu, NULL);
  if (threads < 1) threads = 1;
  pthread_t *th = (pthread_t *)malloc((size_t)threads * sizeof(pthread_t));
  for (int t = 0; t < threads; ++t) pthread_create(&th[t], NULL, so_p1_worker, &jb);
  for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
  free(th);
  pthread_mutex_destroy(&jb.mu);
  int *order;
  long tot = so_p1_schedule(rd, &order);
  long nm = 0;
  for (long s = 0; s < tot; ++s)
    if (order[s] >= 0) nm += jb.cnt[2 * order[s]] + jb.cnt[2 * order[s] + 1];
  so_match *m = (so_match *)malloc((size_t)(nm > 0 ? nm : 1) * sizeof(so_match));
  long k = 0;
  for (long s = 0; s < tot; ++s) {
    int ridx = order[s];
    if (ridx < 0) continue;
    for (int strand = 0; strand < 2; ++strand) {
      size_t b0 = (size_t)ridx * per + (size_t)strand * (size_t)max_hits;
      for (int h = 0; h < jb.cnt[2 * ridx + strand]; ++h) {
        m[k].slot_read = ridx;
        m[k].strand = strand;
        m[k].ref_idx = jb.ri[b0 + h];
        m[k].shift = jb.sh[b0 + h];
        m[k].ref_pos = jb.rp[b0 + h];
        ++k;
      }
    }
  }
  free(order);
  free(jb.ri);
  free(jb.sh);
  free(jb.rp);
  free(jb.cnt);
  *out = m;
  *n_out = (int)nm;
  return 0;
}

typedef struct so_lt13_s so_lt13;
static int so_lt13_build(const so_ref *r, const so_index *ix, so_lt13 **out, char *err,
                         size_t errlen);
static void so_lt13_free(so_lt13 *t);
static int so_run_phase1_lt13(const so_lt13 *t, const so_reads *rd, int threads,
                              so_match **out, int *n_out);

int so_phase1(const char *ref, size_t ref_len, const char *reads,
              size_t reads_len, const so_params *p, so_match **out, int *n_out,
              char *err, size_t errlen) {
  so_ref r;
  so_reads rd;
  so_index *ix = NULL;
  int rc = so_ref_parse(ref, ref_len, &r, err, errlen);
  if (rc == 0) rc = so_index_from_ref(&r, p->seed_len, p->ignore_thres, &ix, err, errlen);
  if (rc == 0) rc = so_reads_parse(reads, reads_len, &rd, err, errlen, so_read_limit(p));
  if (rc == 0) {
    if (p->seeder == 1) {
      so_lt13 *t = NULL;
      rc = so_lt13_build(&r, ix, &t, err, errlen);
      if (rc == 0) rc = so_run_phase1_lt13(t, &rd, p->threads, out, n_out);
      so_lt13_free(t);
    } else {
      rc = so_run_phase1(ix, &rd, p->max_hits, p->threads, out, n_out);
    }
    free(rd.r);
  }
  so_index_free(ix);
  so_ref_free(&r);
  return rc;
}

/* ------------------------------------------------------------------ */
/* lt13 seed-and-extend seeder: the Phase 1 of the reference CLI's GPU   */
/* default (search2Queries, src/search2.cu:48-259), restated per query   */
/* strand in the order the kernel's single block computes it.            */

#define SO_L13_ARR 2304     /* idealArrSize at 48 KB of shared memory per
                               block (src/search2.cu:122-137)             */
#define SO_L13_THREADS 64   /* dimBlock.x (src/search2.cu:151)            */
#define SO_L13_ITERS (SO_L13_ARR / SO_L13_THREADS)
#define SO_L13_POS_BITS 25  /* REF_POS_BITS2 (src/lookupTable13.cu:32)    */
#define SO_L13_POS_MASK 33554431
#define SO_L13_HITS 3       /* maxNumHits = 3 (src/search2.cu:62)         */
#define SO_L13_KEEP 1000    /* the k > 1000 reset (src/lookupTable13.cu:800) */

struct so_lt13_s {
  const so_index *ix;   /* keys = lookup, numTuplesPerHash = actual      */
  int k, nrefs;
  int32_t *vals;        /* _refPos2: total + 1 composites, [0] = -1      */
  long *tbase, *ntup;   /* per reference: first tuple id, tuple count    */
  int32_t *map;         /* refPosHashMap per tuple id (0: never written) */
  long long max_comp;   /* _maxRefPosComposite: entries of the device copy */
};

static void so_lt13_free(so_lt13 *t) {
  if (!t) return;
  free(t->vals);
  free(t->tbase);
  free(t->ntup);
  free(t->map);
  free(t);
}

/* lookupTable13Create (src/lookupTable13.cu:64-242) on top of the SSAHA
 * index of the same tuples: composites refIdx << 25 | pos / k replace the
 * positions, and refPosHashMap holds the hash of every tuple written to the
 * temporary file (the first thres occurrences of each hash).  The map has
 * _maxRefPosComposite entries on the device, one short of the largest
 * composite written (src/lookupTable13.cu:182,374-377); reads at or past
 * that length are undefined in the reference and are 0 here, the value of
 * every entry never written. */
static int so_lt13_build(const so_ref *r, const so_index *ix, so_lt13 **out, char *err,
                         size_t errlen) {
  const int k = ix->k;
  if (r->n > 64) {
    so_err(err, errlen, "lt13 seeding: more than 64 reference sequences (the composite "
           "position keeps the index in the bits of an int above bit 25)");
    return -1;
  }
  if (ix->thres > SO_L13_ARR - SO_L13_KEEP - 2 * SO_L13_THREADS) {
    so_err(err, errlen, "lt13 seeding: ignore threshold above %d (the kernel's shared "
           "arrays would overflow)", SO_L13_ARR - SO_L13_KEEP - 2 * SO_L13_THREADS);
    return -1;
  }
  so_lt13 *t = (so_lt13 *)calloc(1, sizeof(so_lt13));
  t->ix = ix;
  t->k = k;
  t->nrefs = r->n;
  t->tbase = (long *)calloc((size_t)r->n + 1, sizeof(long));
  t->ntup = (long *)calloc((size_t)r->n + 1, sizeof(long));
  long nt = 0;
  for (int i = 0; i < r->n; ++i) {
    t->tbase[i] = nt;
    t->ntup[i] = (long)(r->recs[i].cat_len / (size_t)k);
    if (t->ntup[i] >= (1L << SO_L13_POS_BITS) - 64) {
      so_err(err, errlen, "lt13 seeding: a sequence of %ld tuples does not fit the "
             "composite position", t->ntup[i]);
      so_lt13_free(t);
      return -1;
    }
    nt += t->ntup[i];
  }
  t->vals = (int32_t *)malloc(((size_t)ix->total + 1) * sizeof(int32_t));
  t->vals[0] = -1;
  for (int i = 1; i <= ix->total; ++i)
    t->vals[i] = ((int32_t)ix->ref_idx[i] << SO_L13_POS_BITS) + ix->ref_pos[i] / k;
  t->map = (int32_t *)calloc((size_t)(nt > 0 ? nt : 1), sizeof(int32_t));
  int *seen = (int *)calloc((size_t)ix->nb, sizeof(int));
  for (int ri = 0; ri < r->n; ++ri) {
    const char *s = r->cat + r->recs[ri].cat_start;
    for (long c = 0; c < t->ntup[ri]; ++c) {
      int h = so_hash(s + c * k, k);
      if (++seen[h] <= ix->thres) {
        t->map[t->tbase[ri] + c] = h;
        long long comp = ((long long)ri << SO_L13_POS_BITS) + c;
        if (comp > t->max_comp) t->max_comp = comp;
      }
    }
  }
  free(seen);
  *out = t;
  return 0;
}

static int32_t so_lt13_map_at(const so_lt13 *t, long long v) {
  if (v < 0 || v >= t->max_comp) return 0;
  int r = (int)(v >> SO_L13_POS_BITS);
  long c = (long)(v & SO_L13_POS_MASK);
  if (r >= t->nrefs || c >= t->ntup[r]) return 0;
  return t->map[t->tbase[r] + c];
}

/* getRandNum13_gpu (src/lookupTable13.cu:907-911): K&R's generator on the
 * block's shared seed, which the reference never initialises; it starts at
 * 0 here for every query strand. */
static int so_l13_rand(uint32_t *seed) {
  *seed = *seed * 1103515245u + 12345u;
  return (int)((*seed / 65536u) % 32768u);
}

/* One query strand: lookupTable13MapQry2_gpu (src/lookupTable13.cu:646-868)
 * with the block's 64 threads run in order.  Writes up to 3 hits (records
 * whose reference index is not -1, src/search2.cu:339-377). */
static int so_lt13_query(const so_lt13 *t, const char *seq, int Q, int32_t *ri, int32_t *rp) {
  const so_index *ix = t->ix;
  const int k = t->k;
  char qs[SO_L13_ARR];            /* qrySeq_shr: the strand, zeros after it */
  int nm[SO_L13_ARR], pos[SO_L13_ARR], pos3[SO_L13_ARR];
  int qh[SO_L13_ARR];
  memset(qs, 0, sizeof(qs));
  memcpy(qs, seq, (size_t)Q);
  for (int i = 0; i < SO_L13_ARR; ++i) {
    nm[i] = -1;
    pos[i] = -1;
    pos3[i] = -1;
  }
  /* getHash13_gpu at every offset the kernel hashes (zeros hash as A) */
  const int n_tup = Q - k + 1;
  const int last = (Q / k) * k;
  int hmax = n_tup + 2 > last ? n_tup + 2 : last;
  if (hmax < 0) hmax = 0;
  for (int x = 0; x < hmax && x + k <= SO_L13_ARR; ++x) qh[x] = so_hash(qs + x, k);
  int count = 0, maxm = 0;
  int inc = -1;
  while (inc <= n_tup) {
    ++inc;
    const int h = qh[inc];
    const int nh = ix->actual[h];
    const int iters = (nh + SO_L13_THREADS - 1) / SO_L13_THREADS;
    const int key = ix->lookup[h];
    /* seed and extend every hit of the tuple (src/lookupTable13.cu:722-771) */
    for (int j = 0; j < iters * SO_L13_THREADS; ++j) {
      const int idx = count + j;
      long long val = j < nh ? t->vals[key + j] : -1;
      if (val < 0) {
        nm[idx] = 0;
        continue;
      }
      const int start_val = (int)val;
      int matches = 0, mm = 0, mm2 = 0, inc2 = inc;
      int32_t rth = so_lt13_map_at(t, val);
      while (inc2 < last) {
        if (rth == qh[inc2]) {
          ++val;
          rth = so_lt13_map_at(t, val);
          inc2 += k;
          ++matches;
          mm = 0;
          mm2 = 0;
        } else if (mm < k - 1) {
          ++inc2;
          ++mm;
        } else if (mm2 == 0) {
          ++val;
          rth = so_lt13_map_at(t, val);
          inc2 -= mm;
          mm = 0;
          ++mm2;
        } else {
          break;
        }
      }
      nm[idx] = matches;
      pos[idx] = start_val;
    }
    /* the tail clear (src/lookupTable13.cu:774-783): thread 0 clears from
     * offset for gap entries, the block from offset in steps of 64 */
    const int offset = count + nh;
    const int gap = (SO_L13_ARR - offset) % SO_L13_THREADS;
    for (int i = offset; i < offset + gap; ++i) nm[i] = -1;
    const int it3 = (SO_L13_ARR - offset) / SO_L13_THREADS;
    for (int i = offset; i < offset + it3 * SO_L13_THREADS; ++i) nm[i] = -1;
    /* keep the biggest matches (src/lookupTable13.cu:786-803) */
    int kk = count;
    for (int j = count; j < offset; ++j) {
      if (maxm <= nm[j]) {
        if (maxm < nm[j]) {
          maxm = nm[j];
          kk = 0;
        }
        nm[j] = -1;
        nm[kk] = maxm;
        pos[kk] = pos[j];
        ++kk;
      }
    }
    if (kk > SO_L13_KEEP) kk = 0;
    count = kk;
  }
  /* final selection (src/lookupTable13.cu:808-839): the maximum over
   * [0, count], then the entries equal to it in thread-strided order */
  int fm = 0;
  for (int i = 0; i <= count; ++i)
    if (nm[i] > fm) fm = nm[i];
  int n3 = 0;
  for (int th = 0; th < SO_L13_THREADS; ++th)
    for (int i = 0; i < SO_L13_ITERS; ++i) {
      const int p = i * SO_L13_THREADS + th;
      if (nm[p] == fm) pos3[n3++] = pos[p];
    }
  int pick[SO_L13_HITS];
  if (n3 > SO_L13_HITS) {
    /* arrGetRandomNums13_gpu (src/lookupTable13.cu:882-898) */
    uint32_t seed = 0;
    int got = 0;
    while (got < SO_L13_HITS) {
      int v = so_l13_rand(&seed) % n3;
      int dup = 0;
      for (int i = 0; i < got; ++i) dup |= pick[i] == v;
      if (!dup) pick[got++] = v;
    }
  } else {
    for (int i = 0; i < SO_L13_HITS; ++i) pick[i] = i;
  }
  int n = 0;
  for (int i = 0; i < SO_L13_HITS; ++i) {
    const int v = pos3[pick[i]];
    const int8_t r8 = (int8_t)(v >> SO_L13_POS_BITS);
    if (r8 == -1) continue;
    ri[n] = r8;
    rp[n] = (v & SO_L13_POS_MASK) * k;
    ++n;
  }
  return n;
}

int so_lt13_map(const char *fasta, size_t len, int k, int thres, const char *seq,
                int seq_len, int32_t *ri, int32_t *rp, char *err, size_t errlen) {
  so_ref r;
  so_index *ix = NULL;
  so_lt13 *t = NULL;
  int rc = so_ref_parse(fasta, len, &r, err, errlen);
  if (rc == 0) rc = so_index_from_ref(&r, k, thres, &ix, err, errlen);
  if (rc == 0) rc = so_lt13_build(&r, ix, &t, err, errlen);
  if (rc == 0) rc = so_lt13_query(t, seq, seq_len, ri, rp);
  so_lt13_free(t);
  so_index_free(ix);
  so_ref_free(&r);
  return rc;
}

typedef struct {
  const so_lt13 *t;
  const so_reads *rd;
  int32_t *ri, *rp;  /* per read: 2 x 3 entries */
  int *cnt;          /* per read: [fwd, rev] */
  long next;
  pthread_mutex_t mu;
} so_l13_job;

static void *so_l13_worker(void *arg) {
  so_l13_job *jb = (so_l13_job *)arg;
  char rev[SO_READ_LONGEST + 1];
  for (;;) {
    pthread_mutex_lock(&jb->mu);
    long i = jb->next;
    jb->next += 64;
    pthread_mutex_unlock(&jb->mu);
    if (i >= jb->rd->n) break;
    long e = i + 64 < jb->rd->n ? i + 64 : jb->rd->n;
    for (; i < e; ++i) {
      const so_read *r = &jb->rd->r[i];
      size_t b0 = (size_t)i * 2 * SO_L13_HITS;
      jb->cnt[2 * i] = so_lt13_query(jb->t, r->seq, r->len, jb->ri + b0, jb->rp + b0);
      so_revcomp(r->seq, r->len, rev);
      jb->cnt[2 * i + 1] = so_lt13_query(jb->t, rev, r->len, jb->ri + b0 + SO_L13_HITS,
                                         jb->rp + b0 + SO_L13_HITS);
    }
  }
  return NULL;
}

/* search2Queries' records (src/search2.cu:176-256, 339-377): every read in
 * file order, forward strand then reverse complement, shift 0. */
static int so_run_phase1_lt13(const so_lt13 *t, const so_reads *rd, int threads,
                              so_match **out, int *n_out) {
  so_l13_job jb;
  memset(&jb, 0, sizeof(jb));
  jb.t = t;
  jb.rd = rd;
  size_t nr = (size_t)(rd->n > 0 ? rd->n : 1);
  jb.ri = (int32_t *)malloc(nr * 2 * SO_L13_HITS * sizeof(int32_t));
  jb.rp = (int32_t *)malloc(nr * 2 * SO_L13_HITS * sizeof(int32_t));
  jb.cnt = (int *)calloc(nr * 2, sizeof(int));
  pthread_mutex_init(&jb.mu, NULL);
  if (threads < 1) threads = 1;
  pthread_t *th = (pthread_t *)malloc((size_t)threads * sizeof(pthread_t));
  for (int i = 0; i < threads; ++i) pthread_create(&th[i], NULL, so_l13_worker, &jb);
  for (int i = 0; i < threads; ++i) pthread_join(th[i], NULL);
  free(th);
  pthread_mutex_destroy(&jb.mu);
  long nm = 0;
  for (long i = 0; i < rd->n; ++i) nm += jb.cnt[2 * i] + jb.cnt[2 * i + 1];
  so_match *m = (so_match *)malloc((size_t)(nm > 0 ? nm : 1) * sizeof(so_match));
  long q = 0;
  for (long i = 0; i < rd->n; ++i)
    for (int strand = 0; strand < 2; ++strand) {
      size_t b0 = (size_t)i * 2 * SO_L13_HITS + (size_t)strand * SO_L13_HITS;
      for (int h = 0; h < jb.cnt[2 * i + strand]; ++h) {
        m[q].slot_read = (int32_t)i;
        m[q].strand = strand;
        m[q].ref_idx = jb.ri[b0 + h];
        m[q].shift = 0;
        m[q].ref_pos = jb.rp[b0 + h];
        ++q;
      }
    }
  free(jb.ri);
  free(jb.rp);
  free(jb.cnt);
  *out = m;
  *n_out = (int)nm;
  return 0;
}

/* ------------------------------------------------------------------ */
/* Phase 2                                                             */

/* getNumQueriesPerIteration (src/align.cu:2767-2793) with the per-pair
 * memory of getMemPerRefQryPair (src/align.cu:2739-2756). */
static long so_p2_batch(long long device_mem, int Q, long nm) {
  long per_iter;
  if (device_mem > 0) {
    int mem_pair = (SO_WIN + 1) + (Q + 1) + 4 + 4 + 4 + 2 + 2 * (SO_WIN + Q + 2);
    long gm = (long)(device_mem - SO_MEM_MARGIN);
    per_iter = (int)floor((float)gm / mem_pair);
    if (per_iter > 2147483647L) per_iter = 2147483647L;
  } else {
    per_iter = nm;
  }
  if (per_iter > nm) per_iter = nm;
  if (per_iter >= 2 && per_iter % 2 == 1) --per_iter;
  return per_iter;
}

/* qryNameCmp (src/align.cu:1501-1519) */
static int so_name_cmp(const char *s, const char *t, int size) {
  int i;
  for (i = 0; i < size; ++i) {
    if (s[i] == '\0' && t[i] == '\0') return 0;
    else if (s[i] == '\0' || t[i] == '\0') break;
    else if (s[i] != t[i]) return -1;
  }
  if ((s[i] == '*' && s[i + 1] == '\0') || (t[i] == '*' && t[i + 1] == '\0'))
    return 0;
  return -1;
}

typedef struct {
  char qname[SO_NAME_MAX + 1];
  const char *rname;
  int ref_dist;
  char q[SO_QMAX + 2];
  char w[SO_WIN + 1];
  so_aln a;
  char *qc, *rc;
} so_pair;

typedef struct {
  so_pair *pp;
  long n;
  int Q;
  const so_params *p;
  long next;
  pthread_mutex_t mu;
} so_p2_job;

static void *so_p2_worker(void *arg) {
  so_p2_job *jb = (so_p2_job *)arg;
  for (;;) {
    pthread_mutex_lock(&jb->mu);
    long i = jb->next;
    jb->next += 16;
    pthread_mutex_unlock(&jb->mu);
    if (i >= jb->n) break;
    long e = i + 16 < jb->n ? i + 16 : jb->n;
    for (; i < e; ++i) {
      so_pair *x = &jb->pp[i];
      so_sw(x->q, jb->Q, x->w, SO_WIN, jb->p->match, jb->p->mismatch,
            jb->p->gap_open, jb->p->gap_ext, &x->a, x->qc, x->rc, NULL);
    }
  }
  return NULL;
}

typedef struct { char *b; size_t n, cap; } so_sb;
static void so_sb_put(so_sb *s, const char *p, size_t n) {
  if (s->n + n + 1 > s->cap) {
    while (s->n + n + 1 > s->cap) s->cap = s->cap ? s->cap * 2 : 1 << 16;
    s->b = (char *)realloc(s->b, s->cap);
  }
  memcpy(s->b + s->n, p, n);
  s->n += n;
}

static void so_print_record(so_sb *sb, const so_pair *x) {
  char hdr[512];
  int len = x->a.len;
  so_sb_put(sb, "\n****************************************\n", 42);
  int hn = snprintf(hdr, sizeof(hdr),
                    "Qry: %s | Ref: %s | Score: %.1f | AlignStart: %d | "
                    "AlignEnd: %d | AlignLength: %d\n",
                    x->qname, x->rname, x->a.score, x->a.start + x->ref_dist,
                    x->a.end + x->ref_dist, len);
  so_sb_put(sb, hdr, (size_t)hn);
  so_sb_put(sb, "R: ", 3);
  for (int z = len - 1; z >= 0; --z) so_sb_put(sb, &x->rc[z], 1);
  so_sb_put(sb, "\n   ", 4);
  for (int z = len - 1; z >= 0; --z) {
    char rc = x->rc[z], qc = x->qc[z];
    int ur = (unsigned)(rc - 'a') < 26u ? rc - 32 : rc;
    int uq = (unsigned)(qc - 'a') < 26u ? qc - 32 : qc;
    char ch = (ur == uq || rc == 'N' || qc == 'N') ? '|'
              : (rc == '-' || qc == '-')          ? '-'
                                                  : '.';
    so_sb_put(sb, &ch, 1);
  }
  so_sb_put(sb, "\nQ: ", 4);
  for (int z = len - 1; z >= 0; --z) so_sb_put(sb, &x->qc[z], 1);
  so_sb_put(sb, "\n", 1);
}

/* printCigar (src/output.cu:33-81): runs over the consensus from its last
 * byte to its first; '-' in the reference consensus is D, else '-' in the
 * query consensus is I, else M. */
static void so_print_cigar(so_sb *sb, const char *qc, const char *rc, int len) {
  int run = 0;
  char op = ' ', buf[16];
  for (int z = len - 1; z >= 0; --z) {
    char c = rc[z] == '-' ? 'D' : qc[z] == '-' ? 'I' : 'M';
    if (run > 0 && c != op) {
      int n = snprintf(buf, sizeof(buf), "%d%c", run, op);
      so_sb_put(sb, buf, (size_t)n);
      run = 0;
    }
    op = c;
    ++run;
  }
  if (run > 0) {
    int n = snprintf(buf, sizeof(buf), "%d%c", run, op);
    so_sb_put(sb, buf, (size_t)n);
  }
}

/* printOutputSam (src/output.cu:98-130): one line per record, window start */
static void so_print_sam(so_sb *sb, const so_pair *x) {
  char hdr[512];
  int hn = snprintf(hdr, sizeof(hdr), "%s\t*\t%s\t%d\t255\t", x->qname, x->rname, x->a.start);
  so_sb_put(sb, hdr, (size_t)hn);
  so_print_cigar(sb, x->qc, x->rc, x->a.len);
  so_sb_put(sb, "\t*\t0\t0\t", 7);
  for (int z = x->a.len - 1; z >= 0; --z) so_sb_put(sb, &x->qc[z], 1);
  so_sb_put(sb, "\t*\n", 3);
}

struct so_session {
  so_ref r;
  so_index *ix;
  so_lt13 *l13;  /* seeder 1 only */
  so_params p;
};

int so_session_create(const char *ref, size_t ref_len, const so_params *p,
                      so_session **out, char *err, size_t errlen) {
  so_session *s = (so_session *)calloc(1, sizeof(so_session));
  s->p = *p;
  int rc = so_ref_parse(ref, ref_len, &s->r, err, errlen);
  if (rc == 0) rc = so_index_from_ref(&s->r, p->seed_len, p->ignore_thres, &s->ix, err, errlen);
  if (rc == 0 && p->seeder == 1) rc = so_lt13_build(&s->r, s->ix, &s->l13, err, errlen);
  if (rc != 0) {
    so_session_free(s);
    return rc;
  }
  *out = s;
  return 0;
}

void so_session_free(so_session *s) {
  if (!s) return;
  so_lt13_free(s->l13);
  so_index_free(s->ix);
  so_ref_free(&s->r);
  free(s);
}

int so_align(const char *ref, size_t ref_len, const char *reads,
             size_t reads_len, const so_params *p, char **out, size_t *out_len,
             char *err, size_t errlen) {
  so_session *s = NULL;
  int rc = so_session_create(ref, ref_len, p, &s, err, errlen);
  if (rc == 0) rc = so_session_align(s, reads, reads_len, out, out_len, err, errlen);
  so_session_free(s);
  return rc;
}

int so_session_align(so_session *ss, const char *reads, size_t reads_len,
                     char **out, size_t *out_len, char *err, size_t errlen) {
  const so_params *p = &ss->p;
  so_ref r = ss->r;
  so_reads rd;
  so_match *m = NULL;
  int nm = 0;
  memset(&rd, 0, sizeof(rd));
  int rc = so_reads_parse(reads, reads_len, &rd, err, errlen, so_read_limit(p));
  if (rc == 0)
    rc = p->seeder == 1 ? so_run_phase1_lt13(ss->l13, &rd, p->threads, &m, &nm)
                        : so_run_phase1(ss->ix, &rd, p->max_hits, p->threads, &m, &nm);
  if (rc != 0) {
    free(rd.r);
    return rc;
  }
  int Q = p->qry_len > 0 ? p->qry_len : rd.first_len;
  if (Q < 1 || Q > SO_QMAX) {
    so_err(err, errlen, "query length %d outside 1..%d", Q, SO_QMAX);
    free(rd.r); free(m);
    return -1;
  }
  long per_iter = so_p2_batch(p->device_mem, Q, nm);
  int n_iter = per_iter > 0 ? (int)ceil((float)nm / per_iter) : 0;
  so_sb sb = {0};
  /* query buffers that persist like the reference's: the per-slot host
   * buffer querySeq and the stack buffer tmpQrySeq (src/align.cu:660-728) */
  char *slotq = (char *)calloc((size_t)(per_iter > 0 ? per_iter : 1), (size_t)Q + 1);
  char *tmpq = (char *)calloc((size_t)Q + 2, 1);
  long done = 0;
  for (int it = 0; it < n_iter; ++it) {
    long cnt = per_iter;
    if (it == n_iter - 1) {
      long maxs = (long)n_iter * per_iter;
      cnt = nm < maxs ? nm - (long)(n_iter - 1) * per_iter : per_iter;
    }
    so_pair *pp = (so_pair *)calloc((size_t)cnt, sizeof(so_pair));
    char *cons = (char *)malloc((size_t)cnt * 2 * (size_t)(SO_WIN + Q + 2));
    for (long j = 0; j < cnt; ++j) {
      const so_match *mm = &m[done + j];
      const so_read *rr = &rd.r[mm->slot_read];
      so_pair *x = &pp[j];
      x->qc = cons + (size_t)j * 2 * (size_t)(SO_WIN + Q + 2);
      x->rc = x->qc + (SO_WIN + Q + 2);
      int dist = mm->ref_pos - SO_SHIFT_BASES;
      if (dist < 0) dist = 0;
      x->ref_dist = dist;
      const so_rec *rec = &r.recs[mm->ref_idx];
      unsigned off = (unsigned)rec->seq_off + (unsigned)dist +
                     (rec->bpl > 0 ? (unsigned)dist / rec->bpl : 0u);
      so_fetch_window(r.file, r.file_len, off, x->w);
      x->rname = rec->name;
      /* getSeq2 from the read's sequence offset (src/input.cu:216-258) */
      int avail = rr->len < Q ? rr->len : Q;
      char *dst = (mm->strand == 1) ? tmpq : slotq + (size_t)j * (Q + 1);
      memcpy(dst, rr->seq, (size_t)avail);
      dst[avail] = '\0';
      strcpy(x->qname, rr->name);
      if (mm->strand == 1) {
        char *sq = slotq + (size_t)j * (Q + 1);
        so_revcomp(tmpq, Q, sq);
        strcat(x->qname, "*");
      }
      memcpy(x->q, slotq + (size_t)j * (Q + 1), (size_t)Q);
    }
    so_p2_job jb;
    memset(&jb, 0, sizeof(jb));
    jb.pp = pp;
    jb.n = cnt;
    jb.Q = Q;
    jb.p = p;
    pthread_mutex_init(&jb.mu, NULL);
    int threads = p->threads < 1 ? 1 : p->threads;
    pthread_t *th = (pthread_t *)malloc((size_t)threads * sizeof(pthread_t));
    for (int t = 0; t < threads; ++t) pthread_create(&th[t], NULL, so_p2_worker, &jb);
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&jb.mu);
    if (p->out_format == 1) {  /* SAM: every record, no selection (src/align.cu:756-761) */
      for (long j = 0; j < cnt; ++j) so_print_sam(&sb, &pp[j]);
      free(pp);
      free(cons);
      done += cnt;
      continue;
    }
    /* chooseBestAlignment over this batch (src/align.cu:844-905) */
    long start = 0;
    while (start < cnt) {
      long end = start;
      while (end + 1 < cnt &&
             so_name_cmp(pp[end + 1].qname, pp[end].qname, SO_NAME_MAX) == 0)
        ++end;
      float mx = 0.0f;
      for (long i = start; i <= end; ++i)
        if (mx < pp[i].a.score) mx = pp[i].a.score;
      long keep = -1;
      for (long i = start; i <= end; ++i)
        if (pp[i].a.score == mx) { keep = i; break; }
      for (long i = start; i <= end; ++i)
        if (i != keep) pp[i].a.score = -1.0f;
      start = end + 1;
    }
    for (long j = 0; j < cnt; ++j)
      if (!(pp[j].a.score < 0.0f)) so_print_record(&sb, &pp[j]);
    free(pp);
    free(cons);
    done += cnt;
  }
  free(slotq);
  free(tmpq);
  free(m);
  free(rd.r);
  so_sb_put(&sb, "", 0);
  if (!sb.b) { sb.b = (char *)malloc(1); }
  sb.b[sb.n] = '\0';
  *out = sb.b;
  *out_len = sb.n;
  return 0;
}

/* ------------------------------------------------------------------ */
/* Paired-end pipeline (-q2): the GPU branch of src/main.cu:172-212.    */
/* Phase 1 searchQueries_paired2 (src/search.cu:2084-2200) on           */
/* lookupTable2 (src/lookupTable2.cu:75-300): non-overlapping tuples    */
/* stored as FILE offsets, mapped back by refMapGetIndexAndPos          */
/* (src/refMap.cu:166-242).  Phase 2 alignQueries_paired2               */
/* (src/align.cu:1879-2110): windows of 3Q by getSeq, mate pairs chosen */
/* by chooseBestAlignment_paired3 (src/align.cu:1248-1422), records by  */
/* printOutput_paired2 (src/output.cu:300-362).                          */

#define SO_PE_THRES 1000   /* TUPLE_IGNORE_THRES, src/common.h:75          */
#define SO_PE_HITS 3       /* MAX_NUM_HITS_PAIRED_END, src/common.h:63     */

typedef struct {
  int k, nb;
  int *lookup, *repeats;
  uint32_t *fileoff;       /* total + 1; [0] unused                        */
} so_pe_index;

static void so_pe_index_free(so_pe_index *t) {
  if (!t) return;
  free(t->lookup);
  free(t->repeats);
  free(t->fileoff);
  free(t);
}

/* lookupTable2Create's loop over the reference lines (src/lookupTable2.cu:
 * 99-168): tuples at 0, k, 2k of each line buffer (carried bases first),
 * file offset = header end + bases + line count, one less for the first
 * tuple written after a carry. */
static so_pe_index *so_pe_index_build(const char *b, size_t n, int k) {
  so_pe_index *t = (so_pe_index *)calloc(1, sizeof(so_pe_index));
  t->k = k;
  t->nb = 1 << (2 * k);
  t->lookup = (int *)calloc((size_t)t->nb, sizeof(int));
  t->repeats = (int *)calloc((size_t)t->nb, sizeof(int));
  int *nrep = (int *)calloc((size_t)t->nb, sizeof(int));
  size_t cap = 1024, nw = 0;
  int *wh = (int *)malloc(cap * sizeof(int));
  uint32_t *wo = (uint32_t *)malloc(cap * sizeof(uint32_t));
  char *line = (char *)malloc(2 * SO_LINE_MAX + 16);
  long total = 0;
  int offset = 0, num_bases = 0, num_nl = 0;
  uint32_t ref_pos = 0;
  size_t pos = 0, c;
  while ((c = so_chunk(b, n, pos)) > 0) {
    memcpy(line + offset, b + pos, c);
    line[offset + c] = '\0';
    pos += c;
    int ll = offset + (int)c;
    if (line[ll - 1] == '\n') line[--ll] = '\0';
    if (ll == 0) {
      offset = 0;
    } else if (line[offset] == '>') {
      offset = 0;
      num_bases = 0;
      num_nl = 0;
      ref_pos = (uint32_t)pos;  /* ftell after the header line */
    } else {
      int iters = ll - k + 1, i;
      for (i = 0; i < iters; i += k) {
        int h = so_hash(line + i, k);
        ++t->repeats[h];
        if (t->repeats[h] <= SO_PE_THRES) {
          ++nrep[h];
          ++total;
          if (nw == cap) {
            cap *= 2;
            wh = (int *)realloc(wh, cap * sizeof(int));
            wo = (uint32_t *)realloc(wo, cap * sizeof(uint32_t));
          }
          wh[nw] = h;
          if (offset > 0) {
            wo[nw] = ref_pos + (uint32_t)num_bases + (uint32_t)i + (uint32_t)num_nl - 1u;
            offset = 0;
          } else {
            wo[nw] = ref_pos + (uint32_t)num_bases + (uint32_t)i + (uint32_t)num_nl;
          }
          ++nw;
        } else if (t->repeats[h] == nrep[h] + 1) {
          nrep[h] = 0;
          total -= SO_PE_THRES;
        }
      }
      num_bases += ll;
      ++num_nl;
      offset = ll - i;
      memmove(line, line + i, (size_t)(offset > 0 ? offset : 0));
      if (offset < 0) offset = 0;
      num_bases -= offset;
    }
  }
  t->fileoff = (uint32_t *)calloc((size_t)total + 1, sizeof(uint32_t));
  t->fileoff[0] = UINT32_MAX;
  int start = 1;
  for (int h = 0; h < t->nb; ++h)
    if (t->repeats[h] > 0 && t->repeats[h] <= SO_PE_THRES) {
      t->lookup[h] = start;
      start += t->repeats[h];
    }
  for (size_t w = 0; w < nw; ++w) {
    int h = wh[w];
    if (t->repeats[h] <= SO_PE_THRES) {
      int idx = t->lookup[h] + nrep[h] - 1;
      t->fileoff[idx] = wo[w];
      --nrep[h];
    }
  }
  free(wh);
  free(wo);
  free(line);
  free(nrep);
  return t;
}

/* refMapGetIndexAndPos (src/refMap.cu:166-242) */
static void so_pe_index_pos(const so_ref *r, uint32_t off, int *index, int *pos) {
  int idx = -1;
  if (r->recs[0].seq_off == off) {
    *index = 0;
    *pos = 0;
    return;
  }
  if (r->n == 1) {
    idx = 0;
  } else {
    for (int i = 1; i < r->n; ++i) {
      if (r->recs[i - 1].seq_off == off) {
        *index = i - 1;
        *pos = 0;
        return;
      } else if (r->recs[i].seq_off > off) {
        idx = i - 1;
        break;
      }
    }
    if (idx == -1) idx = r->n - 1;
  }
  const uint32_t so = (uint32_t)r->recs[idx].seq_off;
  const uint32_t bpl = r->recs[idx].bpl;
  if (bpl == 0) {
    *pos = (int)(off - so);
  } else {
    uint32_t tmp = so;
    int nl = 0;
    while (tmp + bpl + 1 <= off) {
      tmp += bpl + 1;
      ++nl;
    }
    *pos = (int)(off - so) - nl;
  }
  *index = idx;
}

typedef struct {
  int8_t index;
  int32_t shift, offset;
  long order;
} so_pe_hit;

static int so_pe_hit_cmp(const void *a, const void *b) {
  const so_pe_hit *x = (const so_pe_hit *)a, *y = (const so_pe_hit *)b;
  if (x->index != y->index) return x->index < y->index ? -1 : 1;
  if (x->shift != y->shift) return x->shift < y->shift ? -1 : 1;
  if (x->offset != y->offset) return x->offset < y->offset ? -1 : 1;
  return x->order < y->order ? -1 : x->order > y->order; /* a stable merge sort */
}

/* lookupTable2MapQry (src/lookupTable2.cu:247-300) with getBestScoringPosition
 * (src/lookupTable2.cu:308-452): the first node of the first min(3, n) largest
 * clusters (the random picks pinned to the first ones) */
static int so_pe_map(const so_pe_index *t, const so_ref *r, const char *seq, int Q,
                     int8_t *ri, int32_t *sh, int32_t *off) {
  const int k = t->k;
  int nq = Q - k + 1;
  long cap = 0, nh = 0;
  for (int i = 0; i < nq; ++i) {
    int h = so_hash(seq + i, k);
    if (t->repeats[h] > SO_PE_THRES) continue;
    cap += t->repeats[h];
  }
  so_pe_hit *hits = (so_pe_hit *)malloc((size_t)(cap > 0 ? cap : 1) * sizeof(so_pe_hit));
  for (int i = 0; i < nq; ++i) {
    int h = so_hash(seq + i, k);
    if (t->repeats[h] > SO_PE_THRES) continue;
    int s0 = t->lookup[h], e0 = s0 + t->repeats[h] - 1;
    for (int j = s0; j <= e0; ++j) {
      int idx, p;
      so_pe_index_pos(r, t->fileoff[j], &idx, &p);
      hits[nh].index = (int8_t)idx;
      hits[nh].shift = p - i;
      hits[nh].offset = p;
      hits[nh].order = nh;
      ++nh;
    }
  }
  int n = 0;
  if (nh == 1) {
    ri[0] = hits[0].index;
    sh[0] = hits[0].shift;
    off[0] = hits[0].offset;
    n = 1;
  } else if (nh > 1) {
    qsort(hits, (size_t)nh, sizeof(so_pe_hit), so_pe_hit_cmp);
    int maxsz = 0, nmax = 0;
    for (long a = 0; a < nh;) {
      long e = a;
      while (e + 1 < nh && hits[e + 1].index == hits[a].index && hits[e + 1].shift == hits[a].shift) ++e;
      int sz = (int)(e - a + 1);
      if (sz > maxsz) {
        maxsz = sz;
        nmax = 1;
      } else if (sz == maxsz) {
        ++nmax;
      }
      a = e + 1;
    }
    int want = nmax < SO_PE_HITS ? nmax : SO_PE_HITS;
    for (long a = 0; a < nh && n < want;) {
      long e = a;
      while (e + 1 < nh && hits[e + 1].index == hits[a].index && hits[e + 1].shift == hits[a].shift) ++e;
      if ((int)(e - a + 1) == maxsz) {
        ri[n] = hits[a].index;
        sh[n] = hits[a].shift;
        off[n] = hits[a].offset;
        ++n;
      }
      a = e + 1;
    }
  }
  free(hits);
  return n;
}

typedef struct {
  int32_t id, mate, rev, read;   /* read: index in its mate file */
  int32_t ref_idx, shift, offset;
} so_pe_match;

/* searchQueries_paired2's records: per pair id, mate 1 forward, mate 1
 * reverse, mate 2 forward, mate 2 reverse; Q = getSeqSize of file 1. */
static int so_pe_phase1(const so_ref *r, const so_pe_index *t, const so_reads *r1,
                        const so_reads *r2, int Q, so_pe_match **out, long *n_out) {
  long cap = 64, n = 0;
  so_pe_match *m = (so_pe_match *)malloc((size_t)cap * sizeof(so_pe_match));
  char rev[SO_READ_LONGEST + 1];
  int8_t ri[SO_PE_HITS];
  int32_t sh[SO_PE_HITS], of[SO_PE_HITS];
  for (int i = 0; i < r1->n; ++i) {
    const so_read *mate[2] = {&r1->r[i], &r2->r[i]};
    for (int mi = 0; mi < 2; ++mi)
      for (int rc = 0; rc < 2; ++rc) {
        const so_read *q = mate[mi];
        const char *seq = q->seq;
        if (rc) {
          so_revcomp(q->seq, q->len, rev);
          seq = rev;
        }
        int nh = so_pe_map(t, r, seq, Q, ri, sh, of);
        for (int h = 0; h < nh; ++h) {
          if (n == cap) {
            cap *= 2;
            m = (so_pe_match *)realloc(m, (size_t)cap * sizeof(so_pe_match));
          }
          m[n].id = i + 1;
          m[n].mate = mi + 1;
          m[n].rev = rc;
          m[n].read = i;
          m[n].ref_idx = ri[h];
          m[n].shift = sh[h];
          m[n].offset = of[h];
          ++n;
        }
      }
  }
  *out = m;
  *n_out = n;
  return 0;
}

/* getNumQrsPerIter_paired (src/align.cu:1812-1852) over the record ids */
static int so_pe_batches(const so_pe_match *m, long n, int max_per, int **out) {
  int old_count = 0, count = 0, old_id = 0, is_new = 0, size = 0;
  int *arr = NULL;
  for (long r = 0; r < n; ++r) {
    ++count;
    int id = m[r].id;
    if (is_new) {
      is_new = 0;
      if (id == old_id)
        arr[size - 1] = old_count;
      else
        count = 1;
    } else if (id != old_id) {
      old_count = count - 1;
    }
    if (count == max_per) {
      arr = (int *)realloc(arr, (size_t)(size + 1) * sizeof(int));
      arr[size++] = count;
      count = count - old_count;
      is_new = 1;
    }
    old_id = id;
  }
  if (!is_new && count <= max_per) {
    arr = (int *)realloc(arr, (size_t)(size + 1) * sizeof(int));
    arr[size++] = count;
  }
  *out = arr;
  return size;
}

/* getSeq (src/input.cu:163-204): up to len bytes from the file offset on,
 * across lines, stopping at a '>' line; out is left untouched when nothing
 * is read (the caller zeroes it first). */
static void so_get_seq(const char *b, size_t n, size_t off, char *out, int len) {
  int cnt = 0, first = 1;
  size_t pos = off, c;
  while ((c = so_chunk(b, n, pos)) > 0) {
    const char *l = b + pos;
    pos += c;
    if (l[0] == '>') break;
    int ll = (int)c - (l[c - 1] == '\n');
    cnt += ll;
    if (cnt > len) ll -= cnt - len;
    if (first) {
      memcpy(out, l, (size_t)ll);
      out[ll] = '\0';
      first = 0;
    } else {
      size_t cur = strlen(out);
      memcpy(out + cur, l, (size_t)ll);
      out[cur + ll] = '\0';
    }
    if (cnt >= len) break;
  }
}

/* getMatePairName (src/align.cu:1434-1467): names end in 1 or 2 (the
 * library refuses others: the reference leaves the previous name there) */
static void so_pe_mate_name(const char *q, char *mate) {
  int len = (int)strlen(q) - 1;
  if (len < 0) return;
  if (q[len] == '*') {
    if (len >= 1 && (q[len - 1] == '1' || q[len - 1] == '2')) {
      memcpy(mate, q, (size_t)(len - 1));
      mate[len - 1] = q[len - 1] == '1' ? '2' : '1';
      mate[len] = '\0';
    }
  } else if (q[len] == '1' || q[len] == '2') {
    memcpy(mate, q, (size_t)len);
    mate[len] = q[len] == '1' ? '2' : '1';
    mate[len + 1] = '\0';
  }
}

typedef struct {
  char qname[SO_NAME_MAX + 1];
  const char *rname;
  int ref_dist, rev, id;
  char *q, *w;
  so_aln a;
  float score;
  char *qc, *rc;
} so_pe_pair;

/* chooseBestAlignment_paired3 (src/align.cu:1248-1422): its rand() pinned
 * to 0 (the first best pair); more than 6 tied pairs fit (the reference's
 * arrays of 6 would overflow) */
static void so_pe_choose(so_pe_pair *x, int size, unsigned min_frag, unsigned max_frag,
                         char *mate) {
  int start = 0, end = size - 1;
  while (start < size) {
    for (int i = start + 1; i < size; ++i)
      if (so_name_cmp(x[i].qname, x[i - 1].qname, SO_NAME_MAX) != 0) {
        end = i - 1;
        break;
      }
    if (end < start) end = size - 1;
    so_pe_mate_name(x[start].qname, mate);
    int start2 = end + 1, end2 = size - 1, has = 0;
    if (start2 < size) {
      for (int i = start2; i < size; ++i) {
        if (so_name_cmp(mate, x[i].qname, SO_NAME_MAX) != 0) {
          end2 = i - 1;
          break;
        } else {
          has = 1;
        }
      }
      if (end2 < start2) {
        if (has) {
          end2 = size - 1;
        } else {
          for (int i = start; i <= end; ++i) x[i].score = -1.0f;
          start = start2;
          continue;
        }
      }
    } else {
      for (int i = start; i <= end; ++i) x[i].score = -1.0f;
      start = start2;
      continue;
    }
    float max_score = 0.0f;
    for (int pass = 0; pass < 2; ++pass) {
      int found = -1, found2 = -1;
      for (int i = start; i <= end; ++i)
        for (int j = start2; j <= end2; ++j) {
          if (!((x[i].rev == 0 && x[j].rev == 1) || (x[j].rev == 0 && x[i].rev == 1))) continue;
          float sum = x[i].score + x[j].score;
          if (pass == 0 ? !(max_score < sum) : !(sum == max_score)) continue;
          int ok = 1;
          if (strcmp(x[i].rname, x[j].rname) == 0) {
            int d;
            if (x[i].rev == 0 && x[j].rev == 1)
              d = (x[j].ref_dist + x[j].a.end) - (x[i].ref_dist + x[i].a.start);
            else
              d = (x[i].ref_dist + x[i].a.end) - (x[j].ref_dist + x[j].a.start);
            ok = (unsigned)d >= min_frag && (unsigned)d <= max_frag;
          }
          if (!ok) continue;
          if (pass == 0) {
            max_score = sum;
          } else if (found < 0) {
            found = i;
            found2 = j;
          }
        }
      if (pass == 1) {
        for (int i = start; i <= end; ++i)
          if (found < 0 || i != found) x[i].score = -1.0f;
        for (int i = start2; i <= end2; ++i)
          if (found < 0 || i != found2) x[i].score = -1.0f;
      }
    }
    start = end2 + 1;
  }
}

/* printOutput_paired2 (src/output.cu:300-362) */
static void so_pe_print(so_sb *sb, const so_pe_pair *x, int size) {
  int old = -1;
  for (int y = 0; y < size; ++y) {
    if (x[y].score == -1.0f) continue;
    if (x[y].id != old) {
      old = x[y].id;
      so_sb_put(sb, "\n*************************************\n", 39);
    } else {
      so_sb_put(sb, "\n", 1);
    }
    char hdr[512];
    int len = x[y].a.len;
    int hn = snprintf(hdr, sizeof(hdr),
                      "Qry: %s | Ref: %s | Score: %.1f | AlignStart: %d | AlignEnd: %d | "
                      "AlignLength: %d\n",
                      x[y].qname, x[y].rname, x[y].score, x[y].a.start + x[y].ref_dist,
                      x[y].a.end + x[y].ref_dist, len);
    so_sb_put(sb, hdr, (size_t)hn);
    so_sb_put(sb, "R: ", 3);
    for (int z = len - 1; z >= 0; --z) so_sb_put(sb, &x[y].rc[z], 1);
    so_sb_put(sb, "\n   ", 4);
    for (int z = len - 1; z >= 0; --z) {
      char rc = x[y].rc[z], qc = x[y].qc[z];
      int ur = (unsigned)(rc - 'a') < 26u ? rc - 32 : rc;
      int uq = (unsigned)(qc - 'a') < 26u ? qc - 32 : qc;
      char ch = (ur == uq || rc == 'N' || qc == 'N') ? '|'
                : (rc == '-' || qc == '-')          ? '-'
                                                    : '.';
      so_sb_put(sb, &ch, 1);
    }
    so_sb_put(sb, "\nQ: ", 4);
    for (int z = len - 1; z >= 0; --z) so_sb_put(sb, &x[y].qc[z], 1);
    so_sb_put(sb, "\n", 1);
  }
}

int so_phase1_paired(const char *ref, size_t ref_len, const char *reads1, size_t len1,
                     const char *reads2, size_t len2, const so_params *p, int32_t **out,
                     long *n_out, char *err, size_t errlen) {
  so_ref r;
  so_reads a, b;
  memset(&a, 0, sizeof(a));
  memset(&b, 0, sizeof(b));
  int rc = so_ref_parse(ref, ref_len, &r, err, errlen);
  if (rc == 0) rc = so_reads_parse(reads1, len1, &a, err, errlen, SO_QSEQ_MAX - 1);
  if (rc == 0) rc = so_reads_parse(reads2, len2, &b, err, errlen, SO_QSEQ_MAX - 1);
  if (rc == 0 && a.n != b.n) {
    so_err(err, errlen, "paired reads: %d and %d reads", a.n, b.n);
    rc = -1;
  }
  if (rc == 0) {
    int Q = p->qry_len > 0 ? p->qry_len : a.first_len;
    so_pe_index *t = so_pe_index_build(ref, ref_len, p->seed_len);
    so_pe_match *m = NULL;
    long n = 0;
    so_pe_phase1(&r, t, &a, &b, Q, &m, &n);
    int32_t *o = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * 7 * sizeof(int32_t));
    for (long i = 0; i < n; ++i) {
      int32_t *f = o + 7 * i;
      f[0] = m[i].id;
      f[1] = m[i].rev;
      f[2] = m[i].mate;
      f[3] = m[i].ref_idx;
      f[4] = m[i].shift;
      f[5] = m[i].offset;
      f[6] = m[i].read;
    }
    free(m);
    so_pe_index_free(t);
    *out = o;
    *n_out = n;
  }
  free(a.r);
  free(b.r);
  so_ref_free(&r);
  return rc;
}

int so_align_paired(const char *ref, size_t ref_len, const char *reads1, size_t len1,
                    const char *reads2, size_t len2, const so_params *p, unsigned min_frag,
                    unsigned max_frag, char **out, size_t *out_len, char *err, size_t errlen) {
  so_ref r;
  so_reads rd[2];
  memset(rd, 0, sizeof(rd));
  int rc = so_ref_parse(ref, ref_len, &r, err, errlen);
  if (rc == 0) rc = so_reads_parse(reads1, len1, &rd[0], err, errlen, SO_QSEQ_MAX - 1);
  if (rc == 0) rc = so_reads_parse(reads2, len2, &rd[1], err, errlen, SO_QSEQ_MAX - 1);
  if (rc == 0 && rd[0].n != rd[1].n) {
    so_err(err, errlen, "paired reads: %d and %d reads", rd[0].n, rd[1].n);
    rc = -1;
  }
  const int Q = p->qry_len > 0 ? p->qry_len : rd[0].first_len;
  if (rc == 0 && (Q < 1 || 3 * Q > 1024)) {
    so_err(err, errlen, "query length %d outside 1..341", Q);
    rc = -1;
  }
  if (rc != 0) {
    free(rd[0].r);
    free(rd[1].r);
    so_ref_free(&r);
    return rc;
  }
  const int R = 3 * Q, comb = R + Q + 2;
  so_pe_index *t = so_pe_index_build(ref, ref_len, p->seed_len);
  so_pe_match *m = NULL;
  long nm = 0;
  so_pe_phase1(&r, t, &rd[0], &rd[1], Q, &m, &nm);
  so_pe_index_free(t);
  /* getNumQueriesPerIteration_paired (src/align.cu:2804-2824) */
  long max_per;
  {
    int mem_pair = (R + 1) + (Q + 1) + 4 + 4 + 4 + 2 + 2 * comb;
    long gm = (long)(p->device_mem - SO_MEM_MARGIN);
    max_per = p->device_mem > 0 ? (int)floor((float)gm / mem_pair) : nm;
    if (max_per > nm) max_per = nm;
  }
  int *per = NULL;
  int n_it = max_per > 0 ? so_pe_batches(m, nm, (int)max_per, &per) : 0;
  so_sb sb = {0};
  char mate[SO_NAME_MAX + 2];
  memset(mate, 0, sizeof(mate));
  long done = 0;
  for (int it = 0; it < n_it; ++it) {
    int cnt = per[it];
    so_pe_pair *x = (so_pe_pair *)calloc((size_t)(cnt > 0 ? cnt : 1), sizeof(so_pe_pair));
    char *buf = (char *)calloc((size_t)(cnt > 0 ? cnt : 1), (size_t)(Q + 1 + R + 1 + 2 * comb));
    for (int j = 0; j < cnt; ++j) {
      const so_pe_match *mm = &m[done + j];
      so_pe_pair *y = &x[j];
      char *slot = buf + (size_t)j * (Q + 1 + R + 1 + 2 * comb);
      y->q = slot;
      y->w = slot + Q + 1;
      y->qc = y->w + R + 1;
      y->rc = y->qc + comb;
      y->id = mm->id;
      y->rev = mm->rev;
      int dist = mm->offset - Q;
      if (dist < 0) dist = 0;
      y->ref_dist = dist;
      const so_rec *rec = &r.recs[mm->ref_idx];
      unsigned woff = (unsigned)rec->seq_off + (unsigned)dist +
                      (rec->bpl > 0 ? (unsigned)dist / rec->bpl : 0u);
      so_get_seq(r.file, r.file_len, woff, y->w, R);
      y->rname = rec->name;
      const so_read *rr = &rd[mm->mate - 1].r[mm->read];
      char tmp[SO_QMAX + 2];
      int L = rr->len < Q ? rr->len : Q;
      memcpy(tmp, rr->seq, (size_t)L);
      tmp[L] = '\0';
      strcpy(y->qname, rr->name);
      if (mm->rev) {
        so_revcomp(tmp, Q, y->q);
        strcat(y->qname, "*");
      } else {
        memcpy(y->q, tmp, (size_t)L + 1);
      }
    }
    for (int j = 0; j < cnt; ++j) {
      so_pe_pair *y = &x[j];
      so_sw(y->q, Q, y->w, R, p->match, p->mismatch, p->gap_open, p->gap_ext, &y->a, y->qc,
            y->rc, NULL);
      y->score = y->a.score;
    }
    if (p->out_format == 1) {
      for (int j = 0; j < cnt; ++j) {
        so_pair tmp;
        memset(&tmp, 0, sizeof(tmp));
        strcpy(tmp.qname, x[j].qname);
        tmp.rname = x[j].rname;
        tmp.a = x[j].a;
        tmp.qc = x[j].qc;
        tmp.rc = x[j].rc;
        so_print_sam(&sb, &tmp);
      }
    } else {
      so_pe_choose(x, cnt, min_frag, max_frag, mate);
      so_pe_print(&sb, x, cnt);
    }
    free(x);
    free(buf);
    done += cnt;
  }
  free(per);
  free(m);
  free(rd[0].r);
  free(rd[1].r);
  so_ref_free(&r);
  so_sb_put(&sb, "", 0);
  if (!sb.b) sb.b = (char *)malloc(1);
  sb.b[sb.n] = '\0';
  *out = sb.b;
  *out_len = sb.n;
  return 0;
}
