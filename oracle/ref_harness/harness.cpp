/*
 * harness.cpp — runs the reference's own code for validation of the oracle.
 * TEST INFRASTRUCTURE ONLY; built from the reference sources where they lie
 * (see Makefile), output only under oracle/_ref/.
 *
 * The reference functions called here are compiled unmodified from the
 * reference's src/ directory.  Only glue the reference keeps in static
 * functions or behind device APIs is restated here, each with its citation:
 *   - the 16-slot loop of searchQueries3 (src/search.cu:275-382) and the
 *     record line of printHeuristicMatches4 (src/search.cu:2230-2240),
 *     run sequentially with mapHits6's random picks pinned to the first ones;
 *   - the per-batch loop of alignQueries3 (src/align.cu:574-808) and the
 *     batch sizing of getNumQueriesPerIteration (src/align.cu:2767-2793);
 *   - chooseBestAlignment (src/align.cu:844-905) with the first maximum kept;
 *   - the query loop of search2Queries (src/search2.cu:176-256) and its
 *     printHeuristicMatches (src/search2.cu:339-377), both static there;
 *   - the paired-end loops of searchQueries_paired2 (src/search.cu:2084-2200,
 *     with printHeuristicMatches3, src/search.cu:1848-1860) and
 *     alignQueries_paired2 (src/align.cu:1879-2110), calling the reference's
 *     lookupTable2, getOffsets_paired2, getSeq, chooseBestAlignment_paired3
 *     and printOutput_paired2.
 * The GPU kernels smithWaterman (src/smithWaterman.cu:360-395) and
 * lookupTable13MapQry2_gpu (src/lookupTable13.cu:646-868) run on the CPU:
 * one fiber per CUDA thread, __syncthreads() yields to the next fiber.
 * lookupTable13MapQry2_gpu reads its block's shared random seed without
 * setting it; the harness zeroes the block's shared variables first.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ucontext.h>

#include <vector>

#include "common.h"
#include "input.h"
#include "hitList.h"
#include "lookupTable13.h"
#include "lookupTable2.h"
#include "lookupTable5.h"
#include "mapHits6.h"
#include "output.h"
#include "preprocess.h"
#include "query.h"
#include "refMap.h"

/* declarations with C++ linkage, as the reference compiles them */
void smithWaterman(char *refSeq, int refSeqLength, char *querySeq, int querySeqLength,
                   float match, float mismatch, float gapOpenPenalty, float gapExtPenalty,
                   float *maxScore, int *startPos, int *endPos, int *alignLength,
                   char *refConsensus, char *queryConsensus, int numQueries, int numReferences);
void smithWaterman_cpu(float *HMatrix, int *rowBacktracker, int *colBacktracker, char *refSeq,
                       int refLen, char *qrySeq, int qryLen, float match, float mismatch,
                       float gapOpenPenalty, float gapExtPenalty, float *alignScore,
                       int *startPos, int *endPos, int *alignLen, char *refConsensus,
                       char *qryConsensus);

/* ---- shim runtime (declared in shim.h) ------------------------------- */
struct ref_dim3 threadIdx, blockIdx, blockDim, gridDim;
/* dynamic shared memory of one block: lookupTable13MapQry2_gpu takes
 * idealArrSize x 21 + 16 bytes (src/search2.cu:122-137), under 48 KB */
int arr_shr[12800];

cudaError_t cudaGetLastError(void) { return 0; }
const char *cudaGetErrorString(cudaError_t) { return "no error"; }
cudaError_t cudaMalloc(void **p, size_t n) {
  *p = calloc(n + 65536, 1);
  return 0;
}
cudaError_t cudaFree(void *p) {
  free(p);
  return 0;
}
cudaError_t cudaMemcpy(void *d, const void *s, size_t n, enum cudaMemcpyKind) {
  memcpy(d, s, n);
  return 0;
}
cudaError_t cudaMemset(void *d, int v, size_t n) {
  memset(d, v, n);
  return 0;
}

static unsigned g_rand = 0;
/* stands in for rand() in array.cu (arrGetRandomNums): 0, 1, 2, ... so the
 * random biggest-cluster picks of mapHits6 become the first ones */
extern "C" int ref_rand(void) { return (int)(g_rand++); }
extern "C" int ref_rand_zero(void) { return 0; }
long long ref_device_mem = 288000000000LL;

static ucontext_t g_main;
static std::vector<ucontext_t> g_fib;
static std::vector<int> g_done;
static std::vector<char> g_stacks;
static int g_cur = 0;

void __syncthreads(void) { swapcontext(&g_fib[g_cur], &g_main); }

struct KernelArgs {
  char *ref;
  int R;
  char *qry;
  int Q;
  float m, x, o, e;
  float *score;
  int *start, *end, *len;
  char *rcons, *qcons;
};
static KernelArgs g_args;

static void sw_body() {
  KernelArgs &a = g_args;
  smithWaterman(a.ref, a.R, a.qry, a.Q, a.m, a.x, a.o, a.e, a.score, a.start, a.end, a.len,
                a.rcons, a.qcons, 1, 1);
}
static void (*g_body)() = sw_body;

static void fiber_entry(int tid) {
  g_body();
  g_done[tid] = 1;
}

/* One CUDA block of T threads for block index b. */
static void run_block(int T, int b) {
  const size_t stack = 64 * 1024;
  g_fib.assign(T, ucontext_t());
  g_done.assign(T, 0);
  g_stacks.resize((size_t)T * stack);
  blockIdx.x = (unsigned)b;
  blockDim.x = (unsigned)T;
  for (int t = 0; t < T; ++t) {
    getcontext(&g_fib[t]);
    g_fib[t].uc_stack.ss_sp = g_stacks.data() + (size_t)t * stack;
    g_fib[t].uc_stack.ss_size = stack;
    g_fib[t].uc_link = &g_main;
    makecontext(&g_fib[t], (void (*)())fiber_entry, 1, t);
  }
  for (;;) {
    int alive = 0;
    for (int t = 0; t < T; ++t) {
      if (g_done[t]) continue;
      g_cur = t;
      threadIdx.x = (unsigned)t;
      swapcontext(&g_main, &g_fib[t]);
      if (!g_done[t]) alive = 1;
    }
    if (!alive) break;
  }
}

extern "C" {

/* The GPU kernel on one pair.  q has Q bytes, r has R bytes. */
int ref_sw_kernel(const char *q, int Q, const char *r, int R, float m, float x, float o, float e,
                  float *score, int *start, int *end, int *len, char *qcons, char *rcons) {
  std::vector<char> qb(Q + 1, 0), rb(R + 1, 0);
  memcpy(qb.data(), q, Q);
  memcpy(rb.data(), r, R);
  g_args = KernelArgs{rb.data(), R, qb.data(), Q, m, x, o, e, score, start, end, len, rcons, qcons};
  *score = 0;
  int T = Q + 1 > R ? Q + 1 : R;
  run_block(T, 0);
  return 0;
}

/* The reference's CPU Smith-Waterman (the timed baseline of the survey). */
int ref_sw_cpu(const char *q, int Q, const char *r, int R, float m, float x, float o, float e,
               float *score, int *start, int *end, int *len, char *qcons, char *rcons) {
  std::vector<float> H((size_t)(Q + 1) * (R + 1), 0.0f);
  std::vector<int> rb((size_t)(Q + 1) * (R + 1), 0), cb((size_t)(Q + 1) * (R + 1), 0);
  std::vector<char> qq(q, q + Q), rr(r, r + R);
  qq.push_back(0);
  rr.push_back(0);
  smithWaterman_cpu(H.data(), rb.data(), cb.data(), rr.data(), R, qq.data(), Q, m, x, o, e, score,
                    start, end, len, rcons, qcons);
  return 0;
}

/* lookupTable5Create on a FASTA file; exports the table in its layout. */
int ref_index(const char *path, int k, int thres, int *n_buckets, int *total, int **lookup,
              int **repeats, char **ref_idx, int **ref_pos) {
  preprocessCreate();
  int nd = 0;
  lookupTable5Create_wrap(path, k, 3, lookup, ref_idx, ref_pos, &nd, repeats, thres);
  *n_buckets = nd;
  int t = 0;
  for (int h = 0; h < nd; ++h)
    if ((*repeats)[h] > 0 && (*repeats)[h] <= thres) t += (*repeats)[h];
  *total = t;
  return 0;
}

/* lookupTable5MapQry on the index built by the last ref_index call. */
int ref_map_query(const char *seq, const char *rev, int len, int is_rev, char *ri, int *sh,
                  int *rp) {
  Query q;
  std::vector<char> s(seq, seq + len), rv(rev, rev + len);
  s.push_back(0);
  rv.push_back(0);
  char name[2] = "q";
  q.name = name;
  q.length = len;
  q.seq = s.data();
  q.revCompSeq = rv.data();
  q.nameOffset = 0;
  q.seqOffset = 0;
  g_rand = 0;
  return lookupTable5MapQry(&q, (uint)len, (uint)is_rev, ri, sh, rp);
}

/* mapHits6GetBestHits with the random picks pinned to the first ones. */
int ref_best_hits(int max_hits, char *ri, int *sh, int *rp, int n, char *o_ri, int *o_sh,
                  int *o_rp) {
  g_rand = 0;
  return mapHits6GetBestHits(max_hits, ri, sh, rp, n, o_ri, o_sh, o_rp);
}

static int qry_name_cmp(const char *s, const char *t, int size) {
  int i;
  for (i = 0; i < size; ++i) {
    if (s[i] == '\0' && t[i] == '\0') return 0;
    else if (s[i] == '\0' || t[i] == '\0') break;
    else if (s[i] != t[i]) return -1;
  }
  if ((s[i] == '*' && s[i + 1] == '\0') || (t[i] == '*' && t[i + 1] == '\0')) return 0;
  return -1;
}

static void choose_best(char *names, int name_len, float *score, int size) {
  int start = 0, end = size - 1;
  while (start < size) {
    int i;
    for (i = start + 1; i < size; ++i)
      if (qry_name_cmp(names + i * name_len, names + (i - 1) * name_len, name_len) != 0) {
        end = i - 1;
        break;
      }
    if (end < start) end = size - 1;
    float mx = 0.0f;
    for (i = start; i <= end; ++i)
      if (mx < score[i]) mx = score[i];
    int keep = -1;
    for (i = start; i <= end; ++i)
      if (score[i] == mx) {
        keep = i;
        break;
      }
    for (i = start; i <= end; ++i)
      if (i != keep) score[i] = -1.0f;
    start = end + 1;
  }
}

/* ---- lt13 seeding: search2Queries' loop, one CPU block per strand ---- */
extern "C" char __start_ref13shr[], __stop_ref13shr[];

struct L13Args {
  int *keys, *vals, *ntup, *map;
  char *qrs;
  uchar *qlen;
  int *qdist;
  char *ri;
  int *rp;
  int k;
};
static L13Args g_l13;

static void l13_body() {
  L13Args &a = g_l13;
  lookupTable13MapQry2_gpu(a.keys, a.vals, a.ntup, a.map, a.qrs, a.qlen, a.qdist,
                           MAX_QRY_SEQ_LENGTH, a.ri, a.rp, 3, a.k, 0, 2304);
}

/* Writes the match file of search2Queries for the reads file: per read,
 * forward then reverse-complement hits (reference index != -1), shift 0.
 * Returns the number of records. */
static long l13_phase1(const char *ref_file, const char *qry_file, FILE *mf, int seed_len,
                       int thres) {
  int total = 0;
  lookupTable13Create(ref_file, seed_len, thres, &total);
  int *keys, *vals, *ntup, *map, nk, nv, maxc;
  lookupTable13CpyHashTableToGPU(&keys, &nk, &vals, &nv, &ntup, &map, &maxc);
  lookupTable13CpyConstMemToGPU();
  FILE *qf = fopen(qry_file, "r");
  Query *q = qryCreate2();
  std::vector<char> qrs(2 * MAX_QRY_SEQ_LENGTH + 64, 0);
  uchar qlen[2];
  int qdist[2] = {0, 0};
  char ri[2 * 3];
  int rp[2 * 3];
  long n = 0;
  while (qryGetNext2(qf, q) != NULL) {
    strcpy(qrs.data(), q->seq);
    qlen[0] = (uchar)q->length;
    strcpy(qrs.data() + MAX_QRY_SEQ_LENGTH, q->revCompSeq);
    qlen[1] = (uchar)q->length;
    qdist[1] = qlen[0];
    memset(ri, -1, sizeof(ri));
    memset(rp, -1, sizeof(rp));
    g_l13 = L13Args{keys, vals, ntup, map, qrs.data(), qlen, qdist, ri, rp, seed_len};
    g_body = l13_body;
    for (int b = 0; b < 2; ++b) {
      memset(__start_ref13shr, 0, (size_t)(__stop_ref13shr - __start_ref13shr));
      memset(arr_shr, 0, sizeof(arr_shr));
      run_block(64, b);
    }
    g_body = sw_body;
    for (int b = 0; b < 2; ++b)
      for (int j = 0; j < 3; ++j) {
        int kk = b * 3 + j;
        if (ri[kk] != -1) {
          fprintf(mf, "%s\t%d\t%d\t%d\t%d\t%lu\t%lu\n", q->name, b, ri[kk], 0, rp[kk],
                  q->nameOffset, q->seqOffset);
          ++n;
        }
      }
  }
  fclose(qf);
  qryDelete(q);
  cudaFree(keys);
  cudaFree(vals);
  cudaFree(ntup);
  cudaFree(map);
  return n;
}

/* The SSAHA -> GPU Smith-Waterman -> best alignment pipeline with the
 * reference's functions, file to file.  device_mem sizes the Phase-2
 * batches as the reference does from its GPU; out_format 1 prints every
 * record with printOutputSam instead of the best ones with printOutput
 * (the branch of src/align.cu:756-768).  Returns the number of match
 * records. */
long ref_pipeline_fmt(const char *ref_file, const char *qry_file, const char *out_file,
                      const char *match_file, long long device_mem, int seed_len, int thres,
                      float m, float x, float o, float e, int out_format, int seeder) {
  preprocessCreate();
  int num_qrs = getSeqCount((char *)qry_file);
  int qry_len = getSeqSize((char *)qry_file);
  refMapCreate(ref_file);
  FILE *mf = fopen(match_file, "w");
  long num_matches = 0;
  const int nt = NUM_THREADS;
  Query *slot[NUM_THREADS];
  for (int j = 0; j < nt; ++j) slot[j] = qryCreate2();
  if (seeder == 1) {
    num_matches = l13_phase1(ref_file, qry_file, mf, seed_len, thres);
  } else {
    int total = 0;
    lookupTable5Create(ref_file, seed_len, MAX_NUM_HITS_SINGLE_END, thres, &total);
    FILE *qf = fopen(qry_file, "r");
    char ri[MAX_NUM_HITS_SINGLE_END];
    int sh[MAX_NUM_HITS_SINGLE_END], rp[MAX_NUM_HITS_SINGLE_END];
    for (int i = 0; i < num_qrs; i += nt) {
      for (int j = 0; j < nt; ++j) qryGetNext2(qf, slot[j]);
      for (int j = 0; j < nt; ++j) {
        for (int strand = 0; strand < 2; ++strand) {
          g_rand = 0;
          int n = lookupTable5MapQry(slot[j], slot[j]->length, strand, ri, sh, rp);
          for (int h = 0; h < n; ++h)
            fprintf(mf, "%s\t%d\t%d\t%d\t%d\t%lu\t%lu\n", slot[j]->name, strand, ri[h], sh[h],
                    rp[h], slot[j]->nameOffset, slot[j]->seqOffset);
          num_matches += n;
        }
      }
    }
    fclose(qf);
  }
  fclose(mf);
  /* Phase 2 */
  const int R = REF_LENGTH, Q = qry_len, comb = R + Q + 2;
  long per_iter;
  {
    int mem_pair = (R + 1) + (Q + 1) + 4 + 4 + 4 + 2 + 2 * (R + Q + 2);
    long gm = (long)(device_mem - GLOBAL_MEM_MARGIN);
    per_iter = (int)floor((float)gm / mem_pair);
    if (per_iter > num_matches) per_iter = num_matches;
    if (per_iter >= 2 && per_iter % 2 == 1) --per_iter;
  }
  int n_iter = per_iter > 0 ? (int)ceil((float)num_matches / per_iter) : 0;
  std::vector<float> score(per_iter > 0 ? per_iter : 1);
  std::vector<int> dist(score.size()), st(score.size()), en(score.size()), ln(score.size());
  std::vector<char> rcons(score.size() * comb), qcons(score.size() * comb);
  std::vector<char> qname(score.size() * MAX_SEQ_NAME_LENGTH), rname(score.size() * MAX_SEQ_NAME_LENGTH);
  std::vector<char> qseq(score.size() * (Q + 1), 0), rseq(score.size() * (R + 1), 0);
  std::vector<char> tmpq(Q + 1, 0);
  mf = fopen(match_file, "r");
  FILE *of = fopen(out_file, "w");
  FILE *qfp = fopen(qry_file, "r");
  FILE *rfp = fopen(ref_file, "r");
  for (int it = 0; it < n_iter; ++it) {
    memset(rseq.data(), 0, rseq.size());
    long cnt = per_iter;
    if (it == n_iter - 1) {
      long maxs = (long)n_iter * per_iter;
      cnt = num_matches < maxs ? num_matches - (long)(n_iter - 1) * per_iter : per_iter;
    }
    for (long j = 0; j < cnt; ++j) {
      uint qno, qso, rno, rso, rfo, rev;
      int ridx;
      getOffsets(mf, &qno, &qso, &rno, &rso, &rfo, &dist[j], &rev, &ridx);
      dist[j] = dist[j] - R / 3 > 0 ? dist[j] - R / 3 : 0;
      refMapGetOffsets(ridx, dist[j], &rno, &rfo);
      getRefSeq2(rfp, rfo, rseq.data() + j * (R + 1), R);
      getSeqName(rfp, rno, rname.data() + j * MAX_SEQ_NAME_LENGTH);
      if (rev == 1) {
        getSeq2(qfp, qso, tmpq.data(), Q);
        qryGetReverseComplement(tmpq.data(), Q, qseq.data() + j * (Q + 1));
        getSeqName(qfp, qno, qname.data() + j * MAX_SEQ_NAME_LENGTH);
        strcat(qname.data() + j * MAX_SEQ_NAME_LENGTH, "*");
      } else {
        getSeq2(qfp, qso, qseq.data() + j * (Q + 1), Q);
        getSeqName(qfp, qno, qname.data() + j * MAX_SEQ_NAME_LENGTH);
      }
    }
    for (long j = 0; j < cnt; ++j) score[j] = 0;
    g_args = KernelArgs{rseq.data(), R, qseq.data(), Q, m, x, o, e, score.data(), st.data(),
                        en.data(), ln.data(), rcons.data(), qcons.data()};
    const int T = Q + 1 > R ? Q + 1 : R;
    for (long j = 0; j < cnt; ++j) run_block(T, (int)j);
    if (out_format == SAM_OUTPUT_FORMAT) {
      printOutputSam((int)cnt, qname.data(), rname.data(), score.data(), st.data(), en.data(),
                     ln.data(), comb, qcons.data(), rcons.data(), of);
    } else {
      choose_best(qname.data(), MAX_SEQ_NAME_LENGTH, score.data(), (int)cnt);
      printOutput((int)cnt, qname.data(), rname.data(), score.data(), dist.data(), st.data(),
                  en.data(), ln.data(), comb, qcons.data(), rcons.data(), of);
    }
  }
  fclose(mf);
  fclose(of);
  fclose(qfp);
  fclose(rfp);
  for (int j = 0; j < nt; ++j) qryDelete(slot[j]);
  refMapFree();
  return num_matches;
}

long ref_pipeline(const char *ref_file, const char *qry_file, const char *out_file,
                  const char *match_file, long long device_mem, int seed_len, int thres,
                  float m, float x, float o, float e) {
  return ref_pipeline_fmt(ref_file, qry_file, out_file, match_file, device_mem, seed_len, thres,
                          m, x, o, e, DEFAULT_OUTPUT_FORMAT, 0);
}

}  // extern "C"

/* prototypes of align.cu's exported functions, C++ linkage as the reference
 * compiles them (align.h also declares its static helpers) */
int getMemPerRefQryPair(int refLength, int queryLength);
int getNumQueriesPerIteration_paired(cudaDeviceProp *deviceProp, int memPerRefQueryPair,
                                     int numTotalQueries);
void chooseBestAlignment_paired3_wrap(char *qryName, int qryNameLen, uint *revComp,
                                      char *refName, int refNameLen, float *score,
                                      int *refDistance, int *alignStart, int *alignEnd, int size,
                                      uint minFragSize, uint maxFragSize);
void getNumQrsPerIter_paired_wrap(const char *file, int maxNumQrsPerIter, int **numQrsPerIter,
                                  int *arrSize);

extern "C" {

/* The paired-end pipeline of src/main.cu:172-212 (GPU branch), file to
 * file.  Returns the number of match records. */
long ref_pipeline_paired(const char *ref_file, const char *q1_file, const char *q2_file,
                         const char *out_file, const char *match_file, long long device_mem,
                         int seed_len, float m, float x, float o, float e, int out_format,
                         unsigned min_frag, unsigned max_frag) {
  preprocessCreate();
  const int num_qrs = getSeqCount((char *)q1_file);
  const int qry_len = getSeqSize((char *)q1_file);
  refMapCreate(ref_file);
  /* Phase 1: searchQueries_paired2 */
  lookupTable2Create(ref_file, seed_len, MAX_NUM_HITS_PAIRED_END, TUPLE_IGNORE_THRES);
  Query *qry1 = qryCreate2(), *qry2 = qryCreate2();
  FILE *mf = fopen(match_file, "w");
  FILE *f1 = fopen(q1_file, "r"), *f2 = fopen(q2_file, "r");
  long num_matches = 0;
  for (int i = 0, id = 0; i < num_qrs; ++i) {
    qry1 = qryGetNext2(f1, qry1);
    qry2 = qryGetNext2(f2, qry2);
    ++id;
    Query *mate[2] = {qry1, qry2};
    for (int mi = 0; mi < 2; ++mi)
      for (int rc = 0; rc < 2; ++rc) {
        g_rand = 0;
        HitList *best = lookupTable2MapQry(mate[mi], (uint)qry_len, (uint)rc);
        for (HitList *h = best; h != NULL; h = h->next) {
          fprintf(mf, "%d\t%s\t%d\t%d\t%d\t%d\t%d\t%u\t%u\n", id, mate[mi]->name, rc, mi + 1,
                  h->index, h->shift, h->offset, (uint)mate[mi]->nameOffset,
                  (uint)mate[mi]->seqOffset);
          ++num_matches;
        }
        if (best != NULL) hitListDelete(best);
      }
  }
  fclose(mf);
  fclose(f1);
  fclose(f2);
  lookupTable2Delete();
  /* Phase 2: alignQueries_paired2 */
  ref_device_mem = device_mem;
  const int Q = qry_len, R = 3 * qry_len, comb = R + Q + 2;
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, 0);
  const int max_qrs = getNumQueriesPerIteration_paired(&prop, getMemPerRefQryPair(R, Q),
                                                       (int)num_matches);
  int *per_iter = NULL, n_iter = 0;
  getNumQrsPerIter_paired_wrap(match_file, max_qrs, &per_iter, &n_iter);
  const size_t cap = max_qrs > 0 ? (size_t)max_qrs : 1;
  std::vector<float> score(cap);
  std::vector<int> dist(cap), st(cap), en(cap), ln(cap), qidx(cap);
  std::vector<uint> rev(cap);
  std::vector<char> rcons(cap * comb), qcons(cap * comb);
  std::vector<char> qname(cap * MAX_SEQ_NAME_LENGTH), rname(cap * MAX_SEQ_NAME_LENGTH);
  std::vector<char> qseq(cap * (Q + 1), 0), rseq(cap * (R + 1), 0);
  std::vector<char> tmpq(Q + 1, 0);
  mf = fopen(match_file, "r");
  f1 = fopen(q1_file, "r");
  f2 = fopen(q2_file, "r");
  FILE *rfp = fopen(ref_file, "r");
  FILE *of = fopen(out_file, "w");
  for (int it = 0; it < n_iter; ++it) {
    const int cnt = per_iter[it];
    memset(rseq.data(), 0, rseq.size());
    for (int j = 0; j < cnt; ++j) {
      uint qno, qso, rno, rso, rfo;
      int mate, ridx;
      getOffsets_paired2(mf, &qno, &qso, &mate, &rno, &rso, &rfo, &dist[j], &rev[j], &ridx,
                         &qidx[j]);
      dist[j] = dist[j] - Q > 0 ? dist[j] - Q : 0;
      refMapGetOffsets(ridx, dist[j], &rno, &rfo);
      getSeq(rfp, rfo, rseq.data() + (size_t)j * (R + 1), R);
      getSeqName(rfp, rno, rname.data() + (size_t)j * MAX_SEQ_NAME_LENGTH);
      FILE *qf = mate == 1 ? f1 : f2;
      if (rev[j] == 1) {
        getSeq(qf, qso, tmpq.data(), Q);
        qryGetReverseComplement(tmpq.data(), Q, qseq.data() + (size_t)j * (Q + 1));
        getSeqName(qf, qno, qname.data() + (size_t)j * MAX_SEQ_NAME_LENGTH);
        strcat(qname.data() + (size_t)j * MAX_SEQ_NAME_LENGTH, "*");
      } else {
        getSeq(qf, qso, qseq.data() + (size_t)j * (Q + 1), Q);
        getSeqName(qf, qno, qname.data() + (size_t)j * MAX_SEQ_NAME_LENGTH);
      }
    }
    for (int j = 0; j < cnt; ++j) score[j] = 0;
    g_args = KernelArgs{rseq.data(), R, qseq.data(), Q, m, x, o, e, score.data(), st.data(),
                        en.data(), ln.data(), rcons.data(), qcons.data()};
    const int T = Q + 1 > R ? Q + 1 : R;
    for (int j = 0; j < cnt; ++j) run_block(T, j);
    if (out_format == SAM_OUTPUT_FORMAT) {
      printOutputSam(cnt, qname.data(), rname.data(), score.data(), st.data(), en.data(),
                     ln.data(), comb, qcons.data(), rcons.data(), of);
    } else {
      chooseBestAlignment_paired3_wrap(qname.data(), MAX_QRY_NAME_LENGTH, rev.data(),
                                       rname.data(), MAX_REF_NAME_LENGTH, score.data(),
                                       dist.data(), st.data(), en.data(), cnt, min_frag,
                                       max_frag);
      printOutput_paired2(cnt, qidx.data(), qname.data(), rname.data(), score.data(),
                          dist.data(), st.data(), en.data(), ln.data(), comb, qcons.data(),
                          rcons.data(), of);
    }
  }
  fclose(mf);
  fclose(f1);
  fclose(f2);
  fclose(rfp);
  fclose(of);
  free(per_iter);
  refMapFree();
  return num_matches;
}

}  // extern "C"
