// C ABI and pipeline orchestration.  Everything on the data path runs on the
// context's stream; the host only parses FASTA structure, sizes buffers and
// reads back the few counts that size the next stage.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "handles.h"
#include "internal.h"


using namespace swift;

bool swift::global_bases(const std::vector<RefRecord>& recs, std::vector<uint32_t>* gbase) {
  gbase->assign(recs.size() + 1, 0);
  uint64_t at = kGPad;
  for (size_t r = 0; r < recs.size(); ++r) {
    (*gbase)[r] = (uint32_t)at;
    at += recs[r].cat_len + kGPad;
    if (at >= (1ull << 32) - 64) return false;
  }
  (*gbase)[recs.size()] = (uint32_t)at;
  return true;
}

// The postings as global positions for the SSAHA seeding kernels (left null
// when the reference is too long for them).
int index_global_positions(swift_index* ix, cudaStream_t st) {
  std::vector<uint32_t> gb;
  if (ix->total <= 0 || !global_bases(ix->recs, &gb)) return SWIFT_OK;
  if (cudaMalloc(&ix->d_gbase, gb.size() * sizeof(uint32_t)) != cudaSuccess ||
      cudaMalloc(&ix->d_gpos, (size_t)ix->total * sizeof(uint32_t)) != cudaSuccess ||
      cudaMemcpyAsync(ix->d_gbase, gb.data(), gb.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                      st) != cudaSuccess)
    return SWIFT_E_CUDA;
  launch_global_positions(st, ix->d_post, ix->total, ix->d_gbase, ix->d_gpos);
  return cudaGetLastError() == cudaSuccess ? SWIFT_OK : SWIFT_E_CUDA;
}

namespace {

int fail(swift_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail(ctx, SWIFT_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define CKLAUNCH()                                                                     \
  do {                                                                                 \
    cudaError_t e_ = cudaGetLastError();                                               \
    if (e_ != cudaSuccess)                                                             \
      return fail(ctx, SWIFT_E_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e_)); \
  } while (0)

// Stream-ordered temporaries released at the end of a call.
struct Scratch {
  cudaStream_t st;
  std::vector<void*> ptrs;
  explicit Scratch(cudaStream_t s) : st(s) {}
  ~Scratch() {
    for (void* p : ptrs) cudaFreeAsync(p, st);
  }
  template <typename T>
  cudaError_t get(T** out, size_t count) {
    void* p = nullptr;
    cudaError_t e = cudaMallocAsync(&p, std::max<size_t>(count * sizeof(T), 16), st);
    if (e != cudaSuccess) return e;
    ptrs.push_back(p);
    *out = (T*)p;
    return cudaSuccess;
  }
};

// Work after side_fork may run on ctx->side as well as ctx->st; SideJoin
// orders ctx->st after it again (at join(), or when it leaves scope, so an
// early error return still joins before the scratch is freed on ctx->st).
int side_fork(swift_ctx* ctx) {
  if (!ctx->side) {
    if (cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->join_ev, cudaEventDisableTiming) != cudaSuccess)
      return fail(ctx, SWIFT_E_CUDA, "side stream: " + std::string(cudaGetErrorString(cudaGetLastError())));
  }
  if (cudaEventRecord(ctx->fork_ev, ctx->st) != cudaSuccess ||
      cudaStreamWaitEvent(ctx->side, ctx->fork_ev, 0) != cudaSuccess)
    return fail(ctx, SWIFT_E_CUDA, "side stream fork failed");
  return SWIFT_OK;
}

struct SideJoin {
  swift_ctx* ctx;
  bool armed = false;
  explicit SideJoin(swift_ctx* c) : ctx(c) {}
  int join() {
    armed = false;
    if (cudaEventRecord(ctx->join_ev, ctx->side) != cudaSuccess ||
        cudaStreamWaitEvent(ctx->st, ctx->join_ev, 0) != cudaSuccess)
      return fail(ctx, SWIFT_E_CUDA, "side stream join failed");
    return SWIFT_OK;
  }
  ~SideJoin() {
    if (armed) join();
  }
};

// text copied to the host in this many record ranges (align_into), for
// calls with at least kOutChunkMin records
constexpr int kOutChunks = 16;
constexpr int64_t kOutChunkMin = 65536;

// Text of records [0, n) written in record ranges; with a host buffer each
// range is copied there on the side stream while the next one is written.
struct TextChunks {
  int n_chunks = 1;
  uint64_t rec_at[kOutChunks + 1] = {}, text_at[kOutChunks + 1] = {};
  // Queues the copies of the range starts' text offsets (offs: exclusive
  // scan of the record sizes); they hold after the caller's next
  // synchronisation of st.
  int plan(swift_ctx* ctx, cudaStream_t st, const uint64_t* offs, int64_t n, bool to_host) {
    n_chunks = to_host && n >= kOutChunkMin ? kOutChunks : 1;
    for (int c = 0; c <= n_chunks; ++c) rec_at[c] = (uint64_t)n * c / n_chunks;
    for (int c = 1; c < n_chunks; ++c)
      CK(cudaMemcpyAsync(&text_at[c], offs + rec_at[c], 8, cudaMemcpyDeviceToHost, st));
    return SWIFT_OK;
  }
  // After that synchronisation: the write kernels into text (total bytes),
  // `done` recorded on st after the last one.  The text goes to host_out
  // when it fits host_cap; the copies are complete once st is synchronised.
  int write(swift_ctx* ctx, cudaStream_t st, FormatArgs fa, bool sam, char* text, uint64_t total,
            char* host_out, size_t host_cap, cudaEvent_t done) {
    text_at[0] = 0;
    text_at[n_chunks] = total;
    fa.text = text;
    const bool to_host = host_out && total > 0 && total <= host_cap;
    SideJoin copies(ctx);
    if (to_host) {
      const int rc = side_fork(ctx);
      if (rc != SWIFT_OK) return rc;
      copies.armed = true;
      while (ctx->copy_ev.size() < (size_t)n_chunks) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->copy_ev.push_back(e);
      }
    }
    for (int c = 0; c < n_chunks; ++c) {
      fa.first = (int64_t)rec_at[c];
      fa.n = (int64_t)rec_at[c + 1];
      if (sam)
        launch_sam_write(st, fa);
      else
        launch_format_write(st, fa);
      CKLAUNCH();
      if (to_host && text_at[c + 1] > text_at[c]) {
        CK(cudaEventRecord(ctx->copy_ev[c], st));
        CK(cudaStreamWaitEvent(ctx->side, ctx->copy_ev[c], 0));
        CK(cudaMemcpyAsync(host_out + text_at[c], text + text_at[c], text_at[c + 1] - text_at[c],
                           cudaMemcpyDeviceToHost, ctx->side));
      }
    }
    CK(cudaEventRecord(done, st));
    return to_host ? copies.join() : SWIFT_OK;
  }
};

void keep_pool(int device) {
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
}

// Records of all read strands -> match arrays in match-file order.
__global__ void fill_matches_kernel(const int32_t* __restrict__ nbest, const int3* __restrict__ best,
                                    int max_hits, int64_t n_reads, const uint64_t* __restrict__ roff,
                                    const int32_t* __restrict__ rep, const uint64_t* __restrict__ rep_off,
                                    int64_t n_rep, int32_t* m_read, int32_t* m_strand, int32_t* m_ri,
                                    int32_t* m_sh, int32_t* m_rp) {
  int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n_reads + n_rep) return;
  int64_t read;
  uint64_t o;
  if (v < n_reads) {
    read = v;
    o = roff[v];
  } else {
    read = rep[v - n_reads];
    o = rep_off[v - n_reads];
  }
  for (int s = 0; s < 2; ++s) {
    const int64_t sid = 2 * read + s;
    const int c = nbest[sid];
    for (int h = 0; h < c; ++h) {
      const int3 b = best[sid * max_hits + h];
      m_read[o] = (int32_t)read;
      m_strand[o] = s;
      m_ri[o] = b.x;
      m_sh[o] = b.y;
      m_rp[o] = b.z;
      ++o;
    }
  }
}

// Splits pairs into the packed score pass and the generic kernel.
__global__ void partition_pairs_kernel(const DevPair* __restrict__ pairs, int64_t n, int all_generic,
                                       int32_t* fast, int32_t* n_fast, int32_t* gen,
                                       int32_t* n_gen) {
  // block-aggregated appends: one atomic per block and list
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < n;
  const bool g = valid && (all_generic || (pairs[i].flags & 1));
  const bool f = valid && !g;
  block_append(g, (int32_t)i, gen, n_gen);
  block_append(f, (int32_t)i, fast, n_fast);
}

// Printed pairs of the packed path that have not been traced yet (with
// bounded selection the candidates already were); also counts all printed
// records.
__global__ void traceback_list_kernel(const DevPair* __restrict__ pairs,
                                      const int32_t* __restrict__ keep,
                                      const int32_t* __restrict__ cand, int64_t n, int all_generic,
                                      int32_t* list, int32_t* cnt, int32_t* printed) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool k = i < n && keep[i];
  const bool t = k && !all_generic && !(pairs[i].flags & 1) && !(cand && cand[i] == (int32_t)i);
  block_append(t, (int32_t)i, list, cnt);
  block_count(k, printed);
}

// Order of the exact score pass: the further a pair's LCS bound lies above
// T, the least score that could make it its group's pick (its candidate's
// score, + 1 after the candidate in group order), the later the pair can
// stop (pairs of reads with no true window, whose candidates score low, run
// to the window's end).  Key: that margin in matches, largest first, so
// pairs stopping alike share warps.  A counting sort by key.
__global__ void exact_key_count_kernel(const int32_t* __restrict__ list, const int32_t* __restrict__ n,
                                       const int32_t* __restrict__ ub, const int32_t* __restrict__ cand,
                                       const DevAln* __restrict__ aln, int match,
                                       int32_t* __restrict__ keys, int32_t* hist) {
  __shared__ int32_t h[kSufBlocks + 1];
  if (threadIdx.x <= kSufBlocks) h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < *n) {
    const int32_t p = list[i], c = cand[p];
    const int margin = (ub[p] - (aln[c].score + (p > c ? 1 : 0))) / match;
    const int k = kSufBlocks - min(kSufBlocks, max(margin, 0));
    keys[i] = k;
    atomicAdd(&h[k], 1);
  }
  __syncthreads();
  if (threadIdx.x <= kSufBlocks && h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], h[threadIdx.x]);
}

// Trace order of the candidates (and of every pair with SAM output): they
// stop early on the suffix LCS values.  Key: the LCS bound's shortfall from
// a whole-query match, largest first: reads with no true window (their trace
// runs to the window's end) come first and share warps, and the pairs that
// stop once their alignment ends share the rest.  A counting sort by key.
__global__ void cand_key_count_kernel(const int32_t* __restrict__ list, const int32_t* __restrict__ n,
                                      const uint16_t* __restrict__ lsuf,
                                      const int32_t* __restrict__ q_len, int Q,
                                      int32_t* __restrict__ keys, int32_t* hist) {
  __shared__ int32_t h[kSufBlocks + 1];
  if (threadIdx.x <= kSufBlocks) h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < *n) {
    const int32_t p = list[i];
    const int shortfall = (q_len ? q_len[p] : Q) - (int)lsuf[(int64_t)p * kSufBlocks];
    const int k = kSufBlocks - min(kSufBlocks, max(shortfall, 0));
    keys[i] = k;
    atomicAdd(&h[k], 1);
  }
  __syncthreads();
  if (threadIdx.x <= kSufBlocks && h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], h[threadIdx.x]);
}

__global__ void stop_key_scatter_kernel(const int32_t* __restrict__ list, const int32_t* __restrict__ n,
                                        const int32_t* __restrict__ keys,
                                        const int32_t* __restrict__ hist, int32_t* fill,
                                        int32_t* __restrict__ out) {
  __shared__ int32_t base[kSufBlocks + 1], cnt[kSufBlocks + 1];
  if (threadIdx.x <= kSufBlocks) cnt[threadIdx.x] = 0;
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int k = 0, r = 0;
  if (i < *n) {
    k = keys[i];
    r = atomicAdd(&cnt[k], 1);
  }
  __syncthreads();
  if (threadIdx.x <= kSufBlocks) {
    int b = 0;
    for (int t = 0; t < (int)threadIdx.x; ++t) b += hist[t];
    base[threadIdx.x] = cnt[threadIdx.x] ? b + atomicAdd(&fill[threadIdx.x], cnt[threadIdx.x]) : 0;
  }
  __syncthreads();
  if (i < *n) out[base[k] + r] = list[i];
}

__global__ void read_counts_kernel(const int32_t* __restrict__ nbest, int64_t n_reads,
                                   uint64_t* __restrict__ cnt) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n_reads) cnt[r] = (uint64_t)(nbest[2 * r] + nbest[2 * r + 1]);
}

// Record counts of a wave's record slots (each slot one read's records).
__global__ void slot_counts_kernel(const int32_t* __restrict__ nbest,
                                   const int32_t* __restrict__ slot_read, int64_t n_slots,
                                   uint64_t* __restrict__ cnt) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n_slots) {
    const int64_t r = slot_read[v];
    cnt[v] = (uint64_t)(nbest[2 * r] + nbest[2 * r + 1]);
  }
}

// out[i] = v[at[i]] for i < n (at[i] == len: total, the value past the end)
__global__ void gather_u64_kernel(const uint64_t* __restrict__ v, int64_t len,
                                  const uint64_t* __restrict__ total, const int64_t* __restrict__ at,
                                  int64_t n, uint64_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = at[i] >= len ? *total : v[at[i]];
}

__global__ void aln_to_ref_layout_kernel(const DevAln* __restrict__ aln, int64_t n, float* score,
                                         int32_t* start, int32_t* end, int32_t* len) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  DevAln a = aln[i];
  score[i] = (float)a.score;
  start[i] = a.start;
  end[i] = a.end;
  len[i] = a.len;
}

struct SeedOut {
  int32_t *m_read = nullptr, *m_strand = nullptr, *m_ri = nullptr, *m_sh = nullptr,
          *m_rp = nullptr;
  int64_t n = 0;
  int64_t overflow = 0;
  int64_t launches = 0;
  // SSAHA seeding: the warp kernels' device time and their sector-model
  // bytes (counters on the device, read with the call's last results)
  double kernel_ms = 0;
  unsigned long long* d_model = nullptr;
};

// lookupTable2's position of every posting (src/lookupTable2.cu:75-218,
// searchQueries_paired2's index): the same tuples and bucket order as an
// SSAHA index with the 1000-repeat threshold, each stored there as a FILE
// offset (header end + bases + line count, one less for the first tuple
// written after a line that carried bases over) and read back through
// refMapGetIndexAndPos (src/refMap.cu:166-242), which counts newlines with
// the record's bases-per-line.  The line walk runs on the host over the
// reference bytes once; the postings keep their order.
int ensure_lt2(swift_ctx* ctx, const swift_index* cidx) {
  swift_index* idx = const_cast<swift_index*>(cidx);
  std::lock_guard<std::mutex> lk(idx->pe_mu);
  if (idx->pe_ready) return SWIFT_OK;
  constexpr int kThres = 1000;  // TUPLE_IGNORE_THRES (src/common.h:75)
  std::vector<char> file(idx->file_len + 1, 0);
  CK(cudaMemcpy(file.data(), idx->d_file, idx->file_len, cudaMemcpyDeviceToHost));
  const swift_index* src = idx;
  if (idx->thres != kThres) {
    const int rc = swift_index_build(ctx, file.data(), idx->file_len, idx->k, kThres,
                                     &idx->pe_sub);
    if (rc != SWIFT_OK) return rc;
    src = idx->pe_sub;
  }
  const int k = idx->k;
  const int nr = (int)idx->recs.size();
  std::vector<int64_t> tb(nr + 1, 0);
  for (int r = 0; r < nr; ++r) tb[r + 1] = tb[r] + (int64_t)(idx->recs[r].cat_len / (uint64_t)k);
  std::vector<int32_t> ppos((size_t)std::max<int64_t>(tb[nr], 1), 0);
  std::vector<int8_t> pidx((size_t)std::max<int64_t>(tb[nr], 1), 0);
  // refMapGetIndexAndPos
  auto index_pos = [&](uint32_t off, int* index, int* pos) {
    if ((uint32_t)idx->recs[0].seq_off == off) {
      *index = 0;
      *pos = 0;
      return;
    }
    int id = -1;
    if (nr == 1) {
      id = 0;
    } else {
      for (int i = 1; i < nr; ++i) {
        if ((uint32_t)idx->recs[i - 1].seq_off == off) {
          *index = i - 1;
          *pos = 0;
          return;
        } else if ((uint32_t)idx->recs[i].seq_off > off) {
          id = i - 1;
          break;
        }
      }
      if (id == -1) id = nr - 1;
    }
    const uint32_t so = (uint32_t)idx->recs[id].seq_off, bpl = idx->recs[id].bpl;
    if (bpl == 0) {
      *pos = (int)(off - so);
    } else {
      const uint32_t nl = off >= so ? (off - so) / (bpl + 1) : 0;
      *pos = (int)(off - so) - (int)nl;
    }
    *index = id;
  };
  // the line walk of lookupTable2Create (lines as fgets cuts them)
  {
    std::vector<uint16_t> seen((size_t)idx->nb, 0);
    std::vector<char> line(2 * 100000 + 16);
    const size_t n = idx->file_len;
    int offset = 0, num_bases = 0, num_nl = 0, ri = -1;
    uint32_t ref_pos = 0;
    size_t pos = 0;
    auto code = [](char c) -> uint32_t {
      const uint32_t u = (uint8_t)c & 0xDFu;
      return u == 'C' ? 1u : u == 'G' ? 2u : u == 'T' ? 3u : 0u;
    };
    while (pos < n) {
      size_t lim = std::min<size_t>(n - pos, 100000 - 1);
      const char* nlp = (const char*)memchr(file.data() + pos, '\n', lim);
      const size_t c = nlp ? (size_t)(nlp - (file.data() + pos)) + 1 : lim;
      memcpy(line.data() + offset, file.data() + pos, c);
      pos += c;
      int ll = offset + (int)c;
      if (line[ll - 1] == '\n') --ll;
      if (ll == 0) {
        offset = 0;
      } else if (line[offset] == '>') {
        offset = 0;
        num_bases = 0;
        num_nl = 0;
        ++ri;
        ref_pos = (uint32_t)pos;
      } else {
        const int iters = ll - k + 1;
        int i;
        for (i = 0; i < iters; i += k) {
          uint32_t h = 0;
          for (int t = k - 1; t >= 0; --t) h = (h << 2) | code(line[i + t]);
          if (seen[h] < 65535) ++seen[h];
          if (seen[h] <= kThres) {
            uint32_t off = ref_pos + (uint32_t)num_bases + (uint32_t)i + (uint32_t)num_nl;
            if (offset > 0) {
              off -= 1u;
              offset = 0;
            }
            const int64_t c0 = (int64_t)num_bases + i;  // position in the record
            if (ri >= 0 && ri < nr && c0 / k < tb[ri + 1] - tb[ri]) {
              int id2, p2;
              index_pos(off, &id2, &p2);
              ppos[tb[ri] + c0 / k] = p2;
              pidx[tb[ri] + c0 / k] = (int8_t)id2;
            }
          }
        }
        num_bases += ll;
        ++num_nl;
        offset = ll - i;
        if (offset > 0) memmove(line.data(), line.data() + i, (size_t)offset);
        else offset = 0;
        num_bases -= offset;
      }
    }
  }
  std::vector<uint2> post((size_t)std::max<int64_t>(src->total, 1));
  if (src->total)
    CK(cudaMemcpy(post.data(), src->d_post, src->total * sizeof(uint2), cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < src->total; ++i) {
    const uint32_t r = post[i].y, c0 = post[i].x;
    const int64_t t = tb[r] + c0 / (uint32_t)k;
    post[i] = make_uint2((uint32_t)ppos[t], (uint32_t)(int32_t)pidx[t]);
  }
  CK(cudaMalloc(&idx->d_post_pe, (size_t)std::max<int64_t>(src->total, 1) * sizeof(uint2)));
  if (src->total)
    CK(cudaMemcpy(idx->d_post_pe, post.data(), src->total * sizeof(uint2), cudaMemcpyHostToDevice));
  // their global positions, when every position stays within 64 of its
  // sequence (the keys then keep to their sequence's range)
  std::vector<uint32_t> gb;
  if (idx->d_gbase && src->total && global_bases(idx->recs, &gb)) {
    std::vector<uint32_t> gpos((size_t)src->total);
    bool ok = true;
    for (int64_t i = 0; i < src->total && ok; ++i) {
      const int32_t pos = (int32_t)post[i].x;
      const uint32_t r = post[i].y;
      ok = r < idx->recs.size() && pos >= -64 && pos <= (int64_t)idx->recs[r].cat_len + 64;
      if (ok) gpos[i] = (uint32_t)((int64_t)gb[r] + pos);
    }
    if (ok) {
      CK(cudaMalloc(&idx->d_gpos_pe, (size_t)src->total * sizeof(uint32_t)));
      CK(cudaMemcpy(idx->d_gpos_pe, gpos.data(), src->total * sizeof(uint32_t),
                    cudaMemcpyHostToDevice));
    }
  }
  idx->pe_ready = true;
  return SWIFT_OK;
}

// SSAHA seeding of every strand of a.rd (lookupTable5MapQry +
// mapHits6GetBestHits per strand): the on-chip kernel, then the strands it
// handed over (more hits than its shared tables hold) on the overflow
// kernel.  a.best / a.nbest / a.overflow_list / a.n_overflow (zeroed) are
// the caller's.
int seed_ssaha(swift_ctx* ctx, Scratch& sc, SeedArgs a, SeedOut* out) {
  cudaStream_t st = ctx->st;
  const int64_t n = a.n_reads, ns = 2 * n;
  int32_t* ovl = a.overflow_list;
  int32_t* novl = a.n_overflow;
  int32_t* nbest = a.nbest;
  CK(sc.get(&a.mid_list, (size_t)std::max<int64_t>(ns, 1)));
  CK(sc.get(&a.big_list, (size_t)std::max<int64_t>(ns, 1)));
  CK(sc.get(&a.n_mid, 2));
  CK(cudaMemsetAsync(a.n_mid, 0, 2 * sizeof(int32_t), st));
  a.n_big = a.n_mid + 1;
  if (!out->d_model) {
    CK(sc.get(&out->d_model, kSeedModelSlots));
    CK(cudaMemsetAsync(out->d_model, 0, kSeedModelSlots * sizeof(unsigned long long), st));
  }
  a.model_bytes = out->d_model;
  CK(cudaEventRecord(ctx->ev[9], st));
  launch_seed(st, a);
  CKLAUNCH();
  CK(cudaEventRecord(ctx->ev[10], st));
  out->launches += n > 0 ? 3 : 0;
  int32_t h_novl = 0;
  CK(cudaMemcpyAsync(&h_novl, novl, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (n > 0) {
    float t = 0;
    cudaEventElapsedTime(&t, ctx->ev[9], ctx->ev[10]);
    out->kernel_ms += t;
  }
  out->overflow += h_novl;
  if (h_novl > 0) {
    std::vector<int32_t> list(h_novl), nb(ns);
    CK(cudaMemcpyAsync(list.data(), ovl, h_novl * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(nb.data(), nbest, ns * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::vector<uint64_t> toff(h_novl);
    std::vector<uint32_t> tsz(h_novl);
    uint64_t tot = 0;
    for (int i = 0; i < h_novl; ++i) {
      uint32_t hits = (uint32_t)(-nb[list[i]]);
      uint32_t S = 64;
      while (S < 2 * hits) S <<= 1;
      toff[i] = tot;
      tsz[i] = S;
      tot += 2 * (uint64_t)S;  // S keys (8 B) + 2 S counters (4 B)
    }
    uint64_t* scratch;
    uint64_t* d_toff;
    uint32_t* d_tsz;
    CK(sc.get(&scratch, tot));
    CK(sc.get(&d_toff, h_novl));
    CK(sc.get(&d_tsz, h_novl));
    CK(cudaMemsetAsync(scratch, 0, tot * sizeof(uint64_t), st));
    CK(cudaMemcpyAsync(d_toff, toff.data(), h_novl * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_tsz, tsz.data(), h_novl * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    a.scratch = scratch;
    launch_seed_overflow(st, a, h_novl, d_toff, d_tsz);
    CKLAUNCH();
    out->launches += 1;
  }
  return SWIFT_OK;
}

// The lt13 tables of an index (seed13.cu), built once on first use: the
// composite of every posting, and refPosHashMap per tuple id, which keeps a
// tuple's hash when it is among the first thres occurrences of that hash in
// file order (lookupTable13Create, src/lookupTable13.cu:101-140).  The
// hashes come from the device; the occurrence ranks are counted on the host
// in one pass over the tuples.
int ensure_lt13(swift_ctx* ctx, const swift_index* cidx) {
  swift_index* idx = const_cast<swift_index*>(cidx);
  std::lock_guard<std::mutex> lk(idx->lt13_mu);
  if (idx->lt13_ready) return SWIFT_OK;
  const int nr = (int)idx->recs.size();
  if (nr > kMaxRefs13)
    return fail(ctx, SWIFT_E_LIMIT, "lt13 seeding: more than 64 reference sequences (the "
                                    "composite position keeps the index above bit 25 of an int)");
  if (idx->thres > kMaxThres13)
    return fail(ctx, SWIFT_E_LIMIT, "lt13 seeding: ignore threshold above 1176 (the reference "
                                    "kernel's shared arrays would overflow)");
  const int k = idx->k;
  std::vector<int64_t> tb(nr + 1, 0), nt(std::max(nr, 1), 0);
  std::vector<uint64_t> tbu(nr + 1, 0);
  for (int r = 0; r < nr; ++r) {
    nt[r] = (int64_t)(idx->recs[r].cat_len / (uint64_t)k);
    if (nt[r] >= (1 << 25) - 64)
      return fail(ctx, SWIFT_E_LIMIT, "lt13 seeding: a sequence's tuples do not fit the "
                                      "composite position");
    tb[r + 1] = tb[r] + nt[r];
    tbu[r + 1] = (uint64_t)tb[r + 1];
  }
  const int64_t n_tup = tb[nr];
  cudaStream_t st = ctx->st;
  std::vector<uint32_t> hash((size_t)std::max<int64_t>(n_tup, 1));
  {
    Scratch sc(st);
    uint64_t* d_tb;
    uint32_t* d_hash;
    CK(sc.get(&d_tb, (size_t)nr + 1));
    CK(sc.get(&d_hash, (size_t)std::max<int64_t>(n_tup, 1)));
    CK(cudaMemcpyAsync(d_tb, tbu.data(), (nr + 1) * 8, cudaMemcpyHostToDevice, st));
    launch_tuple_hash13(st, idx->d_packed, idx->d_recs, d_tb, nr, (uint64_t)n_tup, k, d_hash);
    CKLAUNCH();
    CK(cudaMemcpyAsync(hash.data(), d_hash, n_tup * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  std::vector<int32_t> map((size_t)std::max<int64_t>(n_tup, 1), 0);
  std::vector<uint16_t> seen((size_t)idx->nb, 0);
  int64_t max_comp = 0;
  for (int r = 0; r < nr; ++r)
    for (int64_t c = 0; c < nt[r]; ++c) {
      const int64_t t = tb[r] + c;
      const uint32_t h = hash[t];
      if (seen[h] < 65535) ++seen[h];
      if (seen[h] <= (uint32_t)idx->thres) {
        map[t] = (int32_t)h;
        max_comp = std::max<int64_t>(max_comp, ((int64_t)r << 25) + c);
      }
    }
  CK(cudaMalloc(&idx->d_map13, (size_t)std::max<int64_t>(n_tup, 1) * 4));
  CK(cudaMalloc(&idx->d_vals13, (size_t)std::max<int64_t>(idx->total, 1) * 4));
  CK(cudaMalloc(&idx->d_tbase13, (size_t)std::max(nr, 1) * 8));
  CK(cudaMalloc(&idx->d_ntup13, (size_t)std::max(nr, 1) * 8));
  CK(cudaMemcpyAsync(idx->d_map13, map.data(), n_tup * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(idx->d_tbase13, tb.data(), nr * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(idx->d_ntup13, nt.data(), nr * 8, cudaMemcpyHostToDevice, st));
  launch_composites13(st, idx->d_post, idx->total, k, idx->d_vals13);
  CKLAUNCH();
  CK(cudaStreamSynchronize(st));
  idx->max_comp13 = max_comp;
  idx->n_tup13 = n_tup;
  idx->lt13_ready = true;
  return SWIFT_OK;
}

// Phase 1 for resident reads: fills the match arrays (allocated in sc).
// seeder 0: SSAHA (searchQueries3, with its stale trailing batch); 1: lt13
// seed-and-extend (search2Queries: every read once, 3 hits per strand).
int run_seed(swift_ctx* ctx, const swift_index* idx, const swift_reads* rd, int max_hits,
             int seeder, Scratch& sc, SeedOut* out, std::vector<WaveReq>* wave = nullptr) {
  const int64_t n = rd->n;
  const int64_t ns = 2 * n;
  cudaStream_t st = ctx->st;
  if (seeder == 1) {
    const int rc13 = ensure_lt13(ctx, idx);
    if (rc13 != SWIFT_OK) return rc13;
    max_hits = 3;  // search2Queries fixes maxNumHits at 3 (src/search2.cu:62)
  }
  int3* best;
  int32_t *nbest, *ovl, *novl;
  CK(sc.get(&best, (size_t)std::max<int64_t>(ns, 1) * max_hits));
  CK(sc.get(&nbest, (size_t)std::max<int64_t>(ns, 1)));
  CK(sc.get(&ovl, (size_t)std::max<int64_t>(ns, 1)));
  CK(sc.get(&novl, 2));
  CK(cudaMemsetAsync(novl, 0, 2 * sizeof(int32_t), st));
  if (seeder == 1) {
    Seed13Args s13;
    memset(&s13, 0, sizeof(s13));
    s13.reads = rd->d_bytes;
    s13.rd = rd->d_rd;
    s13.n_reads = n;
    s13.groups = idx->d_groups;
    s13.cstart = idx->d_cstart;
    s13.vals = idx->d_vals13;
    s13.map = idx->d_map13;
    s13.tbase = idx->d_tbase13;
    s13.ntup = idx->d_ntup13;
    s13.nrefs = (int)idx->recs.size();
    s13.max_comp = idx->max_comp13;
    s13.k = idx->k;
    s13.best = best;
    s13.nbest = nbest;
    s13.overflow_list = ovl;
    s13.n_overflow = novl;
    launch_seed13(st, s13, false);
    CKLAUNCH();
    out->launches += ns > 0 ? 1 : 0;
    int32_t h_novl = 0;
    CK(cudaMemcpyAsync(&h_novl, novl, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    out->overflow = h_novl;
    if (h_novl > 0) {  // strands redone with the reference's full array sizes
      s13.list = ovl;
      s13.n_list = h_novl;
      s13.n_overflow = novl + 1;
      launch_seed13(st, s13, true);
      CKLAUNCH();
      out->launches += 1;
    }
  }
  if (seeder != 1) {
    SeedArgs a;
    memset(&a, 0, sizeof(a));
    a.reads = rd->d_bytes;
    a.rd = rd->d_rd;
    a.n_reads = n;
    a.max_len = rd->max_len;
    a.offsets = idx->d_offsets;
    a.groups = idx->d_groups;
    a.cstart = idx->d_cstart;
    a.postings = idx->d_post;
    a.gpos = idx->d_gpos;
    a.gbase = idx->d_gbase;
    a.n_recs = (int)idx->recs.size();
    a.k = idx->k;
    a.max_hits = max_hits;
    a.best = best;
    a.nbest = nbest;
    a.overflow_list = ovl;
    a.n_overflow = novl;
    const int rcs = seed_ssaha(ctx, sc, a, out);
    if (rcs != SWIFT_OK) return rcs;
  }
  if (wave) {
    // a merged wave: each request's records in its order (its reads, then
    // the stale reads of its own 16-read loop), requests one after another
    const size_t W = wave->size();
    std::vector<int32_t> slots;
    std::vector<int64_t> slot_base(W + 1);
    for (size_t r = 0; r < W; ++r) {
      slot_base[r] = (int64_t)slots.size();
      const WaveReq& q = (*wave)[r];
      for (int64_t i = 0; i < q.n; ++i) slots.push_back((int32_t)(q.read0 + i));
      if (seeder != 1) slots.insert(slots.end(), q.repeats.begin(), q.repeats.end());
    }
    slot_base[W] = (int64_t)slots.size();
    const int64_t nv = (int64_t)slots.size();
    int32_t* d_slots;
    int64_t* d_sb;
    uint64_t *cnt, *roff, *tot_d, *d_rec0;
    void* tmp;
    CK(sc.get(&d_slots, (size_t)std::max<int64_t>(nv, 1)));
    CK(sc.get(&d_sb, W + 1));
    CK(sc.get(&cnt, (size_t)std::max<int64_t>(nv, 1)));
    CK(sc.get(&roff, (size_t)std::max<int64_t>(nv, 1)));
    CK(sc.get(&tot_d, 1));
    CK(sc.get(&d_rec0, W + 1));
    CK(sc.get((uint8_t**)&tmp, scan_temp_bytes(nv)));
    if (nv) CK(cudaMemcpyAsync(d_slots, slots.data(), nv * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_sb, slot_base.data(), (W + 1) * 8, cudaMemcpyHostToDevice, st));
    if (nv) slot_counts_kernel<<<(unsigned)((nv + 255) / 256), 256, 0, st>>>(nbest, d_slots, nv, cnt);
    CKLAUNCH();
    out->launches += (nv > 0 ? 1 : 0) + exclusive_scan_u64(st, cnt, roff, nv, tmp, tot_d);
    gather_u64_kernel<<<(unsigned)((W + 1 + 255) / 256), 256, 0, st>>>(roff, nv, tot_d, d_sb,
                                                                       (int64_t)W + 1, d_rec0);
    CKLAUNCH();
    ++out->launches;
    std::vector<uint64_t> rec0(W + 1);
    CK(cudaMemcpyAsync(rec0.data(), d_rec0, (W + 1) * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const uint64_t total = rec0[W];
    for (size_t r = 0; r < W; ++r) {
      (*wave)[r].rec0 = (int64_t)rec0[r];
      (*wave)[r].nm = (int64_t)(rec0[r + 1] - rec0[r]);
    }
    const size_t tn = std::max<uint64_t>(total, 1);
    CK(sc.get(&out->m_read, tn));
    CK(sc.get(&out->m_strand, tn));
    CK(sc.get(&out->m_ri, tn));
    CK(sc.get(&out->m_sh, tn));
    CK(sc.get(&out->m_rp, tn));
    if (nv > 0)  // every slot as a "repeat" entry: read slots[v] at offset roff[v]
      fill_matches_kernel<<<(unsigned)((nv + 255) / 256), 256, 0, st>>>(
          nbest, best, max_hits, 0, nullptr, d_slots, roff, nv, out->m_read, out->m_strand,
          out->m_ri, out->m_sh, out->m_rp);
    CKLAUNCH();
    out->launches += nv > 0 ? 1 : 0;
    out->n = (int64_t)total;
    return SWIFT_OK;
  }
  // per-read record counts -> offsets
  uint64_t *cnt, *roff, *tot_d;
  void* tmp;
  CK(sc.get(&cnt, (size_t)std::max<int64_t>(n, 1)));
  CK(sc.get(&roff, (size_t)std::max<int64_t>(n, 1)));
  CK(sc.get(&tot_d, 1));
  CK(sc.get((uint8_t**)&tmp, scan_temp_bytes(n)));
  if (n > 0) read_counts_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nbest, n, cnt);
  CKLAUNCH();
  out->launches += (n > 0 ? 1 : 0) + exclusive_scan_u64(st, cnt, roff, n, tmp, tot_d);
  CKLAUNCH();
  uint64_t total_in = 0;
  CK(cudaMemcpyAsync(&total_in, tot_d, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
  // the stale trailing batch of searchQueries3; search2Queries has none
  const std::vector<int32_t> no_rep;
  const std::vector<int32_t>& rep = seeder == 1 ? no_rep : rd->repeats;
  std::vector<uint64_t> rep_cnt(rep.size()), rep_off(rep.size());
  std::vector<int32_t> rep_nb(2 * rep.size());
  for (size_t i = 0; i < rep.size(); ++i)
    CK(cudaMemcpyAsync(&rep_nb[2 * i], nbest + 2 * (int64_t)rep[i], 2 * sizeof(int32_t),
                       cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  uint64_t total = total_in;
  for (size_t i = 0; i < rep.size(); ++i) {
    rep_off[i] = total;
    total += (uint64_t)(rep_nb[2 * i] + rep_nb[2 * i + 1]);
  }
  int32_t* d_rep;
  uint64_t* d_rep_off;
  CK(sc.get(&d_rep, std::max<size_t>(rep.size(), 1)));
  CK(sc.get(&d_rep_off, std::max<size_t>(rep.size(), 1)));
  if (!rep.empty()) {
    CK(cudaMemcpyAsync(d_rep, rep.data(), rep.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_rep_off, rep_off.data(), rep.size() * sizeof(uint64_t),
                       cudaMemcpyHostToDevice, st));
  }
  const size_t tn = std::max<uint64_t>(total, 1);
  CK(sc.get(&out->m_read, tn));
  CK(sc.get(&out->m_strand, tn));
  CK(sc.get(&out->m_ri, tn));
  CK(sc.get(&out->m_sh, tn));
  CK(sc.get(&out->m_rp, tn));
  const int64_t nv = n + (int64_t)rep.size();
  if (nv > 0)
    fill_matches_kernel<<<(unsigned)((nv + 255) / 256), 256, 0, st>>>(
        nbest, best, max_hits, n, roff, d_rep, d_rep_off, (int64_t)rep.size(), out->m_read,
        out->m_strand, out->m_ri, out->m_sh, out->m_rp);
  CKLAUNCH();
  out->launches += nv > 0 ? 1 : 0;
  out->n = (int64_t)total;
  return SWIFT_OK;
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// transient: buffers for one call, from the stream-ordered pool of ctx->st
// (freed in stream order by swift_reads_destroy)
int upload_reads(swift_ctx* ctx, const char* b, size_t len, swift_reads** out,
                 double* parse_ms = nullptr, double* h2d_ms = nullptr, bool transient = false,
                 int max_read = kReadMax) {
  // bytes to the device, then the record structure found there (parse.cu)
  cudaStream_t st = ctx->st;
  swift_reads* r = new swift_reads();
  r->device = ctx->device;
  r->len = len;
  if (transient) r->pool_st = st;
  auto t0 = std::chrono::steady_clock::now();
  auto bail = [&](int code, const std::string& m) {
    swift_reads_destroy(r);
    return fail(ctx, code, m);
  };
#define CKR(call)                                                                         \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) return bail(SWIFT_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
  CKR(transient ? cudaMallocAsync(&r->d_bytes, len + 64, st) : cudaMalloc(&r->d_bytes, len + 64));
  CKR(cudaMemcpyAsync(r->d_bytes, b, len, cudaMemcpyHostToDevice, st));
  CKR(cudaStreamSynchronize(st));
  if (h2d_ms) *h2d_ms = ms_since(t0);
  t0 = std::chrono::steady_clock::now();
  {
    Scratch sc(st);
    const uint64_t tiles = parse_tiles(len);
    uint32_t *cnt, *off, *n_nl_d;
    unsigned long long* err;
    ParseSummary* sum;
    void* tmp;
    CKR(sc.get(&cnt, std::max<uint64_t>(tiles, 1)));
    CKR(sc.get(&off, std::max<uint64_t>(tiles, 1)));
    CKR(sc.get(&n_nl_d, 1));
    CKR(sc.get(&err, 1));
    CKR(sc.get(&sum, 1));
    CKR(sc.get((uint8_t**)&tmp, scan_temp_bytes((int64_t)tiles)));
    const ParseSummary init = {INT32_MAX, 0, 0, 0};
    CKR(cudaMemcpyAsync(sum, &init, sizeof(init), cudaMemcpyHostToDevice, st));
    CKR(cudaMemsetAsync(err, 0xFF, sizeof(unsigned long long), st));
    launch_parse_tiles(st, r->d_bytes, len, cnt, err);
    exclusive_scan_u32(st, cnt, off, (int64_t)tiles, tmp, n_nl_d);
    CKR(cudaGetLastError());
    uint32_t n_nl = 0;
    CKR(cudaMemcpyAsync(&n_nl, n_nl_d, 4, cudaMemcpyDeviceToHost, st));
    CKR(cudaStreamSynchronize(st));
    const uint64_t n_lines = n_nl + ((len > 0 && b[len - 1] != '\n') ? 1 : 0);
    uint64_t* nl;
    CKR(sc.get(&nl, std::max<uint64_t>(n_nl, 1)));
    const size_t rd_bytes = std::max<uint64_t>(n_lines / 2, 1) * sizeof(DevRead);
    CKR(transient ? cudaMallocAsync(&r->d_rd, rd_bytes, st) : cudaMalloc(&r->d_rd, rd_bytes));
    launch_parse_newlines(st, r->d_bytes, len, off, nl);
    launch_parse_lines(st, r->d_bytes, len, nl, n_nl, n_lines, r->d_rd, sum, err, max_read);
    CKR(cudaGetLastError());
    unsigned long long h_err = 0;
    ParseSummary h_sum;
    CKR(cudaMemcpyAsync(&h_err, err, sizeof(h_err), cudaMemcpyDeviceToHost, st));
    CKR(cudaMemcpyAsync(&h_sum, sum, sizeof(h_sum), cudaMemcpyDeviceToHost, st));
    CKR(cudaStreamSynchronize(st));
    if (h_err != ~0ull) {
      std::string m;
      const int code = parse_error((uint32_t)(h_err & 0xFF), h_err >> 8, &m, max_read);
      return bail(code, m);
    }
    r->n = (int64_t)(n_lines / 2);
    r->n_gt = (int64_t)((n_lines + 1) / 2);  // '>' occurs only at header starts
    r->first_len = h_sum.first_len;
    r->min_len = r->n ? h_sum.min_len : 0;
    r->max_len = h_sum.max_len;
  }
#undef CKR
  r->repeats = phase1_stale_repeats(r->n, r->n_gt);
  if (parse_ms) *parse_ms = ms_since(t0);
  *out = r;
  return SWIFT_OK;
}

}  // namespace

extern "C" {

void swift_params_default(swift_params* p) {
  p->seed_len = 12;
  p->ignore_thres = 1000;
  p->max_hits = 3;
  p->match = 2;
  p->mismatch = -1;
  p->gap_open = -10;
  p->gap_ext = -1;
  p->qry_len = 0;
  p->device_mem = 0;
  p->out_format = 0;
  p->seeder = 0;
  p->max_read_len = 0;
}

int swift_ctx_create(int device, void* stream, swift_ctx** out) {
  if (!out) return SWIFT_E_ARG;
  swift_ctx* ctx = new swift_ctx();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) {
    if (stream) {
      ctx->st = (cudaStream_t)stream;
    } else {
      e = cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking);
      ctx->own_stream = true;
    }
  }
  if (e == cudaSuccess) {
    size_t fr = 0, tot = 0;
    e = cudaMemGetInfo(&fr, &tot);
    ctx->total_mem = (int64_t)tot;
  }
  for (int i = 0; i < kCtxEvents && e == cudaSuccess; ++i) e = cudaEventCreate(&ctx->ev[i]);
  if (e != cudaSuccess) {
    delete ctx;
    return SWIFT_E_CUDA;
  }
  keep_pool(device);
  *out = ctx;
  return SWIFT_OK;
}

int swift_ctx_destroy(swift_ctx* ctx) {
  if (!ctx) return SWIFT_OK;
  cudaSetDevice(ctx->device);
  if (ctx->st) cudaStreamSynchronize(ctx->st);
  if (ctx->d_text) cudaFree(ctx->d_text);
  for (int i = 0; i < kCtxEvents; ++i)
    if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
  if (ctx->side) {
    cudaStreamSynchronize(ctx->side);
    cudaStreamDestroy(ctx->side);
    cudaEventDestroy(ctx->fork_ev);
    cudaEventDestroy(ctx->join_ev);
  }
  for (cudaEvent_t e : ctx->chunk_ev) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->copy_ev) cudaEventDestroy(e);
  if (ctx->own_stream) cudaStreamDestroy(ctx->st);
  delete ctx;
  return SWIFT_OK;
}

const char* swift_last_error(const swift_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int swift_ctx_set_sw_path(swift_ctx* ctx, int32_t path) {
  if (!ctx || path < 0 || path > 2) return SWIFT_E_ARG;
  ctx->sw_path = path;
  return SWIFT_OK;
}

int swift_ctx_set_tuning(swift_ctx* ctx, int32_t mode) {
  if (!ctx || mode < 0 || mode > 64) return SWIFT_E_ARG;
  ctx->tuning = mode;
  return SWIFT_OK;
}

int swift_ctx_info(const swift_ctx* ctx, int64_t* total_mem, int32_t* sm_count) {
  if (!ctx) return SWIFT_E_ARG;
  if (total_mem) *total_mem = ctx->total_mem;
  if (sm_count) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess)
      return SWIFT_E_CUDA;
    *sm_count = v;
  }
  return SWIFT_OK;
}

void swift_free(void* p) { free(p); }

int swift_peak_dpx(swift_ctx* ctx, double* cells_per_s) {
  if (!ctx || !cells_per_s) return fail(ctx, SWIFT_E_ARG, "null argument");
  CK(cudaSetDevice(ctx->device));
  double ips = 0;
  int rc = measure_dpx_peak(ctx->st, ctx->device, &ips);
  if (rc != SWIFT_OK) return fail(ctx, rc, "calibration kernel failed");
  *cells_per_s = 2.0 * ips;
  return SWIFT_OK;
}

int swift_index_build(swift_ctx* ctx, const char* ref, size_t len, int32_t k, int32_t thres,
                      swift_index** out) {
  if (!ctx || !ref || !out) return fail(ctx, SWIFT_E_ARG, "null argument");
  if (k < 1 || k > 15) return fail(ctx, SWIFT_E_ARG, "seed length outside 1..15");
  if (thres < 0) return fail(ctx, SWIFT_E_ARG, "negative ignore threshold");
  CK(cudaSetDevice(ctx->device));
  HostRef hr;
  int rc = parse_reference(ref, len, &hr, &ctx->err);
  if (rc != SWIFT_OK) return rc;
  cudaStream_t st = ctx->st;
  swift_index* ix = new swift_index();
  ix->device = ctx->device;
  ix->k = k;
  ix->thres = thres;
  ix->file_len = len;
  ix->recs = hr.recs;
  ix->cat_len = hr.cat_len;
  ix->nb = (int64_t)1 << (2 * k);
  const int nr = (int)hr.recs.size();
  std::vector<DevRecord> dr(nr);
  std::vector<uint64_t> tbase(nr + 1, 0);
  for (int i = 0; i < nr; ++i) {
    memset(&dr[i], 0, sizeof(DevRecord));
    dr[i].seq_off = hr.recs[i].seq_off;
    dr[i].cat_start = hr.recs[i].cat_start;
    dr[i].cat_len = hr.recs[i].cat_len;
    dr[i].bpl = hr.recs[i].bpl;
    dr[i].name_len = hr.recs[i].name_len;
    memcpy(dr[i].name, hr.recs[i].name, kNameMax);
    dr[i].regular = hr.recs[i].regular ? 1 : 0;
    tbase[i + 1] = tbase[i] + hr.recs[i].cat_len / (uint64_t)k;
  }
  const uint64_t n_tuples = tbase[nr];
  const int64_t n_lines = (int64_t)hr.line_len.size();
  const int64_t n_words = (int64_t)((hr.cat_len + 15) / 16);
  auto bail = [&](int code, const std::string& m) {
    swift_index_destroy(ix);
    return fail(ctx, code, m);
  };
#define CKI(call)                                                                       \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) return bail(SWIFT_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
  CKI(cudaMalloc(&ix->d_file, len + 64));
  CKI(cudaMalloc(&ix->d_recs, std::max(nr, 1) * sizeof(DevRecord)));
  CKI(cudaMalloc(&ix->d_cat, (size_t)n_words * 16 + 64));
  CKI(cudaMalloc(&ix->d_packed, ((size_t)n_words + 2) * sizeof(uint32_t)));
  CKI(cudaMalloc(&ix->d_odd, (size_t)odd_bits_words(n_words) * sizeof(uint32_t)));
  CKI(cudaMalloc(&ix->d_count, (size_t)ix->nb * sizeof(uint32_t)));
  CKI(cudaMalloc(&ix->d_offsets, ((size_t)ix->nb + 1) * sizeof(uint32_t)));
  {
    Scratch sc(st);
    uint64_t *d_src, *d_dst, *d_tbase;
    uint32_t *d_len, *d_eff, *d_cursor;
    void* tmp;
    CKI(sc.get(&d_src, n_lines));
    CKI(sc.get(&d_dst, n_lines));
    CKI(sc.get(&d_len, n_lines));
    CKI(sc.get(&d_tbase, nr + 1));
    CKI(sc.get(&d_eff, (size_t)ix->nb));
    CKI(sc.get(&d_cursor, (size_t)ix->nb));
    CKI(sc.get((uint8_t**)&tmp, scan_temp_bytes(ix->nb)));
    CKI(cudaMemcpyAsync(ix->d_file, ref, len, cudaMemcpyHostToDevice, st));
    CKI(cudaMemcpyAsync(ix->d_recs, dr.data(), nr * sizeof(DevRecord), cudaMemcpyHostToDevice, st));
    if (n_lines) {
      CKI(cudaMemcpyAsync(d_src, hr.line_src.data(), n_lines * 8, cudaMemcpyHostToDevice, st));
      CKI(cudaMemcpyAsync(d_dst, hr.line_dst.data(), n_lines * 8, cudaMemcpyHostToDevice, st));
      CKI(cudaMemcpyAsync(d_len, hr.line_len.data(), n_lines * 4, cudaMemcpyHostToDevice, st));
    }
    CKI(cudaMemcpyAsync(d_tbase, tbase.data(), (nr + 1) * 8, cudaMemcpyHostToDevice, st));
    CKI(cudaMemsetAsync(ix->d_cat, 0, (size_t)n_words * 16 + 64, st));
    CKI(cudaMemsetAsync(ix->d_packed, 0, ((size_t)n_words + 2) * sizeof(uint32_t), st));
    CKI(cudaMemsetAsync(ix->d_count, 0, (size_t)ix->nb * sizeof(uint32_t), st));
    CKI(cudaMemsetAsync(d_cursor, 0, (size_t)ix->nb * sizeof(uint32_t), st));
    launch_compact_lines(st, ix->d_file, d_src, d_dst, d_len, n_lines, ix->d_cat);
    launch_pack2bit(st, ix->d_cat, n_words, ix->d_packed);
    launch_odd_bits(st, ix->d_cat, n_words, ix->d_odd);
    launch_count_tuples(st, ix->d_packed, ix->d_recs, d_tbase, nr, n_tuples, k, ix->d_count);
    launch_threshold(st, ix->d_count, ix->nb, (uint32_t)thres, d_eff);
    exclusive_scan_u32(st, d_eff, ix->d_offsets, ix->nb, tmp, ix->d_offsets + ix->nb);
    uint32_t total = 0;
    CKI(cudaMemcpyAsync(&total, ix->d_offsets + ix->nb, 4, cudaMemcpyDeviceToHost, st));
    CKI(cudaStreamSynchronize(st));
    ix->total = total;
    CKI(cudaMalloc(&ix->d_post, std::max<size_t>(total, 1) * sizeof(uint2)));
    launch_scatter_tuples(st, ix->d_packed, ix->d_recs, d_tbase, nr, n_tuples, k, (uint32_t)thres,
                          ix->d_count, ix->d_offsets, d_cursor, ix->d_post);
    launch_order_buckets(st, ix->d_offsets, ix->nb, ix->d_post);
    CKI(cudaGetLastError());
    if (index_global_positions(ix, st) != SWIFT_OK) CKI(cudaErrorMemoryAllocation);
    const int64_t ng = (ix->nb + 63) / 64;
    uint32_t *d_bits32, *d_gcnt, *d_grank, *d_nocc;
    CKI(sc.get(&d_bits32, (size_t)(ix->nb + 31) / 32));
    CKI(sc.get(&d_gcnt, (size_t)ng));
    CKI(sc.get(&d_grank, (size_t)ng));
    CKI(sc.get(&d_nocc, 1));
    CKI(cudaMalloc(&ix->d_groups, (size_t)ng * sizeof(uint4)));
    CKI(cudaMalloc(&ix->d_cstart, ((size_t)total + 1) * sizeof(uint32_t)));
    build_bucket_directory(st, ix->d_offsets, ix->nb, d_bits32, d_gcnt, d_grank, tmp, d_nocc,
                           ix->d_groups, ix->d_cstart);
    CKI(cudaGetLastError());
  }
  CKI(cudaStreamSynchronize(st));
#undef CKI
  *out = ix;
  return SWIFT_OK;
}

int swift_index_destroy(swift_index* ix) {
  if (!ix) return SWIFT_OK;
  cudaSetDevice(ix->device);
  cudaFree(ix->d_file);
  cudaFree(ix->d_recs);
  cudaFree(ix->d_cat);
  cudaFree(ix->d_packed);
  cudaFree(ix->d_odd);
  cudaFree(ix->d_count);
  cudaFree(ix->d_offsets);
  cudaFree(ix->d_groups);
  cudaFree(ix->d_cstart);
  cudaFree(ix->d_post);
  cudaFree(ix->d_vals13);
  cudaFree(ix->d_map13);
  cudaFree(ix->d_tbase13);
  cudaFree(ix->d_ntup13);
  cudaFree(ix->d_post_pe);
  cudaFree(ix->d_gpos);
  cudaFree(ix->d_gbase);
  cudaFree(ix->d_gpos_pe);
  if (ix->pe_sub) swift_index_destroy(ix->pe_sub);
  delete ix;
  return SWIFT_OK;
}

int swift_index_info(swift_ctx* ctx, const swift_index* ix, int32_t* n_refs, int64_t* total,
                     int64_t* nb) {
  if (!ix) return fail(ctx, SWIFT_E_ARG, "null index");
  if (n_refs) *n_refs = (int32_t)ix->recs.size();
  if (total) *total = ix->total;
  if (nb) *nb = ix->nb;
  return SWIFT_OK;
}

int swift_index_export(swift_ctx* ctx, const swift_index* ix, int32_t* lookup, int32_t* repeats,
                       int8_t* ref_idx, int32_t* ref_pos) {
  if (!ctx || !ix) return fail(ctx, SWIFT_E_ARG, "null argument");
  CK(cudaSetDevice(ctx->device));
  std::vector<uint32_t> cnt(ix->nb), off(ix->nb + 1);
  std::vector<uint2> post(std::max<int64_t>(ix->total, 1));
  CK(cudaMemcpy(cnt.data(), ix->d_count, ix->nb * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(off.data(), ix->d_offsets, (ix->nb + 1) * 4, cudaMemcpyDeviceToHost));
  if (ix->total) CK(cudaMemcpy(post.data(), ix->d_post, ix->total * 8, cudaMemcpyDeviceToHost));
  for (int64_t h = 0; h < ix->nb; ++h) {
    const bool kept = cnt[h] > 0 && cnt[h] <= (uint32_t)ix->thres;
    if (lookup) lookup[h] = kept ? (int32_t)off[h] + 1 : 0;
    if (repeats) repeats[h] = (int32_t)cnt[h];
  }
  if (ref_idx) {
    ref_idx[0] = -1;
    for (int64_t i = 0; i < ix->total; ++i) ref_idx[i + 1] = (int8_t)post[i].y;
  }
  if (ref_pos) {
    ref_pos[0] = -1;
    for (int64_t i = 0; i < ix->total; ++i) ref_pos[i + 1] = (int32_t)post[i].x;
  }
  return SWIFT_OK;
}

int swift_reads_upload(swift_ctx* ctx, const char* b, size_t len, swift_reads** out) {
  if (!ctx || !b || !out) return fail(ctx, SWIFT_E_ARG, "null argument");
  CK(cudaSetDevice(ctx->device));
  // reads up to the longest the pipeline takes; each call checks its own
  // limit (swift_params.max_read_len)
  return upload_reads(ctx, b, len, out, nullptr, nullptr, false, kSeedReadMax);
}

int swift_reads_destroy(swift_reads* r) {
  if (!r) return SWIFT_OK;
  cudaSetDevice(r->device);
  if (r->pool_st) {
    if (r->d_bytes) cudaFreeAsync(r->d_bytes, r->pool_st);
    if (r->d_rd) cudaFreeAsync(r->d_rd, r->pool_st);
  } else {
    cudaFree(r->d_bytes);
    cudaFree(r->d_rd);
  }
  delete r;
  return SWIFT_OK;
}

namespace {

int seed_records(swift_ctx* ctx, const swift_index* idx, const char* reads, size_t len,
                 int32_t max_hits, int seeder, swift_match* out, int64_t cap, int64_t* n) {
  if (!ctx || !idx || !reads || !n) return fail(ctx, SWIFT_E_ARG, "null argument");
  if (max_hits < 1 || max_hits > 64) return fail(ctx, SWIFT_E_ARG, "max_hits outside 1..64");
  CK(cudaSetDevice(ctx->device));
  swift_reads* rd = nullptr;
  int rc = upload_reads(ctx, reads, len, &rd, nullptr, nullptr, true);
  if (rc != SWIFT_OK) return rc;
  {
    Scratch sc(ctx->st);
    SeedOut so;
    rc = run_seed(ctx, idx, rd, max_hits, seeder, sc, &so);
    if (rc == SWIFT_OK) {
      *n = so.n;
      int64_t w = std::min<int64_t>(so.n, cap);
      if (w > 0 && out) {
        std::vector<int32_t> a(w), b(w), c(w), d(w), f(w);
        cudaStream_t st = ctx->st;
        cudaError_t e = cudaMemcpyAsync(a.data(), so.m_read, w * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(b.data(), so.m_strand, w * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(c.data(), so.m_ri, w * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d.data(), so.m_rp, w * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(f.data(), so.m_sh, w * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
          rc = fail(ctx, SWIFT_E_CUDA, cudaGetErrorString(e));
        } else {
          for (int64_t i = 0; i < w; ++i) {
            out[i].read = a[i];
            out[i].strand = b[i];
            out[i].ref_idx = c[i];
            out[i].ref_pos = d[i];
            out[i].shift = f[i];
          }
        }
      }
    }
  }
  swift_reads_destroy(rd);
  return rc;
}

}  // namespace

int swift_seed(swift_ctx* ctx, const swift_index* idx, const char* reads, size_t len,
               int32_t max_hits, swift_match* out, int64_t cap, int64_t* n) {
  return seed_records(ctx, idx, reads, len, max_hits, 0, out, cap, n);
}

int swift_seed_lt13(swift_ctx* ctx, const swift_index* idx, const char* reads, size_t len,
                    swift_match* out, int64_t cap, int64_t* n) {
  return seed_records(ctx, idx, reads, len, 3, 1, out, cap, n);
}


// alignSequences takes its scores as float (src/align.cu:2904-2921) and the
// reference CLI parses them with atoi (src/main.cu:309-324), so they are
// whole numbers: refuse any other value instead of truncating it.
static int whole_scores(swift_ctx* ctx, float fm, float fx, float fo, float fe, int32_t* m,
                        int32_t* x, int32_t* o, int32_t* e) {
  const float in[4] = {fm, fx, fo, fe};
  int32_t* out[4] = {m, x, o, e};
  for (int i = 0; i < 4; ++i) {
    const float v = in[i];
    if (!(v == v) || v != std::nearbyint(v) || std::fabs(v) > 32767.0f)
      return fail(ctx, SWIFT_E_ARG,
                  "scores must be whole numbers within +-32767 (the reference parses them "
                  "with atoi)");
    *out[i] = (int32_t)v;
  }
  return SWIFT_OK;
}

int swift_sw_batch(swift_ctx* ctx, const char* qry, const char* ref, int32_t Q, int32_t R,
                   int64_t n, float fm, float fx, float fo, float fe, float* score,
                   int32_t* start, int32_t* end, int32_t* len, char* qcons, char* rcons) {
  if (!ctx || !qry || !ref || !score || !start || !end || !len || !qcons || !rcons)
    return fail(ctx, SWIFT_E_ARG, "null argument");
  int32_t m, x, o, e;
  {
    const int rcw = whole_scores(ctx, fm, fx, fo, fe, &m, &x, &o, &e);
    if (rcw != SWIFT_OK) return rcw;
  }
  if (n < 0) return fail(ctx, SWIFT_E_ARG, "negative pair count");
  if (Q < 1 || Q > kMaxQ || R < 1 || R > kMaxR)
    return fail(ctx, SWIFT_E_LIMIT, "Q must be 1..256 and R 1..1024");
  if (n == 0) return SWIFT_OK;
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->st;
  Scratch sc(st);
  auto is_dev = [](const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
  };
  {
    const void* ptrs[] = {qry, ref, score, start, end, len, qcons, rcons};
    for (const void* q : ptrs) {
      cudaPointerAttributes at;
      if (cudaPointerGetAttributes(&at, q) != cudaSuccess) {
        cudaGetLastError();
        continue;
      }
      if (at.type == cudaMemoryTypeDevice && at.device != ctx->device)
        return fail(ctx, SWIFT_E_ARG,
                    "swift_sw_batch: a buffer lives on another device than the context's");
    }
  }
  const int64_t cs = (int64_t)Q + R + 2;
  const char* dq = qry;
  const char* dw = ref;
  if (!is_dev(qry)) {
    char* t;
    CK(sc.get(&t, (size_t)n * (Q + 1)));
    CK(cudaMemcpyAsync(t, qry, (size_t)n * (Q + 1), cudaMemcpyHostToDevice, st));
    dq = t;
  }
  if (!is_dev(ref)) {
    char* t;
    CK(sc.get(&t, (size_t)n * (R + 1)));
    CK(cudaMemcpyAsync(t, ref, (size_t)n * (R + 1), cudaMemcpyHostToDevice, st));
    dw = t;
  }
  DevAln* aln;
  CK(sc.get(&aln, (size_t)n));
  const bool out_dev = is_dev(score);
  char *dqc = qcons, *drc = rcons;
  if (!is_dev(qcons)) CK(sc.get(&dqc, (size_t)n * cs));
  if (!is_dev(rcons)) CK(sc.get(&drc, (size_t)n * cs));
  SwArgs a;
  memset(&a, 0, sizeof(a));
  a.q = dq;
  a.w = dw;
  a.q_stride = Q + 1;
  a.w_stride = R + 1;
  a.Q = Q;
  a.R = R;
  a.match = m;
  a.mismatch = x;
  a.gap_open = o;
  a.gap_ext = e;
  a.n = n;
  a.aln = aln;
  a.qcons = dqc;
  a.rcons = drc;
  a.cons_stride = cs;
  int rc = launch_sw(st, a, &ctx->err);
  if (rc != SWIFT_OK) return rc;
  CKLAUNCH();
  float* dscore = score;
  int32_t *dstart = start, *dend = end, *dlen = len;
  if (!out_dev) {
    CK(sc.get(&dscore, n));
    CK(sc.get(&dstart, n));
    CK(sc.get(&dend, n));
    CK(sc.get(&dlen, n));
  }
  aln_to_ref_layout_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(aln, n, dscore, dstart, dend,
                                                                       dlen);
  CKLAUNCH();
  if (!out_dev) {
    CK(cudaMemcpyAsync(score, dscore, n * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(start, dstart, n * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(end, dend, n * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(len, dlen, n * 4, cudaMemcpyDeviceToHost, st));
  }
  if (dqc != qcons) CK(cudaMemcpyAsync(qcons, dqc, (size_t)n * cs, cudaMemcpyDeviceToHost, st));
  if (drc != rcons) CK(cudaMemcpyAsync(rcons, drc, (size_t)n * cs, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return SWIFT_OK;
}

int swift_sw_batch_noalloc(swift_ctx* ctx, const char* qry, const char* ref, int32_t Q,
                           int32_t R, int64_t n, float fm, float fx, float fo, float fe,
                           float* score, int32_t* start, int32_t* end, int32_t* len,
                           char* qcons, char* rcons) {
  // Same kernels as swift_sw_batch; the per-pair records go to the static
  // array of sw.cu instead of pool memory, and the host never waits.
  if (!ctx || !qry || !ref || !score || !start || !end || !len || !qcons || !rcons)
    return fail(ctx, SWIFT_E_ARG, "null argument");
  int32_t m, x, o, e;
  {
    const int rcw = whole_scores(ctx, fm, fx, fo, fe, &m, &x, &o, &e);
    if (rcw != SWIFT_OK) return rcw;
  }
  if (n < 0) return fail(ctx, SWIFT_E_ARG, "negative pair count");
  if (n > kStaticSwPairs)
    return fail(ctx, SWIFT_E_LIMIT,
                "n_pairs above SWIFT_SW_NOALLOC_MAX_PAIRS (65536), the size of the static "
                "scratch; split the batch or use swift_sw_batch");
  if (Q < 1 || Q > kMaxQ || R < 1 || R > kMaxR)
    return fail(ctx, SWIFT_E_LIMIT, "Q must be 1..256 and R 1..1024");
  CK(cudaSetDevice(ctx->device));
  const void* ptrs[] = {qry, ref, score, start, end, len, qcons, rcons};
  for (const void* q : ptrs) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, q) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, SWIFT_E_ARG, "swift_sw_batch_noalloc takes device pointers only");
    }
    if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
      return fail(ctx, SWIFT_E_ARG, "swift_sw_batch_noalloc takes device pointers only");
    if (at.type == cudaMemoryTypeDevice && at.device != ctx->device)
      return fail(ctx, SWIFT_E_ARG,
                  "swift_sw_batch_noalloc: a buffer lives on another device than the context's");
  }
  DevAln* aln = nullptr;
  int rc = static_sw_scratch(ctx->device, &aln, &ctx->err);
  if (rc != SWIFT_OK) return rc;
  if (n == 0) return SWIFT_OK;
  cudaStream_t st = ctx->st;
  SwArgs a;
  memset(&a, 0, sizeof(a));
  a.q = qry;
  a.w = ref;
  a.q_stride = Q + 1;
  a.w_stride = R + 1;
  a.Q = Q;
  a.R = R;
  a.match = m;
  a.mismatch = x;
  a.gap_open = o;
  a.gap_ext = e;
  a.n = n;
  a.aln = aln;
  a.qcons = qcons;
  a.rcons = rcons;
  a.cons_stride = (int64_t)Q + R + 2;
  rc = launch_sw(st, a, &ctx->err);
  if (rc != SWIFT_OK) return rc;
  CKLAUNCH();
  aln_to_ref_layout_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(aln, n, score, start, end,
                                                                       len);
  CKLAUNCH();
  return SWIFT_OK;
}

static bool device_ptr(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

__global__ void aln_to_i32_kernel(const DevAln* __restrict__ aln, int64_t n, int32_t* score,
                                  int32_t* start, int32_t* end, int32_t* len) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const DevAln a = aln[i];
  score[i] = a.score;
  start[i] = a.start;
  end[i] = a.end;
  len[i] = a.len;
}

int swift_sw_pairs(swift_ctx* ctx, const char* qry, const int64_t* q_off, const int32_t* q_len,
                   const char* ref, const int64_t* r_off, const int32_t* r_len, int64_t n,
                   int32_t m, int32_t x, int32_t o, int32_t e, int32_t* score, int32_t* start,
                   int32_t* end, int32_t* len, char* qcons, char* rcons, int64_t cs, int32_t mode,
                   swift_pairs_stats* stats) {
  if (!ctx || !qry || !q_off || !q_len || !ref || !r_off || !r_len || !score || !start || !end ||
      !len)
    return fail(ctx, SWIFT_E_ARG, "null argument");
  if ((qcons == nullptr) != (rcons == nullptr)) return fail(ctx, SWIFT_E_ARG, "qcons and rcons: both or neither");
  if (n < 0) return fail(ctx, SWIFT_E_ARG, "negative pair count");
  if (mode != 0 && mode != 1) return fail(ctx, SWIFT_E_ARG, "mode must be 0 (batched) or 1 (plain)");
  if (mode == 1 && !(x < 0 && o < 0 && e < 0))
    return fail(ctx, SWIFT_E_ARG,
                "plain mode pads pairs, which is exact only with negative mismatch and gap penalties");
  if (qcons && (cs <= 0 || cs % 4 != 0)) return fail(ctx, SWIFT_E_ARG, "cons_stride must be a positive multiple of 4");
  swift_pairs_stats ps;
  memset(&ps, 0, sizeof(ps));
  ps.pairs = n;
  if (n == 0) {
    if (stats) *stats = ps;
    return SWIFT_OK;
  }
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->st;
  Scratch sc(st);
  const bool in_dev = device_ptr(qry);
  if (in_dev != device_ptr(ref) || in_dev != device_ptr(q_off) || in_dev != device_ptr(q_len) ||
      in_dev != device_ptr(r_off) || in_dev != device_ptr(r_len))
    return fail(ctx, SWIFT_E_ARG, "inputs must be all host or all device memory");
  const bool out_dev = device_ptr(score);
  if (out_dev != device_ptr(start) || out_dev != device_ptr(end) || out_dev != device_ptr(len) ||
      (qcons && (out_dev != device_ptr(qcons) || out_dev != device_ptr(rcons))))
    return fail(ctx, SWIFT_E_ARG, "outputs must be all host or all device memory");
  // inputs on the device
  const char *dq = qry, *dr = ref;
  const int64_t *dqo = q_off, *dro = r_off;
  const int32_t *dql = q_len, *drl = r_len;
  if (!in_dev) {
    int64_t qext = 0, rext = 0;
    for (int64_t i = 0; i < n; ++i) {
      if (q_len[i] < 1 || r_len[i] < 1 || q_off[i] < 0 || r_off[i] < 0)
        return fail(ctx, SWIFT_E_ARG, "pair lengths must be >= 1 and offsets >= 0");
      qext = std::max<int64_t>(qext, q_off[i] + q_len[i]);
      rext = std::max<int64_t>(rext, r_off[i] + r_len[i]);
    }
    char *tq, *tr;
    int64_t *tqo, *tro;
    int32_t *tql, *trl;
    CK(sc.get(&tq, (size_t)qext));
    CK(sc.get(&tr, (size_t)rext));
    CK(sc.get(&tqo, (size_t)n));
    CK(sc.get(&tro, (size_t)n));
    CK(sc.get(&tql, (size_t)n));
    CK(sc.get(&trl, (size_t)n));
    CK(cudaMemcpyAsync(tq, qry, qext, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(tr, ref, rext, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(tqo, q_off, n * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(tro, r_off, n * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(tql, q_len, n * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(trl, r_len, n * 4, cudaMemcpyHostToDevice, st));
    dq = tq; dr = tr; dqo = tqo; dro = tro; dql = tql; drl = trl;
  }
  CK(cudaEventRecord(ctx->ev[0], st));
  // shape limits over all pairs
  int32_t* mx;
  CK(sc.get(&mx, 8));
  const int32_t mx0[8] = {0, 0, 0x7fffffff, 0, 0, 0, 0, 0};
  CK(cudaMemcpyAsync(mx, mx0, sizeof(mx0), cudaMemcpyHostToDevice, st));
  launch_var_max_len(st, dql, drl, n, mx);
  CKLAUNCH();
  int32_t h_mx[8];
  CK(cudaMemcpyAsync(h_mx, mx, sizeof(h_mx), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const int maxQ = h_mx[0], maxR = h_mx[1];
  const int64_t n_long = h_mx[6];
  if (h_mx[2] < 1) return fail(ctx, SWIFT_E_ARG, "pair lengths must be >= 1");
  if (maxQ > kLongMaxQ || maxR > kLongMaxR)
    return fail(ctx, SWIFT_E_LIMIT, "q_len <= 4096 and r_len <= 8192");
  if (mode == 1 && n_long > 0)
    return fail(ctx, SWIFT_E_LIMIT,
                "plain mode takes q_len <= 256 and r_len <= 1024 (768 when q_len > 128)");
  if (n_long > 0 && !(x < 0 && o < 0 && e < 0))
    return fail(ctx, SWIFT_E_ARG,
                "pairs longer than 256 x 1024 need negative mismatch and gap penalties");
  if (qcons && cs < (int64_t)h_mx[3] + 2) return fail(ctx, SWIFT_E_ARG, "cons_stride below q_len + r_len + 2");
  // fixed strides for the pairs of the warp-per-pair kernels (long pairs are
  // read in place)
  const int64_t q_stride = ((int64_t)h_mx[4] + 16) & ~(int64_t)15;
  const int64_t w_stride = ((int64_t)h_mx[5] + 16) & ~(int64_t)15;
  int bias0 = 0;
  // chunks bound the fixed-stride copies and the traceback scratch
  const int64_t chunk = 4 << 20;
  const int64_t nc = std::min<int64_t>(n, chunk);
  char *qbuf, *wbuf;
  DevAln* aln;
  int2* best2;
  uint32_t *key, *hist, *hstart, *fill, *occ, *segpos, *nseg_d, *bad;
  int32_t *sorted, *seg_key, *seg_start, *seg_count;
  void* tmp;
  CK(sc.get(&qbuf, (size_t)(nc * q_stride)));
  CK(sc.get(&wbuf, (size_t)(nc * w_stride)));
  CK(sc.get(&aln, (size_t)nc));
  CK(sc.get(&best2, (size_t)nc));
  CK(sc.get(&key, (size_t)nc));
  CK(sc.get(&sorted, (size_t)nc));
  CK(sc.get(&hist, kVarKeys));
  CK(sc.get(&hstart, kVarKeys + 1));
  CK(sc.get(&fill, kVarKeys));
  CK(sc.get(&occ, kVarKeys));
  CK(sc.get(&segpos, kVarKeys + 1));
  CK(sc.get(&nseg_d, 2));
  CK(sc.get(&bad, 1));
  CK(cudaMemsetAsync(bad, 0, sizeof(uint32_t), st));
  CK(sc.get(&seg_key, kVarKeys));
  CK(sc.get(&seg_start, kVarKeys));
  CK(sc.get(&seg_count, kVarKeys));
  CK(sc.get((uint8_t**)&tmp, scan_temp_bytes(std::max<int64_t>(kVarKeys, nc))));
  // outputs staged on the device when the caller's are host memory
  int32_t *os = score, *ost = start, *oe = end, *ol = len;
  char *oqc = qcons, *orc = rcons;
  if (!out_dev) {
    CK(sc.get(&os, (size_t)nc));
    CK(sc.get(&ost, (size_t)nc));
    CK(sc.get(&oe, (size_t)nc));
    CK(sc.get(&ol, (size_t)nc));
    if (qcons) {
      CK(sc.get(&oqc, (size_t)(nc * cs)));
      CK(sc.get(&orc, (size_t)(nc * cs)));
    }
  }
  uint32_t* dirs[2] = {nullptr, nullptr};
  int64_t dirs_words[2] = {0, 0};
  int launches = 0;
  SideJoin joined(ctx);  // after sc: joins the side stream before sc frees
  for (int64_t c0 = 0; c0 < n; c0 += chunk) {
    const int64_t cn = std::min(chunk, n - c0);
    char* cq = qcons ? (out_dev ? qcons + c0 * cs : oqc) : nullptr;
    char* cr = qcons ? (out_dev ? rcons + c0 * cs : orc) : nullptr;
    VarPairArgs va;
    memset(&va, 0, sizeof(va));
    va.qry = dq;
    va.q_off = dqo + c0;
    va.q_len = dql + c0;
    va.ref = dr;
    va.r_off = dro + c0;
    va.r_len = drl + c0;
    va.n = cn;
    va.qbuf = qbuf;
    va.wbuf = wbuf;
    va.q_stride = q_stride;
    va.w_stride = w_stride;
    va.long_prof = long_prof_ok(m, x, o, kLongMaxQ);
    va.class_ok = 0;
    for (int c = 0; mode == 0 && c < 6; ++c)
      if (fast_params_ok(packed_class_max_q(c), kFastMaxR, m, x, o, e, &bias0)) va.class_ok |= 1u << c;
    va.fast_max_r = kFastMaxR;
    va.key = key;
    va.hist = hist;
    va.bad = bad;
    CK(cudaMemsetAsync(hist, 0, kVarKeys * sizeof(uint32_t), st));
    launch_pack_var(st, va);
    CKLAUNCH();
    ++launches;
    if (mode == 1) {
      // padding bytes must not occur in the pairs (see pack_var_kernel)
      uint32_t h_bad = 0;
      CK(cudaMemcpyAsync(&h_bad, bad, 4, cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      if (h_bad)
        return fail(ctx, SWIFT_E_INPUT, "plain mode: bytes 0x00 and 0x01 are reserved for padding");
      SwArgs sa;
      memset(&sa, 0, sizeof(sa));
      sa.q = qbuf;
      sa.w = wbuf;
      sa.q_stride = q_stride;
      sa.w_stride = w_stride;
      sa.Q = maxQ;
      sa.R = maxR;
      sa.match = m;
      sa.mismatch = x;
      sa.gap_open = o;
      sa.gap_ext = e;
      sa.n = cn;
      sa.aln = aln;
      sa.qcons = cq;
      sa.rcons = cr;
      sa.cons_stride = cs;
      int rc = launch_sw(st, sa, &ctx->err);
      if (rc != SWIFT_OK) return rc;
      CKLAUNCH();
      ++launches;
      ps.segments += 1;
      ps.generic_pairs += cn;
    } else {
      // counting sort by shape key; the segment table goes to the host
      int k = exclusive_scan_u32(st, hist, hstart, kVarKeys, tmp, hstart + kVarKeys);
      launch_var_occupied(st, hist, occ);
      k += exclusive_scan_u32(st, occ, segpos, kVarKeys, tmp, nseg_d);
      launch_var_segments(st, hist, hstart, segpos, seg_key, seg_start, seg_count);
      CK(cudaMemsetAsync(fill, 0, kVarKeys * sizeof(uint32_t), st));
      launch_var_scatter(st, key, cn, hstart, fill, sorted);
      CKLAUNCH();
      launches += k + 3;
      uint32_t nseg = 0;
      CK(cudaMemcpyAsync(&nseg, nseg_d, 4, cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      std::vector<int32_t> hk(nseg), hs(nseg), hc(nseg);
      if (nseg) {
        CK(cudaMemcpyAsync(hk.data(), seg_key, nseg * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(hs.data(), seg_start, nseg * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(hc.data(), seg_count, nseg * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
      }
      // launch groups: packed pairs by row class (their keys are
      // consecutive), generic pairs by exact shape
      struct Group {
        bool gen;
        int Q, R;           // generic: the shape; packed: the class's rows, widest window
        int64_t start, count;
      };
      std::vector<Group> groups;
      std::vector<std::pair<int64_t, int64_t>> long_groups;  // (start, count) per rows class
      std::vector<int> long_class;
      for (uint32_t s = 0; s < nseg; ++s) {
        if ((uint32_t)hk[s] >= kVarLongKey) {
          long_groups.push_back({hs[s], hc[s]});
          long_class.push_back((int)((uint32_t)hk[s] - kVarLongKey));  // 2 class + profile bit
          continue;
        }
        const bool gen = (hk[s] >> 20) & 1;
        const int q = (hk[s] >> 11) & 511, R = hk[s] & 2047;
        if (!gen && !groups.empty() && !groups.back().gen && groups.back().Q == 8 * q) {
          groups.back().R = std::max(groups.back().R, R);
          groups.back().count += hc[s];
          continue;
        }
        groups.push_back({gen, gen ? q : 8 * q, R, hs[s], hc[s]});
      }
      ps.segments += (int64_t)groups.size();
      // launch sizes go to the device (the kernels read counts there)
      std::vector<int32_t> gcount(groups.size());
      for (size_t g = 0; g < groups.size(); ++g) gcount[g] = (int32_t)groups[g].count;
      int32_t* gcount_d = seg_count;  // reuse: the segment counts are on the host now
      if (!groups.empty())
        CK(cudaMemcpyAsync(gcount_d, gcount.data(), groups.size() * 4, cudaMemcpyHostToDevice, st));
      for (size_t gi = 0; gi < groups.size(); ++gi) {
        const Group& G = groups[gi];
        const int Q = G.Q, R = G.R;
        const int64_t cnt = G.count;
        int32_t* list = sorted + G.start;
        int bias = 0;
        if (G.gen || !fast_params_ok(Q, R, m, x, o, e, &bias)) {
          // (a packed class whose longest query the packed scoring does not
          // take runs here too: the int32 kernel takes per-launch shapes, so
          // its pairs go one exact shape at a time)
          if (!G.gen) return fail(ctx, SWIFT_E_DEVICE, "packed class outside the packed scoring");
          SwArgs sa;
          memset(&sa, 0, sizeof(sa));
          sa.q = qbuf;
          sa.w = wbuf;
          sa.q_stride = q_stride;
          sa.w_stride = w_stride;
          sa.Q = Q;
          sa.R = R;
          sa.match = m;
          sa.mismatch = x;
          sa.gap_open = o;
          sa.gap_ext = e;
          sa.n = cnt;
          sa.aln = aln;
          sa.qcons = cq;
          sa.rcons = cr;
          sa.cons_stride = cs;
          sa.list = list;
          sa.count = gcount_d + gi;
          int rc = launch_sw(st, sa, &ctx->err);
          if (rc != SWIFT_OK) return rc;
          CKLAUNCH();
          ++launches;
          ps.generic_pairs += cnt;
          continue;
        }
        // packed trace pass + walk over pairs of one class, per-pair lengths,
        // in sub-chunks that bound the direction scratch
        const int64_t sub = 262144;
        // the class's (lanes, rows per lane) shape: the default, a forced
        // candidate, or the fastest candidate on a sample of these pairs
        // (timed once per context, class and window bin)
        int32_t cg[16], crpl[16];
        const int ncand = packed_shape_candidates(Q, cg, crpl, 16);
        int sg = 0, srpl = 0;
        if (ctx->tuning >= 2 && ctx->tuning - 2 < ncand) {
          sg = cg[ctx->tuning - 2];
          srpl = crpl[ctx->tuning - 2];
        }
        const int tkey = (Q / 8) * 64 + (R + 63) / 64;
        const bool tune = ctx->tuning == 1 && ncand > 1 && !ctx->tuned.count(tkey) &&
                          cnt >= 1024;
        int64_t words = 0;
        for (int c = 0; c < (tune ? ncand : 1); ++c)
          words = std::max(words, trace_scratch_words(Q, R, std::min(cnt, sub),
                                                      tune ? cg[c] : sg, tune ? crpl[c] : srpl));
        if (words > dirs_words[0]) {
          CK(sc.get(&dirs[0], (size_t)words));
          dirs_words[0] = words;
        }
        FastArgs fa;
        memset(&fa, 0, sizeof(fa));
        fa.q = qbuf;
        fa.w = wbuf;
        fa.q_stride = q_stride;
        fa.w_stride = w_stride;
        fa.Q = Q;
        fa.R = R;
        fa.q_len = dql + c0;
        fa.r_len = drl + c0;
        fa.match = m;
        fa.mismatch = x;
        fa.gap_open = o;
        fa.gap_ext = e;
        fa.bias = bias;
        fa.aln = aln;
        fa.best = best2;
        fa.dirs = dirs[0];
        fa.qcons = cq;
        fa.rcons = cr;
        fa.cons_stride = cs;
        fa.list = list;
        fa.count = gcount_d + gi;
        if (tune) {
          // a sample from the middle of the class (its pairs are sorted by
          // window length), each candidate warmed once and timed once
          const int64_t ns = std::min<int64_t>(cnt, 16384);
          int32_t* ns_d;
          CK(sc.get(&ns_d, 1));
          const int32_t ns32 = (int32_t)ns;
          CK(cudaMemcpyAsync(ns_d, &ns32, 4, cudaMemcpyHostToDevice, st));
          FastArgs ta = fa;
          ta.list = list + (cnt - ns) / 2;
          ta.count = ns_d;
          ta.list_offset = 0;
          cudaEvent_t e0 = ctx->ev[9], e1 = ctx->ev[10];
          float best_ms = 0;
          int best = 0;
          for (int c = 0; c < ncand; ++c) {
            ta.shape_g = cg[c];
            ta.shape_rpl = crpl[c];
            float t = 0;
            for (int rep = 0; rep < 2; ++rep) {
              CK(cudaEventRecord(e0, st));
              const int kk = launch_sw_trace(st, ta, ns);
              if (kk == 0) return fail(ctx, SWIFT_E_DEVICE, "trace pass could not launch");
              launches += kk;
              CKLAUNCH();
              CK(cudaEventRecord(e1, st));
              CK(cudaEventSynchronize(e1));
              CK(cudaEventElapsedTime(&t, e0, e1));
              ps.tune_ms += t;
            }
            if (c == 0 || t < best_ms) {
              best_ms = t;
              best = c;
            }
          }
          ctx->tuned[tkey] = {cg[best], crpl[best]};
        }
        if (ctx->tuning == 1) {
          auto it = ctx->tuned.find(tkey);
          if (it != ctx->tuned.end()) {
            sg = it->second.first;
            srpl = it->second.second;
          }
        }
        fa.shape_g = sg;
        fa.shape_rpl = srpl;
        {
          int32_t dg[1], dr[1];
          packed_shape_candidates(Q, dg, dr, 1);
          const int pc = packed_class(Q);
          if (pc >= 0 && pc < 8) {
            ps.shape_lanes[pc] = sg ? sg : dg[0];
            ps.shape_rows[pc] = sg ? srpl : dr[0];
          }
        }
        for (int64_t off = 0; off < cnt; off += sub) {
          fa.list_offset = off;
          const int kk = launch_sw_trace(st, fa, std::min(sub, cnt - off));
          if (kk == 0) return fail(ctx, SWIFT_E_DEVICE, "trace pass could not launch");
          launches += kk;
          CKLAUNCH();
        }
      }
      // long pairs: one CTA each, largest first, in launches of many waves
      // (the block scheduler fills SMs freed by small pairs) whose direction
      // slots, sized per pair, fit one of two scratch regions.  Launches
      // alternate between the context stream and a side stream, each
      // launch's walk on its own stream: a walk (a few threads per SM)
      // overlaps the next launch's fill, and a region is reused only after
      // the walk that read it.
      if (!long_groups.empty()) {
        std::vector<int32_t> hql(cn), hrl(cn);
        CK(cudaMemcpyAsync(hql.data(), dql + c0, cn * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(hrl.data(), drl + c0, cn * 4, cudaMemcpyDeviceToHost, st));
        int64_t n_long = 0;
        for (const auto& g : long_groups) n_long += g.second;
        std::vector<int32_t> ids(n_long);
        int64_t at = 0;
        for (const auto& g : long_groups) {
          CK(cudaMemcpyAsync(ids.data() + at, sorted + g.first, g.second * 4,
                             cudaMemcpyDeviceToHost, st));
          at += g.second;
        }
        CK(cudaStreamSynchronize(st));
        struct LongBatch {
          int rpl;
          bool prof;
          int64_t b0, nb, words;
        };
        std::vector<LongBatch> batches;
        std::vector<int64_t> off(n_long);
        const int64_t region_words = (int64_t)(8.0e9 / 4);
        int64_t max_words = 0;
        at = 0;
        for (size_t lg = 0; lg < long_groups.size(); ++lg) {
          const int64_t cnt = long_groups[lg].second;
          int32_t* g = ids.data() + at;
          std::sort(g, g + cnt, [&](int32_t u, int32_t v) {
            const int64_t cu = (int64_t)hql[u] * hrl[u], cv = (int64_t)hql[v] * hrl[v];
            return cu != cv ? cu > cv : u < v;
          });
          const int rpl = 4 * ((long_class[lg] >> 1) + 1);
          const bool prof = long_class[lg] & 1;
          int64_t b0 = 0;
          while (b0 < cnt) {
            int64_t words = 0, b1 = b0;
            while (b1 < cnt && (b1 == b0 || words + long_slot_words(hrl[g[b1]]) <= region_words)) {
              off[at + b1] = words;
              words += long_slot_words(hrl[g[b1]]);
              ++b1;
            }
            batches.push_back({rpl, prof, at + b0, b1 - b0, words});
            max_words = std::max(max_words, words);
            b0 = b1;
          }
          at += cnt;
          ps.segments += 1;
        }
        int32_t* dlist;
        int64_t* doff;
        CK(sc.get(&dlist, (size_t)n_long));
        CK(sc.get(&doff, (size_t)n_long));
        CK(cudaMemcpyAsync(dlist, ids.data(), n_long * 4, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(doff, off.data(), n_long * 8, cudaMemcpyHostToDevice, st));
        const int n_regions = batches.size() > 1 ? 2 : 1;
        for (int r = 0; r < n_regions; ++r) {
          if (max_words > dirs_words[r]) {
            CK(sc.get(&dirs[r], (size_t)max_words));
            dirs_words[r] = max_words;
          }
        }
        if (n_regions > 1) {
          const int rc = side_fork(ctx);
          if (rc != SWIFT_OK) return rc;
          joined.armed = true;
        }
        for (size_t b = 0; b < batches.size(); ++b) {
          const LongBatch& lb = batches[b];
          cudaStream_t bs = (b & 1) ? ctx->side : st;
          LongArgs la;
          memset(&la, 0, sizeof(la));
          la.qry = dq;
          la.q_off = dqo + c0;
          la.q_len = dql + c0;
          la.ref = dr;
          la.r_off = dro + c0;
          la.r_len = drl + c0;
          la.list = dlist + lb.b0;
          la.n = lb.nb;
          la.max_r = kLongMaxR;
          la.match = m;
          la.mismatch = x;
          la.gap_open = o;
          la.gap_ext = e;
          la.bias = long_bias(o);
          la.dirs = dirs[b & 1];
          la.dir_off = doff + lb.b0;
          la.best = best2;
          la.aln = aln;
          la.qcons = cq;
          la.rcons = cr;
          la.cons_stride = cs;
          const int kk = launch_sw_long(bs, la, lb.rpl, lb.prof);
          if (kk == 0) return fail(ctx, SWIFT_E_DEVICE, "long pass could not launch");
          launches += kk;
          CKLAUNCH();
        }
        if (joined.armed) {
          const int rc = joined.join();
          if (rc != SWIFT_OK) return rc;
        }
      }
    }
    aln_to_i32_kernel<<<(unsigned)((cn + 255) / 256), 256, 0, st>>>(
        aln, cn, out_dev ? score + c0 : os, out_dev ? start + c0 : ost, out_dev ? end + c0 : oe,
        out_dev ? len + c0 : ol);
    CKLAUNCH();
    ++launches;
    if (!out_dev) {
      CK(cudaMemcpyAsync(score + c0, os, cn * 4, cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(start + c0, ost, cn * 4, cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(end + c0, oe, cn * 4, cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(len + c0, ol, cn * 4, cudaMemcpyDeviceToHost, st));
      if (qcons) {
        CK(cudaMemcpyAsync(qcons + c0 * cs, oqc, cn * cs, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(rcons + c0 * cs, orc, cn * cs, cudaMemcpyDeviceToHost, st));
      }
      CK(cudaStreamSynchronize(st));  // the staging buffers are reused by the next chunk
    }
  }
  CK(cudaEventRecord(ctx->ev[1], st));
  CK(cudaEventSynchronize(ctx->ev[1]));
  float t = 0;
  cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[1]);
  ps.ms = t;
  ps.launches = launches + 1;
  if (stats) {
    // cells need the lengths on the host
    if (!in_dev) {
      for (int64_t i = 0; i < n; ++i) ps.cells += (int64_t)q_len[i] * r_len[i];
    } else {
      std::vector<int32_t> a(n), b(n);
      CK(cudaMemcpy(a.data(), q_len, n * 4, cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(b.data(), r_len, n * 4, cudaMemcpyDeviceToHost));
      for (int64_t i = 0; i < n; ++i) ps.cells += (int64_t)a[i] * b[i];
    }
    *stats = ps;
  }
  return SWIFT_OK;
}

// host_out (optional, host_cap bytes): the text is also copied there,
// overlapped with its writing; the copies are complete once ctx->st is
// synchronised.  Text longer than host_cap is not copied.
// The longest read a call takes: the reference's 199 bases unless the
// parameters allow more (up to kSeedReadMax).
static int read_limit(const swift_params* p) {
  return p && p->max_read_len > 0 ? std::min(p->max_read_len, kSeedReadMax) : kReadMax;
}

// wave: a merged batch of requests (the serving loop), each with its own
// query length, stale-read tail and Phase-2 batches; the requests must be
// valid on their own (checked at admission).  Null: rd is one request.
}  // extern "C"
int read_limit_of(const swift_params* p) { return read_limit(p); }
extern "C" {

static int align_resident_impl(swift_ctx* ctx, const swift_index* idx, const swift_reads* rd,
                               const swift_params* p, size_t* out_len, swift_stats* stats,
                               char* host_out, size_t host_cap,
                               std::vector<WaveReq>* wave = nullptr) {
  if (!ctx || !idx || !rd || !p) return fail(ctx, SWIFT_E_ARG, "null argument");
  CK(cudaSetDevice(ctx->device));
  if (p->seed_len != idx->k || p->ignore_thres != idx->thres)
    return fail(ctx, SWIFT_E_ARG, "parameters differ from the index's seed length / threshold");
  if (p->max_hits < 1 || p->max_hits > 64) return fail(ctx, SWIFT_E_ARG, "max_hits outside 1..64");
  if (p->max_read_len < 0 || p->max_read_len > kSeedReadMax)
    return fail(ctx, SWIFT_E_ARG, "max_read_len outside 0..300");
  if (rd->max_len > read_limit(p))
    return fail(ctx, SWIFT_E_LIMIT,
                "reads: read longer than " + std::to_string(read_limit(p)) + " bases" +
                    (read_limit(p) == kReadMax ? " (the reference's query buffer)" : ""));
  if (read_limit(p) > kReadMax && p->seeder == 1 && rd->max_len > kReadMax)
    return fail(ctx, SWIFT_E_LIMIT, "lt13 seeding takes reads of up to 199 bases");
  // the longest query of the call (every query when not a wave)
  int Q = p->qry_len > 0 ? p->qry_len : rd->first_len;
  bool uniform_q = true;
  if (wave) {
    if (wave->empty()) return fail(ctx, SWIFT_E_ARG, "empty wave");
    Q = 0;
    for (const WaveReq& q : *wave) {
      if (q.Q < 1 || q.Q > kMaxQ) return fail(ctx, SWIFT_E_ARG, "wave: query length out of range");
      Q = std::max(Q, (int)q.Q);
      uniform_q = uniform_q && q.Q == (*wave)[0].Q;
    }
  }
  if (Q < 1 || Q > kMaxQ)
    return fail(ctx, SWIFT_E_LIMIT, "query length outside 1.." + std::to_string(kMaxQ));
  if (!wave && rd->n > 0 && rd->min_len < Q)
    return fail(ctx, SWIFT_E_INPUT,
                "a read is shorter than the query length; the reference aligns such reads "
                "against stale buffer contents");
  cudaStream_t st = ctx->st;
  Scratch sc(st);
  swift_stats s;
  memset(&s, 0, sizeof(s));
  CK(cudaEventRecord(ctx->ev[0], st));
  SeedOut so;
  if (p->seeder != 0 && p->seeder != 1) return fail(ctx, SWIFT_E_ARG, "seeder must be 0 or 1");
  int rc = run_seed(ctx, idx, rd, p->max_hits, p->seeder, sc, &so, wave);
  if (rc != SWIFT_OK) return rc;
  CK(cudaEventRecord(ctx->ev[1], st));
  const int64_t nm = so.n;
  const int64_t dev_mem = p->device_mem > 0 ? p->device_mem : ctx->total_mem;
  // records the batches of getNumQueriesPerIteration cover: all of them,
  // unless the float ceil of the batch count comes out one short
  auto processed = [](int64_t nrec, int64_t per) -> int64_t {
    const int it = phase2_iterations(nrec, per);
    if (it <= 0) return 0;
    const int64_t maxs = (int64_t)it * per;
    const int64_t last = nrec < maxs ? nrec - (int64_t)(it - 1) * per : per;
    return (int64_t)(it - 1) * per + last;
  };
  const int64_t per_iter = phase2_batch(dev_mem, Q, nm);
  int64_t nproc = wave ? nm : processed(nm, per_iter);
  // a wave's batch boundaries: each request's own batches (of its own
  // query length), so its best-per-read groups end where they end alone
  std::vector<uint8_t> h_bs;
  if (wave) {
    h_bs.assign((size_t)std::max<int64_t>(nm, 1), 0);
    for (const WaveReq& q : *wave) {
      const int64_t per = phase2_batch(dev_mem, q.Q, q.nm);
      if (processed(q.nm, per) != q.nm)
        return fail(ctx, SWIFT_E_LIMIT, "wave: a request's batches do not cover its records");
      for (int64_t k = 0; k < q.nm; k += std::max<int64_t>(per, 1)) h_bs[q.rec0 + k] = 1;
    }
  }
  const int Qs = (Q + 16) & ~15;
  // consensus stride: Q + R + 2 bytes, rounded to 16 so the walk kernel can
  // store 32-bit words
  const int64_t cs = ((int64_t)Q + kWin + 2 + 15) & ~(int64_t)15;
  const size_t nn = (size_t)std::max<int64_t>(nproc, 1);
  DevPair* pairs;
  char *qbuf, *wbuf, *qcons, *rcons;
  DevAln* aln;
  int32_t* keep;
  uint64_t *bytes, *offs, *tot_d;
  void* tmp;
  CK(sc.get(&pairs, nn));
  CK(sc.get(&qbuf, nn * Qs));
  CK(sc.get(&wbuf, nn * kWinPad));
  CK(sc.get(&aln, nn));
  CK(sc.get(&qcons, nn * cs));
  CK(sc.get(&rcons, nn * cs));
  CK(sc.get(&keep, nn));
  CK(sc.get(&bytes, nn));
  CK(sc.get(&offs, nn));
  CK(sc.get(&tot_d, 1));
  CK(sc.get((uint8_t**)&tmp, scan_temp_bytes(nproc)));
  PairArgs pa;
  memset(&pa, 0, sizeof(pa));
  pa.ref_file = idx->d_file;
  pa.ref_file_len = idx->file_len;
  pa.cat = (const char*)idx->d_cat;
  pa.odd = idx->d_odd;
  pa.recs = idx->d_recs;
  pa.reads = rd->d_bytes;
  pa.rd = rd->d_rd;
  pa.m_read = so.m_read;
  pa.m_strand = so.m_strand;
  pa.m_ri = so.m_ri;
  pa.m_rp = so.m_rp;
  pa.n = nproc;
  pa.Q = Q;
  pa.pairs = pairs;
  pa.qbuf = qbuf;
  pa.wbuf = wbuf;
  pa.Qs = Qs;
  uint8_t* read_cls;
  CK(sc.get(&read_cls, (size_t)std::max<int64_t>(rd->n, 1)));
  pa.read_cls = read_cls;
  pa.n_reads = rd->n;
  // a wave of several query lengths: each record's own, for the pair
  // builder and every Smith-Waterman pass (rows past it match nothing)
  int32_t* pair_q = nullptr;
  uint8_t* d_bs = nullptr;
  if (wave) {
    CK(sc.get(&d_bs, nn));
    if (nm) CK(cudaMemcpyAsync(d_bs, h_bs.data(), nm, cudaMemcpyHostToDevice, st));
    if (!uniform_q) {
      std::vector<int32_t> h_rq((size_t)std::max<int64_t>(rd->n, 1), 0);
      for (const WaveReq& q : *wave)
        std::fill(h_rq.begin() + q.read0, h_rq.begin() + q.read0 + q.n, q.Q);
      int32_t* d_rq;
      CK(sc.get(&d_rq, h_rq.size()));
      CK(cudaMemcpyAsync(d_rq, h_rq.data(), h_rq.size() * 4, cudaMemcpyHostToDevice, st));
      CK(sc.get(&pair_q, nn));
      pa.read_q = d_rq;
      pa.pair_q = pair_q;
    }
  }
  launch_build_pairs(st, pa);
  CKLAUNCH();
  CK(cudaEventRecord(ctx->ev[2], st));
  // split: packed score pass (then traceback of the printed pairs) or the
  // generic kernel (full result at once)
  int bias = 0;
  const bool fast_ok =
      ctx->sw_path != 1 && fast_params_ok(Q, kWin, p->match, p->mismatch, p->gap_open, p->gap_ext, &bias);
  // SAM output prints every record: no selection, every pair traced
  const bool sam = p->out_format == 1;
  const bool bounded = fast_ok && ctx->sw_path == 0 && !sam;
  // counters: 0 packed-path pairs, 1 generic pairs, 2 trace list,
  // 3 pairs the LCS bound keeps (exact-score list), 4 second trace list,
  // 5 printed records
  // counters 8.. : histogram and fill of the early-stop sort (two uses)
  int32_t *fast_list, *gen_list, *tb_list, *cnt;
  CK(sc.get(&fast_list, nn));
  CK(sc.get(&gen_list, nn));
  CK(sc.get(&tb_list, nn));
  CK(sc.get(&cnt, 8 + 4 * (kSufBlocks + 1)));
  CK(cudaMemsetAsync(cnt, 0, (8 + 4 * (kSufBlocks + 1)) * sizeof(int32_t), st));
  int launches = 0;
  if (nproc > 0) {
    partition_pairs_kernel<<<(unsigned)((nproc + 255) / 256), 256, 0, st>>>(
        pairs, nproc, fast_ok ? 0 : 1, fast_list, cnt, gen_list, cnt + 1);
    CKLAUNCH();
    ++launches;
  }
  SwArgs sa;
  memset(&sa, 0, sizeof(sa));
  sa.q = qbuf;
  sa.w = wbuf;
  sa.q_stride = Qs;
  sa.w_stride = kWinPad;
  sa.Q = Q;
  sa.R = kWin;
  sa.match = p->match;
  sa.mismatch = p->mismatch;
  sa.gap_open = p->gap_open;
  sa.gap_ext = p->gap_ext;
  sa.n = nproc;
  sa.aln = aln;
  sa.qcons = qcons;
  sa.rcons = rcons;
  sa.cons_stride = cs;
  sa.q_len = pair_q;
  FastArgs fa2;
  memset(&fa2, 0, sizeof(fa2));
  fa2.q = qbuf;
  fa2.w = wbuf;
  fa2.q_stride = Qs;
  fa2.w_stride = kWinPad;
  fa2.Q = Q;
  fa2.R = kWin;
  fa2.match = p->match;
  fa2.mismatch = p->mismatch;
  fa2.gap_open = p->gap_open;
  fa2.gap_ext = p->gap_ext;
  fa2.bias = bias;
  fa2.aln = aln;
  fa2.qcons = qcons;
  fa2.rcons = rcons;
  fa2.cons_stride = cs;
  fa2.q_len = pair_q;
  int32_t *ub = nullptr, *cand = nullptr;
  // suffix LCS values: early stop of the score and trace passes (bounded
  // selection; every pair traced with SAM output)
  uint16_t* lsuf = nullptr;
  const bool lcs_stop = fast_ok && ctx->sw_path == 0;
  if (bounded) CK(sc.get(&cand, nn));
  if (lcs_stop) {
    CK(sc.get(&ub, nn));
    CK(sc.get(&lsuf, nn * kSufBlocks));
  }
  fa2.ub = ub;
  fa2.lsuf = lsuf;
  // cells computed: [0] score passes and later traces, [1] the candidates'
  // trace pass
  unsigned long long* d_cells;
  CK(sc.get(&d_cells, 2));
  CK(cudaMemsetAsync(d_cells, 0, 2 * sizeof(unsigned long long), st));
  fa2.cells_done = d_cells;
  CK(cudaEventRecord(ctx->ev[7], st));
  if (fast_ok && nproc > 0 && !sam) {
    fa2.list = fast_list;
    fa2.count = cnt;
    // bounded: the LCS bound of every packed pair, with its suffix values
    // (the exact pass runs later on the pairs it cannot rule out); else
    // exact scores
    const int k = bounded ? launch_sw_lcs(st, fa2, nproc) : launch_sw_score(st, fa2, nproc);
    if (k == 0) return fail(ctx, SWIFT_E_DEVICE, "first Smith-Waterman pass could not launch");
    launches += k;
    CKLAUNCH();
  }
  CK(cudaEventRecord(ctx->ev[8], st));
  if (nproc > 0) {
    sa.list = gen_list;
    sa.count = cnt + 1;
    rc = launch_sw(st, sa, &ctx->err);
    if (rc != SWIFT_OK) return rc;
    CKLAUNCH();
    ++launches;
  }
  CK(cudaEventRecord(ctx->ev[3], st));
  FormatArgs fa;
  memset(&fa, 0, sizeof(fa));
  fa.reads = rd->d_bytes;
  fa.rd = rd->d_rd;
  fa.recs = idx->d_recs;
  fa.pairs = pairs;
  fa.aln = aln;
  fa.qcons = qcons;
  fa.rcons = rcons;
  fa.cons_stride = cs;
  fa.n = nproc;
  fa.batch = per_iter > 0 ? per_iter : 1;
  fa.batch_start = d_bs;
  fa.keep = keep;
  fa.bytes = bytes;
  fa.offs = offs;
  fa.ub = ub;
  fa.cand = cand;
  int2* best2 = nullptr;
  if (fast_ok && nproc > 0) CK(sc.get(&best2, nn));
  fa2.best = best2;
  // trace pass + walk over list[0, n), in chunks that bound the direction
  // scratch; `timed`: CUDA events around each chunk's trace pass
  int timed_chunks = 0;
  auto trace_list = [&](int32_t* list, int32_t* count, int64_t n, bool timed) -> int {
    const int64_t chunk = 262144;
    if (n <= 0) return SWIFT_OK;
    const int64_t words = trace_scratch_words(Q, kWin, std::min(n, chunk));
    uint32_t* dirs;
    CK(sc.get(&dirs, (size_t)words));
    fa2.list = list;
    fa2.count = count;
    fa2.dirs = dirs;
    if (timed) {
      const size_t need = 2 * (size_t)((n + chunk - 1) / chunk);
      while (ctx->chunk_ev.size() < need) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        ctx->chunk_ev.push_back(e);
      }
    }
    for (int64_t off = 0; off < n; off += chunk) {
      fa2.list_offset = off;
      cudaEvent_t eb = nullptr, ea = nullptr;
      if (timed) {
        eb = ctx->chunk_ev[2 * timed_chunks];
        ea = ctx->chunk_ev[2 * timed_chunks + 1];
        ++timed_chunks;
      }
      const int k = launch_sw_trace(st, fa2, std::min(chunk, n - off), eb, ea);
      if (k == 0) return fail(ctx, SWIFT_E_DEVICE, "trace pass could not launch");
      launches += k;
      CKLAUNCH();
    }
    fa2.list_offset = 0;
    return SWIFT_OK;
  };
  int32_t h_cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int64_t pruned = 0;
  // list[0, *count) -> out in early-stop order (grid sized by max_n)
  int32_t *keys = nullptr, *sorted = nullptr;
  if (lcs_stop) {
    CK(sc.get(&keys, nn));
    CK(sc.get(&sorted, nn));
  }
  int sort_uses = 0;
  // cand_order: the traces' key (else the exact score pass's)
  auto sort_by_stop = [&](const int32_t* list, const int32_t* count, int64_t max_n,
                          int32_t* out, bool cand_order) -> int {
    if (max_n <= 0) return SWIFT_OK;
    int32_t* hist = cnt + 8 + 2 * (kSufBlocks + 1) * sort_uses;
    int32_t* fill = hist + (kSufBlocks + 1);
    ++sort_uses;
    const unsigned grid = (unsigned)((max_n + 255) / 256);
    if (cand_order)
      cand_key_count_kernel<<<grid, 256, 0, st>>>(list, count, lsuf, pair_q, Q, keys, hist);
    else
      exact_key_count_kernel<<<grid, 256, 0, st>>>(list, count, ub, cand, aln, p->match, keys, hist);
    stop_key_scatter_kernel<<<grid, 256, 0, st>>>(list, count, keys, hist, fill, out);
    CKLAUNCH();
    launches += 2;
    return SWIFT_OK;
  };
  if (sam) {
    // every record is printed: trace every packed-path pair (the trace pass
    // scores it as well)
    CK(cudaEventRecord(ctx->ev[6], st));
    if (fast_ok && nproc > 0) {
      CK(cudaMemcpyAsync(h_cnt, cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      int32_t* sam_list = fast_list;
      if (lsuf) {
        // suffix LCS values for the early stop, then the order that groups
        // pairs stopping alike
        fa2.list = fast_list;
        fa2.count = cnt;
        fa2.list_offset = 0;
        const int k = launch_sw_lcs(st, fa2, h_cnt[0]);
        if (k == 0) return fail(ctx, SWIFT_E_DEVICE, "LCS pass could not launch");
        launches += k;
        CKLAUNCH();
        rc = sort_by_stop(fast_list, cnt, h_cnt[0], sorted, true);
        if (rc != SWIFT_OK) return rc;
        sam_list = sorted;
      }
      fa2.cells_done = d_cells + 1;
      rc = trace_list(sam_list, cnt, h_cnt[0], true);
      if (rc != SWIFT_OK) return rc;
      fa2.cells_done = d_cells;
      fa2.lsuf = nullptr;
    }
  }
  int64_t lcs_kept = 0, cand_n = 0;
  if (bounded && nproc > 0) {
    // candidates (largest LCS bound of their group) traced first; they stop
    // early on the LCS pass's suffix values, in an order that groups pairs
    // stopping alike
    launch_candidates(st, fa, tb_list, cnt + 2);
    CKLAUNCH();
    ++launches;
    CK(cudaMemcpyAsync(h_cnt, cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaEventRecord(ctx->ev[6], st));
    cand_n = h_cnt[2];
    fa2.cells_done = d_cells + 1;
    int32_t* cand_list = tb_list;
    if (lsuf) {
      rc = sort_by_stop(tb_list, cnt + 2, cand_n, sorted, true);
      if (rc != SWIFT_OK) return rc;
      cand_list = sorted;
    }
    rc = trace_list(cand_list, cnt + 2, cand_n, true);
    if (rc != SWIFT_OK) return rc;
    fa2.cells_done = d_cells;
    // pairs whose LCS bound cannot rule them out against their candidate's
    // score get the exact score pass, which drops each pair once its score
    // is settled or provably too low to be its group's pick
    int32_t* k1_list = fast_list;  // free once the LCS pass has run
    launch_prune(st, fa, aln, k1_list, cnt + 3);
    CKLAUNCH();
    ++launches;
    CK(cudaMemcpyAsync(h_cnt, cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    lcs_kept = h_cnt[3];
    if (lcs_kept > 0) {
      int32_t* ex_list = k1_list;
      if (lsuf) {
        rc = sort_by_stop(k1_list, cnt + 3, lcs_kept, sorted, false);
        if (rc != SWIFT_OK) return rc;
        ex_list = sorted;
      }
      fa2.list = ex_list;
      fa2.count = cnt + 3;
      fa2.list_offset = 0;
      fa2.cand = cand;
      launches += launch_sw_score(st, fa2, lcs_kept);
      CKLAUNCH();
      fa2.cand = nullptr;
    }
  }
  if (!sam) {
    launch_select(st, fa);
    CKLAUNCH();
    launches += nproc > 0 ? 1 : 0;
  }
  if (!bounded && !sam) CK(cudaEventRecord(ctx->ev[6], st));
  if (nproc > 0 && !sam) {
    // printed packed-path pairs not traced yet
    int32_t* list2 = bounded ? gen_list : tb_list;  // generic list no longer needed
    traceback_list_kernel<<<(unsigned)((nproc + 255) / 256), 256, 0, st>>>(
        pairs, keep, cand, nproc, fast_ok ? 0 : 1, list2, cnt + 4, cnt + 5);
    CKLAUNCH();
    ++launches;
    CK(cudaMemcpyAsync(h_cnt, cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    rc = trace_list(list2, cnt + 4, h_cnt[4], false);
    if (rc != SWIFT_OK) return rc;
    if (bounded) pruned = std::max<int64_t>(h_cnt[0] - h_cnt[2] - lcs_kept, 0);
  }
  CK(cudaEventRecord(ctx->ev[4], st));
  if (sam)
    launch_sam_sizes(st, fa);
  else
    launch_format_sizes(st, fa);
  CKLAUNCH();
  int scan_k = exclusive_scan_u64(st, bytes, offs, nproc, tmp, tot_d);
  CKLAUNCH();
  uint64_t total = 0;
  CK(cudaMemcpyAsync(&total, tot_d, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(h_cnt, cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
  unsigned long long h_cells2[2] = {0, 0}, h_model[kSeedModelSlots] = {};
  CK(cudaMemcpyAsync(h_cells2, d_cells, sizeof(h_cells2), cudaMemcpyDeviceToHost, st));
  const unsigned long long h_cells = h_cells2[0] + h_cells2[1];
  // a wave: each request's text starts at its first record's offset
  std::vector<uint64_t> h_t0;
  if (wave) {
    const size_t W = wave->size();
    std::vector<int64_t> at(W + 1);
    for (size_t r = 0; r < W; ++r) at[r] = (*wave)[r].rec0;
    at[W] = nproc;
    int64_t* d_at;
    uint64_t* d_t0;
    CK(sc.get(&d_at, W + 1));
    CK(sc.get(&d_t0, W + 1));
    CK(cudaMemcpyAsync(d_at, at.data(), (W + 1) * 8, cudaMemcpyHostToDevice, st));
    gather_u64_kernel<<<(unsigned)((W + 1 + 255) / 256), 256, 0, st>>>(offs, nproc, tot_d, d_at,
                                                                       (int64_t)W + 1, d_t0);
    CKLAUNCH();
    ++launches;
    h_t0.resize(W + 1);
    CK(cudaMemcpyAsync(h_t0.data(), d_t0, (W + 1) * 8, cudaMemcpyDeviceToHost, st));
  }
  if (so.d_model)
    CK(cudaMemcpyAsync(h_model, so.d_model, sizeof(h_model), cudaMemcpyDeviceToHost, st));
  TextChunks chunks;
  rc = chunks.plan(ctx, st, offs, nproc, host_out != nullptr);
  if (rc != SWIFT_OK) return rc;
  CK(cudaStreamSynchronize(st));
  if (wave)
    for (size_t r = 0; r < wave->size(); ++r) {
      (*wave)[r].text0 = h_t0[r];
      (*wave)[r].text1 = h_t0[r + 1];
    }
  if (total + 1 > ctx->text_cap) {
    if (ctx->d_text) cudaFree(ctx->d_text);
    ctx->d_text = nullptr;
    size_t cap = (size_t)(total * 1.25) + 4096;
    CK(cudaMalloc(&ctx->d_text, cap));
    ctx->text_cap = cap;
  }
  rc = chunks.write(ctx, st, fa, sam, ctx->d_text, total, host_out, host_cap, ctx->ev[5]);
  if (rc != SWIFT_OK) return rc;
  CK(cudaEventSynchronize(ctx->ev[5]));
  ctx->text_len = total;
  if (out_len) *out_len = total;
  if (stats) {
    float t;
    cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[1]);
    s.seed_ms = t;
    cudaEventElapsedTime(&t, ctx->ev[1], ctx->ev[2]);
    s.pairs_ms = t;
    cudaEventElapsedTime(&t, ctx->ev[2], ctx->ev[3]);
    s.sw_ms = t;
    // the trace pass of all packed pairs (SAM) or of the candidates
    // (bounded selection), up to their early stop
    double trace_sum = 0;
    for (int c = 0; c < timed_chunks; ++c) {
      cudaEventElapsedTime(&t, ctx->chunk_ev[2 * c], ctx->chunk_ev[2 * c + 1]);
      trace_sum += t;
    }
    s.trace_ms = trace_sum;
    s.trace_cells = (int64_t)h_cells2[1];
    if (!sam) {
      cudaEventElapsedTime(&t, ctx->ev[7], ctx->ev[8]);
      s.first_pass_ms = t;
      s.first_pass_kind = bounded ? 3 : 1;
      s.first_pass_cells = fast_ok ? (int64_t)h_cnt[0] * Q * kWin : 0;
    }
    s.lcs_kept = lcs_kept;
    s.seed_kernel_ms = so.kernel_ms;
    for (int i = 0; i < kSeedModelSlots; ++i) s.seed_model_bytes += (int64_t)h_model[i];
    // the generic kernel computes every cell of its pairs; the packed score
    // and trace passes counted theirs
    s.sw_cells_computed = (int64_t)h_cells + (int64_t)h_cnt[1] * Q * kWin;
    cudaEventElapsedTime(&t, ctx->ev[3], ctx->ev[6]);
    s.select_ms = t;
    cudaEventElapsedTime(&t, ctx->ev[6], ctx->ev[4]);
    s.traceback_ms = t;
    cudaEventElapsedTime(&t, ctx->ev[4], ctx->ev[5]);
    s.format_ms = t;
    cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[5]);
    s.total_ms = t;
    s.reads = rd->n;
    s.records = nm;
    s.cells = nproc * (int64_t)Q * kWin;
    s.out_bytes = (int64_t)total;
    s.seed_overflow_strands = so.overflow;
    s.printed = sam ? nproc : h_cnt[5];
    s.sw_generic_pairs = h_cnt[1];
    s.traced_pairs = sam ? h_cnt[0] : h_cnt[2] + h_cnt[4];
    s.bound_pruned = pruned;
    s.retraced_pairs = bounded ? h_cnt[4] : 0;
    // build_pairs + the Smith-Waterman passes and select (launches) +
    // format sizes, scan, format write (one per record range)
    s.launches = so.launches + (nproc > 0 ? 1 + 1 + chunks.n_chunks : 0) + launches + scan_k;
    *stats = s;
  }
  return SWIFT_OK;
}

// One merged wave of the serving loop (server.cpp): the requests' reads
// FASTA bytes back to back in host memory with their per-read records
// (offsets into those bytes), every request valid on its own.  The text of
// all requests goes to host_out when it fits host_cap (the caller splits it
// with each request's text0 / text1), else it stays on the device for
// swift_fetch_output.
}  // extern "C"
int run_wave(swift_ctx* ctx, const swift_index* idx, const swift_params* p, const char* bytes,
             size_t len, const std::vector<DevRead>& rd, std::vector<WaveReq>* wave,
             char* host_out, size_t host_cap, size_t* out_len, swift_stats* stats) {
  if (!ctx || !idx || !p || !wave || (!bytes && len)) return fail(ctx, SWIFT_E_ARG, "null argument");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->st;
  swift_reads* r = new swift_reads();
  r->device = ctx->device;
  r->len = len;
  r->pool_st = st;
  r->n = (int64_t)rd.size();
  r->n_gt = r->n;
  int32_t mn = INT32_MAX, mx = 0;
  for (const DevRead& d : rd) {
    mn = std::min(mn, d.len);
    mx = std::max(mx, d.len);
  }
  r->min_len = r->n ? mn : 0;
  r->max_len = mx;
  r->first_len = r->n ? rd[0].len : 0;
  int rc = SWIFT_OK;
  if (cudaMallocAsync(&r->d_bytes, len + 64, st) != cudaSuccess ||
      cudaMallocAsync(&r->d_rd, std::max<size_t>(rd.size(), 1) * sizeof(DevRead), st) != cudaSuccess ||
      (len && cudaMemcpyAsync(r->d_bytes, bytes, len, cudaMemcpyHostToDevice, st) != cudaSuccess) ||
      (!rd.empty() && cudaMemcpyAsync(r->d_rd, rd.data(), rd.size() * sizeof(DevRead),
                                      cudaMemcpyHostToDevice, st) != cudaSuccess)) {
    rc = fail(ctx, SWIFT_E_CUDA, std::string("wave upload: ") + cudaGetErrorString(cudaGetLastError()));
  } else {
    rc = align_resident_impl(ctx, idx, r, p, out_len, stats, host_out, host_cap, wave);
    if (rc == SWIFT_OK) {
      const cudaError_t e = cudaStreamSynchronize(st);  // the host copies of the text
      if (e != cudaSuccess) rc = fail(ctx, SWIFT_E_CUDA, cudaGetErrorString(e));
    }
  }
  swift_reads_destroy(r);
  return rc;
}
extern "C" {

int swift_align_resident(swift_ctx* ctx, const swift_index* idx, const swift_reads* rd,
                         const swift_params* p, size_t* out_len, swift_stats* stats) {
  return align_resident_impl(ctx, idx, rd, p, out_len, stats, nullptr, 0);
}

int swift_fetch_output(swift_ctx* ctx, char* dst, size_t cap) {
  if (!ctx || !dst) return fail(ctx, SWIFT_E_ARG, "null argument");
  size_t n = std::min(cap, ctx->text_len);
  if (n) CK(cudaMemcpy(dst, ctx->d_text, n, cudaMemcpyDeviceToHost));
  return SWIFT_OK;
}

int swift_align(swift_ctx* ctx, const swift_index* idx, const char* reads, size_t len,
                const swift_params* p, char** out, size_t* out_len, swift_stats* stats) {
  if (!ctx || !idx || !reads || !p || !out || !out_len) return fail(ctx, SWIFT_E_ARG, "null argument");
  CK(cudaSetDevice(ctx->device));
  swift_reads* rd = nullptr;
  double parse_ms = 0, h2d_ms = 0;
  int rc = upload_reads(ctx, reads, len, &rd, &parse_ms, &h2d_ms, true, read_limit(p));
  if (rc != SWIFT_OK) return rc;
  size_t n = 0;
  rc = swift_align_resident(ctx, idx, rd, p, &n, stats);
  auto t0 = std::chrono::steady_clock::now();
  if (rc == SWIFT_OK) {
    char* h = (char*)malloc(n + 1);
    if (!h) {
      rc = fail(ctx, SWIFT_E_NOMEM, "host output buffer");
    } else {
      cudaError_t e = n ? cudaMemcpy(h, ctx->d_text, n, cudaMemcpyDeviceToHost) : cudaSuccess;
      if (e != cudaSuccess) {
        free(h);
        rc = fail(ctx, SWIFT_E_CUDA, cudaGetErrorString(e));
      } else {
        h[n] = '\0';
        *out = h;
        *out_len = n;
      }
    }
  }
  if (stats) {
    stats->host_parse_ms = parse_ms;
    stats->h2d_ms = h2d_ms;
    stats->d2h_ms = ms_since(t0);
  }
  swift_reads_destroy(rd);
  return rc;
}

int swift_align_into(swift_ctx* ctx, const swift_index* idx, const char* reads, size_t len,
                     const swift_params* p, char* out, size_t cap, size_t* out_len,
                     swift_stats* stats) {
  if (!ctx || !idx || !reads || !p || !out_len) return fail(ctx, SWIFT_E_ARG, "null argument");
  CK(cudaSetDevice(ctx->device));
  swift_reads* rd = nullptr;
  double parse_ms = 0, h2d_ms = 0;
  int rc = upload_reads(ctx, reads, len, &rd, &parse_ms, &h2d_ms, true, read_limit(p));
  if (rc != SWIFT_OK) return rc;
  size_t n = 0;
  // the text is copied to out while it is written
  rc = align_resident_impl(ctx, idx, rd, p, &n, stats, out, out ? cap : 0);
  auto t0 = std::chrono::steady_clock::now();
  if (rc == SWIFT_OK) {
    *out_len = n;
    cudaError_t e = cudaStreamSynchronize(ctx->st);
    if (e != cudaSuccess)
      rc = fail(ctx, SWIFT_E_CUDA, cudaGetErrorString(e));
    else if (n > cap)
      rc = fail(ctx, SWIFT_E_LIMIT, "output buffer too small");
  }
  if (stats) {
    stats->host_parse_ms = parse_ms;
    stats->h2d_ms = h2d_ms;
    stats->d2h_ms = ms_since(t0);
  }
  swift_reads_destroy(rd);
  return rc;
}

// The text goes to a malloc'd buffer (*out) or, with host_out, into
// host_out (host_cap bytes) in record ranges overlapped with its writing.
static int align_paired_impl(swift_ctx* ctx, const swift_index* idx, const char* reads1,
                             size_t len1, const char* reads2, size_t len2, const swift_params* p,
                             uint32_t min_frag, uint32_t max_frag, char** out, char* host_out,
                             size_t host_cap, size_t* out_len, swift_stats* stats) {
  if (!ctx || !idx || !reads1 || !reads2 || !p || !(out || host_out) || !out_len)
    return fail(ctx, SWIFT_E_ARG, "null argument");
  if (p->seed_len != idx->k) return fail(ctx, SWIFT_E_ARG, "seed length differs from the index's");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->st;
  swift_stats s;
  memset(&s, 0, sizeof(s));
  CK(cudaEventRecord(ctx->ev[0], st));
  swift_reads *rd1 = nullptr, *rd2 = nullptr;
  int rc = upload_reads(ctx, reads1, len1, &rd1, nullptr, nullptr, true);
  if (rc != SWIFT_OK) return rc;
  rc = upload_reads(ctx, reads2, len2, &rd2, nullptr, nullptr, true);
  if (rc != SWIFT_OK) {
    swift_reads_destroy(rd1);
    return rc;
  }
  struct Guard {
    swift_reads *a, *b;
    ~Guard() {
      swift_reads_destroy(a);
      swift_reads_destroy(b);
    }
  } guard{rd1, rd2};
  const int64_t n = rd1->n;
  if (rd2->n != n) return fail(ctx, SWIFT_E_INPUT, "the two reads files hold different numbers of reads");
  const int Q = p->qry_len > 0 ? p->qry_len : rd1->first_len;
  if (Q < 1 || Q > kReadMax) return fail(ctx, SWIFT_E_LIMIT, "query length outside 1..199");
  if (n > 0 && (rd1->min_len < Q || rd2->min_len < Q))
    return fail(ctx, SWIFT_E_INPUT, "a read is shorter than the query length; the reference "
                                    "aligns such reads against stale buffer contents");
  // mate names end in 1 or 2 (getMatePairName; otherwise the reference
  // pairs against the name it found before), checked on the device
  if (n) {
    Scratch scn(st);
    int32_t* d_bad;
    CK(scn.get(&d_bad, 1));
    CK(cudaMemsetAsync(d_bad, 0, sizeof(int32_t), st));
    launch_pe_names(st, rd1->d_bytes, rd1->d_rd, rd2->d_bytes, rd2->d_rd, n, d_bad);
    CKLAUNCH();
    int32_t bad = 0;
    CK(cudaMemcpyAsync(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (bad) return fail(ctx, SWIFT_E_INPUT, "paired-end read names must end in 1 or 2");
  }
  rc = ensure_lt2(ctx, idx);
  if (rc != SWIFT_OK) return rc;
  const swift_index* src = idx->pe_sub ? idx->pe_sub : idx;
  Scratch sc(st);
  // Phase 1: both files' strands on the lookupTable2 positions
  constexpr int kHits = 3;  // MAX_NUM_HITS_PAIRED_END (src/common.h:63)
  const int64_t ns = 2 * n;
  int3 *best1, *best2;
  int32_t *nb1, *nb2, *ovl, *novl;
  CK(sc.get(&best1, (size_t)std::max<int64_t>(ns, 1) * kHits));
  CK(sc.get(&best2, (size_t)std::max<int64_t>(ns, 1) * kHits));
  CK(sc.get(&nb1, (size_t)std::max<int64_t>(ns, 1)));
  CK(sc.get(&nb2, (size_t)std::max<int64_t>(ns, 1)));
  CK(sc.get(&ovl, (size_t)std::max<int64_t>(ns, 1)));
  CK(sc.get(&novl, 2));
  SeedOut so;
  for (int f = 0; f < 2; ++f) {
    CK(cudaMemsetAsync(novl, 0, 2 * sizeof(int32_t), st));
    SeedArgs a;
    memset(&a, 0, sizeof(a));
    const swift_reads* r = f == 0 ? rd1 : rd2;
    a.reads = r->d_bytes;
    a.rd = r->d_rd;
    a.n_reads = n;
    a.max_len = r->max_len;
    a.groups = src->d_groups;
    a.cstart = src->d_cstart;
    a.offsets = src->d_offsets;
    a.postings = idx->d_post_pe;
    a.gpos = idx->d_gpos_pe;
    a.gbase = idx->d_gbase;
    a.n_recs = (int)idx->recs.size();
    a.k = idx->k;
    a.max_hits = kHits;
    a.fixed_len = Q;
    a.best = f == 0 ? best1 : best2;
    a.nbest = f == 0 ? nb1 : nb2;
    a.overflow_list = ovl;
    a.n_overflow = novl;
    rc = seed_ssaha(ctx, sc, a, &so);
    if (rc != SWIFT_OK) return rc;
  }
  // records in searchQueries_paired2's order
  PairedArgs pa;
  memset(&pa, 0, sizeof(pa));
  pa.n_pairs = n;
  pa.max_hits = kHits;
  pa.nbest1 = nb1;
  pa.nbest2 = nb2;
  pa.best1 = best1;
  pa.best2 = best2;
  uint64_t *cnt, *roff, *tot_d;
  void* tmp;
  CK(sc.get(&cnt, (size_t)std::max<int64_t>(n, 1)));
  CK(sc.get(&roff, (size_t)std::max<int64_t>(n, 1)));
  CK(sc.get(&tot_d, 1));
  CK(sc.get((uint8_t**)&tmp, scan_temp_bytes(n)));
  launch_pe_records(st, pa, cnt);
  CKLAUNCH();
  int launches = (int)so.launches + (n > 0 ? 1 : 0) + exclusive_scan_u64(st, cnt, roff, n, tmp, tot_d);
  uint64_t nrec = 0;
  CK(cudaMemcpyAsync(&nrec, tot_d, 8, cudaMemcpyDeviceToHost, st));
  std::vector<uint64_t> h_cnt((size_t)std::max<int64_t>(n, 1));
  if (n) CK(cudaMemcpyAsync(h_cnt.data(), cnt, n * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const size_t nr = (size_t)std::max<uint64_t>(nrec, 1);
  CK(sc.get(&pa.m_id, nr));
  CK(sc.get(&pa.m_mate, nr));
  CK(sc.get(&pa.m_rev, nr));
  CK(sc.get(&pa.m_read, nr));
  CK(sc.get(&pa.m_ri, nr));
  CK(sc.get(&pa.m_shift, nr));
  CK(sc.get(&pa.m_off, nr));
  pa.roff = roff;
  pa.n_rec = (int64_t)nrec;
  launch_pe_fill(st, pa);
  CKLAUNCH();
  ++launches;
  CK(cudaEventRecord(ctx->ev[1], st));
  // both reads buffers back to back for names and queries
  char* d_reads;
  DevRead* d_rd;
  CK(sc.get(&d_reads, len1 + len2 + 64));
  CK(sc.get(&d_rd, (size_t)std::max<int64_t>(2 * n, 1)));
  CK(cudaMemcpyAsync(d_reads, rd1->d_bytes, len1, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(d_reads + len1, rd2->d_bytes, len2, cudaMemcpyDeviceToDevice, st));
  if (n) CK(cudaMemcpyAsync(d_rd, rd1->d_rd, n * sizeof(DevRead), cudaMemcpyDeviceToDevice, st));
  launch_shift_reads(st, rd2->d_rd, n, len1, d_rd + n);
  CKLAUNCH();
  // Phase 2 pairs: query Q, window 3Q; the packed passes trace pairs of
  // ACGT bytes with full windows, the generic kernel the others
  const int R = 3 * Q;
  const int64_t qs = (Q + 16) & ~15, ws = (R + 16) & ~15;
  const int64_t cs = ((int64_t)Q + R + 2 + 15) & ~(int64_t)15;  // the walk stores words
  char *qbuf, *wbuf, *qcons, *rcons;
  DevPair* pairs;
  DevAln* aln;
  CK(sc.get(&qbuf, nr * qs));
  CK(sc.get(&wbuf, nr * ws));
  CK(sc.get(&qcons, nr * cs));
  CK(sc.get(&rcons, nr * cs));
  CK(sc.get(&pairs, nr));
  CK(sc.get(&aln, nr));
  CK(cudaMemsetAsync(wbuf, 0, nr * ws, st));
  pa.Q = Q;
  pa.ref_file = idx->d_file;
  pa.cat = (const char*)idx->d_cat;
  pa.odd = idx->d_odd;
  pa.ref_file_len = idx->file_len;
  pa.recs = idx->d_recs;
  pa.reads = d_reads;
  pa.rd = d_rd;
  pa.pairs = pairs;
  pa.qbuf = qbuf;
  pa.wbuf = wbuf;
  pa.q_stride = qs;
  pa.w_stride = ws;
  launch_pe_pairs(st, pa);
  CKLAUNCH();
  ++launches;
  CK(cudaEventRecord(ctx->ev[2], st));
  int bias = 0;
  const bool fast_ok = fast_params_ok(Q, R, p->match, p->mismatch, p->gap_open, p->gap_ext, &bias);
  int32_t *fast_list, *gen_list, *lcnt;
  CK(sc.get(&fast_list, nr));
  CK(sc.get(&gen_list, nr));
  CK(sc.get(&lcnt, 2));
  CK(cudaMemsetAsync(lcnt, 0, 2 * sizeof(int32_t), st));
  if (nrec > 0) {
    partition_pairs_kernel<<<(unsigned)((nrec + 255) / 256), 256, 0, st>>>(
        pairs, (int64_t)nrec, fast_ok ? 0 : 1, fast_list, lcnt, gen_list, lcnt + 1);
    CKLAUNCH();
    ++launches;
    SwArgs sa;
    memset(&sa, 0, sizeof(sa));
    sa.q = qbuf;
    sa.w = wbuf;
    sa.q_stride = qs;
    sa.w_stride = ws;
    sa.Q = Q;
    sa.R = R;
    sa.match = p->match;
    sa.mismatch = p->mismatch;
    sa.gap_open = p->gap_open;
    sa.gap_ext = p->gap_ext;
    sa.n = (int64_t)nrec;
    sa.aln = aln;
    sa.qcons = qcons;
    sa.rcons = rcons;
    sa.cons_stride = cs;
    sa.list = gen_list;
    sa.count = lcnt + 1;
    rc = launch_sw(st, sa, &ctx->err);
    if (rc != SWIFT_OK) return rc;
    CKLAUNCH();
    ++launches;
    if (fast_ok) {
      int32_t h_fast = 0;
      CK(cudaMemcpyAsync(&h_fast, lcnt, 4, cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      const int64_t chunk = 262144;
      int2* best2;
      uint32_t* dirs;
      CK(sc.get(&best2, nr));
      CK(sc.get(&dirs, (size_t)trace_scratch_words(Q, R, std::min<int64_t>(std::max(h_fast, 1), chunk))));
      FastArgs fa2;
      memset(&fa2, 0, sizeof(fa2));
      fa2.q = qbuf;
      fa2.w = wbuf;
      fa2.q_stride = qs;
      fa2.w_stride = ws;
      fa2.Q = Q;
      fa2.R = R;
      fa2.match = p->match;
      fa2.mismatch = p->mismatch;
      fa2.gap_open = p->gap_open;
      fa2.gap_ext = p->gap_ext;
      fa2.bias = bias;
      fa2.aln = aln;
      fa2.qcons = qcons;
      fa2.rcons = rcons;
      fa2.cons_stride = cs;
      fa2.best = best2;
      fa2.list = fast_list;
      fa2.count = lcnt;
      fa2.dirs = dirs;
      for (int64_t off = 0; off < h_fast; off += chunk) {
        fa2.list_offset = off;
        const int kk = launch_sw_trace(st, fa2, std::min<int64_t>(chunk, h_fast - off));
        if (kk == 0) return fail(ctx, SWIFT_E_DEVICE, "trace pass could not launch");
        launches += kk;
        CKLAUNCH();
      }
    }
  }
  CK(cudaEventRecord(ctx->ev[3], st));
  // selection (chooseBestAlignment_paired3 per batch) on the host over the
  // per-record scores, names and coordinates; printing flags to the device
  const bool sam = p->out_format == 1;
  FormatArgs fa;
  memset(&fa, 0, sizeof(fa));
  fa.reads = d_reads;
  fa.rd = d_rd;
  fa.recs = idx->d_recs;
  fa.pairs = pairs;
  fa.aln = aln;
  fa.qcons = qcons;
  fa.rcons = rcons;
  fa.cons_stride = cs;
  fa.n = (int64_t)nrec;
  int32_t* keep;
  int8_t* sep;
  uint64_t *bytes, *offs, *tot2;
  void* tmp2;
  CK(sc.get(&keep, nr));
  CK(sc.get(&sep, nr));
  CK(sc.get(&bytes, nr));
  CK(sc.get(&offs, nr));
  CK(sc.get(&tot2, 1));
  CK(sc.get((uint8_t**)&tmp2, scan_temp_bytes((int64_t)nrec)));
  // Phase-2 batches: getNumQueriesPerIteration_paired (src/align.cu:2804-2824)
  // and getNumQrsPerIter_paired (src/align.cu:1812-1852) over the record ids,
  // which follow from the per-pair record counts; records past the last
  // batch are not aligned in the reference and not printed here
  std::vector<uint8_t> h_bs(nr, 0);
  uint64_t covered = 0;
  {
    const int64_t dev_mem = p->device_mem > 0 ? p->device_mem : ctx->total_mem;
    int64_t max_per;
    {
      const int mem_pair = (R + 1) + (Q + 1) + 4 + 4 + 4 + 2 + 2 * (Q + R + 2);
      const long gm = (long)(dev_mem - 100000000LL);
      max_per = (int)floor((float)gm / mem_pair);
      if (max_per > (int64_t)nrec) max_per = (int64_t)nrec;
    }
    if (max_per > 0) {
      std::vector<int64_t> per;
      int64_t old_count = 0, count = 0, old_id = 0;
      bool is_new = false;
      for (int64_t i = 0; i < n; ++i)
        for (uint64_t t = 0; t < h_cnt[i]; ++t) {
          ++count;
          const int64_t id = i + 1;
          if (is_new) {
            is_new = false;
            if (id == old_id) per.back() = old_count;
            else count = 1;
          } else if (id != old_id) {
            old_count = count - 1;
          }
          if (count == max_per) {
            per.push_back(count);
            count -= old_count;
            is_new = true;
          }
          old_id = id;
        }
      if (!is_new && count <= max_per) per.push_back(count);
      for (int64_t c : per) {
        if (covered < nrec) h_bs[covered] = 1;
        covered += (uint64_t)c;
      }
      covered = std::min<uint64_t>(covered, nrec);
    }
  }
  fa.n = (int64_t)covered;
  int64_t printed = (int64_t)covered;
  if (!sam && covered > 0) {
    // reference-name classes (the pairing compares names, not indices)
    std::vector<int32_t> h_class(idx->recs.size());
    for (size_t r = 0; r < idx->recs.size(); ++r) {
      h_class[r] = (int32_t)r;
      for (size_t q = 0; q < r; ++q)
        if (strcmp(idx->recs[q].name, idx->recs[r].name) == 0) {
          h_class[r] = (int32_t)q;
          break;
        }
    }
    uint8_t* d_bs;
    int32_t* d_class;
    uint32_t *run_flag, *run_of, *n_runs_d;
    int64_t* first;
    void* tmp3;
    CK(sc.get(&d_bs, nr));
    CK(sc.get(&d_class, std::max<size_t>(h_class.size(), 1)));
    CK(sc.get(&run_flag, nr));
    CK(sc.get(&run_of, nr));
    CK(sc.get(&n_runs_d, 1));
    CK(sc.get(&first, nr));
    CK(sc.get((uint8_t**)&tmp3, scan_temp_bytes((int64_t)nrec)));
    CK(cudaMemcpyAsync(d_bs, h_bs.data(), covered, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_class, h_class.data(), h_class.size() * 4, cudaMemcpyHostToDevice, st));
    PairSelArgs ps;
    memset(&ps, 0, sizeof(ps));
    ps.n = (int64_t)covered;
    ps.pairs = pairs;
    ps.aln = aln;
    ps.id = pa.m_id;
    ps.batch_start = d_bs;
    ps.reads = d_reads;
    ps.rd = d_rd;
    ps.ref_class = d_class;
    ps.min_frag = min_frag;
    ps.max_frag = max_frag;
    ps.keep = keep;
    ps.sep = sep;
    launch_pe_runs(st, ps, run_flag);
    CKLAUNCH();
    launches += 1 + exclusive_scan_u32(st, run_flag, run_of, (int64_t)covered, tmp3, n_runs_d);
    uint32_t n_runs = 0;
    CK(cudaMemcpyAsync(&n_runs, n_runs_d, 4, cudaMemcpyDeviceToHost, st));
    launch_pe_run_first(st, ps, run_flag, run_of, first);
    CKLAUNCH();
    CK(cudaStreamSynchronize(st));
    launch_pe_pair_runs(st, ps, first, (int64_t)n_runs);
    CKLAUNCH();
    launch_pe_sep(st, ps);
    CKLAUNCH();
    launches += 3;
    fa.keep = keep;
    fa.pe_sep = sep;
  }
  CK(cudaEventRecord(ctx->ev[4], st));
  fa.bytes = bytes;
  fa.offs = offs;
  if (sam)
    launch_sam_sizes(st, fa);
  else
    launch_format_sizes(st, fa);
  CKLAUNCH();
  launches += (covered > 0 ? 1 : 0) + exclusive_scan_u64(st, bytes, offs, (int64_t)covered, tmp2, tot2);
  uint64_t total = 0;
  CK(cudaMemcpyAsync(&total, tot2, 8, cudaMemcpyDeviceToHost, st));
  TextChunks chunks;
  rc = chunks.plan(ctx, st, offs, (int64_t)covered, host_out != nullptr);
  if (rc != SWIFT_OK) return rc;
  CK(cudaStreamSynchronize(st));
  char* d_text;
  CK(sc.get(&d_text, (size_t)total + 16));
  rc = chunks.write(ctx, st, fa, sam, d_text, total, host_out, host_cap, ctx->ev[5]);
  if (rc != SWIFT_OK) return rc;
  launches += covered > 0 ? chunks.n_chunks : 0;
  *out_len = total;
  if (host_out) {
    CK(cudaStreamSynchronize(st));
    if (total > host_cap) return fail(ctx, SWIFT_E_LIMIT, "output buffer too small");
  } else {
    char* h = (char*)malloc(total + 1);
    if (!h) return fail(ctx, SWIFT_E_NOMEM, "host output buffer");
    if (total) {
      const cudaError_t e = cudaMemcpyAsync(h, d_text, total, cudaMemcpyDeviceToHost, st);
      if (e != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
        free(h);
        return fail(ctx, SWIFT_E_CUDA, "output copy");
      }
    }
    h[total] = '\0';
    *out = h;
  }
  if (stats) {
    float t;
    cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[1]);
    s.seed_ms = t;
    cudaEventElapsedTime(&t, ctx->ev[1], ctx->ev[2]);
    s.pairs_ms = t;
    cudaEventElapsedTime(&t, ctx->ev[2], ctx->ev[3]);
    s.sw_ms = t;
    cudaEventElapsedTime(&t, ctx->ev[3], ctx->ev[4]);
    s.select_ms = t;
    cudaEventElapsedTime(&t, ctx->ev[4], ctx->ev[5]);
    s.format_ms = t;
    cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[5]);
    s.total_ms = t;
    s.reads = 2 * n;
    s.records = (int64_t)nrec;
    s.printed = printed;
    s.cells = (int64_t)nrec * Q * R;
    s.out_bytes = (int64_t)total;
    s.seed_overflow_strands = so.overflow;
    s.launches = launches;
    *stats = s;
  }
  return SWIFT_OK;
}

int swift_align_paired(swift_ctx* ctx, const swift_index* idx, const char* reads1, size_t len1,
                       const char* reads2, size_t len2, const swift_params* p,
                       uint32_t min_frag, uint32_t max_frag, char** out, size_t* out_len,
                       swift_stats* stats) {
  if (!out) return fail(ctx, SWIFT_E_ARG, "null argument");
  return align_paired_impl(ctx, idx, reads1, len1, reads2, len2, p, min_frag, max_frag, out,
                           nullptr, 0, out_len, stats);
}

int swift_align_paired_into(swift_ctx* ctx, const swift_index* idx, const char* reads1,
                            size_t len1, const char* reads2, size_t len2, const swift_params* p,
                            uint32_t min_frag, uint32_t max_frag, char* out, size_t cap,
                            size_t* out_len, swift_stats* stats) {
  if (!out) return fail(ctx, SWIFT_E_ARG, "null argument");
  return align_paired_impl(ctx, idx, reads1, len1, reads2, len2, p, min_frag, max_frag, nullptr,
                           out, cap, out_len, stats);
}

static int read_file(const char* path, std::vector<char>* buf, std::string* err) {
  FILE* f = fopen(path, "rb");
  if (!f) {
    *err = std::string("cannot open ") + path;
    return SWIFT_E_ARG;
  }
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  buf->resize((size_t)std::max(n, 0L));
  size_t got = n > 0 ? fread(buf->data(), 1, (size_t)n, f) : 0;
  fclose(f);
  if ((long)got != n) {
    *err = std::string("short read of ") + path;
    return SWIFT_E_ARG;
  }
  return SWIFT_OK;
}

int swift_align_files(swift_ctx* ctx, const char* qry_path, const char* ref_path,
                      const char* out_path, const swift_params* p) {
  if (!ctx || !qry_path || !ref_path || !out_path || !p) return fail(ctx, SWIFT_E_ARG, "null argument");
  std::vector<char> ref, qry;
  int rc = read_file(ref_path, &ref, &ctx->err);
  if (rc == SWIFT_OK) rc = read_file(qry_path, &qry, &ctx->err);
  if (rc != SWIFT_OK) return rc;
  swift_index* idx = nullptr;
  rc = swift_index_build(ctx, ref.data(), ref.size(), p->seed_len, p->ignore_thres, &idx);
  if (rc != SWIFT_OK) return rc;
  char* out = nullptr;
  size_t n = 0;
  rc = swift_align(ctx, idx, qry.data(), qry.size(), p, &out, &n, nullptr);
  swift_index_destroy(idx);
  if (rc != SWIFT_OK) return rc;
  FILE* f = fopen(out_path, "wb");
  if (!f) {
    free(out);
    return fail(ctx, SWIFT_E_ARG, std::string("cannot write ") + out_path);
  }
  size_t w = fwrite(out, 1, n, f);
  fclose(f);
  free(out);
  if (w != n) return fail(ctx, SWIFT_E_ARG, std::string("short write to ") + out_path);
  return SWIFT_OK;
}

}  // extern "C"
