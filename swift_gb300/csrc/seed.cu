// Phase 1 on the device: SSAHA hit emission and best-cluster selection for
// every read strand.  Restates lookupTable5MapQry (src/lookupTable5.cu:
// 557-603) and mapHits6GetBestHits (src/mapHits6.cu:40-318):
//   hits  = { (refIdx, refPos - i, refPos) : query offset i, posting of the
//             hash of query[i, i+k) }
//   sort by (refIdx, shift, refPos), clusters = runs of equal
//   (refIdx, shift), keep the first max_hits clusters of the biggest size and
//   report each cluster's first hit.
// The sort order is total (equal refIdx, refPos and shift imply equal i), so
// any exact sort reproduces the reference; ties between clusters of the same
// size keep the first ones in sort order.
//
// On-chip paths: one warp per strand.  The warp hashes the strand's k-mers
// (lane t owns the consecutive query offsets t*M .. t*M+M-1, so hits in lane
// order are hits in offset order), looks each up in the compact bucket
// directory and counts postings with a warp scan.  Then
//   - at most 32 hits (most strands): lane t fetches hit t; clusters are the
//     lanes whose (refIdx, shift) match (__match_any_sync), the biggest size
//     is a warp max, a cluster's first hit is its lowest lane, and the first
//     max_hits clusters in key order come from warp minima: no sort at all;
//   - up to 512 hits: the strand goes to a list for the sort kernel, which
//     writes 64-bit keys  refIdx << 41 | (shift + 512) << 9 | i  into shared
//     memory, sorts them (bitonic) and finds run lengths with ballots;
//   - more: a per-strand hash table in global scratch (one CTA each).
//
// Both warp kernels also add up the strand's bytes under the sector model of
// the seeding roofline (2-bit read, one 32-byte sector per directory lookup,
// the 5-byte postings of each occupied bucket in whole sectors, 12 bytes per
// hit out) into model_bytes, when it is given.
#include "internal.h"

namespace swift {
namespace {

constexpr int kSeedWarps = 8;          // warps per block
constexpr int kShiftBias = 512;        // shift >= -(kSeedReadMax - 1) always
constexpr int kFastHits = 32;          // hits of the sort-free path
constexpr int kHashCap = 256;          // hits of the hash-table path
constexpr int kHashSlots = 512;        // its table slots per warp (load <= 1/2)
constexpr int kHashWarps = 4;          // warps per block of the hash-table path
constexpr int kSortCap = 512;          // hits of the sort path

__device__ __forceinline__ uint8_t fwd_code(uint8_t c) {
  uint32_t u = c & 0xDFu;
  return u == 'C' ? 1 : u == 'G' ? 2 : u == 'T' ? 3 : 0;
}
// code of qryGetReverseComplement's output character for input c:
// A->T(3), C->G(2), G->C(1), anything else -> A(0) (case-sensitive)
__device__ __forceinline__ uint8_t rev_code(uint8_t c) {
  return c == 'A' ? 3 : c == 'C' ? 2 : c == 'G' ? 1 : 0;
}

__device__ __forceinline__ uint64_t make_key(uint32_t ri, int32_t shift, int32_t i) {
  return ((uint64_t)ri << 41) | ((uint64_t)(uint32_t)(shift + kShiftBias) << 9) | (uint32_t)i;
}

// words of 16 packed 2-bit codes covering kSeedReadMax bases, plus one word
constexpr int kPackedWords = (kSeedReadMax + 15) / 16 + 1;
// query offsets per lane at most (contiguous ranges of M = ceil(nq / 32));
// the kernels are instantiated for KM = 3, 5, 7 and 10 and launched with the
// smallest that covers the call's longest strand
constexpr int kM = (kSeedReadMax + 31) / 32;

struct WarpSmem {
  uint8_t codes[16 * kPackedWords];  // whole 16-code groups
  uint32_t packed[kPackedWords];
};

// The strand's hits per lane: loads its codes, packs them 2 bits each (code
// i at bits 2 (i % 16) of word i / 16, as the index packs the reference, so
// the hash of [i, i + k) is one funnel shift, k <= 15), and looks up the
// buckets of offsets i0 .. i0 + M - 1 (i0 = lane * M).  Returns the lane's
// postings; beg / cnt per offset.
template <int KM>
__device__ __forceinline__ uint32_t strand_lookups(const SeedArgs& a, const DevRead& rd, int strand,
                                                   int L, int nq, int M, WarpSmem& w, int lane,
                                                   uint32_t (&beg)[KM], uint32_t (&cnt)[KM]) {
  const char* s = a.reads + rd.seq_off;
  for (int i = lane; i < L; i += 32)
    w.codes[i] = strand == 0 ? fwd_code((uint8_t)s[i]) : rev_code((uint8_t)s[L - 1 - i]);
  __syncwarp();
  if (lane < kPackedWords) {
    uint32_t pw = 0;
    if (16 * lane < L) {
      const uint32_t* c4 = reinterpret_cast<const uint32_t*>(w.codes + 16 * lane);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        // codes past L are stale bytes: masked below
        const uint32_t x = c4[q];
        pw |= ((x & 3u) | ((x >> 6) & 0xCu) | ((x >> 12) & 0x30u) | ((x >> 18) & 0xC0u)) << (8 * q);
      }
      const int valid = L - 16 * lane;
      if (valid < 16) pw &= (1u << (2 * valid)) - 1u;
    }
    w.packed[lane] = pw;
  }
  __syncwarp();
  const uint32_t kmask = (1u << (2 * a.k)) - 1u;
  const int i0 = lane * M;
  uint32_t my = 0;
#pragma unroll
  for (int m = 0; m < KM; ++m) {
    const int i = i0 + m;
    beg[m] = cnt[m] = 0;
    if (m < M && i < nq) {
      const uint32_t h =
          __funnelshift_r(w.packed[i >> 4], w.packed[(i >> 4) + 1], 2 * (i & 15)) & kmask;
      // compact bucket directory: occupancy bits and rank, then the start
      // of occupied buckets only
      const uint4 grp = __ldg(&a.groups[h >> 6]);
      const uint64_t bits = ((uint64_t)grp.y << 32) | grp.x;
      if ((bits >> (h & 63)) & 1u) {
        const uint32_t r = grp.z + (uint32_t)__popcll(bits & ((1ull << (h & 63)) - 1));
        const uint32_t b = __ldg(&a.cstart[r]), e = __ldg(&a.cstart[r + 1]);
        beg[m] = b;
        cnt[m] = e - b;
        my += e - b;
      }
    }
  }
  return my;
}

// Posting sectors of the lane's lookups under the roofline's sector model.
template <int KM>
__device__ __forceinline__ uint32_t posting_sectors(const uint32_t (&cnt)[KM]) {
  uint32_t b = 0;
#pragma unroll
  for (int m = 0; m < KM; ++m) b += ((5u * cnt[m] + 31u) >> 5) << 5;
  return b;
}

// 64-bit mixer (the finaliser of MurmurHash3) for table slots
__device__ __forceinline__ uint32_t cluster_mix(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  return (uint32_t)x;
}

// lane 0 adds one strand's model bytes (warp-uniform arguments)
__device__ __forceinline__ void account(const SeedArgs& a, int lane, int L, int nq,
                                        uint32_t post_bytes, int hits_out) {
  if (a.model_bytes && lane == 0)
    atomicAdd(&a.model_bytes[blockIdx.x & (kSeedModelSlots - 1)],
              (unsigned long long)((L + 3) / 4 + 32 * max(nq, 0) + post_bytes + 12 * hits_out));
}

__device__ __forceinline__ int strand_nq(const SeedArgs& a, int L) {
  return (a.fixed_len > 0 ? a.fixed_len : L) - a.k + 1;
}

template <int KM>
__global__ void __launch_bounds__(kSeedWarps * 32) seed_fast_kernel(SeedArgs a) {
  __shared__ __align__(16) WarpSmem smem[kSeedWarps];
  __shared__ uint2 info_all[kSeedWarps][kFastHits];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t sid = (int64_t)blockIdx.x * kSeedWarps + wib;
  if (sid >= 2 * a.n_reads) return;
  const DevRead rd = a.rd[sid >> 1];
  const int strand = (int)(sid & 1);
  const int L = rd.len, nq = strand_nq(a, L);
  if (nq <= 0) {
    if (lane == 0) a.nbest[sid] = 0;
    account(a, lane, L, 0, 0, 0);
    return;
  }
  const int M = (nq + 31) >> 5;
  uint32_t beg[KM], cnt[KM];
  const uint32_t my = strand_lookups<KM>(a, rd, strand, L, nq, M, smem[wib], lane, beg, cnt);
  uint32_t incl = my;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += o;
  }
  const uint32_t n = __shfl_sync(0xffffffffu, incl, 31);
  if (n > (uint32_t)kFastHits) {
    // the hash-table, sort or overflow kernel takes the strand
    if (lane == 0) {
      if (n > (uint32_t)kSortCap) {
        a.overflow_list[atomicAdd(a.n_overflow, 1)] = (int32_t)sid;
        a.nbest[sid] = -(int32_t)n;  // hit count, for sizing the overflow table
      } else if (n > (uint32_t)kHashCap) {
        a.big_list[atomicAdd(a.n_big, 1)] = (int32_t)sid;
      } else {
        a.mid_list[atomicAdd(a.n_mid, 1)] = (int32_t)sid;
      }
    }
    if (n > (uint32_t)kSortCap) account(a, lane, L, nq, 0, 0);  // its lookups
    return;
  }
  const uint32_t post = __reduce_add_sync(0xffffffffu, posting_sectors<KM>(cnt));
  // hit t of the strand is posting t - start of the lookup that starts at
  // the last start at or before t: the starts as one bit mask, each start's
  // (first posting - start, query offset) in shared memory
  uint2* info = info_all[wib];
  uint32_t smask = 0, pos = incl - my;
#pragma unroll
  for (int m = 0; m < KM; ++m) {
    if (cnt[m]) {
      smask |= 1u << pos;
      info[pos] = make_uint2(beg[m] - pos, (uint32_t)(lane * M + m));
      pos += cnt[m];
    }
  }
  smask = __reduce_or_sync(0xffffffffu, smask);
  __syncwarp();
  // cluster key (refIdx, shift + bias); lanes without a hit get distinct
  // keys above every real one
  uint64_t ck = ~0ull - (uint64_t)lane;
  uint32_t ri = 0;
  int32_t shift = 0, qi = 0;
  if ((uint32_t)lane < n) {
    const int st = 31 - __clz(smask & (0xffffffffu >> (31 - lane)));
    const uint2 inf = info[st];
    const uint2 p = __ldg(&a.postings[inf.x + (uint32_t)lane]);
    ri = p.y;
    qi = (int32_t)inf.y;
    shift = (int32_t)p.x - qi;
    ck = ((uint64_t)ri << 32) | (uint32_t)(shift + kShiftBias);
  }
  const uint32_t same = __match_any_sync(0xffffffffu, ck);
  const uint32_t size = (uint32_t)lane < n ? (uint32_t)__popc(same) : 0u;
  const uint32_t biggest = __reduce_max_sync(0xffffffffu, size);
  // a cluster's first hit in key order is its lowest lane (offset order, and
  // two hits of one cluster never share an offset)
  uint32_t cand = __ballot_sync(0xffffffffu, size == biggest && size > 0 &&
                                                 (same & ((1u << lane) - 1u)) == 0u);
  const uint32_t hi = (uint32_t)(ck >> 32), lo = (uint32_t)ck;
  int3* out = a.best + sid * a.max_hits;
  int got = 0;
  while (cand && got < a.max_hits) {  // the smallest cluster keys first
    const bool in = (cand >> lane) & 1u;
    const uint32_t hmin = __reduce_min_sync(0xffffffffu, in ? hi : 0xffffffffu);
    const uint32_t lmin = __reduce_min_sync(0xffffffffu, in && hi == hmin ? lo : 0xffffffffu);
    const uint32_t win = __ballot_sync(0xffffffffu, in && hi == hmin && lo == lmin);
    if (lane == __ffs(win) - 1) out[got] = make_int3((int32_t)ri, shift, shift + qi);
    cand &= ~win;
    ++got;
  }
  if (lane == 0) a.nbest[sid] = got;
  account(a, lane, L, nq, post, got);
}

// The strands of a.mid_list (between kFastHits and kHashCap hits), without a
// sort: every hit enters a per-warp open-addressing table over its cluster
// key (refIdx, shift + bias) that counts the cluster and keeps its smallest
// query offset; the biggest count is a warp max over the table, and the
// first max_hits clusters of that size in key order come from warp minima.
// Warps stride over the list, whose length is on the device.
template <int KM>
__global__ void __launch_bounds__(kHashWarps * 32) seed_hash_kernel(SeedArgs a) {
  constexpr unsigned long long kEmpty = ~0ull;  // above every cluster key
  constexpr int kPerLane = kHashSlots / 32;
  __shared__ unsigned long long tkey_all[kHashWarps][kHashSlots];
  __shared__ uint32_t tcnt_all[kHashWarps][kHashSlots];
  __shared__ uint32_t tmin_all[kHashWarps][kHashSlots];
  __shared__ __align__(16) WarpSmem smem[kHashWarps];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned long long* tkey = tkey_all[wib];
  uint32_t* tcnt = tcnt_all[wib];
  uint32_t* tmin = tmin_all[wib];
  const int64_t n_list = *a.n_mid;
  for (int64_t t = (int64_t)blockIdx.x * kHashWarps + wib; t < n_list;
       t += (int64_t)gridDim.x * kHashWarps) {
    const int64_t sid = a.mid_list[t];
    const DevRead rd = a.rd[sid >> 1];
    const int strand = (int)(sid & 1);
    const int L = rd.len, nq = strand_nq(a, L);
    const int M = (nq + 31) >> 5;
    uint32_t beg[KM], cnt[KM];
    const uint32_t my = strand_lookups<KM>(a, rd, strand, L, nq, M, smem[wib], lane, beg, cnt);
    const uint32_t n = __reduce_add_sync(0xffffffffu, my);  // in (kFastHits, kHashCap]
    const uint32_t post = __reduce_add_sync(0xffffffffu, posting_sectors<KM>(cnt));
    // a power of two at least twice the hits
    uint32_t T = 64;
    while (T < 2 * n) T <<= 1;
    for (uint32_t i = lane; i < T; i += 32) {
      tkey[i] = kEmpty;
      tcnt[i] = 0;
      tmin[i] = 0xffffffffu;
    }
    __syncwarp();
#pragma unroll
    for (int m = 0; m < KM; ++m) {
      const uint32_t i = (uint32_t)(lane * M + m);
      for (uint32_t j = 0; j < cnt[m]; ++j) {
        const uint2 p = __ldg(&a.postings[beg[m] + j]);
        const unsigned long long ck =
            ((unsigned long long)p.y << 32) | (uint32_t)((int32_t)p.x - (int32_t)i + kShiftBias);
        uint32_t slot = cluster_mix(ck) & (T - 1);
        for (uint32_t probe = 0; probe < T; ++probe) {  // T > n: a free slot exists
          const unsigned long long old = atomicCAS(&tkey[slot], kEmpty, ck);
          if (old == kEmpty || old == ck) {
            atomicAdd(&tcnt[slot], 1u);
            atomicMin(&tmin[slot], i);
            break;
          }
          slot = (slot + 1) & (T - 1);
        }
      }
    }
    __syncwarp();
    // the biggest cluster, then its clusters as candidate bits of the lane's
    // slots lane, lane + 32, ...
    uint32_t big = 0;
    for (uint32_t i = lane; i < T; i += 32) big = max(big, tcnt[i]);
    big = __reduce_max_sync(0xffffffffu, big);
    uint32_t cand = 0;
#pragma unroll
    for (int q = 0; q < kPerLane; ++q) {
      const uint32_t i = lane + 32 * q;
      if (i < T && tcnt[i] == big) cand |= 1u << q;
    }
    int got = 0;
    int3* out = a.best + sid * a.max_hits;
    while (got < a.max_hits) {  // the smallest cluster keys first
      unsigned long long mk = kEmpty;
      int mq = -1;
      for (uint32_t c = cand; c; c &= c - 1) {
        const int q = __ffs(c) - 1;
        const unsigned long long k = tkey[lane + 32 * q];
        if (k < mk) {
          mk = k;
          mq = q;
        }
      }
      const uint32_t hi = (uint32_t)(mk >> 32), lo = (uint32_t)mk;
      const uint32_t hmin = __reduce_min_sync(0xffffffffu, hi);
      if (hmin == 0xffffffffu) break;  // no candidate left
      const uint32_t lmin = __reduce_min_sync(0xffffffffu, hi == hmin ? lo : 0xffffffffu);
      const uint32_t win = __ballot_sync(0xffffffffu, mq >= 0 && hi == hmin && lo == lmin);
      if (lane == __ffs(win) - 1) {
        const int32_t shift = (int32_t)lo - kShiftBias;
        out[got] = make_int3((int32_t)hi, shift, shift + (int32_t)tmin[lane + 32 * mq]);
        cand &= ~(1u << mq);
      }
      ++got;
    }
    if (lane == 0) a.nbest[sid] = got;
    account(a, lane, L, nq, post, got);
    __syncwarp();  // the table is cleared for the next strand
  }
}

// The sort path over the strands of a.big_list (between kHashCap and
// kSortCap hits); warps stride over the list, whose length is on the device.
template <int CAP, int KM>
__global__ void __launch_bounds__(kSeedWarps * 32, 6) seed_sort_kernel(SeedArgs a) {
  // the sort pads n <= CAP keys to the next power of two, which must fit
  static_assert(CAP >= 32 && (CAP & (CAP - 1)) == 0, "CAP must be a power of two");
  __shared__ uint64_t keys_all[kSeedWarps][CAP];
  __shared__ __align__(16) WarpSmem smem[kSeedWarps];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint64_t* keys = keys_all[wib];
  const int64_t n_list = *a.n_big;
  for (int64_t t = (int64_t)blockIdx.x * kSeedWarps + wib; t < n_list;
       t += (int64_t)gridDim.x * kSeedWarps) {
    const int64_t sid = a.big_list[t];
    const DevRead rd = a.rd[sid >> 1];
    const int strand = (int)(sid & 1);
    const int L = rd.len, nq = strand_nq(a, L);
    const int M = (nq + 31) >> 5;
    uint32_t beg[KM], cnt[KM];
    const uint32_t my = strand_lookups<KM>(a, rd, strand, L, nq, M, smem[wib], lane, beg, cnt);
    uint32_t incl = my;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += o;
    }
    const uint32_t n = __shfl_sync(0xffffffffu, incl, 31);  // in (kHashCap, CAP]
    const uint32_t post = __reduce_add_sync(0xffffffffu, posting_sectors<KM>(cnt));
    uint32_t pos = incl - my;
#pragma unroll
    for (int m = 0; m < KM; ++m) {
      const int i = lane * M + m;
      for (uint32_t j = 0; j < cnt[m]; ++j) {
        const uint2 p = __ldg(&a.postings[beg[m] + j]);
        keys[pos++] = make_key(p.y, (int32_t)p.x - i, i);
      }
    }
    uint32_t P = 32;
    while (P < n) P <<= 1;
    for (uint32_t i = n + lane; i < P; i += 32) keys[i] = ~0ull;
    __syncwarp();
    // bitonic sort of keys[0, P)
    for (uint32_t size = 2; size <= P; size <<= 1) {
      for (uint32_t stride = size >> 1, ls = __ffs(stride) - 1; stride > 0; stride >>= 1, --ls) {
        for (uint32_t u = lane; u < P / 2; u += 32) {
          const uint32_t i = ((u >> ls) << (ls + 1)) | (u & (stride - 1));
          const uint32_t j = i + stride;
          const bool asc = (i & size) == 0;
          const uint64_t x = keys[i], y = keys[j];
          if ((x > y) == asc) {
            keys[i] = y;
            keys[j] = x;
          }
        }
        __syncwarp();
      }
    }
    // run lengths at run starts, scanning chunks back to front: the biggest
    const uint32_t nch = (n + 31) >> 5;
    auto starts = [&](uint32_t c) {
      const uint32_t idx = c * 32 + lane;
      const bool start = idx < n && (idx == 0 || (keys[idx] >> 9) != (keys[idx - 1] >> 9));
      return __ballot_sync(0xffffffffu, start);
    };
    // the run start ending a run that starts at lane `lane` of a chunk whose
    // starts are bal, if it lies in the same chunk (else 0)
    auto next_in_chunk = [&](uint32_t c, uint32_t bal) -> uint32_t {
      const uint32_t above = lane < 31 ? (bal >> (lane + 1)) << (lane + 1) : 0u;
      return above ? c * 32 + __ffs(above) - 1 : 0u;
    };
    uint32_t next = n, biggest = 0;
    for (int c = (int)nch - 1; c >= 0; --c) {
      const uint32_t bal = starts(c);
      if ((bal >> lane) & 1u) {
        const uint32_t nx = next_in_chunk(c, bal);
        biggest = max(biggest, (nx ? nx : next) - ((uint32_t)c * 32 + lane));
      }
      if (bal) next = (uint32_t)c * 32 + __ffs(bal) - 1;
    }
    biggest = __reduce_max_sync(0xffffffffu, biggest);
    // first max_hits runs of the biggest size, front to back: a chunk's last
    // run stays open until the next start (or the end) closes it
    int got = 0;
    int3* out = a.best + sid * a.max_hits;
    auto emit = [&](uint32_t idx) {  // lane 0; got is warp-uniform
      if (lane == 0) {
        const uint64_t key = keys[idx];
        const int32_t ri = (int32_t)(key >> 41);
        const int32_t shift = (int32_t)((key >> 9) & 0xffffffffu) - kShiftBias;
        const int32_t i = (int32_t)(key & 0x1ff);
        out[got] = make_int3(ri, shift, shift + i);
      }
      ++got;
    };
    uint32_t open = ~0u;  // start of the run open at the last chunk boundary
    for (uint32_t c = 0; c < nch && got < a.max_hits; ++c) {
      const uint32_t bal = starts(c);
      if (!bal) continue;
      if (open != ~0u) {
        if ((uint32_t)(c * 32 + __ffs(bal) - 1) - open == biggest) emit(open);
        open = ~0u;
      }
      const uint32_t nx = next_in_chunk(c, bal);
      uint32_t hb = __ballot_sync(0xffffffffu, ((bal >> lane) & 1u) && nx && nx - (c * 32 + lane) == biggest);
      while (hb && got < a.max_hits) {
        emit(c * 32 + __ffs(hb) - 1);
        hb &= hb - 1;
      }
      open = c * 32 + 31 - __clz(bal);
    }
    if (open != ~0u && got < a.max_hits && n - open == biggest) emit(open);
    if (lane == 0) a.nbest[sid] = got;
    account(a, lane, L, nq, post, got);
    __syncwarp();  // keys are rewritten by the next strand
  }
}

// ---------------------------------------------------------------------------
// Overflow path: one CTA per strand, open-addressing table over cluster keys
// (refIdx, shift) with counts and the smallest query offset (kept as
// 1023 - offset under atomicMax so that the table starts all zero).

constexpr int kOvThreads = 512;

__device__ __forceinline__ uint32_t mix(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  return (uint32_t)x;
}

__global__ void __launch_bounds__(kOvThreads) seed_overflow_kernel(SeedArgs a,
                                                                   const uint64_t* tab_off,
                                                                   const uint32_t* tab_size) {
  __shared__ uint8_t codes[kSeedReadMax + 1];
  __shared__ uint64_t red[kOvThreads / 32];
  const int64_t sid = a.overflow_list[blockIdx.x];
  const int64_t read = sid >> 1;
  const int strand = (int)(sid & 1);
  const DevRead rd = a.rd[read];
  const int L = rd.len, k = a.k, nq = (a.fixed_len > 0 ? a.fixed_len : L) - k + 1;
  const uint32_t S = tab_size[blockIdx.x];
  uint64_t* tk = a.scratch + tab_off[blockIdx.x];
  uint32_t* tc = reinterpret_cast<uint32_t*>(tk + S);
  uint32_t* ti = tc + S;
  const char* s = a.reads + rd.seq_off;
  for (int i = threadIdx.x; i < L; i += blockDim.x)
    codes[i] = strand == 0 ? fwd_code((uint8_t)s[i]) : rev_code((uint8_t)s[L - 1 - i]);
  __syncthreads();
  // insert every hit; each warp walks one query offset's bucket at a time
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = wid; i < nq; i += nw) {
    uint32_t h = 0;
    for (int t = k - 1; t >= 0; --t) h = (h << 2) | codes[i + t];
    uint32_t b = a.offsets[h], e = a.offsets[h + 1];
    for (uint32_t j = b + lane; j < e; j += 32) {
      uint2 p = a.postings[j];
      uint64_t ck = make_key(p.y, (int32_t)p.x - i, 0) >> 9;  // nonzero
      uint32_t slot = mix(ck) & (S - 1);
      for (uint32_t probe = 0; probe < S; ++probe) {
        unsigned long long old = atomicCAS((unsigned long long*)&tk[slot], 0ull,
                                           (unsigned long long)ck);
        if (old == 0ull || old == ck) {
          atomicAdd(&tc[slot], 1u);
          atomicMax(&ti[slot], 1023u - (uint32_t)i);  // zero-initialised table
          break;
        }
        slot = (slot + 1) & (S - 1);
      }
    }
  }
  __syncthreads();
  // biggest cluster size
  uint32_t big = 0;
  for (uint32_t x = threadIdx.x; x < S; x += blockDim.x) big = max(big, tc[x]);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) big = max(big, __shfl_xor_sync(0xffffffffu, big, d));
  if (lane == 0) red[wid] = big;
  __syncthreads();
  big = 0;
  for (int w = 0; w < nw; ++w) big = max(big, (uint32_t)red[w]);
  __syncthreads();
  // the first max_hits cluster keys of that size, smallest first
  uint64_t last = 0;
  int got = 0;
  int3* out = a.best + sid * a.max_hits;
  for (int g = 0; g < a.max_hits; ++g) {
    uint64_t mn = ~0ull;
    for (uint32_t x = threadIdx.x; x < S; x += blockDim.x)
      if (tc[x] == big && tk[x] > last && tk[x] < mn) mn = tk[x];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      uint64_t o = __shfl_xor_sync(0xffffffffu, mn, d);
      mn = o < mn ? o : mn;
    }
    if (lane == 0) red[wid] = mn;
    __syncthreads();
    mn = ~0ull;
    for (int w = 0; w < nw; ++w) mn = red[w] < mn ? red[w] : mn;
    __syncthreads();
    if (mn == ~0ull) break;
    if (threadIdx.x == 0) {
      uint32_t slot = mix(mn) & (S - 1);
      while (tk[slot] != mn) slot = (slot + 1) & (S - 1);
      int32_t ri = (int32_t)(mn >> 32);
      int32_t shift = (int32_t)(mn & 0xffffffffu) - kShiftBias;
      out[got] = make_int3(ri, shift, shift + (int32_t)(1023u - ti[slot]));
    }
    ++got;
    last = mn;
  }
  if (threadIdx.x == 0) a.nbest[sid] = got;
}

}  // namespace

template <int KM>
void launch_seed_km(cudaStream_t st, const SeedArgs& a) {
  const int64_t strands = 2 * a.n_reads;
  const unsigned grid = (unsigned)((strands + kSeedWarps - 1) / kSeedWarps);
  seed_fast_kernel<KM><<<grid, kSeedWarps * 32, 0, st>>>(a);
  // the listed strands: grids of a few waves stride over the lists (their
  // lengths are on the device)
  int dev = 0, sms = 0;
  int64_t cap = 1 << 20;
  if (cudaGetDevice(&dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0)
    cap = (int64_t)sms * 4 * 4;
  const int64_t hash_blocks = std::min<int64_t>((strands + kHashWarps - 1) / kHashWarps, 2 * cap);
  seed_hash_kernel<KM><<<(unsigned)hash_blocks, kHashWarps * 32, 0, st>>>(a);
  const int64_t sort_blocks = std::min<int64_t>((strands + kSeedWarps - 1) / kSeedWarps, cap);
  seed_sort_kernel<kSortCap, KM><<<(unsigned)sort_blocks, kSeedWarps * 32, 0, st>>>(a);
}

void launch_seed(cudaStream_t st, const SeedArgs& a) {
  if (a.n_reads <= 0) return;
  // offsets per lane of the longest strand
  const int nq = (a.fixed_len > 0 ? a.fixed_len : a.max_len) - a.k + 1;
  const int M = std::max(1, (nq + 31) / 32);
  if (M <= 3)
    launch_seed_km<3>(st, a);
  else if (M <= 5)
    launch_seed_km<5>(st, a);
  else if (M <= 7)
    launch_seed_km<7>(st, a);
  else
    launch_seed_km<kM>(st, a);
}

int seed_smem_cap() { return kSortCap; }

void launch_seed_overflow(cudaStream_t st, const SeedArgs& a, int n_overflow,
                          const uint64_t* tab_off, const uint32_t* tab_size) {
  if (n_overflow <= 0) return;
  seed_overflow_kernel<<<n_overflow, kOvThreads, 0, st>>>(a, tab_off, tab_size);
}

}  // namespace swift
