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
//   - up to 512 hits: the strand goes to a list for a hash-table kernel
//     (a table of up to 256 or 1024 slots per warp in shared memory), which
//     counts the clusters without a sort;
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
constexpr int kMidCap = 128;           // hits of the small hash-table path
constexpr int kBigCap = 512;           // hits of the large hash-table path

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

// With global positions (a.gpos), a cluster key is the hit's global
// position minus its query offset: sequence r's keys lie in
// [gbase[r] - 319, gbase[r] + length + 64), and sequences sit kGPad = 512
// positions apart, so the sequence of a key is the last r with
// gbase[r] - 400 <= key (a binary search, for the few clusters emitted),
// and keys order as (refIdx, shift) do.
__device__ __forceinline__ int3 global_cluster(const SeedArgs& a, uint32_t key, int32_t qoff) {
  int lo = 0, hi = a.n_recs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&a.gbase[mid]) - 400u <= key) lo = mid; else hi = mid - 1;
  }
  const int32_t shift = (int32_t)(key - __ldg(&a.gbase[lo]));
  return make_int3(lo, shift, shift + qoff);
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

template <int KM, bool G>
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
      if (n > (uint32_t)kBigCap) {
        a.overflow_list[atomicAdd(a.n_overflow, 1)] = (int32_t)sid;
        a.nbest[sid] = -(int32_t)n;  // hit count, for sizing the overflow table
      } else if (n > (uint32_t)kMidCap) {
        a.big_list[atomicAdd(a.n_big, 1)] = (int32_t)sid;
      } else {
        a.mid_list[atomicAdd(a.n_mid, 1)] = (int32_t)sid;
      }
    }
    if (n > (uint32_t)kBigCap) account(a, lane, L, nq, 0, 0);  // its lookups
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
  // cluster key (refIdx, shift + bias), or the global shift; lanes without
  // a hit get distinct keys above every real one
  uint64_t ck = G ? (uint64_t)(0xffffffffu - (uint32_t)lane) : ~0ull - (uint64_t)lane;
  uint32_t ri = 0, pidx = 0;
  int32_t shift = 0, qi = 0;
  if ((uint32_t)lane < n) {
    const int st = 31 - __clz(smask & (0xffffffffu >> (31 - lane)));
    const uint2 inf = info[st];
    qi = (int32_t)inf.y;
    pidx = inf.x + (uint32_t)lane;
    if (G) {
      ck = (uint64_t)(__ldg(&a.gpos[pidx]) - (uint32_t)qi);
    } else {
      const uint2 p = __ldg(&a.postings[inf.x + (uint32_t)lane]);
      ri = p.y;
      shift = (int32_t)p.x - qi;
      ck = ((uint64_t)ri << 32) | (uint32_t)(shift + kShiftBias);
    }
  }
  const uint32_t same = G ? __match_any_sync(0xffffffffu, (uint32_t)ck)
                          : __match_any_sync(0xffffffffu, ck);
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
    if (lane == __ffs(win) - 1) {
      if (G) {  // the winning hit's own posting
        const uint2 p = __ldg(&a.postings[pidx]);
        out[got] = make_int3((int32_t)p.y, (int32_t)p.x - qi, (int32_t)p.x);
      } else {
        out[got] = make_int3((int32_t)ri, shift, shift + qi);
      }
    }
    cand &= ~win;
    ++got;
  }
  if (lane == 0) a.nbest[sid] = got;
  account(a, lane, L, nq, post, got);
}

// The strands of one list (a.mid_list: kFastHits < hits <= kMidCap;
// a.big_list: kMidCap < hits <= kBigCap), without a sort.  The hits are
// gathered cooperatively, hit h by lane h mod 32: the lookups that have
// postings mark their first hit in a bit mask, and hit h belongs to the last
// mark at or before it (found from the mask words, warp-uniform).  Each hit
// enters a per-warp open-addressing table whose slot holds its cluster's key
// (refIdx, shift + bias) above a 16-bit count: one compare-and-swap claims a
// free slot with count 1, an add counts the hits of a slot already holding
// the key; the table is at most two thirds full.  Hits are gathered and
// entered in passes of half the rounds (every posting load of a pass issued
// before any is used), and what a hit keeps afterwards is its query offset
// and slot: its key and its cluster's size are in the table.  The biggest
// count is a warp max; every lane keeps the three smallest keys of that
// count among its hits (equal keys merged, their offsets minimised), and the
// first clusters in key order, each with its smallest query offset, are
// warp minima over those; beyond three clusters a scan over the hits
// continues from the last key.  A strand's work grows with its hits, not
// with the table: the table is emptied once per warp and each strand empties
// only the slots it used.  Warps stride over the list, whose length is on
// the device.
template <int KM, int CAP, int WARPS, int MIN_BLOCKS, bool G>
__global__ void __launch_bounds__(WARPS * 32, MIN_BLOCKS) seed_hash_kernel(SeedArgs a) {
  constexpr unsigned long long kEmpty = ~0ull;  // above every slot value
  constexpr int kSlots = CAP + CAP / 2;         // load <= 2/3
  constexpr int kRounds = CAP / 32;             // hits per lane at most
  constexpr int kPasses = CAP > 128 ? 2 : 1;    // gather and enter in passes
  constexpr int kPassRounds = kRounds / kPasses;
  constexpr int kKeep = 3;                      // smallest keys kept per lane
  static_assert(32 * KM <= 512 && kSlots <= 2048 && kRounds % kPasses == 0, "meta bit fields");
  __shared__ unsigned long long tab_all[WARPS][kSlots];  // key << 16 | count
  __shared__ uint2 start_all[WARPS][CAP];       // first hit -> (posting - hit, offset)
  __shared__ uint32_t mark_all[WARPS][kRounds];  // first hits as bits
  __shared__ __align__(16) WarpSmem smem[WARPS];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned long long* tab = tab_all[wib];
  uint2* start = start_all[wib];
  uint32_t* mark = mark_all[wib];
  const bool big = CAP > kMidCap;
  const int64_t n_list = big ? *a.n_big : *a.n_mid;
  const int32_t* list = big ? a.big_list : a.mid_list;
  for (int i = lane; i < kSlots; i += 32) tab[i] = kEmpty;
  for (int64_t t = (int64_t)blockIdx.x * WARPS + wib; t < n_list;
       t += (int64_t)gridDim.x * WARPS) {
    if (lane < kRounds) mark[lane] = 0;
    __syncwarp();
    const int64_t sid = list[t];
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
    const uint32_t n = __shfl_sync(0xffffffffu, incl, 31);  // in the list's range
    const uint32_t post = __reduce_add_sync(0xffffffffu, posting_sectors<KM>(cnt));
    uint32_t pos = incl - my;
#pragma unroll
    for (int m = 0; m < KM; ++m) {
      if (cnt[m]) {
        start[pos] = make_uint2(beg[m] - pos, (uint32_t)(lane * M + m));
        atomicOr(&mark[pos >> 5], 1u << (pos & 31));
        pos += cnt[m];
      }
    }
    __syncwarp();
    // per hit: its query offset (bits 0-8) and table slot (bits 9-20)
    uint32_t meta[kRounds];
    uint32_t carry = 0;  // the last first hit before the round (hit 0 is one)
#pragma unroll
    for (int ps = 0; ps < kPasses; ++ps) {
      uint2 ph[kPassRounds];
#pragma unroll
      for (int q = 0; q < kPassRounds; ++q) {
        const int r = ps * kPassRounds + q;
        meta[r] = 0;
        ph[q] = make_uint2(0, 0);
        if (32u * r < n) {
          const uint32_t w = mark[r];
          const uint32_t below = w & (0xffffffffu >> (31 - lane));
          const uint32_t st = below ? 32u * r + 31u - __clz(below) : carry;
          carry = w ? 32u * r + 31u - __clz(w) : carry;
          const uint32_t h = lane + 32u * r;
          if (h < n) {
            const uint2 inf = start[st];
            meta[r] = inf.y;
            if (G)
              ph[q].x = __ldg(&a.gpos[inf.x + h]);
            else
              ph[q] = __ldg(&a.postings[inf.x + h]);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < kPassRounds; ++q) {
        const int r = ps * kPassRounds + q;
        if (lane + 32u * r < n) {
          const unsigned long long key =
              G ? (unsigned long long)(ph[q].x - meta[r])
                : ((unsigned long long)ph[q].y << 32) |
                      (uint32_t)((int32_t)ph[q].x - (int32_t)meta[r] + kShiftBias);
          uint32_t slot = (uint32_t)(((unsigned long long)cluster_mix(key) * kSlots) >> 32);
          for (int probe = 0; probe < kSlots; ++probe) {  // kSlots > n: a free slot exists
            const unsigned long long old = atomicCAS(&tab[slot], kEmpty, (key << 16) | 1ull);
            if (old == kEmpty) break;
            if ((old >> 16) == key) {
              atomicAdd(&tab[slot], 1ull);
              break;
            }
            slot = slot + 1 == (uint32_t)kSlots ? 0u : slot + 1;
          }
          meta[r] |= slot << 9;
        }
      }
    }
    __syncwarp();
    auto slot_of = [&](int r) -> uint32_t { return (meta[r] >> 9) & 4095u; };
    // the biggest cluster over the hits' own slots
    uint32_t bigc = 0;
#pragma unroll
    for (int r = 0; r < kRounds; ++r)
      if (lane + 32u * r < n) bigc = max(bigc, (uint32_t)(tab[slot_of(r)] & 0xFFFFu));
    bigc = __reduce_max_sync(0xffffffffu, bigc);
    // the lane's kKeep smallest keys of that size, ascending
    unsigned long long lk[kKeep];
    uint32_t lo[kKeep];
#pragma unroll
    for (int q = 0; q < kKeep; ++q) {
      lk[q] = kEmpty;
      lo[q] = 0xffffffffu;
    }
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
      if (lane + 32u * r < n) {
        const unsigned long long v = tab[slot_of(r)];
        if ((uint32_t)(v & 0xFFFFu) == bigc) {
          unsigned long long k = v >> 16;
          uint32_t o = meta[r] & 511u;
#pragma unroll
          for (int q = 0; q < kKeep; ++q) {
            if (k == lk[q]) {
              lo[q] = min(lo[q], o);
              k = kEmpty;
            } else if (k < lk[q]) {
              const unsigned long long tk = lk[q];
              const uint32_t to = lo[q];
              lk[q] = k;
              lo[q] = o;
              k = tk;
              o = to;
            }
          }
        }
      }
    }
    int got = 0;
    int3* out = a.best + sid * a.max_hits;
    unsigned long long last = 0;  // every key is above 0
    const int first = min(a.max_hits, kKeep);
    while (got < first) {
      // the lane's first key not taken yet is lk[0]: taken keys shift out
      const uint32_t hmin = __reduce_min_sync(0xffffffffu, (uint32_t)(lk[0] >> 32));
      if (hmin == 0xffffffffu) break;  // no cluster left
      const uint32_t lmin = __reduce_min_sync(
          0xffffffffu, (uint32_t)(lk[0] >> 32) == hmin ? (uint32_t)lk[0] : 0xffffffffu);
      const unsigned long long K = ((unsigned long long)hmin << 32) | lmin;
      const bool mine = lk[0] == K;
      const uint32_t mi = __reduce_min_sync(0xffffffffu, mine ? lo[0] : 0xffffffffu);
      if (lane == 0) {
        const int32_t shift = (int32_t)lmin - kShiftBias;
        out[got] = G ? global_cluster(a, lmin, (int32_t)mi)
                     : make_int3((int32_t)hmin, shift, shift + (int32_t)mi);
      }
      if (mine) {
#pragma unroll
        for (int q = 0; q + 1 < kKeep; ++q) {
          lk[q] = lk[q + 1];
          lo[q] = lo[q + 1];
        }
        lk[kKeep - 1] = kEmpty;
      }
      last = K;
      ++got;
    }
    // more than kKeep clusters wanted (and kKeep found): scan the hits for
    // the next keys
    if (got == kKeep) {
      while (got < a.max_hits) {
        unsigned long long mk = kEmpty;
#pragma unroll
        for (int r = 0; r < kRounds; ++r) {
          if (lane + 32u * r < n) {
            const unsigned long long v = tab[slot_of(r)];
            const unsigned long long k = v >> 16;
            if ((uint32_t)(v & 0xFFFFu) == bigc && k > last && k < mk) mk = k;
          }
        }
        const uint32_t hmin = __reduce_min_sync(0xffffffffu, (uint32_t)(mk >> 32));
        if (hmin == 0xffffffffu) break;  // no cluster left
        const uint32_t lmin = __reduce_min_sync(
            0xffffffffu, (uint32_t)(mk >> 32) == hmin ? (uint32_t)mk : 0xffffffffu);
        const unsigned long long K = ((unsigned long long)hmin << 32) | lmin;
        uint32_t mi = 0xffffffffu;
#pragma unroll
        for (int r = 0; r < kRounds; ++r)
          if (lane + 32u * r < n && (tab[slot_of(r)] >> 16) == K) mi = min(mi, meta[r] & 511u);
        mi = __reduce_min_sync(0xffffffffu, mi);
        if (lane == 0) {
          const int32_t shift = (int32_t)lmin - kShiftBias;
          out[got] = G ? global_cluster(a, lmin, (int32_t)mi)
                       : make_int3((int32_t)hmin, shift, shift + (int32_t)mi);
        }
        last = K;
        ++got;
      }
    }
    if (lane == 0) a.nbest[sid] = got;
    account(a, lane, L, nq, post, got);
    __syncwarp();
    // empty the slots this strand used (marks are cleared, starts rewritten)
#pragma unroll
    for (int r = 0; r < kRounds; ++r)
      if (lane + 32u * r < n) tab[slot_of(r)] = kEmpty;
    __syncwarp();
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

template <bool G>
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
      uint64_t ck;  // nonzero
      if (G) {
        ck = (uint64_t)(a.gpos[j] - (uint32_t)i);
      } else {
        const uint2 p = a.postings[j];
        ck = make_key(p.y, (int32_t)p.x - i, 0) >> 9;
      }
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
      if (G) {
        out[got] = global_cluster(a, (uint32_t)mn, (int32_t)(1023u - ti[slot]));
      } else {
        int32_t ri = (int32_t)(mn >> 32);
        int32_t shift = (int32_t)(mn & 0xffffffffu) - kShiftBias;
        out[got] = make_int3(ri, shift, shift + (int32_t)(1023u - ti[slot]));
      }
    }
    ++got;
    last = mn;
  }
  if (threadIdx.x == 0) a.nbest[sid] = got;
}

}  // namespace

template <int KM, bool G>
void launch_seed_kg(cudaStream_t st, const SeedArgs& a) {
  const int64_t strands = 2 * a.n_reads;
  const unsigned grid = (unsigned)((strands + kSeedWarps - 1) / kSeedWarps);
  seed_fast_kernel<KM, G><<<grid, kSeedWarps * 32, 0, st>>>(a);
  // the listed strands: grids of a few waves stride over the lists (their
  // lengths are on the device)
  int dev = 0, sms = 0;
  int64_t cap = 1 << 16;
  if (cudaGetDevice(&dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0)
    cap = (int64_t)sms * 8;
  constexpr int kMidWarps = 8, kBigWarps = 4;
  const int64_t mid_blocks = std::min<int64_t>((strands + kMidWarps - 1) / kMidWarps, 2 * cap);
  seed_hash_kernel<KM, kMidCap, kMidWarps, 5, G>
      <<<(unsigned)mid_blocks, kMidWarps * 32, 0, st>>>(a);
  const int64_t big_blocks = std::min<int64_t>((strands + kBigWarps - 1) / kBigWarps, 4 * cap);
  seed_hash_kernel<KM, kBigCap, kBigWarps, 5, G>
      <<<(unsigned)big_blocks, kBigWarps * 32, 0, st>>>(a);
}

template <int KM>
void launch_seed_km(cudaStream_t st, const SeedArgs& a) {
  if (a.gpos)
    launch_seed_kg<KM, true>(st, a);
  else
    launch_seed_kg<KM, false>(st, a);
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

int seed_smem_cap() { return kBigCap; }

void launch_seed_overflow(cudaStream_t st, const SeedArgs& a, int n_overflow,
                          const uint64_t* tab_off, const uint32_t* tab_size) {
  if (n_overflow <= 0) return;
  if (a.gpos)
    seed_overflow_kernel<true><<<n_overflow, kOvThreads, 0, st>>>(a, tab_off, tab_size);
  else
    seed_overflow_kernel<false><<<n_overflow, kOvThreads, 0, st>>>(a, tab_off, tab_size);
}

}  // namespace swift
