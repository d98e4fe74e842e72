// lt13 seed-and-extend seeding: the Phase 1 of the reference CLI's GPU
// default (search2Queries, src/search2.cu:48-259), on the same tuples as the
// SSAHA index.
//
// Index (lookupTable13Create, src/lookupTable13.cu:64-242): the SSAHA
// buckets with composite values refIdx << 25 | pos / k, plus refPosHashMap,
// the hash of every tuple among the first thres occurrences of its hash, by
// composite.  Here the map is dense per tuple id (tbase[r] + pos / k); a
// composite at or past the largest one written (the device copy of the
// reference is one entry short of it, src/lookupTable13.cu:182,374), past
// its sequence's tuples or into a sequence that has none reads 0, the value
// of every entry the reference never writes.
//
// Query strand (lookupTable13MapQry2_gpu, src/lookupTable13.cu:646-868),
// one warp per strand:
//   1. the strand's bytes in shared memory with zeros after them, and the
//      k-mer hash at every offset the kernel reads (NUL hashes as A);
//   2. every (tuple offset, hit) pair of the strand is extended in parallel
//      across the warp's lanes (the extension depends only on the hit's
//      composite and the offset);
//   3. lane 0 replays the reference block's bookkeeping over the results in
//      tuple order: each tuple's results land at [count, count + hits), the
//      array past them reads -1, and the running maximum compacts the
//      entries that reach it to the front (reset past 1000 entries);
//   4. the entries equal to the maximum over [0, count], in the order of the
//      reference's 64-thread strided scan, give up to 3 hits; with more,
//      K&R's generator picks 3 distinct ones.  The reference reads that
//      generator's seed from shared memory it never sets; it starts at 0.
// A strand whose entries outgrow the fast kernel's shared arrays is redone
// by a kernel sized for the reference's full arrays (2304 entries).
#include "internal.h"

namespace swift {
namespace {

constexpr int kPosBits = 25;
constexpr int kPosMask = (1 << kPosBits) - 1;
constexpr int kKeep = 1000;      // the k > 1000 reset
constexpr int kRefThreads = 64;  // the reference block's threads: the final scan's stride
constexpr int kHits = 3;
// strand bytes + zero padding: tuple offsets run to Q - k + 2 <= 200 (reads <=
// 199 bases), hashes read 16 more codes, a multiple of 16 for the packed words
constexpr int kQBuf = 208;
static_assert(kQBuf % 16 == 0 && kQBuf >= kReadMax + 3, "strand buffer too small");
constexpr int kWarps = 4;

__device__ __forceinline__ uint32_t code13(uint8_t c) {
  const uint32_t u = c & 0xDFu;  // hashCodes_gpu: A/a, N/n and others 0
  return u == 'C' ? 1u : u == 'G' ? 2u : u == 'T' ? 3u : 0u;
}

struct Lt13Shared {
  int nrefs;
  int64_t max_comp;
  int64_t tbase[kMaxRefs13];
  int32_t ntup[kMaxRefs13];  // below 2^25 per reference (the index refuses more)
};

__device__ __forceinline__ int32_t map_at(const Seed13Args& a, const Lt13Shared& s, int64_t v) {
  if (v < 0 || v >= s.max_comp) return 0;
  const int r = (int)(v >> kPosBits);
  const int64_t c = v & kPosMask;
  if (r >= s.nrefs || c >= s.ntup[r]) return 0;
  return a.map[s.tbase[r] + c];
}

// K&R's rand (getRandNum13_gpu, src/lookupTable13.cu:907-911)
__device__ __forceinline__ int rand13(uint32_t* seed) {
  *seed = *seed * 1103515245u + 12345u;
  return (int)((*seed / 65536u) % 32768u);
}

template <int CAP, int GCAP>
struct WarpBuf {
  char q[kQBuf];
  uint32_t packed[kQBuf / 16 + 2];  // 2-bit codes of q, 16 per word
  int32_t qh[kQBuf];
  int32_t hoff[kQBuf + 1];   // exclusive prefix of hits per tuple offset
  uint32_t hstart[kQBuf];    // bucket start per tuple offset
  int16_t ht[kQBuf];         // tuple offsets with hits, in order
  int16_t snm[GCAP];         // staged extension results
  int32_t spos[GCAP];
  int16_t nm[CAP];           // numMatches_shr (live part)
  int32_t pos[CAP];          // refPos_shr
};

template <int CAP, int GCAP>
__global__ void __launch_bounds__(kWarps * 32) seed13_kernel(Seed13Args a) {
  extern __shared__ __align__(16) uint8_t smem13[];
  Lt13Shared& sh = *reinterpret_cast<Lt13Shared*>(smem13);
  WarpBuf<CAP, GCAP>* bufs =
      reinterpret_cast<WarpBuf<CAP, GCAP>*>(smem13 + ((sizeof(Lt13Shared) + 15) & ~(size_t)15));
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    sh.nrefs = a.nrefs;
    sh.max_comp = a.max_comp;
  }
  for (int r = threadIdx.x; r < a.nrefs; r += blockDim.x) {
    sh.tbase[r] = a.tbase[r];
    sh.ntup[r] = (int32_t)a.ntup[r];
  }
  __syncthreads();
  WarpBuf<CAP, GCAP>& b = bufs[wib];
  const int64_t n_items = a.list ? a.n_list : 2 * a.n_reads;
  for (int64_t item = (int64_t)blockIdx.x * kWarps + wib; item < n_items;
       item += (int64_t)gridDim.x * kWarps) {
    const int64_t sid = a.list ? a.list[item] : item;
    const int64_t read = sid >> 1;
    const int strand = (int)(sid & 1);
    const DevRead rr = a.rd[read];
    const int Q = rr.len;
    const char* src = a.reads + rr.seq_off;
    // 1. strand bytes (qryGetReverseComplement: A->T, C->G, G->C, else A)
    for (int i = lane; i < kQBuf; i += 32) {
      char c = 0;
      if (i < Q) {
        if (strand == 0) {
          c = src[i];
        } else {
          const char f = src[Q - 1 - i];
          c = f == 'A' ? 'T' : f == 'C' ? 'G' : f == 'G' ? 'C' : 'A';
        }
      }
      b.q[i] = c;
    }
    __syncwarp();
    const int k = a.k;
    const int n_tup = Q - k + 1;
    const int n_inc = n_tup >= -1 ? n_tup + 2 : 0;  // offsets 0 .. Q - k + 2
    const int last = (Q / k) * k;
    const int xh = max(n_inc, last);
    // getHash13_gpu: sum 4^i code(q[x + i]) is the 2k-bit little-endian
    // field at bit 2x of the packed codes
    for (int w = lane; w < kQBuf / 16 + 2; w += 32) {
      uint32_t v = 0;
      if (w < kQBuf / 16)
        for (int i = 0; i < 16; ++i) v |= code13((uint8_t)b.q[16 * w + i]) << (2 * i);
      b.packed[w] = v;
    }
    __syncwarp();
    const uint64_t hmask = (1ull << (2 * k)) - 1;
    for (int x = lane; x < xh; x += 32) {
      const int wi = x >> 4;
      const uint64_t two = (uint64_t)b.packed[wi] | ((uint64_t)b.packed[wi + 1] << 32);
      b.qh[x] = (int32_t)((two >> (2 * (x & 15))) & hmask);
    }
    __syncwarp();
    // hits per tuple offset and their prefix
    int carry = 0, nht = 0;
    for (int x0 = 0; x0 < n_inc; x0 += 32) {
      const int x = x0 + lane;
      int nh = 0;
      if (x < n_inc) {
        // compact bucket directory: occupancy bits and rank per 64 buckets,
        // then the starts of occupied buckets
        const uint32_t h = (uint32_t)b.qh[x];
        const uint4 grp = __ldg(&a.groups[h >> 6]);
        const uint64_t bits = ((uint64_t)grp.y << 32) | grp.x;
        uint32_t s0 = 0;
        if ((bits >> (h & 63)) & 1u) {
          const uint32_t r = grp.z + (uint32_t)__popcll(bits & ((1ull << (h & 63)) - 1));
          s0 = __ldg(&a.cstart[r]);
          nh = (int)(__ldg(&a.cstart[r + 1]) - s0);
        }
        b.hstart[x] = s0;
      }
      int incl = nh;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += t;
      }
      if (x < n_inc) b.hoff[x] = carry + incl - nh;
      carry += __shfl_sync(0xffffffffu, incl, 31);
      // tuple offsets with hits, in order
      const uint32_t hb = __ballot_sync(0xffffffffu, nh > 0);
      if (nh > 0) b.ht[nht + __popc(hb & ((1u << lane) - 1))] = (int16_t)x;
      nht += __popc(hb);
    }
    if (lane == 0) b.hoff[n_inc] = carry;
    __syncwarp();
    // 2-3. extensions in rounds of whole tuples that fit the staging arrays,
    // then the block's bookkeeping by lane 0.  Only tuple offsets with hits
    // change the state: an offset without hits clears the entries past
    // count, which the next offset with hits overwrites or clears too, so
    // only a run of them after the last offset with hits is felt (live =
    // count at the end).
    int count = 0, maxm = 0, live = 0;
    bool over = false;
    int u0 = 0;
    while (u0 < nht && !over) {
      const int base = b.hoff[b.ht[u0]];
      int u1 = u0 + 1;
      if (b.hoff[b.ht[u0] + 1] - base > GCAP) {
        over = true;
        break;
      }
      while (u1 < nht && b.hoff[b.ht[u1] + 1] - base <= GCAP) ++u1;
      const int g0 = base, g1 = b.hoff[b.ht[u1 - 1] + 1];
      const int t0 = b.ht[u0], t1 = b.ht[u1 - 1] + 1;
      for (int g = g0 + lane; g < g1; g += 32) {
        int lo = t0, hi = t1 - 1;  // the tuple offset holding hit g
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (b.hoff[mid] <= g) lo = mid;
          else hi = mid - 1;
        }
        const int inc = lo;
        const int32_t v0 = a.vals[b.hstart[inc] + (g - b.hoff[inc])];
        int64_t val = v0;
        int matches = 0, mm = 0, mm2 = 0, inc2 = inc;
        int32_t rth = map_at(a, sh, val);
        while (inc2 < last) {
          if (rth == b.qh[inc2]) {
            ++val;
            rth = map_at(a, sh, val);
            inc2 += k;
            ++matches;
            mm = 0;
            mm2 = 0;
          } else if (mm < k - 1) {
            ++inc2;
            ++mm;
          } else if (mm2 == 0) {
            ++val;
            rth = map_at(a, sh, val);
            inc2 -= mm;
            mm = 0;
            ++mm2;
          } else {
            break;
          }
        }
        b.snm[g - g0] = (int16_t)matches;
        b.spos[g - g0] = v0;
      }
      __syncwarp();
      if (lane == 0) {
        for (int u = u0; u < u1 && !over; ++u) {
          const int t = b.ht[u];
          const int nh = b.hoff[t + 1] - b.hoff[t];
          const int offset = count + nh;
          if (offset > CAP) {
            over = true;
            break;
          }
          const int gs = b.hoff[t] - g0;
          for (int j = 0; j < nh; ++j) {
            b.nm[count + j] = b.snm[gs + j];
            b.pos[count + j] = b.spos[gs + j];
          }
          for (int p = offset; p < live; ++p) b.nm[p] = -1;
          live = offset;
          int kk = count;
          for (int j = count; j < offset; ++j) {
            if (maxm <= b.nm[j]) {
              if (maxm < b.nm[j]) {
                maxm = b.nm[j];
                kk = 0;
              }
              b.nm[j] = -1;
              b.nm[kk] = (int16_t)maxm;
              b.pos[kk] = b.pos[j];
              ++kk;
            }
          }
          if (kk > kKeep) kk = 0;
          count = kk;
        }
      }
      over = __shfl_sync(0xffffffffu, over ? 1 : 0, 0) != 0;
      __syncwarp();
      u0 = u1;
    }
    if (lane == 0 && nht > 0 && b.ht[nht - 1] < n_inc - 1) {
      for (int p = count; p < live; ++p) b.nm[p] = -1;
      live = min(live, count);
    }
    // 4. final selection (lane 0)
    if (lane == 0) {
      if (over) {
        a.nbest[sid] = 0;
        const int slot = atomicAdd(a.n_overflow, 1);
        a.overflow_list[slot] = (int32_t)sid;
      } else {
        int fm = 0;
        for (int i = 0; i <= count && i < live; ++i) fm = max(fm, (int)b.nm[i]);
        int total3 = 0;
        for (int p = 0; p < live; ++p) total3 += b.nm[p] == fm;
        // refPos3: the entries equal to fm in the strided order of the
        // reference's 64 threads; the picks index into it
        int pick[kHits] = {0, 1, 2};
        const int n_pick = total3 > kHits ? kHits : total3;
        if (total3 > kHits) {
          uint32_t seed = 0;
          int got = 0;
          while (got < kHits) {
            const int v = rand13(&seed) % total3;
            bool dup = false;
            for (int i = 0; i < got; ++i) dup |= pick[i] == v;
            if (!dup) pick[got++] = v;
          }
        }
        int nb = 0;
        for (int i = 0; i < n_pick; ++i) {
          int32_t v = -1;
          int c = 0;
          for (int t = 0; t < min(kRefThreads, live) && v < 0; ++t)
            for (int p = t; p < live; p += kRefThreads)
              if (b.nm[p] == fm) {
                if (c == pick[i]) {
                  v = b.pos[p];
                  break;
                }
                ++c;
              }
          if ((int8_t)(v >> kPosBits) == -1) continue;  // printHeuristicMatches skips -1
          a.best[sid * kHits + nb] = make_int3(v >> kPosBits, 0, (v & kPosMask) * k);
          ++nb;
        }
        a.nbest[sid] = nb;
      }
    }
    __syncwarp();
  }
}

template <int CAP, int GCAP>
size_t seed13_smem() {
  return ((sizeof(Lt13Shared) + 15) & ~(size_t)15) + kWarps * sizeof(WarpBuf<CAP, GCAP>);
}

template <int CAP, int GCAP>
void launch_seed13_cfg(cudaStream_t st, const Seed13Args& a, int64_t n_items) {
  const size_t smem = seed13_smem<CAP, GCAP>();
  cudaFuncSetAttribute(seed13_kernel<CAP, GCAP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  const int64_t blocks = std::min<int64_t>((n_items + kWarps - 1) / kWarps, 152 * 64);
  seed13_kernel<CAP, GCAP><<<(unsigned)std::max<int64_t>(blocks, 1), kWarps * 32, smem, st>>>(a);
}

// hash of every tuple, by tuple id
__global__ void tuple_hash13_kernel(const uint32_t* __restrict__ packed,
                                    const DevRecord* __restrict__ recs,
                                    const uint64_t* __restrict__ tbase, int n_recs,
                                    uint64_t n_tuples, int k, uint32_t* __restrict__ out) {
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (; t < n_tuples; t += stride) {
    int lo = 0, hi = n_recs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tbase[mid] <= t) lo = mid;
      else hi = mid - 1;
    }
    const uint64_t gp = recs[lo].cat_start + (t - tbase[lo]) * (uint64_t)k;
    const uint64_t wi = gp >> 4;
    const uint32_t shf = (uint32_t)(gp & 15) * 2;
    const uint64_t two = (uint64_t)packed[wi] | ((uint64_t)packed[wi + 1] << 32);
    out[t] = (uint32_t)((two >> shf) & ((1ull << (2 * k)) - 1));
  }
}

// postings (ref_pos, ref_idx) -> composites
__global__ void composite_kernel(const uint2* __restrict__ post, int64_t n, int k,
                                 int32_t* __restrict__ vals) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) {
    const uint2 p = post[i];
    vals[i] = (int32_t)((p.y << kPosBits) + p.x / (uint32_t)k);
  }
}

}  // namespace

void launch_tuple_hash13(cudaStream_t st, const uint32_t* packed, const DevRecord* recs,
                         const uint64_t* tbase, int n_recs, uint64_t n_tuples, int k,
                         uint32_t* out) {
  if (n_tuples == 0) return;
  const uint64_t blocks = std::min<uint64_t>((n_tuples + 255) / 256, 152 * 16);
  tuple_hash13_kernel<<<(unsigned)blocks, 256, 0, st>>>(packed, recs, tbase, n_recs, n_tuples, k,
                                                        out);
}

void launch_composites13(cudaStream_t st, const uint2* post, int64_t n, int k, int32_t* vals) {
  if (n <= 0) return;
  const int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 16);
  composite_kernel<<<(unsigned)blocks, 256, 0, st>>>(post, n, k, vals);
}

void launch_seed13(cudaStream_t st, const Seed13Args& a, bool full) {
  const int64_t n_items = a.list ? a.n_list : 2 * a.n_reads;
  if (n_items <= 0) return;
  if (full)
    launch_seed13_cfg<kFullArr13, kFullStage13>(st, a, n_items);
  else
    launch_seed13_cfg<512, 256>(st, a, n_items);
}

}  // namespace swift
