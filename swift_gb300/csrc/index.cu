// SSAHA index build on the device (restates lookupTable5Create,
// src/lookupTable5.cu:101-252):
//   1. sequence lines of the FASTA bytes are compacted into one base string
//      per record (warp per line, coalesced);
//   2. the bases become 2-bit hash codes, 16 per 32-bit word, read with
//      128-bit loads;
//   3. every non-overlapping k-mer ("tuple", positions 0, k, 2k, ... of each
//      record) is hashed and counted;
//   4. counts above the ignore threshold are dropped and an exclusive scan
//      gives the bucket starts;
//   5. tuples scatter into their buckets; each bucket is then ordered the
//      way the reference leaves it (reverse order of occurrence).
// Per tuple the build reads 3 bytes of packed codes and writes 8 bytes of
// posting; the count and start arrays are 2 x 4^k x 4 bytes.
#include "internal.h"

namespace swift {

__device__ __forceinline__ uint32_t base_code(uint8_t c) {
  // getHash codes (src/preprocess.cu:30-48): C/c 1, G/g 2, T/t 3, else 0
  uint32_t u = c & 0xDFu;  // fold case for letters
  return u == 'C' ? 1u : u == 'G' ? 2u : u == 'T' ? 3u : 0u;
}

__global__ void compact_lines_kernel(const char* __restrict__ file,
                                     const uint64_t* __restrict__ src,
                                     const uint64_t* __restrict__ dst,
                                     const uint32_t* __restrict__ len, int64_t n_lines,
                                     uint8_t* __restrict__ cat) {
  const int lane = threadIdx.x & 31;
  int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (; w < n_lines; w += nw) {
    const char* s = file + src[w];
    uint8_t* d = cat + dst[w];
    const uint32_t L = len[w];
    for (uint32_t i = lane; i < L; i += 32) d[i] = (uint8_t)s[i];
  }
}

__global__ void pack2bit_kernel(const uint8_t* __restrict__ cat, int64_t n_words,
                                uint32_t* __restrict__ packed) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; t < n_words; t += stride) {
    const uint4 v = reinterpret_cast<const uint4*>(cat)[t];
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
    uint32_t out = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int b = 0; b < 4; ++b) out |= base_code((uint8_t)(w[q] >> (8 * b))) << (2 * (4 * q + b));
    packed[t] = out;
  }
}

// Hash of the k bases starting at global base position gp: the little-endian
// 2-bit field [2gp, 2gp+2k) of the packed codes is exactly sum 4^i code_i.
__device__ __forceinline__ uint32_t tuple_hash(const uint32_t* __restrict__ packed, uint64_t gp,
                                               int k) {
  const uint64_t wi = gp >> 4;
  const uint32_t sh = (uint32_t)(gp & 15) * 2;
  const uint64_t two = (uint64_t)packed[wi] | ((uint64_t)packed[wi + 1] << 32);
  return (uint32_t)((two >> sh) & ((1ull << (2 * k)) - 1));
}

// Tuple t of the whole reference -> (record, position in record).
__device__ __forceinline__ int tuple_record(const uint64_t* __restrict__ tbase, int n_recs,
                                            uint64_t t) {
  int lo = 0, hi = n_recs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (tbase[mid] <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void count_tuples_kernel(const uint32_t* __restrict__ packed,
                                    const DevRecord* __restrict__ recs,
                                    const uint64_t* __restrict__ tbase, int n_recs,
                                    uint64_t n_tuples, int k, uint32_t* __restrict__ count) {
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (; t < n_tuples; t += stride) {
    int r = tuple_record(tbase, n_recs, t);
    uint64_t p = (t - tbase[r]) * (uint64_t)k;
    uint32_t h = tuple_hash(packed, recs[r].cat_start + p, k);
    atomicAdd(&count[h], 1u);
  }
}

__global__ void threshold_kernel(const uint32_t* __restrict__ count, int64_t nb, uint32_t thres,
                                 uint32_t* __restrict__ eff) {
  int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; h < nb; h += stride) {
    uint32_t c = count[h];
    eff[h] = c <= thres ? c : 0u;
  }
}

__global__ void scatter_tuples_kernel(const uint32_t* __restrict__ packed,
                                      const DevRecord* __restrict__ recs,
                                      const uint64_t* __restrict__ tbase, int n_recs,
                                      uint64_t n_tuples, int k, uint32_t thres,
                                      const uint32_t* __restrict__ count,
                                      const uint32_t* __restrict__ offsets,
                                      uint32_t* __restrict__ cursor, uint2* __restrict__ post) {
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (; t < n_tuples; t += stride) {
    int r = tuple_record(tbase, n_recs, t);
    uint64_t p = (t - tbase[r]) * (uint64_t)k;
    uint32_t h = tuple_hash(packed, recs[r].cat_start + p, k);
    if (count[h] <= thres) {
      uint32_t slot = offsets[h] + atomicAdd(&cursor[h], 1u);
      post[slot] = make_uint2((uint32_t)p, (uint32_t)r);
    }
  }
}

// Orders each bucket by descending (record, position): the reference fills
// buckets back to front in occurrence order (src/lookupTable5.cu:224-227).
__global__ void order_buckets_kernel(const uint32_t* __restrict__ offsets, int64_t nb,
                                     uint2* __restrict__ post) {
  int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; h < nb; h += stride) {
    uint32_t b = offsets[h], e = offsets[h + 1];
    if (e - b < 2) continue;
    for (uint32_t i = b + 1; i < e; ++i) {
      uint2 v = post[i];
      uint64_t kv = ((uint64_t)v.y << 32) | v.x;
      uint32_t j = i;
      while (j > b) {
        uint2 u = post[j - 1];
        uint64_t ku = ((uint64_t)u.y << 32) | u.x;
        if (ku >= kv) break;
        post[j] = u;
        --j;
      }
      post[j] = v;
    }
  }
}

// Compact bucket directory for seeding.  The bucket-start table has 4^k
// entries (64 MiB at k = 12) and seeding looks up one entry per query
// position at random; most buckets are empty.  The directory keeps, per
// group of 64 buckets, the occupancy bits and the number of occupied buckets
// before the group (16 bytes), and the starts of occupied buckets only:
// a few tens of MB for a 50 Mbp reference, which stay in L2.
__global__ void bucket_bits_kernel(const uint32_t* __restrict__ offsets, int64_t nb,
                                   uint32_t* __restrict__ bits32) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = warp; w * 32 < nb; w += nwarps) {
    const int64_t h = w * 32 + lane;
    const bool occ = h < nb && offsets[h + 1] > offsets[h];
    const uint32_t b = __ballot_sync(0xffffffffu, occ);
    if (lane == 0) bits32[w] = b;
  }
}

__global__ void group_count_kernel(const uint32_t* __restrict__ bits32, int64_t nw32, int64_t ng,
                                   uint32_t* __restrict__ gcnt) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; g < ng; g += stride) {
    const uint32_t lo = bits32[2 * g], hi = 2 * g + 1 < nw32 ? bits32[2 * g + 1] : 0u;
    gcnt[g] = (uint32_t)(__popc(lo) + __popc(hi));
  }
}

__global__ void group_pack_kernel(const uint32_t* __restrict__ bits32, int64_t nw32,
                                  const uint32_t* __restrict__ grank, int64_t ng,
                                  uint4* __restrict__ groups) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; g < ng; g += stride) {
    const uint32_t lo = bits32[2 * g], hi = 2 * g + 1 < nw32 ? bits32[2 * g + 1] : 0u;
    groups[g] = make_uint4(lo, hi, grank[g], 0u);
  }
}

__global__ void compact_starts_kernel(const uint32_t* __restrict__ offsets, int64_t nb,
                                      const uint4* __restrict__ groups,
                                      const uint32_t* __restrict__ n_occ,
                                      uint32_t* __restrict__ cstart) {
  int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if (h == 0) cstart[*n_occ] = offsets[nb];
  for (; h < nb; h += stride) {
    const uint32_t b = offsets[h];
    if (offsets[h + 1] > b) {
      const uint4 g = groups[h >> 6];
      const uint64_t bits = ((uint64_t)g.y << 32) | g.x;
      const uint32_t r = g.z + (uint32_t)__popcll(bits & ((1ull << (h & 63)) - 1));
      cstart[r] = b;
    }
  }
}

static inline unsigned grid_for(int64_t n, int threads, unsigned cap = 152u * 32u) {
  int64_t g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > (int64_t)cap) g = cap;
  return (unsigned)g;
}

void launch_compact_lines(cudaStream_t st, const char* file, const uint64_t* src,
                          const uint64_t* dst, const uint32_t* len, int64_t n_lines,
                          uint8_t* cat) {
  if (n_lines <= 0) return;
  compact_lines_kernel<<<grid_for(n_lines * 32, 256), 256, 0, st>>>(file, src, dst, len, n_lines,
                                                                    cat);
}

// Bit b of odd[t]: byte 32 t + b of cat is not one of ACGTacgt (the zero
// padding after the last base counts as such).
__global__ void odd_bits_kernel(const uint8_t* __restrict__ cat, int64_t n_out,
                                uint32_t* __restrict__ odd) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; t < n_out; t += stride) {
    uint32_t bits = 0;
    for (int b = 0; b < 32; ++b) {
      const uint32_t u = cat[32 * t + b] & 0xDFu;
      if (!(u == 'A' || u == 'C' || u == 'G' || u == 'T')) bits |= 1u << b;
    }
    odd[t] = bits;
  }
}

void launch_odd_bits(cudaStream_t st, const uint8_t* cat, int64_t n_words, uint32_t* odd) {
  // the last word reads bytes up to 32 * odd_bits_words(n_words) - 1 <
  // 16 * n_words + 64
  const int64_t n_out = odd_bits_words(n_words);
  odd_bits_kernel<<<grid_for(n_out, 256), 256, 0, st>>>(cat, n_out, odd);
}

void launch_pack2bit(cudaStream_t st, const uint8_t* cat, int64_t n_words, uint32_t* packed) {
  if (n_words <= 0) return;
  pack2bit_kernel<<<grid_for(n_words, 256), 256, 0, st>>>(cat, n_words, packed);
}

void launch_count_tuples(cudaStream_t st, const uint32_t* packed, const DevRecord* recs,
                         const uint64_t* tbase, int n_recs, uint64_t n_tuples, int k,
                         uint32_t* count) {
  if (n_tuples == 0) return;
  count_tuples_kernel<<<grid_for((int64_t)n_tuples, 256), 256, 0, st>>>(packed, recs, tbase,
                                                                        n_recs, n_tuples, k, count);
}

void launch_threshold(cudaStream_t st, const uint32_t* count, int64_t nb, uint32_t thres,
                      uint32_t* eff) {
  threshold_kernel<<<grid_for(nb, 256), 256, 0, st>>>(count, nb, thres, eff);
}

void launch_scatter_tuples(cudaStream_t st, const uint32_t* packed, const DevRecord* recs,
                           const uint64_t* tbase, int n_recs, uint64_t n_tuples, int k,
                           uint32_t thres, const uint32_t* count, const uint32_t* offsets,
                           uint32_t* cursor, uint2* post) {
  if (n_tuples == 0) return;
  scatter_tuples_kernel<<<grid_for((int64_t)n_tuples, 256), 256, 0, st>>>(
      packed, recs, tbase, n_recs, n_tuples, k, thres, count, offsets, cursor, post);
}

int build_bucket_directory(cudaStream_t st, const uint32_t* offsets, int64_t nb, uint32_t* bits32,
                           uint32_t* gcnt, uint32_t* grank, void* scan_tmp, uint32_t* n_occ,
                           uint4* groups, uint32_t* cstart) {
  const int64_t nw32 = (nb + 31) / 32, ng = (nb + 63) / 64;
  bucket_bits_kernel<<<grid_for(nw32 * 32, 256), 256, 0, st>>>(offsets, nb, bits32);
  group_count_kernel<<<grid_for(ng, 256), 256, 0, st>>>(bits32, nw32, ng, gcnt);
  int k = exclusive_scan_u32(st, gcnt, grank, ng, scan_tmp, n_occ);
  group_pack_kernel<<<grid_for(ng, 256), 256, 0, st>>>(bits32, nw32, grank, ng, groups);
  compact_starts_kernel<<<grid_for(nb, 256), 256, 0, st>>>(offsets, nb, groups, n_occ, cstart);
  return k + 4;
}

void launch_order_buckets(cudaStream_t st, const uint32_t* offsets, int64_t nb, uint2* post) {
  order_buckets_kernel<<<grid_for(nb, 256), 256, 0, st>>>(offsets, nb, post);
}

namespace {
__global__ void global_pos_kernel(const uint2* __restrict__ post, int64_t n,
                                  const uint32_t* __restrict__ gbase, uint32_t* __restrict__ gpos) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    gpos[i] = gbase[post[i].y] + post[i].x;
}
}  // namespace

void launch_global_positions(cudaStream_t st, const uint2* post, int64_t n, const uint32_t* gbase,
                             uint32_t* gpos) {
  if (n > 0) global_pos_kernel<<<grid_for(n, 256), 256, 0, st>>>(post, n, gbase, gpos);
}

}  // namespace swift
