// Phase 2 on explicit pairs of varying lengths: the pairs are copied into
// fixed-stride buffers and sorted by shape, so every launch of the existing
// Smith-Waterman passes covers pairs of one (Q, R).
//
// Shape key: bits 0-10 window length R (<= 1024); for pairs of the packed
// passes bits 11-19 hold Q's row class / 8 (var_rows: the rows of the
// trace shape that takes Q exactly), for the others (a byte outside
// ACGTacgt, or a shape or scoring the packed passes do not take) bit 20 is
// set and bits 11-19 hold Q itself.  A counting sort over the 2^21 keys
// orders the pairs by key: packed pairs of one row class form one set of
// launches (sorted by window length, so a warp's pairs sweep similar
// widths), generic pairs one launch per exact shape.
#include "internal.h"

namespace swift {
namespace {

constexpr int kVarWarps = 8;

__device__ __forceinline__ bool acgt(uint8_t c) {
  const uint32_t u = c & 0xDFu;
  return u == 'A' || u == 'C' || u == 'G' || u == 'T';
}

// One warp per pair: query and window bytes to their fixed-stride slots,
// the pair's shape key, and its histogram count.  Windows are padded with
// NUL and queries with 0x01, so padded rows and columns never match each
// other or a real base ('N' included): with negative mismatch and gap
// penalties every padded cell then stays below the maximum of the real
// ones, and padding changes no result.  Real bytes 0x00 and 0x01 would
// break that, so they are reported (bad).
__global__ void __launch_bounds__(kVarWarps * 32) pack_var_kernel(VarPairArgs a) {
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * kVarWarps + wib;
  if (i >= a.n) return;
  const int Q = a.q_len[i], R = a.r_len[i];
  if (var_pair_long(Q, R)) {  // read in place by the long kernel
    bool other = false;  // a byte outside ACGTN (either case)
    const char* qs = a.qry + a.q_off[i];
    const char* ws = a.ref + a.r_off[i];
    for (int t = lane; t < Q; t += 32) other |= !acgt((uint8_t)qs[t]) && ((uint8_t)qs[t] & 0xDFu) != 'N';
    for (int t = lane; t < R; t += 32) other |= !acgt((uint8_t)ws[t]) && ((uint8_t)ws[t] & 0xDFu) != 'N';
    other = __any_sync(0xffffffffu, other);
    if (lane == 0) {
      const int c = Q <= 1024 ? 0 : Q <= 2048 ? 1 : Q <= 3072 ? 2 : 3;
      const uint32_t key = kVarLongKey + 2 * (uint32_t)c + ((other || !a.long_prof) ? 0u : 1u);
      a.key[i] = key;
      atomicAdd(&a.hist[key], 1u);
    }
    return;
  }
  const char* qs = a.qry + a.q_off[i];
  const char* ws = a.ref + a.r_off[i];
  char* qd = a.qbuf + i * a.q_stride;
  char* wd = a.wbuf + i * a.w_stride;
  bool odd = false, bad = false;
  for (int t = lane; t < a.q_stride; t += 32) {
    const char c = t < Q ? qs[t] : '\x01';
    qd[t] = c;
    if (t < Q && !acgt((uint8_t)c)) odd = true;
    if (t < Q && (uint8_t)c < 2) bad = true;
  }
  for (int t = lane; t < a.w_stride; t += 32) {
    const char c = t < R ? ws[t] : '\0';
    wd[t] = c;
    if (t < R && !acgt((uint8_t)c)) odd = true;
    if (t < R && (uint8_t)c < 2) bad = true;
  }
  odd = __any_sync(0xffffffffu, odd);
  bad = __any_sync(0xffffffffu, bad);
  if (lane == 0 && bad) atomicOr(a.bad, 1u);
  if (lane == 0) {
    const int cls = packed_class(Q);
    const bool gen = odd || R > a.fast_max_r || Q < 1 || R < 1 || cls < 0 ||
                     !((a.class_ok >> cls) & 1u);
    const uint32_t key = gen ? (1u << 20) | ((uint32_t)Q << 11) | (uint32_t)R
                             : ((uint32_t)(var_rows(Q) >> 3) << 11) | (uint32_t)R;
    a.key[i] = key;
    atomicAdd(&a.hist[key], 1u);
  }
}

// Occupied keys -> segment table (key, first position, size), in key order.
__global__ void var_segments_kernel(const uint32_t* __restrict__ hist,
                                    const uint32_t* __restrict__ start,
                                    const uint32_t* __restrict__ seg_pos, uint32_t n_keys,
                                    int32_t* seg_key, int32_t* seg_start, int32_t* seg_count) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_keys || hist[k] == 0) return;
  const uint32_t s = seg_pos[k];
  seg_key[s] = (int32_t)k;
  seg_start[s] = (int32_t)start[k];
  seg_count[s] = (int32_t)hist[k];
}

__global__ void occupied_kernel(const uint32_t* __restrict__ hist, uint32_t n_keys,
                                uint32_t* __restrict__ occ) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n_keys) occ[k] = hist[k] ? 1u : 0u;
}

__global__ void var_scatter_kernel(const uint32_t* __restrict__ key, int64_t n,
                                   const uint32_t* __restrict__ start, uint32_t* fill,
                                   int32_t* __restrict__ sorted) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = key[i];
  sorted[start[k] + atomicAdd(&fill[k], 1u)] = (int32_t)i;
}

// out: max q_len, max r_len, min length, max q_len + r_len, then max q_len
// and r_len over the pairs of the warp-per-pair kernels (not long), count
// of long pairs
__global__ void max_len_kernel(const int32_t* __restrict__ q_len, const int32_t* __restrict__ r_len,
                               int64_t n, int32_t* out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int mq = 0, mr = 0, lo = 0x7fffffff, ms = 0, sq = 0, sr = 0, nl = 0;
  for (; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int Q = q_len[i], R = r_len[i];
    mq = max(mq, Q);
    mr = max(mr, R);
    lo = min(lo, min(Q, R));
    ms = max(ms, Q + R);
    if (var_pair_long(Q, R)) {
      ++nl;
    } else {
      sq = max(sq, Q);
      sr = max(sr, R);
    }
  }
  atomicMax(&out[0], mq);
  atomicMax(&out[1], mr);
  atomicMin(&out[2], lo);
  atomicMax(&out[3], ms);
  atomicMax(&out[4], sq);
  atomicMax(&out[5], sr);
  atomicAdd(&out[6], nl);
}

}  // namespace

void launch_var_max_len(cudaStream_t st, const int32_t* q_len, const int32_t* r_len, int64_t n,
                        int32_t* out) {
  if (n <= 0) return;
  const int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 8);
  max_len_kernel<<<(unsigned)blocks, 256, 0, st>>>(q_len, r_len, n, out);
}

void launch_pack_var(cudaStream_t st, const VarPairArgs& a) {
  if (a.n <= 0) return;
  pack_var_kernel<<<(unsigned)((a.n + kVarWarps - 1) / kVarWarps), kVarWarps * 32, 0, st>>>(a);
}

void launch_var_occupied(cudaStream_t st, const uint32_t* hist, uint32_t* occ) {
  occupied_kernel<<<(kVarKeys + 255) / 256, 256, 0, st>>>(hist, kVarKeys, occ);
}

void launch_var_segments(cudaStream_t st, const uint32_t* hist, const uint32_t* start,
                         const uint32_t* seg_pos, int32_t* seg_key, int32_t* seg_start,
                         int32_t* seg_count) {
  var_segments_kernel<<<(kVarKeys + 255) / 256, 256, 0, st>>>(hist, start, seg_pos, kVarKeys,
                                                              seg_key, seg_start, seg_count);
}

void launch_var_scatter(cudaStream_t st, const uint32_t* key, int64_t n, const uint32_t* start,
                        uint32_t* fill, int32_t* sorted) {
  if (n <= 0) return;
  var_scatter_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(key, n, start, fill, sorted);
}

}  // namespace swift
