// LCS bound of a pair's Smith-Waterman score, bit-parallel.
//
// The matched positions of any local alignment of query q and window w form
// a common subsequence of q and w, so an alignment with M matches has
// M <= LCS(q, w); every other column of it (mismatch, gap) scores below
// zero on the packed path (mismatch, gap_open, gap_ext < 0), so its score is
// at most match * M <= match * LCS(q, w).  That bound is far cheaper than
// any recurrence over the cells and already rules out most pairs that
// cannot be their read's best; the exact score pass then runs only on the
// pairs it leaves, and the suffix values let it and the trace pass stop
// early.
//
// LCS by the bit-vector recurrence of Allison and Dix as simplified by
// Hyyro (one pass over the window, the query as a bit vector V of Q bits,
// all ones at the start):
//     U = V & PM[w_j];   V = (V + U) | (V & ~PM[w_j])
// with PM[c] the query positions holding base class c; LCS = zeros of V.
// One thread per pair; V lives in registers as NW 32-bit words (one carry
// chain per column), PM in shared memory, [class][word][thread], so the
// four loads of a column are conflict-free.
//
// The window is scanned from its last column to its first, against the
// query reversed (LCS(q, w) = LCS(reverse q, reverse w)): after the columns
// c..R the zeros of V are LCS(q, w[c..R]), so the same pass also yields the
// suffix values the trace pass stops early with.  The reversed query sits
// in the top Q bits of the 32 * NW; the bits below it match nothing, stay
// one and never carry.
#include "internal.h"

namespace swift {
namespace {

constexpr int kLcsThreads = 256;
static_assert(kSufSteps == 16, "suffix LCS values are taken per 16-byte block of the window");

// base class of four ACGTacgt bytes at once: A 0, C 1, G 2, T 3 (any map
// works as long as query and window share it)
__device__ __forceinline__ uint32_t class4(uint32_t x) { return ((x >> 1) ^ (x >> 2)) & 0x03030303u; }

// bit b of each byte (b = 0 or 1) of four classes to four adjacent bits
__device__ __forceinline__ uint32_t plane4(uint32_t cls, int b) {
  return (((cls >> b) & 0x01010101u) * 0x10204080u) >> 28;
}

// s = v + u over NW words, carry propagated word to word
template <int NW>
__device__ __forceinline__ void add_words(const uint32_t* v, const uint32_t* u, uint32_t* s);
template <>
__device__ __forceinline__ void add_words<1>(const uint32_t* v, const uint32_t* u, uint32_t* s) {
  s[0] = v[0] + u[0];
}
template <>
__device__ __forceinline__ void add_words<2>(const uint32_t* v, const uint32_t* u, uint32_t* s) {
  asm("add.cc.u32 %0, %2, %4;\n\t"
      "addc.u32 %1, %3, %5;"
      : "=r"(s[0]), "=r"(s[1])
      : "r"(v[0]), "r"(v[1]), "r"(u[0]), "r"(u[1]));
}
template <>
__device__ __forceinline__ void add_words<4>(const uint32_t* v, const uint32_t* u, uint32_t* s) {
  asm("add.cc.u32 %0, %4, %8;\n\t"
      "addc.cc.u32 %1, %5, %9;\n\t"
      "addc.cc.u32 %2, %6, %10;\n\t"
      "addc.u32 %3, %7, %11;"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3])
      : "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(u[0]), "r"(u[1]), "r"(u[2]), "r"(u[3]));
}
template <>
__device__ __forceinline__ void add_words<10>(const uint32_t* v, const uint32_t* u, uint32_t* s) {
  asm("add.cc.u32 %0, %10, %20;\n\t"
      "addc.cc.u32 %1, %11, %21;\n\t"
      "addc.cc.u32 %2, %12, %22;\n\t"
      "addc.cc.u32 %3, %13, %23;\n\t"
      "addc.cc.u32 %4, %14, %24;\n\t"
      "addc.cc.u32 %5, %15, %25;\n\t"
      "addc.cc.u32 %6, %16, %26;\n\t"
      "addc.cc.u32 %7, %17, %27;\n\t"
      "addc.cc.u32 %8, %18, %28;\n\t"
      "addc.u32 %9, %19, %29;"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]),
        "=r"(s[7]), "=r"(s[8]), "=r"(s[9])
      : "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
        "r"(v[8]), "r"(v[9]), "r"(u[0]), "r"(u[1]), "r"(u[2]), "r"(u[3]), "r"(u[4]), "r"(u[5]),
        "r"(u[6]), "r"(u[7]), "r"(u[8]), "r"(u[9]));
}
template <>
__device__ __forceinline__ void add_words<8>(const uint32_t* v, const uint32_t* u, uint32_t* s) {
  asm("add.cc.u32 %0, %8, %16;\n\t"
      "addc.cc.u32 %1, %9, %17;\n\t"
      "addc.cc.u32 %2, %10, %18;\n\t"
      "addc.cc.u32 %3, %11, %19;\n\t"
      "addc.cc.u32 %4, %12, %20;\n\t"
      "addc.cc.u32 %5, %13, %21;\n\t"
      "addc.cc.u32 %6, %14, %22;\n\t"
      "addc.u32 %7, %15, %23;"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]),
        "=r"(s[7])
      : "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
        "r"(u[0]), "r"(u[1]), "r"(u[2]), "r"(u[3]), "r"(u[4]), "r"(u[5]), "r"(u[6]), "r"(u[7]));
}

// NW 32-bit words hold the query: Q <= 32 * NW (a.Q, the launch's longest;
// a.q_len, when given, each pair's own)
template <int NW>
__global__ void __launch_bounds__(kLcsThreads) sw_lcs_kernel(FastArgs a) {
  __shared__ uint32_t pm_all[4 * NW * kLcsThreads];
  const int64_t nlist = *a.count - a.list_offset;
  const int64_t t = (int64_t)blockIdx.x * kLcsThreads + threadIdx.x;
  if (t >= nlist) return;  // no block-wide synchronisation below
  const int32_t p = a.list[a.list_offset + t];
  const int Q = a.q_len ? a.q_len[p] : a.Q, R = a.R;
  // query base classes as two bit planes; positions >= Q match nothing
  const uint32_t* q4 = reinterpret_cast<const uint32_t*>(a.q + (int64_t)p * a.q_stride);
  uint32_t b0[NW], b1[NW], qmask[NW];
#pragma unroll
  for (int wd = 0; wd < NW; ++wd) {
    b0[wd] = b1[wd] = 0;
#pragma unroll
    for (int g = 0; g < 8; ++g) {
      const int i = 32 * wd + 4 * g;
      if (i < Q) {  // the query row holds Q bytes and zero padding up to q_stride
        const uint32_t cls = class4(q4[i >> 2]);
        b0[wd] |= plane4(cls, 0) << (4 * g);
        b1[wd] |= plane4(cls, 1) << (4 * g);
      }
    }
    const int lo = 32 * wd;
    qmask[wd] = Q >= lo + 32 ? ~0u : Q <= lo ? 0u : (1u << (Q - lo)) - 1u;
  }
  // query position i to bit 32 * NW - 1 - i
  uint32_t r0[NW], r1[NW], rmask[NW];
#pragma unroll
  for (int wd = 0; wd < NW; ++wd) {
    r0[wd] = __brev(b0[NW - 1 - wd]);
    r1[wd] = __brev(b1[NW - 1 - wd]);
    rmask[wd] = __brev(qmask[NW - 1 - wd]);
  }
  uint32_t* pm = pm_all + threadIdx.x;
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int wd = 0; wd < NW; ++wd)
      pm[(c * NW + wd) * kLcsThreads] =
          ((c & 1) ? r0[wd] : ~r0[wd]) & ((c & 2) ? r1[wd] : ~r1[wd]) & rmask[wd];
  uint32_t v[NW];
#pragma unroll
  for (int wd = 0; wd < NW; ++wd) v[wd] = ~0u;
  auto column = [&](uint32_t c) {
    const uint32_t* row = pm + c * (NW * kLcsThreads);
    uint32_t m[NW], u[NW], s[NW];
#pragma unroll
    for (int wd = 0; wd < NW; ++wd) {
      m[wd] = row[wd * kLcsThreads];
      u[wd] = v[wd] & m[wd];
    }
    add_words<NW>(v, u, s);
#pragma unroll
    for (int wd = 0; wd < NW; ++wd) v[wd] = s[wd] | (v[wd] & ~m[wd]);
  };
  auto zeros = [&]() {
    int z = 0;
#pragma unroll
    for (int wd = 0; wd < NW; ++wd) z += __popc(~v[wd] & rmask[wd]);
    return z;
  };
  // suffix values: entry m after the columns 16 m + 1 .. R (one-based), that
  // is after the 16-byte block m of the window
  uint16_t* suf = a.lsuf ? a.lsuf + (int64_t)p * kSufBlocks : nullptr;
  // window: 16 bytes per load (rows are 16-byte aligned, w_stride a
  // multiple of 16, R <= w_stride), last block first
  const uint4* w16 = reinterpret_cast<const uint4*>(a.w + (int64_t)p * a.w_stride);
  const int full = R >> 4;
  if (R & 15) {
    const uint4 x = __ldg(w16 + full);
    const uint32_t xs[4] = {x.x, x.y, x.z, x.w};
    for (int j = R - 1; j >= 16 * full; --j) {
      const int o = j & 15;
      column((class4(xs[o >> 2]) >> (8 * (o & 3))) & 3u);
    }
    if (suf) suf[full] = (uint16_t)zeros();
  }
  for (int k = full - 1; k >= 0; --k) {
    const uint4 x = __ldg(w16 + k);
    const uint32_t xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
    for (int h = 3; h >= 0; --h) {
      const uint32_t cls = class4(xs[h]);
#pragma unroll
      for (int b = 3; b >= 0; --b) column((cls >> (8 * b)) & 3u);
    }
    if (suf) suf[k] = (uint16_t)zeros();
  }
  a.ub[p] = a.match * zeros();
}

}  // namespace

int launch_sw_lcs(cudaStream_t st, const FastArgs& a, int64_t max_pairs) {
  if (max_pairs <= 0) return 0;
  if (a.w_stride % 16 != 0 || a.q_stride % 4 != 0 || a.R > a.w_stride) return 0;
  // suffix values: one per 16-column block
  if (a.lsuf && a.R > kSufSteps * kSufBlocks) return 0;
  const unsigned grid = (unsigned)((max_pairs + kLcsThreads - 1) / kLcsThreads);
#define SWIFT_LCS(NW_)                                                        \
  if (a.Q <= 32 * NW_) {                                                      \
    sw_lcs_kernel<NW_><<<grid, kLcsThreads, 0, st>>>(a);                      \
    return 1;                                                                 \
  }
  SWIFT_LCS(1)
  SWIFT_LCS(2)
  SWIFT_LCS(4)
  SWIFT_LCS(8)
  SWIFT_LCS(10)
#undef SWIFT_LCS
  return 0;
}

}  // namespace swift
