// Phase 2 for long pairs (queries up to 4096, windows up to 8192 bases):
// one CTA per pair, the reference kernel's recurrence and tie rules
// (src/smithWaterman.cu:510-645, 911-1026) in int32 cells.
//
// Cells use the packed passes' encoding, Hx = 16 H + onehot(direction) + B,
// so one add-max chain gives H and the reference's direction with its tie
// precedence, and the next cells' gap penalties come from the code bits; at
// these lengths 16 H exceeds 16 bits, so a cell is one 32-bit lane.
//
// Layout.  The 256 threads own consecutive strips of RPL query rows (RPL =
// 4, 8, 12 or 16, the smallest that covers the query).  Within a warp, lane
// t sweeps the window one column behind lane t-1 (shuffles carry the bottom
// row down).  Between warps, lane 31 writes its bottom row's H and UP
// candidate per column to a shared ring that lane 0 of the next warp reads;
// warp w runs two 32-column stages behind warp w-1, one __syncthreads per
// stage, so every value is written before it is read and a ring of 128
// columns is never overrun.  Each thread streams its 2-bit direction codes
// per wavefront step to global scratch (four steps per 16-byte store);
// sw_long_walk_kernel then walks the reference's traceback, one thread per
// pair, carrying the cell score to tell NONE from LEFT.
#include <type_traits>

#include "internal.h"

namespace swift {
namespace {

constexpr int kLW = 8;           // warps per CTA
constexpr int kLT = kLW * 32;    // threads per CTA
constexpr int kStage = 32;       // wavefront steps per stage
constexpr int kRing = 128;       // ring columns between neighbouring warps
constexpr int kWild = 0x100;     // 'N' matches every byte

__device__ __forceinline__ int upcase(uint8_t c) {
  return (unsigned)(c - 'a') < 26u ? c - 'a' + 'A' : c;
}

constexpr int kColMask = (1 << 17) - 1;

__device__ __forceinline__ uint32_t prmt_b(uint32_t a, uint32_t b, uint32_t s) {
  uint32_t d;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(s));
  return d;
}

// base class of an ACGTN pair byte: A 0, C 1, G 2, T 3, N 4 (either case)
__device__ __forceinline__ int class5(uint8_t c) {
  const int u = upcase(c);
  return u == 'C' ? 1 : u == 'G' ? 2 : u == 'T' ? 3 : u == 'N' ? 4 : 0;
}

// PROF: the pair holds only ACGTN bytes (either case) and 16 m Q stays below
// 2^18.  Then the substitution score is one byte permute of a per-row
// profile (window classes A, C, G, T, N), and a row's first maximum is one
// max over keys 2^17 H' + (2^17 - 1 - column), H' = H + B / 16 (16 H + B
// times 2^13, whose low 17 bits are zero): the largest H, and on equal H the
// smallest column.  Other pairs compare bytes.
template <int RPL, bool PROF>
__global__ void __launch_bounds__(kLT, 2) sw_long_kernel(LongArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t item = (int64_t)blockIdx.x;
  if (item >= a.n) return;
  const int32_t p = a.list[item];
  const int Q = a.q_len[p], R = a.r_len[p];
  const char* qg = a.qry + a.q_off[p];
  const char* wg = a.ref + a.r_off[p];
  // shared: up-cased window (int16 per column), rings for the 7 warp boundaries
  int16_t* wu = reinterpret_cast<int16_t*>(smem);                    // [R + 1]
  int32_t* ring = reinterpret_cast<int32_t*>(smem + ((2 * (a.max_r + 1) + 15) & ~15));
  // ring[(b * 2 + 0) * kRing + col % kRing]: UP candidate of boundary b's upper row
  // ring[(b * 2 + 1) * kRing + col % kRing]: its H (code bits cleared)
  for (int c = tid; c < R; c += kLT) {
    if (PROF) {  // byte-permute selector: the class's byte, sign-extended
      const uint32_t k = (uint32_t)class5((uint8_t)wg[c]);
      wu[c + 1] = (int16_t)(k | ((k | 8u) << 4) | ((k | 8u) << 8) | ((k | 8u) << 12));
    } else {
      const int u = upcase((uint8_t)wg[c]);
      wu[c + 1] = (int16_t)(u == 'N' ? kWild : u);
    }
  }
  const int B = a.bias;
  const int B8 = B + 8;
  const int CU = 16 * a.gap_open + 2, CL = 16 * a.gap_open + 1;
  const int KU = 8 * (a.gap_ext - a.gap_open), KL = 16 * (a.gap_ext - a.gap_open);
  const int SM = 16 * a.match + 4, SX = 16 * a.mismatch + 4;
  int qv[RPL], h16p[RPL], xl[RPL], bestv[RPL], bestc[RPL];
  uint32_t pf0[PROF ? RPL : 1], pf1[PROF ? RPL : 1];
  const uint32_t sm8 = (uint32_t)(uint8_t)(int8_t)SM, sx8 = (uint32_t)(uint8_t)(int8_t)SX;
#pragma unroll
  for (int k = 0; k < RPL; ++k) {
    const int i = tid * RPL + k;
    if (PROF) {
      // scores against window classes A C G T (pf0) and N (pf1 byte 0);
      // rows past the query mismatch everything (and stay out of the maximum)
      const int qc = i < Q ? class5((uint8_t)qg[i]) : -1;
      uint32_t v0 = 0;
#pragma unroll
      for (int w = 0; w < 4; ++w)
        v0 |= ((qc == w || qc == 4) ? sm8 : sx8) << (8 * w);
      pf0[k] = v0;
      pf1[k] = qc >= 0 ? sm8 : sx8;
      bestv[k] = B * 8192 + kColMask;  // H = 0 at column 0: no H = 0 cell beats it
    } else {
      if (i < Q) {
        const int u = upcase((uint8_t)qg[i]);
        qv[k] = u == 'N' ? kWild : u;
      } else {
        qv[k] = -1;  // past the query: matches nothing (kept out of the maximum)
      }
      bestv[k] = B;
    }
    h16p[k] = B;
    xl[k] = B;
    bestc[k] = 0;
  }
  const int S4 = (R + 31 + 3) & ~3;  // steps of one thread's direction words
  // the pair's own slot: 256 threads x S4 words from dir_off[item]
  uint32_t* dirs = a.dirs + a.dir_off[item] + (int64_t)tid * S4;
  __syncthreads();
  int send_u = B, send_h = B, diag = B;
  // One wavefront step: this lane's column j against its RPL rows.  FULL:
  // every lane's column lies in 1..R (a warp-uniform fact of the step), so
  // no lane is masked and the rows' state updates in place.
  auto step = [&](const int s, auto full) -> uint32_t {
    constexpr bool kFull = decltype(full)::value;
    int up = __shfl_up_sync(0xffffffffu, send_u, 1);
    const int rh = __shfl_up_sync(0xffffffffu, send_h, 1);
    const int j = s - lane + 1;  // this lane's column
    const bool in = kFull || (j >= 1 && j <= R);
    if (lane == 0) {
      if (warp == 0) {
        up = B;  // row 0
      } else if (in) {
        up = ring[((warp - 1) * 2 + 0) * kRing + (j & (kRing - 1))];
      }
    }
    uint32_t acc = 0;
    if (in) {
      const int rv = wu[j];
      const int cj = kColMask - j;
      int dg = diag;
#pragma unroll
      for (int k = 0; k < RPL; ++k) {
        int sc;
        if (PROF) {
          sc = (int)prmt_b(pf0[k], pf1[k], (uint32_t)(uint16_t)rv);
        } else {
          const bool hit = qv[k] == rv || qv[k] == kWild || (rv == kWild && qv[k] >= 0);
          sc = hit ? SM : SX;
        }
        // DIAG against LEFT off the chain down the rows, then UP and NONE
        const int dl = __viaddmax_s32(dg, sc, xl[k] + CL);
        const int hx = __vimax3_s32(dl, up + CU, B8);
        dg = h16p[k];
        const int h16 = hx & ~15;
        h16p[k] = h16;
        up = (hx & 2) * KU + h16;
        xl[k] = (hx & 1) * KL + h16;
        if (PROF) {
          bestv[k] = max(bestv[k], h16 * 8192 + cj);
        } else if (h16 > bestv[k]) {
          bestv[k] = h16;
          bestc[k] = j;
        }
        // 2 DIAG, 1 UP, 0 LEFT / NONE: code bits 2..1 to bits 2k+1..2k
        if (k == 0) {
          acc |= ((uint32_t)hx >> 1) & 3u;
        } else {
          acc |= ((uint32_t)hx << (2 * k - 1)) & (3u << (2 * k));
        }
      }
      send_u = up;
      send_h = h16p[RPL - 1];
      if (lane == 31 && warp + 1 < kLW) {
        ring[(warp * 2 + 0) * kRing + (j & (kRing - 1))] = up;
        ring[(warp * 2 + 1) * kRing + (j & (kRing - 1))] = send_h;
      }
    }
    // the diagonal of the next step: lane above's bottom H at this column
    // (lane 0: from the ring; column 0 is H = 0)
    if (lane == 0) {
      diag = (warp == 0 || !in) ? B : ring[((warp - 1) * 2 + 1) * kRing + (j & (kRing - 1))];
    } else {
      diag = rh;
    }
    return acc;
  };
  const int steps = R + 31;                          // a warp's wavefront
  // warps whose rows all lie past the query compute nothing (their lanes'
  // rows are out of the maximum, and the walk never reads them); the stage
  // count follows the last warp that computes
  const int act = min(kLW, (Q + 32 * RPL - 1) / (32 * RPL));
  const int n_stages = 2 * (act - 1) + (steps + kStage - 1) / kStage;
  for (int stage = 0; stage < n_stages; ++stage) {
    const int s_lo = (stage - 2 * warp) * kStage;
    if (warp < act && s_lo >= 0 && s_lo < steps) {
#pragma unroll 1
      for (int s0 = s_lo; s0 < s_lo + kStage; s0 += 4) {
        uint4 v;
        if (s0 >= 31 && s0 + 3 <= R - 1) {  // lane 31 past column 0, lane 0 short of R + 1
          v.x = step(s0, std::true_type());
          v.y = step(s0 + 1, std::true_type());
          v.z = step(s0 + 2, std::true_type());
          v.w = step(s0 + 3, std::true_type());
        } else {
          v.x = step(s0, std::false_type());
          v.y = step(s0 + 1, std::false_type());
          v.z = step(s0 + 2, std::false_type());
          v.w = step(s0 + 3, std::false_type());
        }
        if (s0 < S4) __stcg(reinterpret_cast<uint4*>(dirs + s0), v);
      }
    }
    __syncthreads();
  }
  // first maximum in row-major order: per thread, then over the CTA
  int bv = 0, br = 0x7fffffff, bc = 0;
#pragma unroll
  for (int k = 0; k < RPL; ++k) {
    const int i = tid * RPL + k;
    const int v = PROF ? (bestv[k] >> 17) << 4 : bestv[k];
    if (i < Q && v > bv) {
      bv = v;
      br = i + 1;
      bc = PROF ? kColMask - (bestv[k] & kColMask) : bestc[k];
    }
  }
  __shared__ int red_v[kLW], red_r[kLW], red_c[kLW];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    const int ov = __shfl_xor_sync(0xffffffffu, bv, d);
    const int orr = __shfl_xor_sync(0xffffffffu, br, d);
    const int oc = __shfl_xor_sync(0xffffffffu, bc, d);
    if (ov > bv || (ov == bv && orr < br)) {
      bv = ov;
      br = orr;
      bc = oc;
    }
  }
  if (lane == 0) {
    red_v[warp] = bv;
    red_r[warp] = br;
    red_c[warp] = bc;
  }
  __syncthreads();
  if (tid == 0) {
    for (int w = 1; w < kLW; ++w) {
      if (red_v[w] > bv || (red_v[w] == bv && red_r[w] < br)) {
        bv = red_v[w];
        br = red_r[w];
        bc = red_c[w];
      }
    }
    const int score = bv > B ? (bv - B) >> 4 : 0;
    a.best[p] = make_int2(score, score > 0 ? br * (R + 1) + bc : 0);
  }
}

// Traceback walk over the long kernel's direction codes, one thread per
// pair (the same rules as sw_walk_kernel).
template <int RPL>
__global__ void __launch_bounds__(128) sw_long_walk_kernel(LongArgs a) {
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.n) return;
  const int32_t p = a.list[item];
  const int R = a.r_len[p];
  const char* qg = a.qry + a.q_off[p];
  const char* wg = a.ref + a.r_off[p];
  const int S4 = (R + 31 + 3) & ~3;
  const uint32_t* dirs = a.dirs + a.dir_off[item];
  const int W = R + 1;
  // four consecutive steps of one thread per load: a diagonal run of the
  // walk stays in one thread's rows and moves one step back per cell
  int64_t last = -1;
  uint4 words = make_uint4(0, 0, 0, 0);
  auto code_at = [&](int i, int jj) -> uint32_t {
    const int t = (i - 1) / RPL, k = (i - 1) % RPL, ln = t & 31;
    const int64_t at = (int64_t)t * S4 + (jj + ln - 1);
    if ((at & ~(int64_t)3) != last) {
      last = at & ~(int64_t)3;
      words = __ldcg(reinterpret_cast<const uint4*>(dirs + last));
    }
    const int q = (int)(at & 3);
    const uint32_t word = q == 0 ? words.x : q == 1 ? words.y : q == 2 ? words.z : words.w;
    return (word >> (2 * k)) & 3u;
  };
  enum : int { kNone = 0, kDiag = 1, kUp = 2, kLeft = 3 };
  auto dir_of = [](uint32_t code, int h) -> int {
    return code == 2u ? kDiag : code == 1u ? kUp : (h == 0 ? kNone : kLeft);
  };
  const int m = a.match, x = a.mismatch, o = a.gap_open, e = a.gap_ext;
  char* qc = a.qcons ? a.qcons + (int64_t)p * a.cons_stride : nullptr;
  char* rc = a.rcons ? a.rcons + (int64_t)p * a.cons_stride : nullptr;
  const int2 b = a.best[p];
  int cr = b.y / W, cc = b.y % W;
  int h = b.x;
  int d = (cr == 0 || cc == 0) ? kNone : dir_of(code_at(cr, cc), h);
  int nr = cr, nc = cc, nh = h, nd = kNone;
  auto advance = [&]() {
    nr = cr - ((d == kDiag || d == kUp) ? 1 : 0);
    nc = cc - ((d == kDiag || d == kLeft) ? 1 : 0);
    if (d == kNone) {
      nh = h;
      nd = kNone;
      return;
    }
    const uint32_t pc = (nr == 0 || nc == 0) ? 0u : code_at(nr, nc);
    if (d == kDiag) {
      const int qb = upcase((uint8_t)qg[cr - 1]), rb = upcase((uint8_t)wg[cc - 1]);
      nh = h - ((qb == rb || qb == 'N' || rb == 'N') ? m : x);
    } else {
      // the gap costs gap_ext when the predecessor itself moved the same way
      const bool same = nr != 0 && nc != 0 && (d == kUp ? pc == 1u : pc == 0u);
      nh = h - (same ? e : o);
    }
    nd = (nr == 0 || nc == 0) ? kNone : dir_of(pc, nh);
  };
  advance();
  int tick = -1, nref = -1, start = 0;
  auto emit = [&](char r, char q) {
    ++tick;
    if (qc) {
      rc[tick] = r;
      qc[tick] = q;
    }
  };
  while ((cr != nr || cc != nc) && nc != 0 && nr != 0) {
    char rch = '-';
    if (nc != cc) { rch = wg[cc - 1]; ++nref; }
    emit(rch, nr == cr ? '-' : qg[cr - 1]);
    start = cc;
    cr = nr; cc = nc; h = nh; d = nd;
    if (d == kNone) break;
    advance();
  }
  if ((cr != nr || cc != nc) && (nc == 0 || nr == 0)) {
    char rch = '-';
    if (nc != cc) { rch = wg[cc - 1]; ++nref; }
    emit(rch, nr == cr ? '-' : qg[cr - 1]);
    start = cc;
  }
  DevAln out;
  out.score = b.x;
  out.start = start;
  out.end = start + nref;
  out.len = tick + 1;
  a.aln[p] = out;
}

template <int RPL>
int launch_long_rpl(cudaStream_t st, const LongArgs& a, bool prof) {
  const size_t smem = ((2 * (a.max_r + 1) + 15) & ~15) + (size_t)(kLW - 1) * 2 * kRing * 4;
  if (prof)
    sw_long_kernel<RPL, true><<<(unsigned)a.n, kLT, smem, st>>>(a);
  else
    sw_long_kernel<RPL, false><<<(unsigned)a.n, kLT, smem, st>>>(a);
  sw_long_walk_kernel<RPL><<<(unsigned)((a.n + 127) / 128), 128, 0, st>>>(a);
  return 2;
}

}  // namespace

int long_rows_per_lane(int Q) {
  return Q <= 4 * kLT ? 4 : Q <= 8 * kLT ? 8 : Q <= 12 * kLT ? 12 : Q <= 16 * kLT ? 16 : 0;
}

int64_t long_slot_words(int R) { return (int64_t)kLT * ((R + 31 + 3) & ~3); }

int long_bias(int gap_open) { return ((-(16 * gap_open + 1)) + 15) & ~15; }

bool long_prof_ok(int m, int x, int gap_open, int max_q) {
  return 16 * m + 4 <= 127 && 16 * x + 4 >= -128 &&
         16ll * m * max_q + long_bias(gap_open) + 16 < (1ll << 18);
}

int launch_sw_long(cudaStream_t st, const LongArgs& a, int rpl, bool prof) {
  if (a.n <= 0) return 0;
  // shared memory: window (2 B per column) + rings, 23 KB at the longest window
  if (((2 * (a.max_r + 1) + 15) & ~15) + (kLW - 1) * 2 * kRing * 4 > 48 * 1024) return 0;
  if (prof && (a.bias != long_bias(a.gap_open) ||
               !long_prof_ok(a.match, a.mismatch, a.gap_open, 256 * rpl)))
    return 0;
  switch (rpl) {
    case 4: return launch_long_rpl<4>(st, a, prof);
    case 8: return launch_long_rpl<8>(st, a, prof);
    case 12: return launch_long_rpl<12>(st, a, prof);
    case 16: return launch_long_rpl<16>(st, a, prof);
    default: return 0;
  }
}

}  // namespace swift
