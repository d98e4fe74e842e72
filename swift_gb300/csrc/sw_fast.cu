// Phase 2, score pass: the maximum score and its first row-major cell for
// every pair, in packed 16-bit lanes with the DPX add-max instructions.
// Same recurrence and tie rules as sw.cu (the reference kernel's,
// src/smithWaterman.cu:510-645); traceback strings for the pairs that are
// printed come from a second pass (sw.cu) after best-per-read selection.
//
// Encoding.  Each cell is kept as Hx = 16*H + code + B, where code is the
// one-hot direction the reference would store (NONE 8, DIAG 4, UP 2,
// LEFT 1) and B is a bias that keeps every candidate non-negative.  The
// candidates enter a plain max as
//     DIAG: 16*(H[i-1][j-1] + s) + 4 + B
//     UP:   16*(H[i-1][j] + pen) + 2 + B
//     LEFT: 16*(H[i][j-1] + pen) + 1 + B
//     NONE: 8 + B   (H = 0)
// so the max yields H and, on equal H, the reference's precedence
// NONE > DIAG > UP > LEFT of its strict '>' updates.  The gap penalty of a
// neighbour is its gap_ext when the neighbour's own code is UP (for the
// cell below) or LEFT (for the cell to the right), else gap_open; the bits
// 2 and 1 of Hx give that directly:
//     xU = (Hx & ~15) + (Hx & 2) * 8 (e - o)     -> UP candidate + const
//     xL = (Hx & ~15) + (Hx & 1) * 16 (e - o)    -> LEFT candidate + const
// Two pairs share one 32-bit register (low / high 16 bits).
//
// Layout.  A warp holds four pairs: each 16-lane half runs two pairs packed
// in 16-bit halves.  Lane t of a half owns query rows t*RPL+1 .. t*RPL+RPL
// and sweeps the window one column behind lane t-1 (anti-diagonal wavefront
// of row strips); the bottom row's UP candidate and H pass down with two
// shuffles per column.  The substitution score comes from a per-row profile
// register pair selected by one byte-permute per cell.  The first maximum
// of every row is tracked with a packed compare (16-bit integer patterns
// compared as non-negative half floats, whose order they share) and two
// selects.
//
// Preconditions (checked by the caller; other pairs take sw.cu): query and
// window bytes in {A,C,G,T,a,c,g,t}, window length = R (no NUL padding),
// mismatch, gap_open, gap_ext < 0, gap_ext >= gap_open, |16*score+4| < 128,
// 16 * match * Q + B < 31744.
#include <cuda_fp16.h>

#include "internal.h"

namespace swift {
namespace {

constexpr int kFastWarps = 8;
constexpr int kFastMaxR = 512;  // window columns the score pass takes

__device__ __forceinline__ uint32_t base_class(uint32_t c) {
  uint32_t u = c & 0xDFu;
  return u == 'C' ? 1u : u == 'G' ? 2u : u == 'T' ? 3u : 0u;
}

// per-half 0xFFFF where a > b, for non-negative 16-bit integers below 0x7C00
__device__ __forceinline__ uint32_t gt_mask(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("set.gt.u32.f16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}

// byte permute with sign replication (PTX prmt, default mode): selector
// nibble bit 3 replicates the sign of the chosen byte
__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t s) {
  uint32_t d;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(s));
  return d;
}

__device__ __forceinline__ uint32_t sel(uint32_t m, uint32_t a, uint32_t b) {
  // m ? a : b, bitwise
  return (a & m) | (b & ~m);
}

template <int RPL>
__global__ void __launch_bounds__(kFastWarps * 32) sw_score_kernel(FastArgs a) {
  __shared__ uint32_t wsel_all[kFastWarps * 2][kFastMaxR + 1];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int half = lane >> 4, sl = lane & 15;
  const int64_t nlist = *a.count;
  const int64_t base = ((int64_t)blockIdx.x * kFastWarps + wib) * 4 + 2 * half;
  if (((int64_t)blockIdx.x * kFastWarps + wib) * 4 >= nlist) return;  // whole warp
  const int Q = a.Q, R = a.R;
  // the two pairs of this half-warp (a missing second pair repeats the first)
  const bool has0 = base < nlist, has1 = base + 1 < nlist;
  const int32_t p0 = has0 ? a.list[base] : a.list[nlist - 1];
  const int32_t p1 = has1 ? a.list[base + 1] : p0;
  const char* q0 = a.q + (int64_t)p0 * a.q_stride;
  const char* q1 = a.q + (int64_t)p1 * a.q_stride;
  const char* w0 = a.w + (int64_t)p0 * a.w_stride;
  const char* w1 = a.w + (int64_t)p1 * a.w_stride;
  uint32_t* wsel = wsel_all[wib * 2 + half];
  for (int c = sl; c < R; c += 16) {
    uint32_t s0 = base_class((uint8_t)w0[c]), s1 = base_class((uint8_t)w1[c]);
    wsel[c + 1] = s0 | ((s0 | 8u) << 4) | ((4u + s1) << 8) | (((4u + s1) | 8u) << 12);
  }
  __syncwarp();
  const uint32_t B = (uint32_t)a.bias;
  const uint32_t BB = B | (B << 16);
  const uint32_t B8 = BB + 0x00080008u;
  const uint32_t CU = (uint32_t)(uint16_t)(int16_t)(16 * a.gap_open + 2) * 0x00010001u;
  const uint32_t CL = (uint32_t)(uint16_t)(int16_t)(16 * a.gap_open + 1) * 0x00010001u;
  const uint32_t KU = (uint32_t)(8 * (a.gap_ext - a.gap_open));
  const uint32_t KL = (uint32_t)(16 * (a.gap_ext - a.gap_open));
  const uint32_t sm = (uint32_t)(uint8_t)(int8_t)(16 * a.match + 4);
  const uint32_t sx = (uint32_t)(uint8_t)(int8_t)(16 * a.mismatch + 4);
  // per-row state
  uint32_t prof0[RPL], prof1[RPL], h16p[RPL], xl[RPL], bestv[RPL], bestc[RPL];
#pragma unroll
  for (int k = 0; k < RPL; ++k) {
    const int i = sl * RPL + k;
    uint32_t c0 = i < Q ? base_class((uint8_t)q0[i]) : 0u;
    uint32_t c1 = i < Q ? base_class((uint8_t)q1[i]) : 0u;
    uint32_t t0 = 0, t1 = 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      t0 |= ((uint32_t)c == c0 ? sm : sx) << (8 * c);
      t1 |= ((uint32_t)c == c1 ? sm : sx) << (8 * c);
    }
    prof0[k] = t0;
    prof1[k] = t1;
    h16p[k] = BB;          // H[i][0] = 0
    xl[k] = BB;            // LEFT candidate base of column 0 (NONE)
    bestv[k] = BB;
    bestc[k] = 0;
  }
  uint32_t send_u = BB, send_h = BB, diag = BB;
  const int steps = R + 15;
  for (int s = 0; s < steps; ++s) {
    uint32_t up = __shfl_up_sync(0xffffffffu, send_u, 1, 16);
    const uint32_t rh = __shfl_up_sync(0xffffffffu, send_h, 1, 16);
    if (sl == 0) up = BB;  // row 0: H = 0, NONE
    const int j = s - sl + 1;
    if (j >= 1 && j <= R) {
      const uint32_t ws = wsel[j];
      const uint32_t jj = (uint32_t)j * 0x00010001u;
      uint32_t dg = diag;
#pragma unroll
      for (int k = 0; k < RPL; ++k) {
        const uint32_t sc = prmt(prof0[k], prof1[k], ws);
        const uint32_t t1 = __viaddmax_s16x2(xl[k], CL, B8);
        const uint32_t t2 = __viaddmax_s16x2(up, CU, t1);
        const uint32_t hx = __viaddmax_s16x2(dg, sc, t2);
        dg = h16p[k];
        const uint32_t h16 = hx & 0xFFF0FFF0u;
        h16p[k] = h16;
        up = (hx & 0x00020002u) * KU + h16;
        xl[k] = (hx & 0x00010001u) * KL + h16;
        const uint32_t m = gt_mask(h16, bestv[k]);
        bestv[k] = sel(m, h16, bestv[k]);
        bestc[k] = sel(m, jj, bestc[k]);
      }
      send_u = up;
      send_h = h16p[RPL - 1];
    }
    diag = sl == 0 ? BB : rh;
  }
  // first maximum in row-major order, per packed pair
#pragma unroll
  for (int hp = 0; hp < 2; ++hp) {
    const int sh = 16 * hp;
    uint32_t bv = 0, bc = 0, br = 0x7fffffffu;
    const int nrows = Q - sl * RPL;
#pragma unroll
    for (int k = 0; k < RPL; ++k) {
      const uint32_t v = (bestv[k] >> sh) & 0xFFFFu;
      if (k < nrows && v > bv) {
        bv = v;
        bc = (bestc[k] >> sh) & 0xFFFFu;
        br = (uint32_t)(sl * RPL + k + 1);
      }
    }
#pragma unroll
    for (int d = 8; d > 0; d >>= 1) {
      uint32_t ov = __shfl_xor_sync(0xffffffffu, bv, d, 16);
      uint32_t oc = __shfl_xor_sync(0xffffffffu, bc, d, 16);
      uint32_t orr = __shfl_xor_sync(0xffffffffu, br, d, 16);
      if (ov > bv || (ov == bv && orr < br)) {
        bv = ov;
        bc = oc;
        br = orr;
      }
    }
    const bool has = hp == 0 ? has0 : has1;
    if (sl == 0 && has) {
      const int32_t p = hp == 0 ? p0 : p1;
      const int score = bv > B ? (int)((bv - B) >> 4) : 0;
      a.aln[p].score = score;
      a.cell[p] = score > 0 ? (int32_t)(br * (uint32_t)(R + 1) + bc) : 0;
    }
  }
}

}  // namespace

int fast_rows_per_lane(int Q) {
  if (Q <= 32) return 2;
  if (Q <= 64) return 4;
  if (Q <= 112) return 7;
  if (Q <= 128) return 8;
  if (Q <= 192) return 12;
  if (Q <= 256) return 16;
  return 0;
}

bool fast_params_ok(int Q, int R, int m, int x, int o, int e, int* bias) {
  if (R < 1 || R > kFastMaxR || fast_rows_per_lane(Q) == 0) return false;
  if (!(x < 0 && o < 0 && e < 0 && e >= o && m > 0)) return false;
  if (16 * m + 4 > 127 || 16 * x + 4 < -128) return false;
  int b = -(16 * o + 1);
  b = (b + 15) & ~15;
  if (16 * (e - o) >= 2048) return false;
  if (16 * m * Q + b + 16 * (e - o) + 16 >= 31744) return false;
  *bias = b;
  return true;
}

int launch_sw_score(cudaStream_t st, const FastArgs& a, int64_t max_pairs) {
  if (max_pairs <= 0) return 0;
  const int64_t warps = (max_pairs + 3) / 4;
  const unsigned grid = (unsigned)((warps + kFastWarps - 1) / kFastWarps);
  switch (fast_rows_per_lane(a.Q)) {
    case 2: sw_score_kernel<2><<<grid, kFastWarps * 32, 0, st>>>(a); break;
    case 4: sw_score_kernel<4><<<grid, kFastWarps * 32, 0, st>>>(a); break;
    case 7: sw_score_kernel<7><<<grid, kFastWarps * 32, 0, st>>>(a); break;
    case 8: sw_score_kernel<8><<<grid, kFastWarps * 32, 0, st>>>(a); break;
    case 12: sw_score_kernel<12><<<grid, kFastWarps * 32, 0, st>>>(a); break;
    case 16: sw_score_kernel<16><<<grid, kFastWarps * 32, 0, st>>>(a); break;
    default: return 0;
  }
  return 1;
}

}  // namespace swift
