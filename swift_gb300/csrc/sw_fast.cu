// Launchers of the packed passes (kernels in sw_packed.cuh) and the bound
// pass: the relaxed-recurrence upper bound of every pair's score.
#include "sw_packed.cuh"

namespace swift {

// the trace pass (per-pair lengths) and walk of the shapes in kExtraShapes,
// compiled in sw_shapes_{a,b,c}.cu: 1 when the shape was theirs
int launch_trace_var_a(int G, int RPL, unsigned grid, size_t smem, cudaStream_t st, const FastArgs& a);
int launch_trace_var_b(int G, int RPL, unsigned grid, size_t smem, cudaStream_t st, const FastArgs& a);
int launch_trace_var_c(int G, int RPL, unsigned grid, size_t smem, cudaStream_t st, const FastArgs& a);
int launch_walk_a(int G, int RPL, unsigned grid, cudaStream_t st, const FastArgs& a);
int launch_walk_b(int G, int RPL, unsigned grid, cudaStream_t st, const FastArgs& a);
int launch_walk_c(int G, int RPL, unsigned grid, cudaStream_t st, const FastArgs& a);

namespace {

// Upper bound of every pair's score: the same recurrence with every gap
// charged gap_ext (>= gap_open), so by induction each cell is at least the
// reference's cell and the maximum is an upper bound of the score.  Without
// directions a cell is one plain 16-bit H; with Z = -gap_ext
//     H + Z = max(H[i-1][j-1] + (s - gap_ext), H[i-1][j], H[i][j-1], Z)
//     H     = (H + Z) + gap_ext
// i.e. a byte permute, a three-way max, an add-max and one plain add per two
// cells, against six ALU operations of the exact pass.  Rows past the query
// (all mismatch) stay strictly below the maximum of the rows above, as in the
// exact pass.  Writes a.ub[p] = the bound.
constexpr int kBdWarps = 4;

template <int G, int RPL>
__global__ void __launch_bounds__(kBdWarps * 32) sw_bound_kernel(FastArgs a) {
  constexpr int kGroups = 32 / G;
  constexpr int kPairs = 2 * kGroups;
  extern __shared__ uint16_t wsel16_all[];  // [warps * groups][R + 1]
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane / G, sl = lane % G;
  const int64_t nlist = *a.count - a.list_offset;
  const int64_t warp = (int64_t)blockIdx.x * kBdWarps + wib;
  if (warp * kPairs >= nlist) return;  // whole warp
  const int64_t base = warp * kPairs + 2 * g;
  const int Q = a.Q, R = a.R;
  const int32_t* list = a.list + a.list_offset;
  const bool has0 = base < nlist, has1 = base + 1 < nlist;
  const int32_t p0 = has0 ? list[base] : list[nlist - 1];
  const int32_t p1 = has1 ? list[base + 1] : p0;
  // each pair's query length (rows past it are all-mismatch rows)
  const int Q0 = a.q_len ? a.q_len[p0] : Q, Q1 = a.q_len ? a.q_len[p1] : Q;
  const char* q0 = a.q + (int64_t)p0 * a.q_stride;
  const char* q1 = a.q + (int64_t)p1 * a.q_stride;
  const char* w0 = a.w + (int64_t)p0 * a.w_stride;
  const char* w1 = a.w + (int64_t)p1 * a.w_stride;
  uint16_t* wsel = wsel16_all + (wib * kGroups + g) * (R + 1);
  for (int c = sl; c < R; c += G) {
    uint32_t s0 = base_class((uint8_t)w0[c]), s1 = base_class((uint8_t)w1[c]);
    wsel[c + 1] = (uint16_t)(s0 | ((s0 | 8u) << 4) | ((4u + s1) << 8) | (((4u + s1) | 8u) << 12));
  }
  __syncwarp();
  const uint32_t Z = (uint32_t)(-a.gap_ext);
  const uint32_t ZZ = Z * 0x00010001u;
  // per-half add of gap_ext as one 32-bit add: every half it meets is at
  // least Z = -gap_ext, so no borrow crosses between the halves
  const uint32_t EE = (uint32_t)((int32_t)a.gap_ext * 65537);
  const uint32_t sm = (uint32_t)(uint8_t)(int8_t)(a.match - a.gap_ext);
  const uint32_t sx = (uint32_t)(uint8_t)(int8_t)(a.mismatch - a.gap_ext);
  const uint32_t all_x = sx * 0x01010101u;
  uint32_t prof0[RPL], prof1[RPL], h[RPL];
#pragma unroll
  for (int k = 0; k < RPL; ++k) {
    const int i = sl * RPL + k;
    prof0[k] = i < Q0 ? all_x ^ ((sm ^ sx) << (8 * base_class((uint8_t)q0[i]))) : all_x;
    prof1[k] = i < Q1 ? all_x ^ ((sm ^ sx) << (8 * base_class((uint8_t)q1[i]))) : all_x;
    h[k] = 0;  // H[i][0] = 0
  }
  const uint32_t not_first = sl == 0 ? 0u : 1u;  // row 0 above lane 0: H = 0
  const uint16_t* wcol = wsel + 1 - sl;          // lane sl holds column s - sl + 1
  // maximum of the lane's cells per block of kSufSteps wavefront steps
  uint32_t* blk = reinterpret_cast<uint32_t*>(wsel16_all + kBdWarps * kGroups * (R + 1)) +
                  (wib * 32 + lane) * kSufBlocks;
  uint32_t best = ZZ, send = 0, prev_up = 0;
  // One wavefront step; `check` only in the G - 1 steps at either end, where
  // some lanes are outside the window.  The running maximum takes only the
  // cells of `track` steps: a lane holds whole rows, and the cell right of
  // an untracked cell, one step later, is at least its value + gap_ext, so
  // the maximum of tracked cells - gap_ext bounds every cell.  The last
  // column of every row is tracked (the last main step and the checked
  // steps).
  auto step = [&](int s, bool check, bool track) {
    uint32_t up = __shfl_up_sync(0xffffffffu, send, 1, G) * not_first;
    // the diagonal of the lane's first row is the lane above's last row one
    // column back: what arrived as `up` one step earlier
    uint32_t dg = prev_up;
    prev_up = up;
    if (check) {
      const int j = s - sl + 1;
      if (j < 1 || j > R) return;
    }
    const uint32_t ws = wcol[s];
    uint32_t hpair = 0;
#pragma unroll
    for (int k = 0; k < RPL; ++k) {
      const uint32_t sc = prmt(prof0[k], prof1[k], ws);
      const uint32_t t = __vimax3_s16x2(up, h[k], ZZ);
      const uint32_t hz = __viaddmax_s16x2(dg, sc, t);
      dg = h[k];
      up = hz + EE;
      h[k] = up;
      if (!track) {
      } else if (k & 1) {
        best = __vimax3_s16x2(best, hpair, hz);
      } else if (k == RPL - 1) {
        best = __vimax_s16x2_relu(best, hz);
      } else {
        hpair = hz;
      }
    }
    send = up;
  };
  const int steps = R + G - 1;
  auto flush = [&](int s) {
    if ((s & (kSufSteps - 1)) == kSufSteps - 1) {
      blk[s / kSufSteps] = best;
      best = ZZ;
    }
  };
  if (R >= G) {
    for (int s = 0; s < G - 1; ++s) {
      step(s, true, true);
      flush(s);
    }
    // steady state in pairs of steps, the maximum taken on the second
    int s = G - 1;
    for (; s + 1 < R - 1; s += 2) {
      step(s, false, false);
      flush(s);
      step(s + 1, false, true);
      flush(s + 1);
    }
    for (; s < R; ++s) {
      step(s, false, true);
      flush(s);
    }
    for (s = R; s < steps; ++s) {
      step(s, true, true);
      flush(s);
    }
  } else {
    for (int s = 0; s < steps; ++s) {
      step(s, true, true);
      flush(s);
    }
  }
  const int nblk = (steps + kSufSteps - 1) / kSufSteps;
  if (steps % kSufSteps) blk[nblk - 1] = best;
  // suffix maxima over blocks, across the group's lanes: suf[m] bounds every
  // cell the wavefront reaches at step kSufSteps * m or later, which covers
  // all cells right of column kSufSteps * m
  uint32_t suf = ZZ;
  for (int b = nblk - 1; b >= 0; --b) {
    suf = __vimax_s16x2_relu(suf, blk[b]);
    uint32_t v = suf;
#pragma unroll
    for (int d = G / 2; d > 0; d >>= 1) v = __vimax_s16x2_relu(v, __shfl_xor_sync(0xffffffffu, v, d, G));
    if (sl == 0) {
      // tracked maximum (H + Z) - Z, plus Z = -gap_ext for the untracked cells
      const int32_t v0 = (int32_t)(v & 0xFFFFu), v1 = (int32_t)(v >> 16);
      if (a.suf) {
        if (has0) a.suf[(int64_t)p0 * kSufBlocks + b] = (uint16_t)v0;
        if (has1) a.suf[(int64_t)p1 * kSufBlocks + b] = (uint16_t)v1;
      }
      if (b == 0) {
        if (has0) a.ub[p0] = v0;
        if (has1) a.ub[p1] = v1;
      }
    }
  }
}

struct Shape {
  int G, RPL;
};

// lanes per group and rows per lane for a query length (Q <= 320)
Shape shape_for(int Q) {
  if (Q <= 32) return {8, 4};
  if (Q <= 64) return {8, 8};
  if (Q <= 104) return {8, 13};
  if (Q <= 128) return {8, 16};
  if (Q <= 208) return {16, 13};
  if (Q <= 256) return {16, 16};
  if (Q <= 320) return {32, 10};
  return {0, 0};
}

// the compiled (lanes, rows per lane) shapes of the exact passes
constexpr Shape kShapes[] = {{8, 4}, {4, 8}, {8, 8}, {4, 16}, {8, 13}, {8, 16},
                             {16, 8}, {16, 13}, {16, 16}, {32, 7}, {32, 10}};
constexpr int kNumShapes = (int)(sizeof(kShapes) / sizeof(kShapes[0]));
// shapes of the per-pair-length trace pass and walk only (swift_sw_pairs'
// query length classes between the row counts above)
constexpr Shape kExtraShapes[] = {{8, 5},   {8, 6},   {8, 7},   {8, 9},   {8, 10},  {8, 11},
                                  {8, 12},  {8, 14},  {8, 15},  {16, 9},  {16, 10}, {16, 11},
                                  {16, 12}, {16, 14}, {16, 15}, {32, 8},  {32, 9}};

// The launch's shape: a.shape when set (it must cover a.Q), else the
// default for a.Q.
Shape shape_of(const FastArgs& a) {
  if (a.shape_g > 0) {
    for (const Shape& c : kShapes)
      if (c.G == a.shape_g && c.RPL == a.shape_rpl && c.G * c.RPL >= a.Q) return c;
    for (const Shape& c : kExtraShapes)
      if (c.G == a.shape_g && c.RPL == a.shape_rpl && c.G * c.RPL >= a.Q) return c;
    return {0, 0};
  }
  return shape_for(a.Q);
}

template <bool TRACE, bool VAR>
int launch_shape(cudaStream_t st, const FastArgs& a, int64_t max_pairs) {
  const Shape s = shape_of(a);
  if (s.G == 0 || max_pairs <= 0) return 0;
  const int pairs_per_warp = 2 * (32 / s.G);
  const int64_t warps = (max_pairs + pairs_per_warp - 1) / pairs_per_warp;
  const unsigned grid = (unsigned)((warps + kPkWarps - 1) / kPkWarps);
  const int tb = kPkWarps * 32;
  const size_t smem = (size_t)kPkWarps * (32 / s.G) * (a.R + 1) * sizeof(uint32_t);
#define SWIFT_PK(G_, R_)                                                  \
  if (s.G == G_ && s.RPL == R_) {                                          \
    if (smem > 48 * 1024)                                                  \
      cudaFuncSetAttribute(sw_packed_kernel<G_, R_, TRACE, VAR>,           \
                           cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                           (int)smem);                                     \
    sw_packed_kernel<G_, R_, TRACE, VAR><<<grid, tb, smem, st>>>(a);       \
    return 1;                                                              \
  }
  SWIFT_PK(8, 4)
  SWIFT_PK(4, 8)
  SWIFT_PK(8, 8)
  SWIFT_PK(4, 16)
  SWIFT_PK(8, 13)
  SWIFT_PK(8, 16)
  SWIFT_PK(16, 8)
  SWIFT_PK(16, 13)
  SWIFT_PK(16, 16)
  SWIFT_PK(32, 7)
  SWIFT_PK(32, 10)
#undef SWIFT_PK
  if (TRACE && VAR)
    return launch_trace_var_a(s.G, s.RPL, grid, smem, st, a) ||
           launch_trace_var_b(s.G, s.RPL, grid, smem, st, a) ||
           launch_trace_var_c(s.G, s.RPL, grid, smem, st, a);
  return 0;
}

// lanes per group and rows per lane of the bound pass: three registers per
// row (against four in the exact passes) leave room for longer strips, which
// spread the per-step work over more cells
Shape bound_shape_for(int Q) {
  if (Q <= 32) return {4, 8};
  if (Q <= 64) return {4, 16};
  if (Q <= 100) return {4, 25};
  if (Q <= 128) return {4, 32};
  if (Q <= 200) return {8, 25};
  if (Q <= 256) return {8, 32};
  if (Q <= 320) return {16, 20};
  return {0, 0};
}

int launch_bound(cudaStream_t st, const FastArgs& a, int64_t max_pairs) {
  const Shape s = bound_shape_for(a.Q);
  if (s.G == 0 || max_pairs <= 0) return 0;
  const int pairs_per_warp = 2 * (32 / s.G);
  const int64_t warps = (max_pairs + pairs_per_warp - 1) / pairs_per_warp;
  const unsigned grid = (unsigned)((warps + kBdWarps - 1) / kBdWarps);
  if (a.R + s.G - 1 > kSufSteps * kSufBlocks) return 0;
  const size_t smem = (size_t)kBdWarps * (32 / s.G) * (a.R + 1) * sizeof(uint16_t) +
                      (size_t)kBdWarps * 32 * kSufBlocks * sizeof(uint32_t) + 16;
#define SWIFT_BD(G_, R_)                                                  \
  if (s.G == G_ && s.RPL == R_) {                                          \
    if (smem > 48 * 1024)                                                  \
      cudaFuncSetAttribute(sw_bound_kernel<G_, R_>,                        \
                           cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                           (int)smem);                                     \
    sw_bound_kernel<G_, R_><<<grid, kBdWarps * 32, smem, st>>>(a);         \
    return 1;                                                              \
  }
  SWIFT_BD(4, 8)
  SWIFT_BD(4, 16)
  SWIFT_BD(4, 25)
  SWIFT_BD(4, 32)
  SWIFT_BD(8, 25)
  SWIFT_BD(8, 32)
  SWIFT_BD(16, 20)
#undef SWIFT_BD
  return 0;
}

int launch_walk(cudaStream_t st, const FastArgs& a, int64_t max_pairs) {
  const Shape s = shape_of(a);
  if (s.G == 0 || max_pairs <= 0) return 0;
  const unsigned grid = (unsigned)((max_pairs + kWalkThreads - 1) / kWalkThreads);
#define SWIFT_WK(G_, R_)                                      \
  if (s.G == G_ && s.RPL == R_) {                              \
    sw_walk_kernel<G_, R_><<<grid, kWalkThreads, 0, st>>>(a);  \
    return 1;                                                  \
  }
  SWIFT_WK(8, 4)
  SWIFT_WK(4, 8)
  SWIFT_WK(8, 8)
  SWIFT_WK(4, 16)
  SWIFT_WK(8, 13)
  SWIFT_WK(8, 16)
  SWIFT_WK(16, 8)
  SWIFT_WK(16, 13)
  SWIFT_WK(16, 16)
  SWIFT_WK(32, 7)
  SWIFT_WK(32, 10)
#undef SWIFT_WK
  return launch_walk_a(s.G, s.RPL, grid, st, a) || launch_walk_b(s.G, s.RPL, grid, st, a) ||
         launch_walk_c(s.G, s.RPL, grid, st, a);
}

}  // namespace


bool fast_params_ok(int Q, int R, int m, int x, int o, int e, int* bias) {
  if (R < 1 || R > kFastMaxR || shape_for(Q).G == 0) return false;
  if (!(x < 0 && o < 0 && e < 0 && e >= o && m > 0)) return false;
  if (16 * m + 4 > 127 || 16 * x + 4 < -128) return false;
  int b = -(16 * o + 1);
  b = (b + 15) & ~15;
  if (16 * (e - o) >= 2048) return false;
  if (16 * m * Q + b + 16 * (e - o) + 16 >= 0x7C00) return false;
  *bias = b;
  return true;
}

int64_t trace_scratch_words(int Q, int R, int64_t pairs, int shape_g, int shape_rpl) {
  FastArgs a;
  memset(&a, 0, sizeof(a));
  a.Q = Q;
  a.shape_g = shape_g;
  a.shape_rpl = shape_rpl;
  const Shape s = shape_of(a);
  if (s.G == 0) return 0;
  const int64_t groups = (pairs + 1) / 2 + 32;  // round up to whole warps
  return groups * (int64_t)s.G * ((s.RPL + 7) / 8) * steps8(R, s.G);
}

int packed_shape_candidates(int Q, int32_t* g, int32_t* rpl, int cap) {
  // the shape whose rows are Q's row class exactly (8 lanes up to 128 rows,
  // 16 up to 256, then 32), then the other shapes of the trace pass with up
  // to about an eighth more rows
  const int rows = var_rows(Q);
  if (rows < 0 || cap < 1) return 0;
  const int dg = rows <= 128 ? 8 : rows <= 256 ? 16 : 32;
  const Shape d = {dg, rows / dg};
  int n = 0;
  g[n] = d.G;
  rpl[n] = d.RPL;
  ++n;
  auto add = [&](const Shape& c) {
    const int r = c.G * c.RPL;
    if (r >= rows && r <= rows + rows / 8 + 8 && !(c.G == d.G && c.RPL == d.RPL) && n < cap) {
      g[n] = c.G;
      rpl[n] = c.RPL;
      ++n;
    }
  };
  for (const Shape& c : kShapes) add(c);
  for (const Shape& c : kExtraShapes) add(c);
  return n;
}

int launch_sw_score(cudaStream_t st, const FastArgs& a, int64_t max_pairs) {
  return a.q_len ? launch_shape<false, true>(st, a, max_pairs)
                 : launch_shape<false, false>(st, a, max_pairs);
}

int launch_sw_bound(cudaStream_t st, const FastArgs& a, int64_t max_pairs) {
  return launch_bound(st, a, max_pairs);
}

int launch_sw_trace(cudaStream_t st, const FastArgs& a, int64_t max_pairs, cudaEvent_t before,
                    cudaEvent_t after) {
  if (a.cons_stride % 4 != 0) return 0;  // the walk stores 32-bit words
  FastArgs b = a;
  b.chunk = max_pairs;
  b.one = 1;
  b.four = 4;
  if (before && cudaEventRecord(before, st) != cudaSuccess) return 0;
  int k = a.q_len ? launch_shape<true, true>(st, b, max_pairs) : launch_shape<true, false>(st, b, max_pairs);
  if (after && cudaEventRecord(after, st) != cudaSuccess) return 0;
  return k + launch_walk(st, b, max_pairs);
}

}  // namespace swift
