// Launchers of the packed passes (kernels in sw_packed.cuh).
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
