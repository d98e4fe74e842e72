// Packed trace pass (per-pair lengths) and walk for the (lanes, rows per
// lane) shapes {8, 5}, {8, 6}, {8, 7}, {8, 9}, {8, 10}, {8, 11}: the row counts
// between those of the other packed shapes, which swift_sw_pairs' query
// length classes take exactly.  Kernels in sw_packed.cuh; their own
// translation unit so that the shapes compile in parallel.
#include "sw_packed.cuh"

namespace swift {

int launch_trace_var_a(int G, int RPL, unsigned grid, size_t smem, cudaStream_t st,
                        const FastArgs& a) {
#define SWIFT_PKX(G_, R_)                                                  \
  if (G == G_ && RPL == R_) {                                              \
    if (smem > 48 * 1024)                                                  \
      cudaFuncSetAttribute(sw_packed_kernel<G_, R_, true, true>,           \
                           cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                           (int)smem);                                     \
    sw_packed_kernel<G_, R_, true, true><<<grid, kPkWarps * 32, smem, st>>>(a); \
    return 1;                                                              \
  }
  SWIFT_PKX(8, 5)
  SWIFT_PKX(8, 6)
  SWIFT_PKX(8, 7)
  SWIFT_PKX(8, 9)
  SWIFT_PKX(8, 10)
  SWIFT_PKX(8, 11)
#undef SWIFT_PKX
  return 0;
}

int launch_walk_a(int G, int RPL, unsigned grid, cudaStream_t st, const FastArgs& a) {
#define SWIFT_WKX(G_, R_)                                      \
  if (G == G_ && RPL == R_) {                                  \
    sw_walk_kernel<G_, R_><<<grid, kWalkThreads, 0, st>>>(a);  \
    return 1;                                                  \
  }
  SWIFT_WKX(8, 5)
  SWIFT_WKX(8, 6)
  SWIFT_WKX(8, 7)
  SWIFT_WKX(8, 9)
  SWIFT_WKX(8, 10)
  SWIFT_WKX(8, 11)
#undef SWIFT_WKX
  return 0;
}

}  // namespace swift
