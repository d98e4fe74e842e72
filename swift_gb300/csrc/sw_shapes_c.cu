// Packed trace pass (per-pair lengths) and walk for the (lanes, rows per
// lane) shapes {16, 12}, {16, 14}, {16, 15}, {32, 8}, {32, 9}: the row counts
// between those of the other packed shapes, which swift_sw_pairs' query
// length classes take exactly.  Kernels in sw_packed.cuh; their own
// translation unit so that the shapes compile in parallel.
#include "sw_packed.cuh"

namespace swift {

int launch_trace_var_c(int G, int RPL, unsigned grid, size_t smem, cudaStream_t st,
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
  SWIFT_PKX(16, 12)
  SWIFT_PKX(16, 14)
  SWIFT_PKX(16, 15)
  SWIFT_PKX(32, 8)
  SWIFT_PKX(32, 9)
#undef SWIFT_PKX
  return 0;
}

int launch_walk_c(int G, int RPL, unsigned grid, cudaStream_t st, const FastArgs& a) {
#define SWIFT_WKX(G_, R_)                                      \
  if (G == G_ && RPL == R_) {                                  \
    sw_walk_kernel<G_, R_><<<grid, kWalkThreads, 0, st>>>(a);  \
    return 1;                                                  \
  }
  SWIFT_WKX(16, 12)
  SWIFT_WKX(16, 14)
  SWIFT_WKX(16, 15)
  SWIFT_WKX(32, 8)
  SWIFT_WKX(32, 9)
#undef SWIFT_WKX
  return 0;
}

}  // namespace swift
