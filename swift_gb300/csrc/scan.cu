// Device-wide exclusive prefix sums (reduce -> scan of tile sums -> scan).
// Used for index bucket starts, record compaction and output text offsets.
#include "internal.h"

namespace swift {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kTile = kScanThreads * kScanItems;

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    T o = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v += o;
  }
  return v;
}

// Exclusive scan of one value per thread across the block; returns the
// exclusive prefix and writes the block total to *total.
template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T* total) {
  __shared__ T warp_sums[kScanThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  T inc = warp_incl_scan(v);
  if (lane == 31) warp_sums[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    T s = lane < kScanThreads / 32 ? warp_sums[lane] : T(0);
    s = warp_incl_scan(s);
    if (lane < kScanThreads / 32) warp_sums[lane] = s;
  }
  __syncthreads();
  T base = wid ? warp_sums[wid - 1] : T(0);
  *total = warp_sums[kScanThreads / 32 - 1];
  __syncthreads();
  return base + inc - v;
}

template <typename T>
__global__ void tile_reduce(const T* __restrict__ in, int64_t n, T* __restrict__ sums) {
  const int64_t base = (int64_t)blockIdx.x * kTile;
  T s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  T tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <typename T>
__global__ void tile_scan(const T* __restrict__ in, T* __restrict__ out, int64_t n,
                          const T* __restrict__ tile_base, T* total_out) {
  const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kScanItems;
  T v[kScanItems];
  T s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + k;
    v[k] = i < n ? in[i] : T(0);
    s += v[k];
  }
  T tot;
  T pre = block_excl_scan(s, &tot) + (tile_base ? tile_base[blockIdx.x] : T(0));
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + k;
    if (i < n) out[i] = pre;
    pre += v[k];
  }
  if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == kScanThreads - 1)
    *total_out = pre;
}

template <typename T>
size_t temp_elems(int64_t n) {
  size_t t = 0;
  while (n > kTile) {
    n = (n + kTile - 1) / kTile;
    t += 2 * (size_t)n;
  }
  return t;
}

template <typename T>
int scan_rec(cudaStream_t st, const T* in, T* out, int64_t n, T* temp, T* total) {
  if (n <= 0) {
    if (total) cudaMemsetAsync(total, 0, sizeof(T), st);
    return 0;
  }
  int64_t tiles = (n + kTile - 1) / kTile;
  if (tiles == 1) {
    tile_scan<T><<<1, kScanThreads, 0, st>>>(in, out, n, nullptr, total);
    return 1;
  }
  T* sums = temp;
  T* sums_scan = temp + tiles;
  tile_reduce<T><<<(unsigned)tiles, kScanThreads, 0, st>>>(in, n, sums);
  int k = scan_rec<T>(st, sums, sums_scan, tiles, temp + 2 * tiles, nullptr);
  tile_scan<T><<<(unsigned)tiles, kScanThreads, 0, st>>>(in, out, n, sums_scan, total);
  return k + 2;
}

}  // namespace

size_t scan_temp_bytes(int64_t n) { return (temp_elems<uint64_t>(n) + 16) * sizeof(uint64_t); }

int exclusive_scan_u32(cudaStream_t st, const uint32_t* in, uint32_t* out, int64_t n,
                       void* temp, uint32_t* total_dev) {
  return scan_rec<uint32_t>(st, in, out, n, (uint32_t*)temp, total_dev);
}

int exclusive_scan_u64(cudaStream_t st, const uint64_t* in, uint64_t* out, int64_t n,
                       void* temp, uint64_t* total_dev) {
  return scan_rec<uint64_t>(st, in, out, n, (uint64_t*)temp, total_dev);
}

}  // namespace swift
