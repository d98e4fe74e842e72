// Phase 2: Smith-Waterman with traceback, the semantics of the reference's
// GPU kernel smithWaterman (src/smithWaterman.cu:360-395, 510-645, 911-1026):
//
//   H[i][0] = H[0][j] = 0, every boundary cell has direction NONE
//   s = match if U(q[i-1]) == U(r[j-1]) or either is 'N', else mismatch
//   d = H[i-1][j-1] + s
//   t = H[i-1][j] + (dir[i-1][j] == UP   ? gap_ext : gap_open)
//   l = H[i][j-1] + (dir[i][j-1] == LEFT ? gap_ext : gap_open)
//   H = 0, dir = NONE; d > H -> DIAG; t > H -> UP; l > H -> LEFT (strict)
//
// (the gap penalty depends on the neighbour's own chosen direction; there
// is no separate E/F matrix).  Score = max H; the reported cell is the first
// maximum in row-major order.  The traceback walks directions from that cell
// and stops before a NONE cell or after a cell whose predecessor lies in row
// 0 or column 0; it emits reversed consensus strings from the original
// (not upper-cased) bytes.
//
// Kernel layout: one warp per pair.  Lane t owns query rows t*RPL+1 ..
// t*RPL+RPL and sweeps the window columns one step behind lane t-1 (an
// anti-diagonal wavefront of row strips).  The bottom row's H and its
// downward gap candidate pass to the next lane with one shuffle per step.
// 2-bit directions of the lane's rows are packed per column into shared
// memory; lane 0 walks them for the traceback.
#include <mutex>

#include "internal.h"

namespace swift {
namespace {

constexpr int kSwWarps = 4;
enum : uint32_t { kNone = 0, kDiag = 1, kUp = 2, kLeft = 3 };

__device__ __forceinline__ uint32_t upper(uint32_t c) {
  return (c - 'a') < 26u ? c - 'a' + 'A' : c;
}

template <int RPL>
struct DirWord;
template <>
struct DirWord<4> { using T = uint8_t; };
template <>
struct DirWord<8> { using T = uint16_t; };
template <>
struct DirWord<10> { using T = uint32_t; };

// One pair on one warp; base is the warp's shared-memory slice.
template <int RPL>
__device__ __forceinline__ void generic_pair(const SwArgs& a, int64_t pair, uint8_t* base,
                                             int lane) {
  using DW = typename DirWord<RPL>::T;
  const int Q = a.q_len ? a.q_len[pair] : a.Q, R = a.R;
  uint8_t* wsh = base;                                  // R bytes (rounded to 16)
  DW* dirs = reinterpret_cast<DW*>(base + ((R + 15) & ~15));  // (R+1) x 32
  const char* qg = a.q + pair * a.q_stride;
  const char* wg = a.w + pair * a.w_stride;
  for (int c = lane; c < R; c += 32) wsh[c] = (uint8_t)wg[c];
  const int m = a.match, x = a.mismatch, go = a.gap_open, ge = a.gap_ext;
  // my rows
  uint32_t qu[RPL];
  int hprev[RPL], eleft[RPL], best[RPL], bestj[RPL];
  int nrows = Q - lane * RPL;
  nrows = nrows < 0 ? 0 : (nrows > RPL ? RPL : nrows);
#pragma unroll
  for (int k = 0; k < RPL; ++k) {
    int i = lane * RPL + k;
    qu[k] = i < Q ? upper((uint8_t)qg[i]) : 0u;
    hprev[k] = 0;
    eleft[k] = go;  // H[i][0] = 0 with direction NONE
    best[k] = 0;
    bestj[k] = 0;
  }
  __syncwarp();
  int send_h = 0, send_f = go, diag_h = 0;
  const int steps = R + 31;
  for (int s = 0; s < steps; ++s) {
    int recv_h = __shfl_up_sync(0xffffffffu, send_h, 1);
    int recv_f = __shfl_up_sync(0xffffffffu, send_f, 1);
    if (lane == 0) {
      recv_h = 0;
      recv_f = go;
    }
    const int j = s - lane + 1;
    if (j >= 1 && j <= R && nrows > 0) {
      const uint32_t wc = upper(wsh[j - 1]);
      const bool wn = wc == 'N';
      int hd = diag_h;
      int fu = recv_f;
      uint32_t bits = 0;
#pragma unroll
      for (int k = 0; k < RPL; ++k) {
        if (k < nrows) {
          const int sc = (qu[k] == wc || qu[k] == 'N' || wn) ? m : x;
          const int d = hd + sc, t = fu, l = eleft[k];
          int v = 0;
          uint32_t dir = kNone;
          if (v < d) { v = d; dir = kDiag; }
          if (v < t) { v = t; dir = kUp; }
          if (v < l) { v = l; dir = kLeft; }
          hd = hprev[k];
          hprev[k] = v;
          fu = v + (dir == kUp ? ge : go);
          eleft[k] = v + (dir == kLeft ? ge : go);
          if (best[k] < v) {
            best[k] = v;
            bestj[k] = j;
          }
          bits |= dir << (2 * k);
        }
      }
      dirs[j * 32 + lane] = (DW)bits;
      send_h = hprev[nrows - 1];
      send_f = fu;
    }
    diag_h = recv_h;
  }
  // first maximum in row-major order
  int bh = 0, bcell = 0x7fffffff;
#pragma unroll
  for (int k = 0; k < RPL; ++k) {
    if (k < nrows && bh < best[k]) {
      bh = best[k];
      bcell = (lane * RPL + k + 1) * (R + 1) + bestj[k];
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    int oh = __shfl_xor_sync(0xffffffffu, bh, d);
    int oc = __shfl_xor_sync(0xffffffffu, bcell, d);
    if (oh > bh || (oh == bh && oc < bcell)) {
      bh = oh;
      bcell = oc;
    }
  }
  __syncwarp();
  if (lane != 0) return;
  const int cell_max = bh > 0 ? bcell : 0;
  const int W = R + 1;
  auto dir_at = [&](int cell) -> uint32_t {
    int i = cell / W, jj = cell % W;
    if (i == 0 || jj == 0) return kNone;
    int ln = (i - 1) / RPL, k = (i - 1) % RPL;
    return ((uint32_t)dirs[jj * 32 + ln] >> (2 * k)) & 3u;
  };
  // consensus strings are optional (coordinates only when the caller passes none)
  const bool cons = a.qcons != nullptr;
  char* qc = cons ? a.qcons + pair * a.cons_stride : nullptr;
  char* rc = cons ? a.rcons + pair * a.cons_stride : nullptr;
  auto put = [&](int t, char r, char q) {
    if (cons) {
      rc[t] = r;
      qc[t] = q;
    }
  };
  int cur = cell_max, cr = cur / W, cc = cur % W, nxt;
  uint32_t d0 = dir_at(cur);
  nxt = d0 == kUp ? cur - W : d0 == kLeft ? cur - 1 : d0 == kDiag ? cur - W - 1 : cur;
  int nr = nxt / W, nc = nxt % W;
  int tick = -1, nref = -1, start = 0;
  while ((cr != nr || cc != nc) && nc != 0 && nr != 0) {
    ++tick;
    char rch = '-';
    if (nc != cc) { rch = wg[cc - 1]; ++nref; }
    put(tick, rch, nr == cr ? '-' : qg[cr - 1]);
    start = cc;
    cur = nxt; cr = nr; cc = nc;
    uint32_t dd = dir_at(cur);
    if (dd == kNone) break;
    nxt = dd == kUp ? cur - W : dd == kLeft ? cur - 1 : cur - W - 1;
    nr = nxt / W; nc = nxt % W;
  }
  if ((cr != nr || cc != nc) && (nc == 0 || nr == 0)) {
    ++tick;
    char rch = '-';
    if (nc != cc) { rch = wg[cc - 1]; ++nref; }
    put(tick, rch, nr == cr ? '-' : qg[cr - 1]);
    start = cc;
  }
  DevAln out;
  out.score = bh;
  out.start = start;
  out.end = start + nref;
  out.len = tick + 1;
  a.aln[pair] = out;
}

// Warps stride over the pairs (the list's length is known on the device
// only, so the grid is capped rather than sized by it).  W warps per block:
// fewer for long windows, whose direction words fill more shared memory.
template <int RPL, int W>
__global__ void __launch_bounds__(W * 32) sw_generic_kernel(SwArgs a, int per_warp_bytes) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint8_t* base = smem + (size_t)wib * per_warp_bytes;
  const int64_t n = a.list ? (int64_t)*a.count : a.n;
  for (int64_t i = (int64_t)blockIdx.x * W + wib; i < n; i += (int64_t)gridDim.x * W) {
    generic_pair<RPL>(a, a.list ? (int64_t)a.list[i] : i, base, lane);
    __syncwarp();
  }
}

template <int RPL>
int per_warp_bytes(int R) {
  return ((R + 15) & ~15) + (R + 1) * 32 * (int)sizeof(typename DirWord<RPL>::T);
}

constexpr size_t kGenericSmemMax = 200 * 1024;

template <int RPL, int W>
int launch_generic_w(cudaStream_t st, const SwArgs& a, int pw) {
  const size_t smem = (size_t)pw * W;
  // the opt-in above 48 KB is a per-device function attribute: set it on
  // every launch (cheap), so a second device or context needs no state here
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(sw_generic_kernel<RPL, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return SWIFT_E_CUDA;
  int64_t blocks = (a.n + W - 1) / W;
  if (a.list) {  // the list's length is on the device: a few waves stride over it
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0)
      blocks = std::min<int64_t>(blocks, (int64_t)sms * 16 * 4 / W);
  }
  sw_generic_kernel<RPL, W><<<(unsigned)blocks, W * 32, smem, st>>>(a, pw);
  return SWIFT_OK;
}

template <int RPL>
int launch_generic(cudaStream_t st, const SwArgs& a, std::string* err) {
  int pw = per_warp_bytes<RPL>(a.R);
  pw = (pw + 15) & ~15;
  int rc;
  if ((size_t)pw * kSwWarps <= kGenericSmemMax)
    rc = launch_generic_w<RPL, kSwWarps>(st, a, pw);
  else if ((size_t)pw * 2 <= kGenericSmemMax)
    rc = launch_generic_w<RPL, 2>(st, a, pw);
  else if ((size_t)pw <= kGenericSmemMax)
    rc = launch_generic_w<RPL, 1>(st, a, pw);
  else {
    *err = "window too long for the on-chip traceback";
    return SWIFT_E_LIMIT;
  }
  if (rc != SWIFT_OK) *err = "generic kernel: shared-memory opt-in failed";
  return rc;
}

}  // namespace

// Per-pair results for swift_sw_batch_noalloc, held in module memory that is
// reserved when the module loads, so that call needs no allocation.  Each
// record is written by the kernel before anything reads it: nothing here has
// to start at zero.  Every caller on a device shares this one array.
__device__ __align__(256) DevAln g_static_aln[kStaticSwPairs];

int static_sw_scratch(int device, DevAln** out, std::string* err) {
  // The symbol's address is looked up once per device, with that device
  // current (the caller has made it so), and kept.
  constexpr int kDevices = 64;
  static std::mutex mu;
  static DevAln* addr[kDevices] = {};
  if (device < 0 || device >= kDevices) {
    *err = "device ordinal outside 0..63";
    return SWIFT_E_ARG;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_aln);
    if (e != cudaSuccess) {
      *err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return SWIFT_E_CUDA;
    }
    addr[device] = static_cast<DevAln*>(p);
  }
  *out = addr[device];
  return SWIFT_OK;
}

int launch_sw(cudaStream_t st, const SwArgs& a, std::string* err) {
  if (a.n <= 0) return SWIFT_OK;
  if (a.Q < 1 || a.Q > kMaxQ || a.R < 1 || a.R > kMaxR) {
    *err = "Smith-Waterman dimensions outside 1..320 x 1..1024";
    return SWIFT_E_LIMIT;
  }
  if (a.Q <= 128) return launch_generic<4>(st, a, err);
  if (a.Q <= 256) return launch_generic<8>(st, a, err);
  return launch_generic<10>(st, a, err);
}

}  // namespace swift

// ---------------------------------------------------------------------------
// Peak of the packed-int16 max-plus instruction (__vimax3_s16x2_relu: the
// three-way max with zero floor of two 16-bit cells), measured on this GPU:
// one full wave of 256-thread blocks, eight independent chains per thread.
// Two cells per instruction is the Smith-Waterman roofline denominator.
namespace swift {
namespace {
constexpr int kCalIters = 4096;
__global__ void __launch_bounds__(256) dpx_calibration_kernel(uint32_t* out, uint32_t seed) {
  uint32_t x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = seed * (threadIdx.x + 1) + k * 0x01010101u;
  const uint32_t c = seed + 0x00010001u;
  for (int it = 0; it < kCalIters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = __vimax3_s16x2_relu(x[k], x[(k + 1) & 7], c);
  }
  uint32_t acc = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) acc ^= x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}
}  // namespace

int measure_dpx_peak(cudaStream_t st, int device, double* instr_per_s) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return SWIFT_E_CUDA;
  const int blocks = sms * 8, threads = 256;
  uint32_t* out = nullptr;
  if (cudaMallocAsync(&out, (size_t)blocks * threads * 4, st) != cudaSuccess) return SWIFT_E_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0, st);
    dpx_calibration_kernel<<<blocks, threads, 0, st>>>(out, 7u + rep);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    double ops = (double)blocks * threads * kCalIters * 8.0 / 32.0;  // warp instructions
    if (ms > 0 && rep > 0) best = ops * 32.0 / (ms * 1e-3) > best ? ops * 32.0 / (ms * 1e-3) : best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(out, st);
  cudaError_t e = cudaStreamSynchronize(st);
  *instr_per_s = best;  // lane instructions per second
  return e == cudaSuccess ? SWIFT_OK : SWIFT_E_CUDA;
}

}  // namespace swift
