// Phase-2 pair construction on the device, one warp per match record.
// Restates the per-record part of alignQueries3 (src/align.cu:693-728):
//   refDistance = max(0, refPos - 100)
//   file offset = seqOffset[refIdx] + refDistance + refDistance / basesPerLine
//                 (refMapGetOffsets, src/refMap.cu:148-155, 32-bit unsigned)
//   window      = getRefSeq2 (src/input.cu:348-403): up to 300 characters
//                 from that offset, newlines skipped, stopping at a header
//                 line or end of file, then leading / trailing N trimmed
//                 with the reference's pointer arithmetic, NUL padded
//   query       = the first Q characters of the read (getSeq2,
//                 src/input.cu:216-258); for strand 1 the reverse complement
//                 of those Q characters (qryGetReverseComplement).
// The window bytes are compacted with ballots: each step the warp reads 32
// file bytes, drops newlines and appends the rest.
#include "internal.h"

namespace swift {
namespace {

constexpr int kPairWarps = 8;

__device__ __forceinline__ bool is_acgt(char c) {
  const uint32_t u = (uint8_t)c & 0xDFu;
  return u == 'A' || u == 'C' || u == 'G' || u == 'T';
}

__device__ __forceinline__ char comp_char(char c) {
  return c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : 'A';
}

// four bytes from p (any alignment): two aligned loads and a funnel shift
// (the second load stays inside the buffer's padding past the last read)
__device__ __forceinline__ uint32_t load4(const char* p) {
  const uintptr_t ad = (uintptr_t)p;
  const uint32_t* wp = reinterpret_cast<const uint32_t*>(ad & ~(uintptr_t)3);
  return __funnelshift_r(wp[0], wp[1], (uint32_t)(ad & 3) * 8);
}

// comp_char of four upper-case A, C, G, T bytes at once: A <-> T differ in
// 0x15, C <-> G in 0x04, and bit 1 is clear exactly for A and T
__device__ __forceinline__ uint32_t comp4(uint32_t x) {
  return x ^ ((((~x) >> 1) & 0x01010101u) * 0x11u | 0x04040404u);
}

// Per read: 0 when its query (the first Q bytes, Q <= its length) is all
// upper-case A, C, G, T, so that both strands' queries are whole-word
// copies; else 1 (the per-byte path of build_pairs_kernel).
constexpr int kClsRounds = 10;  // queries up to 320 bytes

__global__ void read_class_kernel(PairArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= a.n_reads) return;
  const DevRead rd = a.rd[r];
  const int Q = a.read_q ? a.read_q[r] : a.Q;
  bool bad = rd.len < Q || Q > 32 * kClsRounds;
  const char* s = a.reads + rd.seq_off;
  if (!bad) {
    // every byte loaded before any is tested
    char c[kClsRounds];
#pragma unroll
    for (int t = 0; t < kClsRounds; ++t) c[t] = lane + 32 * t < Q ? s[lane + 32 * t] : 'A';
#pragma unroll
    for (int t = 0; t < kClsRounds; ++t)
      bad |= !(c[t] == 'A' || c[t] == 'C' || c[t] == 'G' || c[t] == 'T');
  }
  bad = __any_sync(0xffffffffu, bad);
  if (lane == 0) a.read_cls[r] = bad ? 1 : 0;
}

// getRefSeq2's walk over the file bytes: up to 300 characters from file
// offset off, newlines dropped, stopping at a header line or end of file.
// The first kPre 32-byte rounds are loaded up front so the warp waits for
// memory once, not once per round.
__device__ int fetch_window(const PairArgs& a, uint32_t off, char* tmp, int lane) {
  constexpr int kPre = 11;
  char pre[kPre];
#pragma unroll
  for (int t = 0; t < kPre; ++t) {
    const uint64_t p = (uint64_t)off + 32 * t + lane;
    pre[t] = p < a.ref_file_len ? a.ref_file[p] : '\0';
  }
  int got = 0;
  bool done = false;
  // one 32-byte round: drop newlines, stop at a header line or end of file
  auto round = [&](char c, uint64_t p) {
    const bool stop = p >= a.ref_file_len || c == '>';
    const uint32_t stop_bal = __ballot_sync(0xffffffffu, stop);
    const int first_stop = stop_bal ? __ffs(stop_bal) - 1 : 32;
    const bool keep = lane < first_stop && c != '\n';
    const uint32_t keep_bal = __ballot_sync(0xffffffffu, keep);
    const int rank = __popc(keep_bal & ((1u << lane) - 1));
    if (keep && got + rank < kWin) tmp[got + rank] = c;
    got += __popc(keep_bal);
    if (got > kWin) got = kWin;
    done = first_stop < 32 || got >= kWin;
  };
#pragma unroll
  for (int t = 0; t < kPre; ++t) {
    if (!done) round(pre[t], (uint64_t)off + 32 * t + lane);
  }
  for (uint64_t pos = (uint64_t)off + 32 * kPre; !done; pos += 32) {
    const uint64_t p = pos + (uint64_t)lane;
    round(p < a.ref_file_len ? a.ref_file[p] : '\0', p);
  }
  return got;
}

__global__ void __launch_bounds__(kPairWarps * 32) build_pairs_kernel(PairArgs a) {
  __shared__ char tmp_all[kPairWarps][kWinPad + 32];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t j = (int64_t)blockIdx.x * kPairWarps + wib;
  if (j >= a.n) return;
  char* tmp = tmp_all[wib];
  const int32_t read = a.m_read[j], strand = a.m_strand[j], ri = a.m_ri[j], rp = a.m_rp[j];
  // the read's record and class, loaded with the reference record's
  const DevRead rd = a.rd[read];
  const int Q = a.read_q ? a.read_q[read] : a.Q;  // the read's request's query length
  const bool words = a.read_cls && a.read_cls[read] == 0;
  const int32_t dist = rp - kShiftBases > 0 ? rp - kShiftBases : 0;
  const DevRecord& rec = a.recs[ri];
  int got = 0;
  char* wout = a.wbuf + j * kWinPad;
  bool odd = false;  // a byte the packed score pass does not take
  int wl = 0;
  // Common case: a whole window inside a record of regular lines with only
  // ACGTacgt bytes (no N to trim): a straight copy of the concatenated bases,
  // 16 bytes per lane.
  bool direct = false;
  static_assert(kWinPad % 16 == 0 && kWin % 4 == 0 && kWinPad - kWin == 4,
                "the last lane's fourth word is the padding");
  uint32_t w[5] = {0, 0, 0, 0, 0};
  uint32_t sh = 0;
  if (rec.regular && a.odd) {
    const uint64_t avail = rec.cat_len > (uint64_t)dist ? rec.cat_len - (uint64_t)dist : 0;
    if (avail >= (uint64_t)kWin) {
      // the window's words are loaded while the bitmap of non-ACGT
      // positions is (both in bounds of the record's concatenated bases)
      if (lane < kWinPad / 16) {
        // four output words from five aligned loads (the reads past the
        // window's end stay inside the cat buffer's padding)
        const uintptr_t ad = (uintptr_t)(a.cat + rec.cat_start + dist + 16 * lane);
        const uint32_t* wp = reinterpret_cast<const uint32_t*>(ad & ~(uintptr_t)3);
        sh = (uint32_t)(ad & 3) * 8;
#pragma unroll
        for (int q = 0; q < 5; ++q) w[q] = wp[q];
      }
      const uint64_t g0 = rec.cat_start + (uint64_t)dist, g1 = g0 + kWin - 1;
      const uint64_t w0 = g0 >> 5;
      uint32_t bits = 0;
      if ((uint64_t)lane <= (g1 >> 5) - w0) {
        bits = a.odd[w0 + lane];
        if (lane == 0) bits &= ~0u << (g0 & 31);
        if (w0 + lane == (g1 >> 5)) bits &= ~0u >> (31 - (g1 & 31));
      }
      direct = !__any_sync(0xffffffffu, bits != 0);
    }
  }
  if (direct) {
    if (lane < kWinPad / 16) {
      uint4 o;
      o.x = __funnelshift_r(w[0], w[1], sh);
      o.y = __funnelshift_r(w[1], w[2], sh);
      o.z = __funnelshift_r(w[2], w[3], sh);
      o.w = lane == kWinPad / 16 - 1 ? 0u : __funnelshift_r(w[3], w[4], sh);
      *reinterpret_cast<uint4*>(wout + 16 * lane) = o;
    }
    wl = kWin;
  } else {
    if (rec.regular) {
      // the window is concatenated positions dist .. dist + 299 of the record
      const uint64_t avail = rec.cat_len > (uint64_t)dist ? rec.cat_len - (uint64_t)dist : 0;
      got = avail < (uint64_t)kWin ? (int)avail : kWin;
      const char* src = a.cat + rec.cat_start + dist;
#pragma unroll
      for (int t = 0; t < (kWin + 31) / 32; ++t) {
        const int i = lane + 32 * t;
        if (i < got) tmp[i] = src[i];
      }
    } else {
      // the file offset refMapGetOffsets gives (only irregular records
      // read the file bytes)
      const uint32_t off = (uint32_t)rec.seq_off + (uint32_t)dist +
                           (rec.bpl > 0 ? (uint32_t)dist / rec.bpl : 0u);
      got = fetch_window(a, off, tmp, lane);
    }
    __syncwarp();
    // N trimming (see the restatement notes at the top of this file)
    int lead = 0;
    {
      bool isn = false;
      for (int base = 0; base < got; base += 32) {
        int i = base + lane;
        isn = i < got && (tmp[i] == 'N' || tmp[i] == 'n');
        uint32_t notn = __ballot_sync(0xffffffffu, !isn && i < got);
        if (notn) {
          lead = base + __ffs(notn) - 1;
          break;
        }
        lead = base + 32 < got ? base + 32 : got;
      }
    }
    int len = got;
    if (lead == 0 && got > 0) {
      for (int base = ((got - 1) / 32) * 32; base >= 0; base -= 32) {
        int i = base + lane;
        bool notn = i < got && !(tmp[i] == 'N' || tmp[i] == 'n');
        uint32_t b = __ballot_sync(0xffffffffu, notn);
        if (b) {
          len = base + 31 - __clz(b) + 1;
          break;
        }
        len = base;
      }
    }
    wl = len - lead;
    if (wl < 0) wl = 0;
    for (int i = lane; i < kWinPad; i += 32) {
      const char c = i < wl ? tmp[lead + i] : '\0';
      wout[i] = c;
      if (i < wl && !is_acgt(c)) odd = true;
    }
  }  // window not copied directly
  // query
  const char* s = a.reads + rd.seq_off;
  if (a.pair_q && lane == 0) a.pair_q[j] = Q;
  const int avail = rd.len < Q ? rd.len : Q;
  char* qout = a.qbuf + j * (int64_t)a.Qs;
  if (words) {
    // upper-case A, C, G, T only (avail = Q, not odd): whole words, the
    // reverse complement byte-reversed and complemented four at a time
    for (int i0 = 4 * lane; i0 < a.Qs; i0 += 128) {
      uint32_t word = 0;
      if (i0 + 4 <= Q) {
        word = strand == 0 ? load4(s + i0) : comp4(__byte_perm(load4(s + Q - 4 - i0), 0u, 0x0123));
      } else if (i0 < Q) {
        for (int b = 0; b < Q - i0; ++b) {
          const char c = strand == 0 ? s[i0 + b] : comp_char(s[Q - 1 - i0 - b]);
          word |= (uint32_t)(uint8_t)c << (8 * b);
        }
      }
      *reinterpret_cast<uint32_t*>(qout + i0) = word;
    }
  } else
  // four bytes per lane, one 32-bit store each (Qs is a multiple of 16)
  for (int i0 = 4 * lane; i0 < a.Qs; i0 += 128) {
    uint32_t word = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int i = i0 + b;
      if (i < Q) {
        char c;
        if (strand == 0) {
          c = i < avail ? s[i] : '\0';
        } else {
          const int src = Q - 1 - i;
          c = comp_char(src < avail ? s[src] : '\0');
        }
        if (!is_acgt(c)) odd = true;
        word |= (uint32_t)(uint8_t)c << (8 * b);
      }
    }
    *reinterpret_cast<uint32_t*>(qout + i0) = word;
  }
  odd = __any_sync(0xffffffffu, odd) || wl != kWin;
  if (lane == 0) {
    DevPair pr;
    pr.read = read;
    pr.strand = strand;
    pr.ref_idx = ri;
    pr.ref_dist = dist;
    pr.win_len = wl;
    pr.flags = odd ? 1 : 0;
    a.pairs[j] = pr;
  }
}

}  // namespace

void launch_build_pairs(cudaStream_t st, const PairArgs& a) {
  if (a.n <= 0) return;
  if (a.read_cls && a.n_reads > 0)
    read_class_kernel<<<(unsigned)((a.n_reads * 32 + 255) / 256), 256, 0, st>>>(a);
  unsigned grid = (unsigned)((a.n + kPairWarps - 1) / kPairWarps);
  build_pairs_kernel<<<grid, kPairWarps * 32, 0, st>>>(a);
}

}  // namespace swift
