// Reads FASTA parsed on the device: the bytes are copied once and the
// record structure is found with a scan, so the host never walks the text.
// Rules are those of qryGetNext2 (src/query.cu:174-213), getSeqCount and
// getSeqSize (src/input.cu:475-524) for the inputs the reference reads
// correctly (one header line, then exactly one sequence line, per read);
// anything else is reported as an error rather than reproduced (the
// reference loops forever on an empty line and overflows its buffers on
// long names or reads).
//   pass 1: per 64-byte tile, newline count and byte checks (NUL, >= 128,
//           '>' not at a line start)
//   scan:   tile newline counts -> newline positions
//   pass 2: per line, header/sequence alternation, lengths, and the
//           per-read record (name offset, sequence offset, lengths)
#include "internal.h"

namespace swift {
namespace {

constexpr int kTile = 64;

__device__ __forceinline__ void report(unsigned long long* err, uint64_t off, uint32_t code) {
  atomicMin(err, (unsigned long long)((off << 8) | code));
}

// bit 7 of each byte of x that is zero (exact: no carry crosses bytes)
__device__ __forceinline__ uint32_t zero_bytes(uint32_t x) {
  return ~(((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x) & 0x80808080u;
}

// a whole tile as four 16-byte loads (b 16-byte aligned)
__device__ __forceinline__ void load_tile(const uint8_t* __restrict__ b, uint64_t lo, uint32_t w[16]) {
  const uint4* p = reinterpret_cast<const uint4*>(b + lo);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint4 v = __ldg(p + q);
    w[4 * q] = v.x;
    w[4 * q + 1] = v.y;
    w[4 * q + 2] = v.z;
    w[4 * q + 3] = v.w;
  }
}

__global__ void tile_scan_bytes(const uint8_t* __restrict__ b, uint64_t n, uint32_t* __restrict__ cnt,
                                unsigned long long* err) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t lo = t * kTile;
  if (lo >= n) return;
  const uint64_t hi = lo + kTile < n ? lo + kTile : n;
  uint32_t c = 0;
  uint8_t prev = lo == 0 ? '\n' : b[lo - 1];
  if (hi - lo == kTile && ((uintptr_t)b & 15) == 0) {
    // four bytes per word: newlines counted, and any NUL, byte >= 128 or
    // '>' not after a newline sends the tile to the byte loop below, which
    // reports the first offending offset
    uint32_t w[16];
    load_tile(b, lo, w);
    uint32_t prev_nl = prev == '\n' ? 0x80u : 0u, bad = 0;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const uint32_t x = w[k];
      const uint32_t nlm = zero_bytes(x ^ 0x0A0A0A0Au);
      c += __popc(nlm);
      bad |= (x & 0x80808080u) | zero_bytes(x) | (zero_bytes(x ^ 0x3E3E3E3Eu) & ~((nlm << 8) | prev_nl));
      prev_nl = nlm >> 24;
    }
    if (!bad) {
      cnt[t] = c;
      return;
    }
    c = 0;
  }
  for (uint64_t i = lo; i < hi; ++i) {
    const uint8_t x = b[i];
    if (x == '\n') ++c;
    if (x == 0 || x >= 128) report(err, i, kParseBadByte);
    if (x == '>' && prev != '\n') report(err, i, kParseGtInLine);
    prev = x;
  }
  cnt[t] = c;
}

__global__ void tile_newlines(const uint8_t* __restrict__ b, uint64_t n,
                              const uint32_t* __restrict__ off, uint64_t* __restrict__ nl) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t lo = t * kTile;
  if (lo >= n) return;
  const uint64_t hi = lo + kTile < n ? lo + kTile : n;
  uint32_t o = off[t];
  if (hi - lo == kTile && ((uintptr_t)b & 15) == 0) {
    uint32_t w[16];
    load_tile(b, lo, w);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      for (uint32_t nlm = zero_bytes(w[k] ^ 0x0A0A0A0Au); nlm; nlm &= nlm - 1)
        nl[o++] = lo + 4 * k + ((__ffs(nlm) - 1) >> 3);
    }
    return;
  }
  for (uint64_t i = lo; i < hi; ++i)
    if (b[i] == '\n') nl[o++] = i;
}

__global__ void lines_to_reads(const uint8_t* __restrict__ b, uint64_t n,
                               const uint64_t* __restrict__ nl, uint64_t n_nl, uint64_t n_lines,
                               DevRead* __restrict__ rd, ParseSummary* sum,
                               unsigned long long* err, int max_read) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  // the read length of this line, if it is a well-formed sequence line;
  // reduced over the warp before the atomics (one address for all reads)
  int32_t mn = INT32_MAX, mx = INT32_MIN;
  auto line = [&]() {
    const uint64_t start = i == 0 ? 0 : nl[i - 1] + 1;
    const uint64_t end = i < n_nl ? nl[i] : n;
    const uint64_t len = end - start;
    if (len == 0) {
      report(err, start, kParseEmptyLine);
      return;
    }
    const bool header = b[start] == '>';
    if ((i & 1) == 0) {
      if (!header) {
        report(err, start, i == 0 ? kParseSeqNoHeader : kParseMultiLine);
        return;
      }
      if (len - 1 > (uint64_t)(kNameMax - 2)) report(err, start, kParseNameLong);
      if (i + 1 >= n_lines) report(err, start, kParseTrailingHeader);
      return;
    }
    if (header) {  // the header before this one has no sequence line
      report(err, i == 1 ? 0 : nl[i - 2] + 1, kParseHeaderNoSeq);
      return;
    }
    if (len > (uint64_t)max_read) {
      report(err, start, kParseReadLong);
      return;
    }
    const uint64_t h0 = i == 1 ? 0 : nl[i - 2] + 1;
    const uint64_t r = i >> 1;
    DevRead d;
    d.name_off = h0;
    d.seq_off = start;
    d.len = (int32_t)len;
    d.name_len = (int32_t)(start - 1 - h0 - 1);
    rd[r] = d;
    mn = mx = (int32_t)len;
    if (r == 0) sum->first_len = (int32_t)len - (end == n ? 1 : 0);  // strlen(line) - 1
  };
  if (i < n_lines) line();
  mn = __reduce_min_sync(0xffffffffu, mn);
  mx = __reduce_max_sync(0xffffffffu, mx);
  if ((threadIdx.x & 31) == 0 && mn != INT32_MAX) {
    atomicMin(&sum->min_len, mn);
    atomicMax(&sum->max_len, mx);
  }
}

}  // namespace

unsigned parse_tiles(uint64_t n) { return (unsigned)((n + kTile - 1) / kTile); }

void launch_parse_tiles(cudaStream_t st, const char* b, uint64_t n, uint32_t* cnt,
                        unsigned long long* err) {
  const uint64_t tiles = (n + kTile - 1) / kTile;
  if (tiles == 0) return;
  tile_scan_bytes<<<(unsigned)((tiles + 255) / 256), 256, 0, st>>>((const uint8_t*)b, n, cnt, err);
}

void launch_parse_newlines(cudaStream_t st, const char* b, uint64_t n, const uint32_t* off,
                           uint64_t* nl) {
  const uint64_t tiles = (n + kTile - 1) / kTile;
  if (tiles == 0) return;
  tile_newlines<<<(unsigned)((tiles + 255) / 256), 256, 0, st>>>((const uint8_t*)b, n, off, nl);
}

void launch_parse_lines(cudaStream_t st, const char* b, uint64_t n, const uint64_t* nl,
                        uint64_t n_nl, uint64_t n_lines, DevRead* rd, ParseSummary* sum,
                        unsigned long long* err, int max_read) {
  if (n_lines == 0) return;
  lines_to_reads<<<(unsigned)((n_lines + 255) / 256), 256, 0, st>>>((const uint8_t*)b, n, nl, n_nl,
                                                                   n_lines, rd, sum, err, max_read);
}

int parse_error(uint32_t code, uint64_t off, std::string* msg, int max_read) {
  const std::string at = " at offset " + std::to_string(off);
  switch (code) {
    case kParseBadByte: *msg = "reads: byte outside 7-bit text" + at; return SWIFT_E_INPUT;
    case kParseGtInLine: *msg = "reads: '>' inside a line" + at; return SWIFT_E_INPUT;
    case kParseEmptyLine:
      *msg = "reads: empty line" + at + " (the reference reader loops forever on it)";
      return SWIFT_E_INPUT;
    case kParseSeqNoHeader: *msg = "reads: sequence line without a header" + at; return SWIFT_E_INPUT;
    case kParseMultiLine:
      *msg = "reads: second sequence line" + at + " (multi-line reads are not supported)";
      return SWIFT_E_INPUT;
    case kParseHeaderNoSeq: *msg = "reads: header without a sequence line" + at; return SWIFT_E_INPUT;
    case kParseTrailingHeader:
      *msg = "reads: trailing header without a sequence line" + at;
      return SWIFT_E_INPUT;
    case kParseNameLong: *msg = "reads: read name longer than 48 characters" + at; return SWIFT_E_LIMIT;
    case kParseReadLong:
      *msg = "reads: read longer than " + std::to_string(max_read) + " bases" +
             (max_read == kReadMax ? std::string(" (the reference's query buffer)") : std::string()) +
             at;
      return SWIFT_E_LIMIT;
    default: *msg = "reads: malformed input" + at; return SWIFT_E_INPUT;
  }
}

}  // namespace swift
