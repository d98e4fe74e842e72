// Paired-end Phase 1 records and Phase 2 pairs on the device (the GPU branch
// of src/main.cu:172-212).
//
// Records (searchQueries_paired2, src/search.cu:2084-2200): per pair id, the
// hits of mate 1 forward, mate 1 reverse complement, mate 2 forward, mate 2
// reverse complement, each strand's best clusters from the SSAHA seeding
// kernel run on the lookupTable2 positions (api.cu builds them).
//
// Pairs (alignQueries_paired2, src/align.cu:1976-2043): the window is
// getSeq's (src/input.cu:163-204) 3Q bytes from the file offset of
// max(0, offset - Q) in the record (refMapGetOffsets): lines read on from
// there, newlines dropped, stopping before a line that starts with '>' or
// after 3Q bytes; no N trimming.  The query is the first Q bases of the
// mate's read line, reverse-complemented for reverse-strand records
// (qryGetReverseComplement over those Q bases).
#include "internal.h"

namespace swift {
namespace {

__global__ void pe_count_kernel(const int32_t* __restrict__ nb1, const int32_t* __restrict__ nb2,
                                int64_t n, uint64_t* __restrict__ cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) cnt[i] = (uint64_t)(nb1[2 * i] + nb1[2 * i + 1] + nb2[2 * i] + nb2[2 * i + 1]);
}

__global__ void pe_fill_kernel(PairedArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n_pairs) return;
  uint64_t o = a.roff[i];
  for (int mate = 0; mate < 2; ++mate) {
    const int32_t* nb = mate == 0 ? a.nbest1 : a.nbest2;
    const int3* best = mate == 0 ? a.best1 : a.best2;
    for (int s = 0; s < 2; ++s) {
      const int64_t sid = 2 * i + s;
      for (int h = 0; h < nb[sid]; ++h) {
        const int3 b = best[sid * a.max_hits + h];
        a.m_id[o] = (int32_t)(i + 1);
        a.m_mate[o] = mate + 1;
        a.m_rev[o] = s;
        a.m_read[o] = (int32_t)i;
        a.m_ri[o] = b.x;
        a.m_shift[o] = b.y;
        a.m_off[o] = b.z;
        ++o;
      }
    }
  }
}

__device__ __forceinline__ char revcomp_base(char c) {
  return c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : 'A';
}

// one warp per record; the window's bytes are compacted with ballots (each
// round the warp reads 32 file bytes, drops newlines, stops at a header)
constexpr int kPeWarps = 8;

__global__ void __launch_bounds__(kPeWarps * 32) pe_pairs_kernel(PairedArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t j = (int64_t)blockIdx.x * kPeWarps + (threadIdx.x >> 5);
  if (j >= a.n_rec) return;
  const int Q = a.Q, R = 3 * a.Q;
  const int mate = a.m_mate[j], rev = a.m_rev[j], read = a.m_read[j], ri = a.m_ri[j];
  int dist = a.m_off[j] - Q;
  if (dist < 0) dist = 0;
  const DevRecord& rec = a.recs[ri];
  const uint32_t woff = (uint32_t)rec.seq_off + (uint32_t)dist +
                        (rec.bpl > 0 ? (uint32_t)dist / rec.bpl : 0u);
  // getSeq over the reference file bytes ('>' only starts header lines)
  char* w = a.wbuf + j * a.w_stride;
  bool odd = false;  // a byte outside ACGT or a short window: the generic kernel
  int got = 0;
  // Common case: the window inside a record of regular lines with only
  // ACGTacgt bytes (the bitmap): getSeq's bytes are the concatenated bases,
  // copied 16 per lane; a lowercase base (bit 0x20 of a letter) is odd here.
  bool direct = false;
  if (rec.regular && a.odd && a.w_stride % 16 == 0) {
    const uint64_t avail = rec.cat_len > (uint64_t)dist ? rec.cat_len - (uint64_t)dist : 0;
    if (avail >= (uint64_t)R) {
      const uint64_t g0 = rec.cat_start + (uint64_t)dist, g1 = g0 + R - 1;
      const uint64_t w0 = g0 >> 5, nw = (g1 >> 5) - w0 + 1;  // at most 20 words (R <= 597)
      uint32_t bits = 0;
      if ((uint64_t)lane < nw) {
        bits = a.odd[w0 + lane];
        if (lane == 0) bits &= ~0u << (g0 & 31);
        if ((uint64_t)lane == nw - 1) bits &= ~0u >> (31 - (g1 & 31));
      }
      direct = !__any_sync(0xffffffffu, bits != 0);
    }
  }
  if (direct) {
    for (int c = lane; 16 * c < R; c += 32) {
      // four output words from five aligned loads (reads past the window's
      // end stay inside the cat buffer's padding); bytes past R are zero
      const uintptr_t ad = (uintptr_t)(a.cat + rec.cat_start + dist + 16 * c);
      const uint32_t* wp = reinterpret_cast<const uint32_t*>(ad & ~(uintptr_t)3);
      const uint32_t sh = (uint32_t)(ad & 3) * 8;
      uint32_t x[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int keep = R - 16 * c - 4 * q;  // valid bytes of this word
        const uint32_t v = __funnelshift_r(wp[q], wp[q + 1], sh);
        x[q] = keep >= 4 ? v : keep <= 0 ? 0u : v & ((1u << (8 * keep)) - 1u);
      }
      odd |= ((x[0] | x[1] | x[2] | x[3]) & 0x20202020u) != 0;
      *reinterpret_cast<uint4*>(w + 16 * c) = make_uint4(x[0], x[1], x[2], x[3]);
    }
    got = R;
  }
  for (uint64_t pos = woff; !direct; pos += 32) {
    const uint64_t p = pos + (uint64_t)lane;
    const char c = p < a.ref_file_len ? a.ref_file[p] : '\0';
    const bool stop = p >= a.ref_file_len || c == '>';
    const uint32_t sb = __ballot_sync(0xffffffffu, stop);
    const int first_stop = sb ? __ffs(sb) - 1 : 32;
    const bool keep = lane < first_stop && c != '\n';
    const uint32_t kb = __ballot_sync(0xffffffffu, keep);
    const int at = got + __popc(kb & ((1u << lane) - 1));
    if (keep && at < R) {
      w[at] = c;
      odd |= !(c == 'A' || c == 'C' || c == 'G' || c == 'T');
    }
    got += __popc(kb);
    if (first_stop < 32 || got >= R) break;
  }
  if (got > R) got = R;
  // query: the mate's read, first Q bases
  const int64_t cr = mate == 1 ? (int64_t)read : a.n_pairs + read;
  const DevRead rr = a.rd[cr];
  const char* s = a.reads + rr.seq_off;
  char* q = a.qbuf + j * a.q_stride;
  // four bytes per lane, one 32-bit store each (q_stride is a multiple of 16)
  for (int t0 = 4 * lane; t0 < a.q_stride; t0 += 128) {
    uint32_t word = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int t = t0 + b;
      if (t < Q) {
        const char c = rev ? revcomp_base(s[Q - 1 - t]) : s[t];
        odd |= !(c == 'A' || c == 'C' || c == 'G' || c == 'T');
        word |= (uint32_t)(uint8_t)c << (8 * b);
      }
    }
    *reinterpret_cast<uint32_t*>(q + t0) = word;
  }
  odd = __any_sync(0xffffffffu, odd);
  if (lane == 0) {
    DevPair p;
    p.read = (int32_t)cr;
    p.strand = rev;
    p.ref_idx = ri;
    p.ref_dist = dist;
    p.win_len = got;
    p.flags = (odd || got != R) ? 1 : 0;
    a.pairs[j] = p;
  }
}

__global__ void aln_from_arrays_kernel(const float* __restrict__ score,
                                       const int32_t* __restrict__ start,
                                       const int32_t* __restrict__ end,
                                       const int32_t* __restrict__ len, int64_t n,
                                       DevAln* __restrict__ aln) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  DevAln d;
  d.score = (int32_t)score[i];
  d.start = start[i];
  d.end = end[i];
  d.len = len[i];
  aln[i] = d;
}

// the second reads file's records after the first's: offsets shifted by the
// first buffer's length
__global__ void shift_reads_kernel(const DevRead* __restrict__ in, int64_t n, uint64_t by,
                                   DevRead* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  DevRead r = in[i];
  r.name_off += by;
  r.seq_off += by;
  out[i] = r;
}


// ---- mate pairing (chooseBestAlignment_paired3, src/align.cu:1248-1422) ----
// Names end in 1 or 2 (checked on the host), so qryNameCmp is equality of
// the read names ("core", the trailing '*' of reverse records aside) and the
// mate name is the core with its last character swapped.  Within a batch the
// reference walks runs of records with one core: a run whose next run has
// the mate core is paired with it and the walk resumes after both; otherwise
// the run is dropped and the walk resumes at the next run.  Whether run r
// starts a step follows from the last run h < r whose next run is not its
// mate: steps start at h + 1, h + 3, ...

__device__ __forceinline__ bool core_equal(const PairSelArgs& a, int64_t x, int64_t y) {
  const DevRead rx = a.rd[a.pairs[x].read], ry = a.rd[a.pairs[y].read];
  if (rx.name_len != ry.name_len) return false;
  const char* px = a.reads + rx.name_off + 1;
  const char* py = a.reads + ry.name_off + 1;
  for (int i = 0; i < rx.name_len; ++i)
    if (px[i] != py[i]) return false;
  return true;
}

// is the core of record y the mate name of record x's core?
__device__ __forceinline__ bool core_is_mate(const PairSelArgs& a, int64_t x, int64_t y) {
  const DevRead rx = a.rd[a.pairs[x].read], ry = a.rd[a.pairs[y].read];
  if (rx.name_len != ry.name_len || rx.name_len < 1) return false;
  const char* px = a.reads + rx.name_off + 1;
  const char* py = a.reads + ry.name_off + 1;
  const int L = rx.name_len;
  for (int i = 0; i < L - 1; ++i)
    if (px[i] != py[i]) return false;
  return py[L - 1] == (px[L - 1] == '1' ? '2' : '1');
}

// per record: 1 where a run of one core starts (batch starts included)
__global__ void pe_run_start_kernel(PairSelArgs a, uint32_t* flag) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.n) return;
  flag[j] = (a.batch_start[j] || !core_equal(a, j, j - 1)) ? 1u : 0u;
}

// per run: its first record, from the run index of each record
__global__ void pe_run_first_kernel(PairSelArgs a, const uint32_t* flag, const uint32_t* run_of,
                                    int64_t* first) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.n) return;
  if (flag[j]) first[run_of[j]] = j;
}

__device__ __forceinline__ bool opposite(const PairSelArgs& a, int64_t i, int64_t j) {
  const int ri = a.pairs[i].strand, rj = a.pairs[j].strand;
  return (ri == 0 && rj == 1) || (rj == 0 && ri == 1);
}

__device__ __forceinline__ bool frag_ok(const PairSelArgs& a, int64_t i, int64_t j) {
  const DevPair pi = a.pairs[i], pj = a.pairs[j];
  if (a.ref_class[pi.ref_idx] != a.ref_class[pj.ref_idx]) return true;  // other reference names
  const DevAln ai = a.aln[i], aj = a.aln[j];
  int d;
  if (pi.strand == 0 && pj.strand == 1)
    d = (pj.ref_dist + aj.end) - (pi.ref_dist + ai.start);
  else
    d = (pi.ref_dist + ai.end) - (pj.ref_dist + aj.start);
  return (uint32_t)d >= a.min_frag && (uint32_t)d <= a.max_frag;
}

// per run: the pairing step it starts, if it starts one
__global__ void pe_pair_runs_kernel(PairSelArgs a, const int64_t* first, int64_t n_runs) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_runs) return;
  // m(h): run h's next run lies in its batch and carries its mate core
  auto run_end = [&](int64_t h) { return h + 1 < n_runs ? first[h + 1] : a.n; };
  auto mates = [&](int64_t h) {
    if (h + 1 >= n_runs) return false;
    const int64_t nx = first[h + 1];
    if (a.batch_start[nx]) return false;
    return core_is_mate(a, first[h], nx);
  };
  int64_t h = r - 1;
  while (h >= 0 && !a.batch_start[first[h + 1]] && mates(h)) --h;
  // runs h + 1 .. r - 1 all pair with their next run: steps alternate
  if (((r - h - 1) & 1) != 0) return;  // run r is the mate run of r - 1
  const int64_t s1 = first[r], e1 = run_end(r);
  if (!mates(r)) {
    for (int64_t i = s1; i < e1; ++i) a.keep[i] = 0;
    return;
  }
  const int64_t s2 = e1, e2 = run_end(r + 1);
  int best = 0;
  for (int64_t i = s1; i < e1; ++i)
    for (int64_t j = s2; j < e2; ++j) {
      if (!opposite(a, i, j)) continue;
      const int sum = a.aln[i].score + a.aln[j].score;
      if (best < sum && frag_ok(a, i, j)) best = sum;
    }
  int64_t f1 = -1, f2 = -1;
  for (int64_t i = s1; i < e1 && f1 < 0; ++i)
    for (int64_t j = s2; j < e2; ++j)
      if (opposite(a, i, j) && a.aln[i].score + a.aln[j].score == best && frag_ok(a, i, j)) {
        f1 = i;
        f2 = j;
        break;
      }
  for (int64_t i = s1; i < e1; ++i) a.keep[i] = i == f1 ? 1 : 0;
  for (int64_t j = s2; j < e2; ++j) a.keep[j] = j == f2 ? 1 : 0;
}

// printOutput_paired2's separator: a kept record opens with the line of '*'
// unless a kept record of the same pair id precedes it in the batch (ids are
// non-decreasing)
__global__ void pe_sep_kernel(PairSelArgs a) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.n) return;
  int8_t sep = 0;
  if (a.keep[j]) {
    sep = 1;
    if (!a.batch_start[j]) {
      for (int64_t i = j - 1; i >= 0 && a.id[i] == a.id[j]; --i) {
        if (a.keep[i]) {
          sep = 0;
          break;
        }
        if (a.batch_start[i]) break;
      }
    }
  }
  a.sep[j] = sep;
}

// getMatePairName reads the name's last character: 1 or 2 on both files
__global__ void pe_names_kernel(const char* __restrict__ b1, const DevRead* __restrict__ rd1,
                                const char* __restrict__ b2, const DevRead* __restrict__ rd2,
                                int64_t n, int32_t* bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int f = 0; f < 2; ++f) {
    const DevRead r = f == 0 ? rd1[i] : rd2[i];
    const char last = r.name_len > 0 ? (f == 0 ? b1 : b2)[r.name_off + r.name_len] : 0;
    if (last != '1' && last != '2') *bad = 1;
  }
}
}  // namespace

void launch_pe_names(cudaStream_t st, const char* b1, const DevRead* rd1, const char* b2,
                     const DevRead* rd2, int64_t n, int32_t* bad) {
  if (n <= 0) return;
  pe_names_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(b1, rd1, b2, rd2, n, bad);
}

void launch_pe_records(cudaStream_t st, const PairedArgs& a, uint64_t* cnt) {
  if (a.n_pairs <= 0) return;
  pe_count_kernel<<<(unsigned)((a.n_pairs + 255) / 256), 256, 0, st>>>(a.nbest1, a.nbest2,
                                                                       a.n_pairs, cnt);
}

void launch_pe_fill(cudaStream_t st, const PairedArgs& a) {
  if (a.n_pairs <= 0) return;
  pe_fill_kernel<<<(unsigned)((a.n_pairs + 255) / 256), 256, 0, st>>>(a);
}

void launch_pe_pairs(cudaStream_t st, const PairedArgs& a) {
  if (a.n_rec <= 0) return;
  pe_pairs_kernel<<<(unsigned)((a.n_rec + kPeWarps - 1) / kPeWarps), kPeWarps * 32, 0, st>>>(a);
}

void launch_aln_from_arrays(cudaStream_t st, const float* score, const int32_t* start,
                            const int32_t* end, const int32_t* len, int64_t n, DevAln* aln) {
  if (n <= 0) return;
  aln_from_arrays_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(score, start, end, len, n,
                                                                       aln);
}

void launch_pe_runs(cudaStream_t st, const PairSelArgs& a, uint32_t* flag) {
  if (a.n <= 0) return;
  pe_run_start_kernel<<<(unsigned)((a.n + 255) / 256), 256, 0, st>>>(a, flag);
}

void launch_pe_run_first(cudaStream_t st, const PairSelArgs& a, const uint32_t* flag,
                         const uint32_t* run_of, int64_t* first) {
  if (a.n <= 0) return;
  pe_run_first_kernel<<<(unsigned)((a.n + 255) / 256), 256, 0, st>>>(a, flag, run_of, first);
}

void launch_pe_pair_runs(cudaStream_t st, const PairSelArgs& a, const int64_t* first,
                         int64_t n_runs) {
  if (n_runs <= 0) return;
  pe_pair_runs_kernel<<<(unsigned)((n_runs + 127) / 128), 128, 0, st>>>(a, first, n_runs);
}

void launch_pe_sep(cudaStream_t st, const PairSelArgs& a) {
  if (a.n <= 0) return;
  pe_sep_kernel<<<(unsigned)((a.n + 255) / 256), 256, 0, st>>>(a);
}

void launch_shift_reads(cudaStream_t st, const DevRead* in, int64_t n, uint64_t by,
                        DevRead* out) {
  if (n <= 0) return;
  shift_reads_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, n, by, out);
}

}  // namespace swift
