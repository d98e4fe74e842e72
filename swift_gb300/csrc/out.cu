// Best alignment per read and the default text record, on the device.
//
// Selection restates chooseBestAlignment (src/align.cu:844-905) with the
// tie pinned to the first maximum: within one Phase-2 batch, consecutive
// records whose query names compare equal under qryNameCmp
// (src/align.cu:1501-1519: equal, or equal but for one trailing '*') form a
// group; the group keeps its first record with the maximum score (maximum
// starting from 0.0 with strict comparison) and drops the others.
//
// Formatting restates printOutput (src/output.cu:154-201), or for SAM output
// printOutputSam (src/output.cu:98-130, below):
//   "\n****************************************\n"
//   "Qry: %s | Ref: %s | Score: %.1f | AlignStart: %d | AlignEnd: %d | "
//   "AlignLength: %d\n"
//   "R: " reversed ref consensus "\n"
//   "   " match line ('|' equal ignoring case or an 'N', '-' gap, '.') "\n"
//   "Q: " reversed query consensus "\n"
// Scores are integers, so "%.1f" prints them with ".0".  A size pass and an
// exclusive scan give every record its output offset; a warp per record then
// writes its text.
#include "internal.h"

namespace swift {
namespace {


// Query name of record j: the read's header text, plus '*' for strand 1.
__device__ __forceinline__ int qname_len(const FormatArgs& a, const DevPair& p) {
  return a.rd[p.read].name_len + (p.strand ? 1 : 0);
}
__device__ __forceinline__ char qname_at(const FormatArgs& a, const DevPair& p, int i) {
  const DevRead& r = a.rd[p.read];
  if (i < r.name_len) return a.reads[r.name_off + 1 + i];
  if (p.strand && i == r.name_len) return '*';
  return '\0';
}

__device__ bool names_equal(const FormatArgs& a, const DevPair& s, const DevPair& t) {
  // records of one read: the same name, or it and it + "*" (either strand),
  // which the comparison below finds equal whenever the name and its '*'
  // fit the slot
  if (s.read == t.read && a.rd[s.read].name_len + 1 < kNameMax) return true;
  // qryNameCmp over the 50-byte name slots
  int i;
  for (i = 0; i < kNameMax; ++i) {
    char cs = qname_at(a, s, i), ct = qname_at(a, t, i);
    if (cs == '\0' && ct == '\0') return true;
    if (cs == '\0' || ct == '\0') break;
    if (cs != ct) return false;
  }
  if (i >= kNameMax) return false;
  char s0 = qname_at(a, s, i), s1 = qname_at(a, s, i + 1);
  char t0 = qname_at(a, t, i), t1 = qname_at(a, t, i + 1);
  return (s0 == '*' && s1 == '\0') || (t0 == '*' && t1 == '\0');
}

// Record j opens a Phase-2 batch: every a.batch records, or where the wave's
// per-request flags say so.
__device__ __forceinline__ bool opens_batch(const FormatArgs& a, int64_t j) {
  return a.batch_start ? a.batch_start[j] != 0 : j % a.batch == 0;
}
// last record of the best-per-read group that starts at j
__device__ __forceinline__ int64_t group_end(const FormatArgs& a, int64_t j) {
  int64_t e = j;
  while (e + 1 < a.n && !opens_batch(a, e + 1) && names_equal(a, a.pairs[e + 1], a.pairs[e])) ++e;
  return e;
}

__global__ void select_kernel(FormatArgs a) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.n) return;
  if (!opens_batch(a, j) && names_equal(a, a.pairs[j], a.pairs[j - 1])) return;  // not a group start
  const int64_t e = group_end(a, j);
  int mx = 0;
  for (int64_t i = j; i <= e; ++i) mx = max(mx, a.aln[i].score);
  int64_t keep = -1;
  for (int64_t i = j; i <= e; ++i)
    if (a.aln[i].score == mx) {
      keep = i;
      break;
    }
  for (int64_t i = j; i <= e; ++i) a.keep[i] = i == keep ? 1 : 0;
}

// Bounded selection, step 1: per best-per-read group (the groups of
// select_kernel) the candidate is the first pair with the largest key, the
// exact score for pairs of the generic kernel and the upper bound for the
// others.  Every pair learns its group's candidate; packed-path candidates
// are listed for the trace pass.
__global__ void candidate_kernel(FormatArgs a, int32_t* list, int32_t* cnt) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool app = false;
  int32_t cand = 0;
  if (j < a.n) {
    if (opens_batch(a, j) || !names_equal(a, a.pairs[j], a.pairs[j - 1])) {
      const int64_t e = group_end(a, j);
      int64_t best = j;
      int bk = -1;
      for (int64_t i = j; i <= e; ++i) {
        const int k = (a.pairs[i].flags & 1) ? a.aln[i].score : a.ub[i];
        if (k > bk) {
          bk = k;
          best = i;
        }
      }
      for (int64_t i = j; i <= e; ++i) a.cand[i] = (int32_t)best;
      cand = (int32_t)best;
      app = !(a.pairs[best].flags & 1);
    }
  }
  block_append(app, cand, list, cnt);
}

// Bounded selection, step 2 (after the candidates' exact scores): a
// packed-path pair other than the candidate can still be its group's first
// maximum only if its bound exceeds the candidate's score, or equals it and
// the pair comes first.  Those are listed for the exact score pass; the rest
// get score -1, below any score, so select_kernel never keeps them.
__global__ void prune_kernel(FormatArgs a, DevAln* aln, int32_t* list, int32_t* cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool app = false;
  if (i < a.n && !(a.pairs[i].flags & 1)) {
    const int32_t c = a.cand[i];
    if (c != (int32_t)i) {
      const int S = aln[c].score, u = a.ub[i];
      if (u > S || (u == S && i < c)) {
        app = true;
      } else {
        aln[i].score = -1;
      }
    }
  }
  block_append(app, (int32_t)i, list, cnt);
}

__device__ __forceinline__ int ndigits(int v) {
  unsigned u = v < 0 ? (unsigned)(-(int64_t)v) : (unsigned)v;
  int n = 1;
  while (u >= 10) {
    u /= 10;
    ++n;
  }
  return n + (v < 0 ? 1 : 0);
}

__device__ __forceinline__ char* put_int(char* o, int v) {
  char buf[12];
  int n = 0;
  unsigned u = v < 0 ? (unsigned)(-(int64_t)v) : (unsigned)v;
  do {
    buf[n++] = (char)('0' + u % 10);
    u /= 10;
  } while (u);
  if (v < 0) *o++ = '-';
  while (n) *o++ = buf[--n];
  return o;
}

__device__ __forceinline__ char* put_str(char* o, const char* s) {
  while (*s) *o++ = *s++;
  return o;
}

constexpr int kLitQry = 5;            // "Qry: "
constexpr int kLitRef = 8;            // " | Ref: "
constexpr int kLitScore = 10;         // " | Score: "
constexpr int kLitStart = 15;         // " | AlignStart: "
constexpr int kLitEnd = 13;           // " | AlignEnd: "
constexpr int kLitLen = 16;           // " | AlignLength: "

__device__ uint64_t record_bytes(const FormatArgs& a, int64_t j) {
  const DevPair p = a.pairs[j];
  const DevAln al = a.aln[j];
  const int dist = p.ref_dist;
  uint64_t n = a.pe_sep ? (a.pe_sep[j] ? 39 : 1) : 42;
  n += kLitQry + qname_len(a, p) + kLitRef + a.recs[p.ref_idx].name_len;
  n += kLitScore + ndigits(al.score) + 2;
  n += kLitStart + ndigits(al.start + dist) + kLitEnd + ndigits(al.end + dist);
  n += kLitLen + ndigits(al.len) + 1;
  const uint64_t L = al.len > 0 ? (uint64_t)al.len : 0;
  n += 3 * (3 + L + 1);
  return n;
}

__global__ void format_sizes_kernel(FormatArgs a) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.n) return;
  a.bytes[j] = a.keep[j] ? record_bytes(a, j) : 0;
}

constexpr int kFmtWarps = 8;
constexpr int kFmtPerWarp = 4;  // records a warp looks at (about one in four is printed)

// The literal pieces of a header line, one after another:
//   "Qry: " | " | Ref: " | " | Score: " | ".0 | AlignStart: " | " | AlignEnd: "
//   | " | AlignLength: " | "\nR: "
__device__ const char kHdrLit[] =
    "Qry:  | Ref:  | Score: .0 | AlignStart:  | AlignEnd:  | AlignLength: \nR: ";
__device__ __forceinline__ void lit_piece(char* o, int src, int n, int lane) {
  if (lane < n) o[lane] = kHdrLit[src + lane];
}

// v's decimal digits (and sign) to o, ndigits(v) bytes
__device__ __forceinline__ void put_int_at(char* o, int v, int nd) {
  unsigned u = v < 0 ? (unsigned)(-(int64_t)v) : (unsigned)v;
  if (v < 0) *o = '-';
  for (int i = nd - 1; i >= (v < 0 ? 1 : 0); --i) {
    o[i] = (char)('0' + u % 10);
    u /= 10;
  }
}

// One warp per kFmtPerWarp consecutive records; a printed record's header
// is written by the lanes in parallel straight into the text: every piece
// (separator, literals, the two names, the four numbers, one lane each) at
// an offset all lanes compute from the piece lengths.
__global__ void __launch_bounds__(kFmtWarps * 32) format_write_kernel(FormatArgs a) {
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t j0 = a.first + ((int64_t)blockIdx.x * kFmtWarps + wib) * kFmtPerWarp;
  const int64_t jt = j0 + lane;
  uint32_t todo = __ballot_sync(0xffffffffu, lane < kFmtPerWarp && jt < a.n && a.keep[jt]);
  while (todo) {
    const int64_t j = j0 + __ffs(todo) - 1;
    todo &= todo - 1;
    const DevPair p = a.pairs[j];
    const DevAln al = a.aln[j];
    const DevRead rd = a.rd[p.read];
    const DevRecord& rec = a.recs[p.ref_idx];
    const int sepn = !a.pe_sep ? 42 : a.pe_sep[j] ? 39 : 1;
    const int ql = rd.name_len + (p.strand ? 1 : 0);
    const int rl = (int)rec.name_len;
    const int v0 = al.score, v1 = al.start + p.ref_dist, v2 = al.end + p.ref_dist, v3 = al.len;
    const int n0 = ndigits(v0), n1 = ndigits(v1), n2 = ndigits(v2), n3 = ndigits(v3);
    char* o = a.text + a.offs[j];
    // separator line
    for (int i = lane; i < sepn; i += 32) o[i] = (i == 0 || i == sepn - 1) ? '\n' : '*';
    char* q = o + sepn;
    lit_piece(q, 0, 5, lane);  // "Qry: "
    q += 5;
    for (int i = lane; i < ql; i += 32) q[i] = i < rd.name_len ? a.reads[rd.name_off + 1 + i] : '*';
    q += ql;
    lit_piece(q, 5, 8, lane);  // " | Ref: "
    q += 8;
    for (int i = lane; i < rl; i += 32) q[i] = rec.name[i];
    q += rl;
    lit_piece(q, 13, 10, lane);  // " | Score: "
    char* d0 = q + 10;
    q = d0 + n0;
    lit_piece(q, 23, 17, lane);  // ".0 | AlignStart: "
    char* d1 = q + 17;
    q = d1 + n1;
    lit_piece(q, 40, 13, lane);  // " | AlignEnd: "
    char* d2 = q + 13;
    q = d2 + n2;
    lit_piece(q, 53, 16, lane);  // " | AlignLength: "
    char* d3 = q + 16;
    q = d3 + n3;
    lit_piece(q, 69, 4, lane);  // "\nR: "
    if (lane < 4) {
      const int v = lane == 0 ? v0 : lane == 1 ? v1 : lane == 2 ? v2 : v3;
      const int nd = lane == 0 ? n0 : lane == 1 ? n1 : lane == 2 ? n2 : n3;
      char* d = lane == 0 ? d0 : lane == 1 ? d1 : lane == 2 ? d2 : d3;
      put_int_at(d, v, nd);
    }
    char* out = q + 4;
    const int L = al.len > 0 ? al.len : 0;
    const char* rc = a.rcons + j * a.cons_stride;
    const char* qc = a.qcons + j * a.cons_stride;
    // "R: " already written; reversed strings
    for (int z = lane; z < L; z += 32) {
      const char r = rc[L - 1 - z], qq = qc[L - 1 - z];
      out[z] = r;
      const int ur = (unsigned)(r - 'a') < 26u ? r - 32 : r;
      const int uq = (unsigned)(qq - 'a') < 26u ? qq - 32 : qq;
      const char m = (ur == uq || r == 'N' || qq == 'N') ? '|' : (r == '-' || qq == '-') ? '-' : '.';
      out[L + 4 + z] = m;
      out[2 * L + 8 + z] = qq;
    }
    if (lane < 9) {
      // "\n   " after R, "\nQ: " after the match line, "\n" at the end
      const int at = lane < 4 ? L + lane : lane < 8 ? 2 * L + lane : 3 * L + 8;
      out[at] = lane == 0 || lane == 4 || lane == 8 ? '\n' : lane < 4 ? ' ' : lane == 5 ? 'Q' : lane == 6 ? ':' : ' ';
    }
  }
}

// SAM records (printOutputSam, src/output.cu:98-130): every record of the
// batch, no best selection, one line each:
//   qname "\t*\t" rname "\t" alignStart "\t255\t" CIGAR "\t*\t0\t0\t"
//   reversed query consensus "\t*\n"
// alignStart is the window coordinate (no reference distance added).  The
// CIGAR (printCigar, src/output.cu:33-81) walks the consensus from its last
// byte to its first: '-' in the reference consensus is D, else '-' in the
// query consensus is I, else M; each run prints as its length and letter.
__device__ __forceinline__ char cigar_op(char r, char q) {
  return r == '-' ? 'D' : q == '-' ? 'I' : 'M';
}

__device__ int cigar_bytes(const char* rc, const char* qc, int L) {
  int n = 0, run = 0;
  char op = ' ';
  for (int z = L - 1; z >= 0; --z) {
    const char c = cigar_op(rc[z], qc[z]);
    if (run > 0 && c != op) {
      n += ndigits(run) + 1;
      run = 0;
    }
    op = c;
    ++run;
  }
  if (run > 0) n += ndigits(run) + 1;
  return n;
}

__global__ void sam_sizes_kernel(FormatArgs a) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.n) return;
  const DevPair p = a.pairs[j];
  const DevAln al = a.aln[j];
  const int L = al.len > 0 ? al.len : 0;
  uint64_t n = qname_len(a, p) + 3 + a.recs[p.ref_idx].name_len + 1 + ndigits(al.start) + 5;
  n += cigar_bytes(a.rcons + j * a.cons_stride, a.qcons + j * a.cons_stride, L);
  n += 7 + L + 3;
  a.bytes[j] = n;
}

// header + CIGAR: names (<= 50 bytes each), 11 digits, 9 literal bytes, and
// at most 2 bytes of CIGAR per consensus byte (<= Q + R <= 199 + 597 of them
// for paired-end windows of 3Q)
constexpr int kSamHead = 1792;

// consensus bytes of one record, and the run starts of its CIGAR operations
constexpr int kSamMaxL = 800;

__global__ void __launch_bounds__(kFmtWarps * 32) sam_write_kernel(FormatArgs a) {
  __shared__ char head_all[kFmtWarps][kSamHead];
  __shared__ char ops_all[kFmtWarps][kSamMaxL];
  __shared__ uint32_t starts_all[kFmtWarps][kSamMaxL / 32];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t j = a.first + (int64_t)blockIdx.x * kFmtWarps + wib;
  if (j >= a.n) return;
  const DevPair p = a.pairs[j];
  const DevAln al = a.aln[j];
  const int L = al.len > 0 ? al.len : 0;
  const char* rc = a.rcons + j * a.cons_stride;
  const char* qc = a.qcons + j * a.cons_stride;
  char* head = head_all[wib];
  char* ops = ops_all[wib];
  uint32_t* starts = starts_all[wib];
  // the operations in printing order (last consensus byte first), and a bit
  // per position that starts a run
  for (int t = lane; t < L; t += 32) ops[t] = cigar_op(rc[L - 1 - t], qc[L - 1 - t]);
  __syncwarp();
  for (int c0 = 0; c0 < L; c0 += 32) {
    const int t = c0 + lane;
    const bool st = t < L && (t == 0 || ops[t] != ops[t - 1]);
    const uint32_t m = __ballot_sync(0xffffffffu, st);
    if (lane == 0) starts[c0 >> 5] = m;
  }
  __syncwarp();
  int hn = 0;
  if (lane == 0) {
    char* o = head;
    const int ql = qname_len(a, p);
    for (int i = 0; i < ql; ++i) *o++ = qname_at(a, p, i);
    o = put_str(o, "\t*\t");
    const DevRecord& rec = a.recs[p.ref_idx];
    for (uint32_t i = 0; i < rec.name_len; ++i) *o++ = rec.name[i];
    *o++ = '\t';
    o = put_int(o, al.start);
    o = put_str(o, "\t255\t");
    int prev = -1;
    for (int c = 0; c < (L + 31) / 32; ++c) {
      uint32_t m = starts[c];
      while (m) {
        const int t = 32 * c + __ffs(m) - 1;
        m &= m - 1;
        if (prev >= 0) {
          o = put_int(o, t - prev);
          *o++ = ops[prev];
        }
        prev = t;
      }
    }
    if (prev >= 0) {
      o = put_int(o, L - prev);
      *o++ = ops[prev];
    }
    o = put_str(o, "\t*\t0\t0\t");
    hn = (int)(o - head);
  }
  hn = __shfl_sync(0xffffffffu, hn, 0);
  __syncwarp();
  char* out = a.text + a.offs[j];
  for (int i = lane; i < hn; i += 32) out[i] = head[i];
  out += hn;
  for (int z = lane; z < L; z += 32) out[z] = qc[L - 1 - z];
  if (lane == 0) {
    out[L] = '\t';
    out[L + 1] = '*';
    out[L + 2] = '\n';
  }
}

}  // namespace

void launch_sam_sizes(cudaStream_t st, const FormatArgs& a) {
  if (a.n <= 0) return;
  sam_sizes_kernel<<<(unsigned)((a.n + 255) / 256), 256, 0, st>>>(a);
}

void launch_sam_write(cudaStream_t st, const FormatArgs& a) {
  const int64_t n = a.n - a.first;
  if (n <= 0) return;
  sam_write_kernel<<<(unsigned)((n + kFmtWarps - 1) / kFmtWarps), kFmtWarps * 32, 0, st>>>(a);
}

void launch_select(cudaStream_t st, const FormatArgs& a) {
  if (a.n <= 0) return;
  select_kernel<<<(unsigned)((a.n + 255) / 256), 256, 0, st>>>(a);
}

void launch_candidates(cudaStream_t st, const FormatArgs& a, int32_t* list, int32_t* cnt) {
  if (a.n <= 0) return;
  candidate_kernel<<<(unsigned)((a.n + 255) / 256), 256, 0, st>>>(a, list, cnt);
}

void launch_prune(cudaStream_t st, const FormatArgs& a, DevAln* aln, int32_t* list, int32_t* cnt) {
  if (a.n <= 0) return;
  prune_kernel<<<(unsigned)((a.n + 255) / 256), 256, 0, st>>>(a, aln, list, cnt);
}

void launch_format_sizes(cudaStream_t st, const FormatArgs& a) {
  if (a.n <= 0) return;
  format_sizes_kernel<<<(unsigned)((a.n + 255) / 256), 256, 0, st>>>(a);
}

void launch_format_write(cudaStream_t st, const FormatArgs& a) {
  const int64_t n = a.n - a.first;
  if (n <= 0) return;
  const int64_t warps = (n + kFmtPerWarp - 1) / kFmtPerWarp;
  format_write_kernel<<<(unsigned)((warps + kFmtWarps - 1) / kFmtWarps), kFmtWarps * 32, 0, st>>>(a);
}

}  // namespace swift
