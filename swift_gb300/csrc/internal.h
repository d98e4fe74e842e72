// Internal declarations shared by the host and device translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/swift_gb300.h"

namespace swift {

// Limits of the reference's data layout (src/common.h:37-57).
constexpr int kNameMax = 50;      // MAX_QRY_NAME_LENGTH / MAX_REF_NAME_LENGTH
constexpr int kReadMax = 199;     // MAX_QRY_SEQ_LENGTH - 1
constexpr int kWin = 300;         // REF_LENGTH
constexpr int kWinPad = 304;      // window stride in device buffers
constexpr int kShiftBases = 100;  // REF_LENGTH / 3 (src/align.cu:668)
constexpr int kMaxRefs = 127;     // refIdx is a char in the reference
constexpr int kLineMax = 100000;  // MAX_LINE_LENGTH (fgets chunking)
constexpr int kP1Slots = 16;      // NUM_THREADS of searchQueries3
constexpr int kSeedReadMax = 300;  // longest strand the seeding kernels take
constexpr int kMaxQ = 320;        // query rows supported by the SW kernels
constexpr int kMaxR = 1024;       // window columns supported by the SW kernels

// ---------------------------------------------------------------------------
// host-side FASTA structure (host_parse.cpp)

struct RefRecord {
  uint64_t name_off;   // file offset of the header line ('>')
  uint64_t seq_off;    // file offset just past the header line
  uint32_t bpl;        // bases per line as refMapCreate computes it
  uint32_t name_len;
  uint64_t cat_start;  // start in the concatenated sequence
  uint64_t cat_len;    // bases in the record
  char name[kNameMax];
  // every sequence line but the last holds bpl bytes, the last at most bpl,
  // and lines follow each other directly: file offset seq_off + c + c / bpl
  // then is concatenated position c, so a window is a contiguous copy
  bool regular;
};

struct HostRef {
  std::vector<RefRecord> recs;
  // sequence lines: file offset, destination in the concatenation, length
  std::vector<uint64_t> line_src, line_dst;
  std::vector<uint32_t> line_len;
  uint64_t cat_len = 0;
};

int parse_reference(const char* b, size_t n, HostRef* out, std::string* err);

// One request of a merged wave (the serving loop): its reads in the wave's
// reads buffers and what is its own when it runs alone.  rec0 / nm and
// text0 / text1 are filled by the pipeline.
struct WaveReq {
  int64_t read0 = 0, n = 0;       // its reads: wave reads [read0, read0 + n)
  int32_t Q = 0;                  // its query length
  std::vector<int32_t> repeats;   // stale reads of its 16-read loop (wave read ids)
  int64_t rec0 = 0, nm = 0;       // its records in the wave's record arrays
  uint64_t text0 = 0, text1 = 0;  // its text in the wave's output
};

// Phase-1 slot schedule of searchQueries3: read index per slot call, -1 for
// a slot never filled.  Returns the list of reads whose records follow the
// in-order ones (slots that re-ran a stale read after end of file).
std::vector<int32_t> phase1_stale_repeats(int64_t n_reads, int64_t n_gt);

// Phase-2 batch size of getNumQueriesPerIteration (src/align.cu:2767-2793).
int64_t phase2_batch(int64_t device_mem, int Q, int64_t n_matches);
int phase2_iterations(int64_t n_matches, int64_t per_iter);

// ---------------------------------------------------------------------------
// device-side layouts

struct DevRecord {        // per reference sequence
  uint64_t seq_off;
  uint64_t cat_start;
  uint64_t cat_len;
  uint32_t bpl;
  uint32_t name_len;
  char name[kNameMax];
  uint8_t regular;        // see RefRecord::regular
  char pad[5];
};

struct DevRead {          // per read
  uint64_t name_off;      // offset of '>' in the reads buffer
  uint64_t seq_off;
  int32_t len;
  int32_t name_len;
};

// A reads FASTA parsed on the host with the device parser's rules
// (parse.cu), reads up to max_read bases: the per-read records (offsets
// into b) and the lengths the pipeline needs.
struct HostReads {
  std::vector<DevRead> rd;
  int64_t n = 0, n_gt = 0;
  int32_t first_len = 0, min_len = 0, max_len = 0;
};
int parse_reads_host(const char* b, size_t n, int max_read, HostReads* out, std::string* err);

// One Phase-2 pair (one match record).
struct DevPair {
  int32_t read;
  int32_t strand;
  int32_t ref_idx;
  int32_t ref_dist;       // max(0, refPos - 100)
  int32_t win_len;        // window bases after N trimming
  int32_t flags;          // bit 0: needs the generic SW kernel
};

// Result of one Smith-Waterman pair.
struct DevAln {
  int32_t score;
  int32_t start, end, len;
};

// ---------------------------------------------------------------------------
// kernels' host launchers (one per .cu file)

// index.cu
void launch_compact_lines(cudaStream_t st, const char* file, const uint64_t* src,
                          const uint64_t* dst, const uint32_t* len, int64_t n_lines,
                          uint8_t* cat);
void launch_pack2bit(cudaStream_t st, const uint8_t* cat, int64_t n_words, uint32_t* packed);
// words of the odd-base bitmap of a cat buffer of n_words 16-byte words
// (the bitmap's reads of cat stay inside the buffer's 64 bytes of padding)
inline int64_t odd_bits_words(int64_t n_words) { return (n_words * 16 + 31) / 32 + 1; }
void launch_odd_bits(cudaStream_t st, const uint8_t* cat, int64_t n_words, uint32_t* odd);
void launch_count_tuples(cudaStream_t st, const uint32_t* packed, const DevRecord* recs,
                         const uint64_t* tbase, int n_recs, uint64_t n_tuples, int k,
                         uint32_t* count);
void launch_threshold(cudaStream_t st, const uint32_t* count, int64_t nb, uint32_t thres,
                      uint32_t* eff);
// Compact bucket directory (index.cu): groups[g] = (occupancy bits of
// buckets 64 g .. 64 g + 63 as lo, hi words, occupied buckets before the
// group, 0); cstart[r] = start of the r-th occupied bucket, cstart[n_occ] =
// total.  Scratch: bits32 (nb / 32), gcnt and grank (nb / 64), scan_tmp.
int build_bucket_directory(cudaStream_t st, const uint32_t* offsets, int64_t nb, uint32_t* bits32,
                           uint32_t* gcnt, uint32_t* grank, void* scan_tmp, uint32_t* n_occ,
                           uint4* groups, uint32_t* cstart);
void launch_scatter_tuples(cudaStream_t st, const uint32_t* packed, const DevRecord* recs,
                           const uint64_t* tbase, int n_recs, uint64_t n_tuples, int k,
                           uint32_t thres, const uint32_t* count, const uint32_t* offsets,
                           uint32_t* cursor, uint2* post);
void launch_order_buckets(cudaStream_t st, const uint32_t* offsets, int64_t nb, uint2* post);
// gpos[i] = gbase[post[i].y] + post[i].x (the seeding kernels' global positions)
void launch_global_positions(cudaStream_t st, const uint2* post, int64_t n, const uint32_t* gbase,
                             uint32_t* gpos);
// Per sequence its first global position: kGPad, then kGPad past the end of
// the one before; false when the last end passes 2^32 - 64 (seeding then
// keeps (ref_pos, ref_idx) keys).
bool global_bases(const std::vector<RefRecord>& recs, std::vector<uint32_t>* gbase);

#ifdef __CUDACC__
// Appends the ids whose flag is set to list with one atomic per block on
// cnt (list order within and across blocks is arbitrary).  Every thread of
// the block calls it, blocks of at most 1024 threads.
__device__ __forceinline__ void block_append(bool flag, int32_t id, int32_t* list, int32_t* cnt) {
  __shared__ int32_t wsum[32];
  __shared__ int32_t base;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  const uint32_t b = __ballot_sync(0xffffffffu, flag);
  if (lane == 0) wsum[wid] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    int32_t t = 0;
    for (int w = 0; w < nw; ++w) {
      const int32_t c = wsum[w];
      wsum[w] = t;
      t += c;
    }
    base = t ? atomicAdd(cnt, t) : 0;
  }
  __syncthreads();
  if (flag) list[base + wsum[wid] + __popc(b & ((1u << lane) - 1))] = id;
  __syncthreads();  // wsum and base free for the next call
}

// Adds the block's count of set flags to cnt with one atomic.
__device__ __forceinline__ void block_count(bool flag, int32_t* cnt) {
  const int32_t c = __syncthreads_count(flag);
  if (threadIdx.x == 0 && c) atomicAdd(cnt, c);
}
#endif

// scan.cu
size_t scan_temp_bytes(int64_t n);
// Each returns the number of kernels it launched.
int exclusive_scan_u32(cudaStream_t st, const uint32_t* in, uint32_t* out, int64_t n,
                       void* temp, uint32_t* total_dev);
int exclusive_scan_u64(cudaStream_t st, const uint64_t* in, uint64_t* out, int64_t n,
                       void* temp, uint64_t* total_dev);

// seed.cu
struct SeedArgs {
  const char* reads;          // reads file bytes
  const DevRead* rd;
  int64_t n_reads;
  const uint32_t* offsets;    // bucket starts, 4^k + 1 entries
  const uint4* groups;        // compact bucket directory (index.cu)
  const uint32_t* cstart;
  const uint2* postings;      // (ref_pos, ref_idx)
  const uint32_t* gpos;       // optional, same order: gbase[ref_idx] + ref_pos
  const uint32_t* gbase;      // with gpos: per sequence its first global position
  int n_recs;
  int k;
  int max_hits;
  int fixed_len;              // > 0: every strand has this many bases (the
                              // strand string's first fixed_len; paired end)
  int3* best;                 // per strand: max_hits x (ri, shift, rp)
  int32_t* nbest;             // per strand
  int32_t* overflow_list;     // strands too big for the on-chip paths
  int32_t* n_overflow;
  int max_len;                // longest read (sizes the per-lane offsets)
  int32_t* mid_list;          // strands for the small hash-table kernel (zeroed count)
  int32_t* n_mid;
  int32_t* big_list;          // strands for the large hash-table kernel (zeroed count)
  int32_t* n_big;
  unsigned long long* model_bytes;  // optional: kSeedModelSlots counters of
                                    // the roofline's sector-model bytes
  uint64_t* scratch;          // overflow path: per-strand hash tables
};
constexpr int kSeedModelSlots = 64;
// global positions: sequences kGPad apart, the first at kGPad
constexpr uint32_t kGPad = 512;
// The sort-free kernel over every strand, then the two hash-table kernels
// over the strands it listed; strands beyond those go to a.overflow_list.
void launch_seed(cudaStream_t st, const SeedArgs& a);

// seed13.cu: lt13 seed-and-extend seeding (search2Queries)
constexpr int kMaxRefs13 = 64;      // refIdx << 25 in an int
constexpr int kFullArr13 = 2304;    // the reference block's shared arrays (idealArrSize)
constexpr int kFullStage13 = 1280;  // staged hits of one tuple offset (ignore threshold <= 1176)
constexpr int kMaxThres13 = 1176;   // kFullArr13 - 1000 kept - 2 x 64 padding
struct Seed13Args {
  const char* reads;
  const DevRead* rd;
  int64_t n_reads;
  const uint4* groups;        // compact bucket directory of the SSAHA index
  const uint32_t* cstart;
  const int32_t* vals;        // composites per posting
  const int32_t* map;         // refPosHashMap per tuple id
  const int64_t* tbase;       // per reference: first tuple id
  const int64_t* ntup;        // per reference: tuples
  int nrefs;
  int64_t max_comp;
  int k;
  const int32_t* list;        // strands to map (null: all 2 x n_reads)
  int64_t n_list;
  int3* best;                 // per strand: 3 x (ref_idx, 0, ref_pos)
  int32_t* nbest;
  int32_t* overflow_list;     // strands whose entries outgrow the fast kernel
  int32_t* n_overflow;
};
void launch_seed13(cudaStream_t st, const Seed13Args& a, bool full);
void launch_tuple_hash13(cudaStream_t st, const uint32_t* packed, const DevRecord* recs,
                         const uint64_t* tbase, int n_recs, uint64_t n_tuples, int k,
                         uint32_t* out);
void launch_composites13(cudaStream_t st, const uint2* post, int64_t n, int k, int32_t* vals);
void launch_seed_overflow(cudaStream_t st, const SeedArgs& a, int n_overflow,
                          const uint64_t* tab_off, const uint32_t* tab_size);
int seed_smem_cap();

// parse.cu: reads FASTA structure found on the device
enum : uint32_t {
  kParseBadByte = 1,
  kParseGtInLine,
  kParseEmptyLine,
  kParseSeqNoHeader,
  kParseMultiLine,
  kParseHeaderNoSeq,
  kParseTrailingHeader,
  kParseNameLong,
  kParseReadLong,
};
struct ParseSummary {
  int32_t min_len, max_len, first_len, pad;
};
unsigned parse_tiles(uint64_t n);
void launch_parse_tiles(cudaStream_t st, const char* b, uint64_t n, uint32_t* cnt,
                        unsigned long long* err);
void launch_parse_newlines(cudaStream_t st, const char* b, uint64_t n, const uint32_t* off,
                           uint64_t* nl);
void launch_parse_lines(cudaStream_t st, const char* b, uint64_t n, const uint64_t* nl,
                        uint64_t n_nl, uint64_t n_lines, DevRead* rd, ParseSummary* sum,
                        unsigned long long* err, int max_read);
int parse_error(uint32_t code, uint64_t off, std::string* msg, int max_read = kReadMax);

// pairs.cu
struct PairArgs {
  const char* ref_file;
  uint64_t ref_file_len;
  const char* cat;            // concatenated record sequences
  const uint32_t* odd;        // optional: bit p of odd[p / 32] set where cat[p] is not ACGTacgt
  const DevRecord* recs;
  const char* reads;
  const DevRead* rd;
  const int32_t* m_read;      // per record: read, strand, ref idx, ref pos
  const int32_t* m_strand;
  const int32_t* m_ri;
  const int32_t* m_rp;
  int64_t n;
  int Q;
  const int32_t* read_q;      // optional: query length per read (reads of
                              // requests with different query lengths)
  int32_t* pair_q;            // optional out: each record's query length
  DevPair* pairs;
  char* qbuf;                 // n x Qs
  char* wbuf;                 // n x kWinPad
  int Qs;                     // query stride (>= every query length + 1)
  uint8_t* read_cls;          // optional scratch, n_reads bytes: per read 0 when its
                              // query bytes are all A, C, G or T (word-wise copy)
  int64_t n_reads;
};
void launch_build_pairs(cudaStream_t st, const PairArgs& a);

// paired.cu: *bad = 1 when a read name of either file does not end in 1 or 2
void launch_pe_names(cudaStream_t st, const char* b1, const DevRead* rd1, const char* b2,
                     const DevRead* rd2, int64_t n, int32_t* bad);
// paired.cu: paired-end records and pairs
struct PairedArgs {
  int64_t n_pairs;            // reads per file
  int max_hits;
  const int32_t *nbest1, *nbest2;   // per strand of each file
  const int3 *best1, *best2;
  const uint64_t* roff;       // per pair: first record
  int64_t n_rec;
  int32_t *m_id, *m_mate, *m_rev, *m_read, *m_ri, *m_shift, *m_off;
  int Q;
  const char* ref_file;
  uint64_t ref_file_len;
  const char* cat;            // optional: the index's concatenated sequences and
  const uint32_t* odd;        // their non-ACGTacgt bitmap (direct window copies)
  const DevRecord* recs;
  const char* reads;          // both reads files, the second after the first
  const DevRead* rd;          // file 1's reads, then file 2's
  DevPair* pairs;
  char* qbuf;                 // n_rec x q_stride
  char* wbuf;                 // n_rec x w_stride, zeroed by the caller
  int64_t q_stride, w_stride; // >= Q + 1 and 3Q + 1, multiples of 16
};
void launch_pe_records(cudaStream_t st, const PairedArgs& a, uint64_t* cnt);
void launch_pe_fill(cudaStream_t st, const PairedArgs& a);
void launch_pe_pairs(cudaStream_t st, const PairedArgs& a);
void launch_aln_from_arrays(cudaStream_t st, const float* score, const int32_t* start,
                            const int32_t* end, const int32_t* len, int64_t n, DevAln* aln);
void launch_shift_reads(cudaStream_t st, const DevRead* in, int64_t n, uint64_t by,
                        DevRead* out);
// mate pairing (chooseBestAlignment_paired3) and printOutput_paired2 flags
struct PairSelArgs {
  int64_t n;                  // records
  const DevPair* pairs;
  const DevAln* aln;
  const int32_t* id;          // pair id per record (non-decreasing)
  const uint8_t* batch_start; // 1 at the first record of each Phase-2 batch
  const char* reads;          // both reads files (names)
  const DevRead* rd;
  const int32_t* ref_class;   // per reference: its name's class (equal names, equal class)
  uint32_t min_frag, max_frag;
  int32_t* keep;              // out: printed
  int8_t* sep;                // out: 1 opens with the line of '*'
};
void launch_pe_runs(cudaStream_t st, const PairSelArgs& a, uint32_t* flag);
void launch_pe_run_first(cudaStream_t st, const PairSelArgs& a, const uint32_t* flag,
                         const uint32_t* run_of, int64_t* first);
void launch_pe_pair_runs(cudaStream_t st, const PairSelArgs& a, const int64_t* first,
                         int64_t n_runs);
void launch_pe_sep(cudaStream_t st, const PairSelArgs& a);

// sw.cu
struct SwArgs {
  const char* q;              // query i at q + i*q_stride
  const char* w;              // window i at w + i*w_stride
  int64_t q_stride, w_stride;
  int Q, R;
  int match, mismatch, gap_open, gap_ext;
  int64_t n;
  DevAln* aln;
  char* qcons;                // reversed consensus strings, stride cons_stride
  char* rcons;
  int64_t cons_stride;
  const int32_t* list;        // optional: pair ids to process ...
  const int32_t* count;       // ... and their number (device); grid sized by n
  const int32_t* q_len;       // optional: query length per pair (<= Q)
};
// Static scratch of swift_sw_batch_noalloc (sw.cu): room for this many pairs.
constexpr int64_t kStaticSwPairs = SWIFT_SW_NOALLOC_MAX_PAIRS;
int static_sw_scratch(int device, DevAln** out, std::string* err);
int launch_sw(cudaStream_t st, const SwArgs& a, std::string* err);

// pairs_var.cu: explicit pairs of varying lengths, sorted by shape
constexpr uint32_t kVarKeys = 1u << 21;  // shape keys: generic bit, Q (9 bits), R (11 bits)
// the top eight keys: long pairs (sw_long.cu) by rows-per-lane class (key
// bits 2-1) and whether they hold only ACGTN bytes (bit 0)
constexpr uint32_t kVarLongKey = kVarKeys - 8;
// pairs beyond the warp-per-pair kernels' shapes go to the long kernel
__host__ __device__ inline bool var_pair_long(int Q, int R) {
  return Q > 256 || R > 1024 || (Q > 128 && R > 768);
}
struct VarPairArgs {
  const char* qry;            // query bytes of pair i at qry + q_off[i], q_len[i] of them
  const int64_t* q_off;
  const int32_t* q_len;
  const char* ref;            // window bytes at ref + r_off[i], r_len[i] of them
  const int64_t* r_off;
  const int32_t* r_len;
  int64_t n;
  char* qbuf;                 // fixed strides, NUL padded
  char* wbuf;
  int64_t q_stride, w_stride;
  uint32_t class_ok;          // bit c: the packed passes take this scoring for class c
  bool long_prof;             // the long kernel's profile path takes this scoring
  int fast_max_r;
  uint32_t* key;              // per pair
  uint32_t* hist;             // per key
  uint32_t* bad;              // set when a pair holds byte 0x00 or 0x01
};
void launch_var_max_len(cudaStream_t st, const int32_t* q_len, const int32_t* r_len, int64_t n,
                        int32_t* out);
void launch_pack_var(cudaStream_t st, const VarPairArgs& a);
void launch_var_occupied(cudaStream_t st, const uint32_t* hist, uint32_t* occ);
void launch_var_segments(cudaStream_t st, const uint32_t* hist, const uint32_t* start,
                         const uint32_t* seg_pos, int32_t* seg_key, int32_t* seg_start,
                         int32_t* seg_count);
void launch_var_scatter(cudaStream_t st, const uint32_t* key, int64_t n, const uint32_t* start,
                        uint32_t* fill, int32_t* sorted);

// sw_long.cu: long pairs (queries up to 4096, windows up to 8192), one CTA each
constexpr int kLongMaxQ = 4096;
constexpr int kLongMaxR = 8192;
struct LongArgs {
  const char* qry;            // pair i: qry + q_off[i], q_len[i] bytes; ref likewise
  const int64_t* q_off;
  const int32_t* q_len;
  const char* ref;
  const int64_t* r_off;
  const int32_t* r_len;
  const int32_t* list;        // pair ids of this launch
  int64_t n;
  int max_r;                  // longest window of the launch
  int match, mismatch, gap_open, gap_ext, bias;
  uint32_t* dirs;             // direction scratch: the slot of item i at dirs + dir_off[i],
  const int64_t* dir_off;     // long_slot_words(R of its pair) words
  int2* best;                 // per pair: (score, first maximum cell)
  DevAln* aln;
  char* qcons;                // optional reversed consensus strings
  char* rcons;
  int64_t cons_stride;
};
int long_rows_per_lane(int Q);           // 4, 8, 12 or 16; 0 beyond 4096
int64_t long_slot_words(int R);          // direction words of one pair (16-byte multiple)
// the long kernel's cell bias for a gap-open penalty, and whether its
// profile path takes a scoring for queries up to max_q rows; prof: every
// pair of the launch holds only ACGTN bytes (either case) and
// long_prof_ok(...) holds
int long_bias(int gap_open);
bool long_prof_ok(int m, int x, int gap_open, int max_q);
int launch_sw_long(cudaStream_t st, const LongArgs& a, int rpl, bool prof);

// sw_fast.cu: packed 16-bit passes (score of every pair; trace of printed pairs)
// Suffix LCS values: window columns per block (the wavefront steps between
// two early-stop tests), blocks per pair.
constexpr int kSufSteps = 16;
constexpr int kSufBlocks = 32;
struct FastArgs {
  const char* q;
  const char* w;
  int64_t q_stride, w_stride;
  int Q, R;
  int match, mismatch, gap_open, gap_ext;
  int bias;
  const int32_t* list;        // pair ids
  const int32_t* count;       // number of ids (device)
  int64_t list_offset;        // first id of this launch
  DevAln* aln;                // score pass: .score; trace pass: all fields
  const int32_t* q_len;       // trace pass: per-pair query and window lengths
  const int32_t* r_len;       // (pairs of one launch may differ), or null
  int32_t* ub;                // LCS bound pass: upper bound of the score per pair
  int2* best;                 // trace pass: (score, first maximum cell) per pair
  uint32_t* dirs;             // trace pass: direction scratch
  int64_t chunk;              // trace pass: pairs of this launch
  char* qcons;                // trace pass: reversed consensus strings
  char* rcons;
  int64_t cons_stride;
  unsigned long long* cells_done;  // optional: score and trace passes add the
                                   // cells they computed (early stop counted)
  int shape_g, shape_rpl;     // optional: the (lanes, rows per lane) shape of the
                              // exact passes and walk; 0: the default for Q
  uint32_t one, four;         // trace pass: 1 and 4, as values the compiler cannot
                              // fold (set by launch_sw_trace)
  uint16_t* lsuf;             // LCS bound pass writes, per pair, kSufBlocks suffix
                              // LCS values: entry m = LCS(query, window columns
                              // kSufSteps * m + 1 .. R); the score and trace
                              // passes read them to stop early; may be null
  const int32_t* cand;        // score pass with lsuf, optional: per pair its
                              // best-per-read group's candidate, whose score
                              // (aln) is known; a pair stops once it provably
                              // cannot reach that score (or tie it from before
                              // the candidate) and then reports a score below
};
bool fast_params_ok(int Q, int R, int m, int x, int o, int e, int* bias);
constexpr int kFastMaxR = 512;  // window columns the packed passes take
// Packed shape class of a query length (the (lanes, rows) shapes of the
// packed passes, shortest first), and the longest query of each class.
__host__ __device__ inline int packed_class(int Q) {
  return Q <= 32 ? 0 : Q <= 64 ? 1 : Q <= 104 ? 2 : Q <= 128 ? 3 : Q <= 208 ? 4 : Q <= 256 ? 5
       : Q <= 320 ? 6 : -1;
}
__host__ __device__ inline int packed_class_max_q(int c) {
  return c == 0 ? 32 : c == 1 ? 64 : c == 2 ? 104 : c == 3 ? 128 : c == 4 ? 208 : c == 5 ? 256
       : 320;
}
// Row class of a query of swift_sw_pairs' packed pairs: the rows of the
// trace-pass shape that takes it exactly (a multiple of 8 up to 128, of 16
// up to 256, of 32 up to 320, at least 32); -1 beyond 320.
__host__ __device__ inline int var_rows(int Q) {
  return Q <= 32 ? 32 : Q <= 128 ? (Q + 7) & ~7 : Q <= 256 ? (Q + 15) & ~15
       : Q <= 320 ? (Q + 31) & ~31 : -1;
}
int64_t trace_scratch_words(int Q, int R, int64_t pairs, int shape_g = 0, int shape_rpl = 0);
// The compiled shapes of the per-pair-length trace pass the autotuner tries
// for the queries of Q's row class (the exact fit, its default, first);
// returns how many.
int packed_shape_candidates(int Q, int32_t* g, int32_t* rpl, int cap);
int launch_sw_score(cudaStream_t st, const FastArgs& a, int64_t max_pairs);
// before / after (optional) are recorded around the trace pass alone
int launch_sw_trace(cudaStream_t st, const FastArgs& a, int64_t max_pairs,
                    cudaEvent_t before = nullptr, cudaEvent_t after = nullptr);
// sw_lcs.cu: a.ub[p] = match * LCS(query, window) for the listed pairs, and
// with a.lsuf the suffix LCS values
int launch_sw_lcs(cudaStream_t st, const FastArgs& a, int64_t max_pairs);
int measure_dpx_peak(cudaStream_t st, int device, double* lane_instr_per_s);

// out.cu
struct FormatArgs {
  const char* reads;
  const DevRead* rd;
  const DevRecord* recs;
  const DevPair* pairs;
  const DevAln* aln;
  const char* qcons;
  const char* rcons;
  int64_t cons_stride;
  int64_t n;
  int64_t first;              // write kernels: records [first, n)
  int64_t batch;              // Phase-2 batch size (best-per-read groups stop at batch ends)
  const uint8_t* batch_start; // optional: 1 at each record that opens a batch (per
                              // request of a wave); replaces the uniform batch size
  int32_t* keep;              // per record: 1 if printed
  uint64_t* bytes;            // per record: text bytes
  uint64_t* offs;             // per record: text offset
  char* text;
  const int32_t* ub;          // bounded selection: upper bound per packed-path pair
  int32_t* cand;              // bounded selection: the group's candidate per pair
  const int8_t* pe_sep;       // paired-end records (printOutput_paired2): 1 opens a
                              // pair with a line of 37 '*', 0 a blank line; null:
                              // the single-end record's 40 '*'
};
void launch_select(cudaStream_t st, const FormatArgs& a);
void launch_candidates(cudaStream_t st, const FormatArgs& a, int32_t* list, int32_t* cnt);
void launch_prune(cudaStream_t st, const FormatArgs& a, DevAln* aln, int32_t* list, int32_t* cnt);
void launch_format_sizes(cudaStream_t st, const FormatArgs& a);
void launch_format_write(cudaStream_t st, const FormatArgs& a);
// SAM output: every record, sizes then text (keep is not read)
void launch_sam_sizes(cudaStream_t st, const FormatArgs& a);
void launch_sam_write(cudaStream_t st, const FormatArgs& a);

}  // namespace swift
