// The library's opaque handles (swift_ctx, swift_index, swift_reads), shared
// by the files that implement the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "internal.h"

constexpr int kCtxEvents = 12;

struct swift_ctx {
  int device = 0;
  cudaStream_t st = nullptr;
  bool own_stream = false;
  std::string err;
  int64_t total_mem = 0;
  cudaEvent_t ev[kCtxEvents] = {};
  char* d_text = nullptr;
  size_t text_len = 0, text_cap = 0;
  int sw_path = 0;  // 0 bounded selection, 1 generic kernel only, 2 exact score of every pair
  cudaStream_t side = nullptr;  // second stream for concurrent launches, made on first use
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  std::vector<cudaEvent_t> chunk_ev;  // per-chunk timing of the trace pass, grown on use
  std::vector<cudaEvent_t> copy_ev;   // text ranges ready for their host copy, grown on use
  // swift_sw_pairs: 1 autotune the packed shape per (query class, window
  // bin), 0 default shapes, k >= 2 the (k-2)-th candidate of every class
  int tuning = 1;
  std::map<int, std::pair<int, int>> tuned;  // (class, window bin) -> (lanes, rows per lane)
};

struct swift_index {
  int device = 0;
  int k = 12, thres = 1000;
  char* d_file = nullptr;
  uint64_t file_len = 0;
  swift::DevRecord* d_recs = nullptr;
  std::vector<swift::RefRecord> recs;
  uint8_t* d_cat = nullptr;
  uint32_t* d_packed = nullptr;
  uint32_t* d_odd = nullptr;    // non-ACGT positions of d_cat, one bit each
  uint64_t cat_len = 0;
  uint32_t* d_count = nullptr;
  uint32_t* d_offsets = nullptr;
  uint4* d_groups = nullptr;   // compact bucket directory for seeding
  uint32_t* d_cstart = nullptr;
  uint2* d_post = nullptr;
  // the postings as global positions (gbase[ref_idx] + ref_pos), for the
  // SSAHA seeding kernels: half the bytes, and 32-bit cluster keys; null
  // when the reference is too long for 32-bit positions
  uint32_t* d_gpos = nullptr;
  uint32_t* d_gbase = nullptr;
  int64_t total = 0;
  int64_t nb = 0;
  // lt13 seeding (seed13.cu), built on first use
  std::mutex lt13_mu;
  bool lt13_ready = false;
  int32_t* d_vals13 = nullptr;   // composite per posting
  int32_t* d_map13 = nullptr;    // refPosHashMap per tuple id
  int64_t* d_tbase13 = nullptr;  // per reference: first tuple id, tuples
  int64_t* d_ntup13 = nullptr;
  int64_t max_comp13 = 0;
  int64_t n_tup13 = 0;           // tuples over all references
  // paired-end seeding (lookupTable2 positions), built on first use: the
  // postings of an index with the 1000-repeat threshold (this one, or
  // pe_sub when this one has another threshold) with lookupTable2's
  // positions
  std::mutex pe_mu;
  bool pe_ready = false;
  swift_index* pe_sub = nullptr;
  uint2* d_post_pe = nullptr;
  uint32_t* d_gpos_pe = nullptr;  // its global positions (null: keys as pairs)
};

struct swift_reads {
  int device = 0;
  char* d_bytes = nullptr;
  uint64_t len = 0;
  swift::DevRead* d_rd = nullptr;
  int64_t n = 0;          // reads
  int64_t n_gt = 0;       // '>' bytes (getSeqCount)
  int32_t first_len = 0;  // getSeqSize
  int32_t min_len = 0, max_len = 0;
  std::vector<int32_t> repeats;
  cudaStream_t pool_st = nullptr;  // buffers from this stream's pool (one call's reads)
};

// api.cu: one merged wave of serving requests (server.cpp); see its comment.
int run_wave(swift_ctx* ctx, const swift_index* idx, const swift_params* p, const char* bytes,
             size_t len, const std::vector<swift::DevRead>& rd, std::vector<swift::WaveReq>* wave,
             char* host_out, size_t host_cap, size_t* out_len, swift_stats* stats);
int read_limit_of(const swift_params* p);
// api.cu: the index's postings as global positions (for the seeding kernels);
// SWIFT_OK also when the reference is too long for them (left null)
int index_global_positions(swift_index* ix, cudaStream_t st);
