// Index persistence for warm starts (serving): the device index written to
// one binary file and read back without re-parsing or re-hashing the
// reference.  It carries what lookupTable13Create2 reads back in the
// reference (src/lookupTable13.cu:257-322: bucket starts and counts,
// composite values, refPosHashMap; there as three text files the commented
// dump of lookupTable13Create writes, src/lookupTable13.cu:227-241), plus
// what this library's pipeline needs: the reference bytes (windows and
// names), the sequence records, the SSAHA postings and bucket directory,
// and the concatenated and 2-bit packed sequence.
//
// Layout (little-endian): a fixed header, then the sections in a fixed
// order, each a plain array.  A 64-bit checksum over the payload guards
// against truncated or damaged files; a file that fails any check is
// refused with SWIFT_E_INPUT.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "handles.h"
#include "../../include/swift_gb300.h"

using namespace swift;

namespace {

constexpr char kMagic[8] = {'S', 'W', 'G', 'B', 'I', 'D', 'X', '1'};
constexpr uint32_t kVersion = 1;

struct FileHeader {
  char magic[8];
  uint32_t version;
  int32_t k, thres;
  uint32_t n_recs;
  uint64_t file_len, cat_len, nb, total;
  uint32_t has_lt13, reserved;
  int64_t max_comp13, n_tup13;
  uint64_t payload_bytes;
  uint64_t checksum;
};
static_assert(sizeof(FileHeader) == 96, "header layout");

// one sequence record, fixed width
struct FileRecord {
  uint64_t name_off, seq_off;
  uint32_t bpl, name_len;
  uint64_t cat_start, cat_len;
  char name[kNameMax];
  uint8_t regular;
  uint8_t pad[5];
};
static_assert(sizeof(FileRecord) == 96, "record layout");

// word-wise FNV-1a-style mix over the payload (8 bytes per step)
struct Checksum {
  uint64_t h = 1469598103934665603ull;
  void add(const void* p, size_t n) {
    const uint8_t* b = (const uint8_t*)p;
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
      uint64_t w;
      memcpy(&w, b + i, 8);
      h = (h ^ w) * 1099511628211ull;
    }
    for (; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
  }
};

int fail(swift_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

struct Section {
  void* dev;        // device array (save: source; load: destination)
  size_t bytes;
};

uint64_t n_words_of(uint64_t cat_len) { return (cat_len + 15) / 16; }

std::vector<Section> sections(const swift_index* ix, bool lt13) {
  const uint64_t nw = n_words_of(ix->cat_len);
  const uint64_t ng = (uint64_t)(ix->nb + 63) / 64;
  const size_t nr = ix->recs.size();
  std::vector<Section> s = {
      {ix->d_file, ix->file_len},
      {ix->d_count, (size_t)ix->nb * 4},
      {ix->d_offsets, ((size_t)ix->nb + 1) * 4},
      {ix->d_groups, ng * sizeof(uint4)},
      {ix->d_cstart, ((size_t)ix->total + 1) * 4},
      {ix->d_post, (size_t)ix->total * sizeof(uint2)},
      {ix->d_cat, nw * 16},
      {ix->d_packed, (nw + 2) * 4},
  };
  if (lt13) {
    s.push_back({ix->d_vals13, (size_t)ix->total * 4});
    s.push_back({ix->d_map13, (size_t)ix->n_tup13 * 4});
    s.push_back({ix->d_tbase13, nr * 8});
    s.push_back({ix->d_ntup13, nr * 8});
  }
  return s;
}

}  // namespace

extern "C" {

int swift_index_save(swift_ctx* ctx, const swift_index* cix, const char* path) {
  if (!ctx || !cix || !path) return fail(ctx, SWIFT_E_ARG, "null argument");
  swift_index* ix = const_cast<swift_index*>(cix);
  if (cudaSetDevice(ix->device) != cudaSuccess) return fail(ctx, SWIFT_E_CUDA, "cudaSetDevice");
  std::lock_guard<std::mutex> lk(ix->lt13_mu);
  const bool lt13 = ix->lt13_ready;
  FileHeader h;
  memset(&h, 0, sizeof(h));
  memcpy(h.magic, kMagic, 8);
  h.version = kVersion;
  h.k = ix->k;
  h.thres = ix->thres;
  h.n_recs = (uint32_t)ix->recs.size();
  h.file_len = ix->file_len;
  h.cat_len = ix->cat_len;
  h.nb = (uint64_t)ix->nb;
  h.total = (uint64_t)ix->total;
  h.has_lt13 = lt13 ? 1 : 0;
  h.max_comp13 = ix->max_comp13;
  h.n_tup13 = ix->n_tup13;
  std::vector<FileRecord> recs(ix->recs.size());
  for (size_t i = 0; i < recs.size(); ++i) {
    const RefRecord& r = ix->recs[i];
    FileRecord& f = recs[i];
    memset(&f, 0, sizeof(f));
    f.name_off = r.name_off;
    f.seq_off = r.seq_off;
    f.bpl = r.bpl;
    f.name_len = r.name_len;
    f.cat_start = r.cat_start;
    f.cat_len = r.cat_len;
    memcpy(f.name, r.name, kNameMax);
    f.regular = r.regular ? 1 : 0;
  }
  // payload to host memory, checksum, then one write
  const std::vector<Section> secs = sections(ix, lt13);
  size_t payload = recs.size() * sizeof(FileRecord);
  for (const Section& s : secs) payload += s.bytes;
  std::vector<uint8_t> buf(payload);
  size_t at = 0;
  memcpy(buf.data(), recs.data(), recs.size() * sizeof(FileRecord));
  at += recs.size() * sizeof(FileRecord);
  for (const Section& s : secs) {
    if (s.bytes) {
      const cudaError_t e = cudaMemcpy(buf.data() + at, s.dev, s.bytes, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return fail(ctx, SWIFT_E_CUDA, cudaGetErrorString(e));
    }
    at += s.bytes;
  }
  Checksum c;
  c.add(buf.data(), buf.size());
  h.payload_bytes = payload;
  h.checksum = c.h;
  FILE* f = fopen(path, "wb");
  if (!f) return fail(ctx, SWIFT_E_ARG, std::string("cannot write ") + path);
  const bool ok = fwrite(&h, sizeof(h), 1, f) == 1 &&
                  (payload == 0 || fwrite(buf.data(), 1, payload, f) == payload);
  const bool closed = fclose(f) == 0;
  if (!ok || !closed) return fail(ctx, SWIFT_E_ARG, std::string("write failed: ") + path);
  return SWIFT_OK;
}

int swift_index_load(swift_ctx* ctx, const char* path, swift_index** out) {
  if (!ctx || !path || !out) return fail(ctx, SWIFT_E_ARG, "null argument");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, SWIFT_E_CUDA, "cudaSetDevice");
  FILE* f = fopen(path, "rb");
  if (!f) return fail(ctx, SWIFT_E_ARG, std::string("cannot read ") + path);
  FileHeader h;
  const bool got = fread(&h, sizeof(h), 1, f) == 1;
  if (!got || memcmp(h.magic, kMagic, 8) != 0 || h.version != kVersion) {
    fclose(f);
    return fail(ctx, SWIFT_E_INPUT, "not an index file of this version");
  }
  if (h.k < 1 || h.k > 15 || h.nb != (1ull << (2 * h.k)) || h.n_recs > 127 ||
      h.has_lt13 > 1 || h.total > h.cat_len || h.payload_bytes > (1ull << 44)) {
    fclose(f);
    return fail(ctx, SWIFT_E_INPUT, "index file header is inconsistent");
  }
  std::vector<uint8_t> buf(h.payload_bytes);
  const bool full = h.payload_bytes == 0 || fread(buf.data(), 1, h.payload_bytes, f) == h.payload_bytes;
  const bool extra = fgetc(f) != EOF;
  fclose(f);
  if (!full || extra) return fail(ctx, SWIFT_E_INPUT, "index file is truncated or has trailing bytes");
  Checksum c;
  c.add(buf.data(), buf.size());
  if (c.h != h.checksum) return fail(ctx, SWIFT_E_INPUT, "index file checksum mismatch");
  swift_index* ix = new swift_index();
  ix->device = ctx->device;
  ix->k = h.k;
  ix->thres = h.thres;
  ix->file_len = h.file_len;
  ix->cat_len = h.cat_len;
  ix->nb = (int64_t)h.nb;
  ix->total = (int64_t)h.total;
  ix->recs.resize(h.n_recs);
  const size_t rec_bytes = (size_t)h.n_recs * sizeof(FileRecord);
  if (rec_bytes > buf.size()) {
    delete ix;
    return fail(ctx, SWIFT_E_INPUT, "index file is truncated");
  }
  for (uint32_t i = 0; i < h.n_recs; ++i) {
    FileRecord fr;
    memcpy(&fr, buf.data() + (size_t)i * sizeof(FileRecord), sizeof(fr));
    RefRecord& r = ix->recs[i];
    r.name_off = fr.name_off;
    r.seq_off = fr.seq_off;
    r.bpl = fr.bpl;
    r.name_len = std::min<uint32_t>(fr.name_len, kNameMax - 1);
    r.cat_start = fr.cat_start;
    r.cat_len = fr.cat_len;
    memcpy(r.name, fr.name, kNameMax);
    r.name[kNameMax - 1] = '\0';
    r.regular = fr.regular != 0;
  }
  {  // every record inside the reference bytes and the concatenated
     // sequence, records in file order and back to back in the sequence:
     // the kernels index with these offsets, so a file that passes the
     // checksum yet holds others is refused here
    uint64_t cat_at = 0, seq_at = 0;
    for (uint32_t i = 0; i < h.n_recs; ++i) {
      const RefRecord& r = ix->recs[i];
      const bool ok = r.name_off + r.name_len <= h.file_len && r.seq_off <= h.file_len &&
                      r.seq_off >= seq_at && r.name_off < r.seq_off &&
                      r.cat_start == cat_at && r.cat_len <= h.cat_len - cat_at &&
                      r.cat_len <= (h.file_len - r.seq_off) && r.bpl <= h.file_len;
      if (!ok) {
        delete ix;
        return fail(ctx, SWIFT_E_INPUT, "index file: a sequence record lies outside the "
                                        "reference or out of order");
      }
      cat_at = r.cat_start + r.cat_len;
      seq_at = r.seq_off;
    }
    if (cat_at != h.cat_len) {
      delete ix;
      return fail(ctx, SWIFT_E_INPUT, "index file: sequence records do not cover the sequence");
    }
  }
  const uint64_t nw = n_words_of(ix->cat_len);
  const uint64_t ng = (h.nb + 63) / 64;
  const size_t nr = h.n_recs;
  {  // the sections' sizes follow from the header: check before allocating
    uint64_t need = rec_bytes + h.file_len + h.nb * 4 + (h.nb + 1) * 4 + ng * sizeof(uint4) +
                    (h.total + 1) * 4 + h.total * sizeof(uint2) + nw * 16 + (nw + 2) * 4;
    if (h.has_lt13)
      need += h.total * 4 + (uint64_t)std::max<int64_t>(h.n_tup13, 0) * 4 + nr * 16;
    if (need != buf.size() || h.n_tup13 < 0) {
      delete ix;
      return fail(ctx, SWIFT_E_INPUT, "index file sections do not match its header");
    }
  }
  auto bail = [&](int code, const std::string& m) {
    swift_index_destroy(ix);
    return fail(ctx, code, m);
  };
#define CKL(call)                                                                              \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) return bail(SWIFT_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
  CKL(cudaMalloc(&ix->d_file, h.file_len + 64));
  CKL(cudaMalloc(&ix->d_recs, std::max<size_t>(nr, 1) * sizeof(DevRecord)));
  CKL(cudaMalloc(&ix->d_count, h.nb * 4));
  CKL(cudaMalloc(&ix->d_offsets, (h.nb + 1) * 4));
  CKL(cudaMalloc(&ix->d_groups, ng * sizeof(uint4)));
  CKL(cudaMalloc(&ix->d_cstart, (h.total + 1) * 4));
  CKL(cudaMalloc(&ix->d_post, std::max<uint64_t>(h.total, 1) * sizeof(uint2)));
  CKL(cudaMalloc(&ix->d_cat, nw * 16 + 64));
  CKL(cudaMalloc(&ix->d_packed, (nw + 2) * 4));
  CKL(cudaMalloc(&ix->d_odd, (size_t)odd_bits_words((int64_t)nw) * 4));
  if (h.has_lt13) {
    ix->n_tup13 = h.n_tup13;
    ix->max_comp13 = h.max_comp13;
    CKL(cudaMalloc(&ix->d_vals13, std::max<uint64_t>(h.total, 1) * 4));
    CKL(cudaMalloc(&ix->d_map13, (size_t)std::max<int64_t>(h.n_tup13, 1) * 4));
    CKL(cudaMalloc(&ix->d_tbase13, std::max<size_t>(nr, 1) * 8));
    CKL(cudaMalloc(&ix->d_ntup13, std::max<size_t>(nr, 1) * 8));
  }
  const std::vector<Section> secs = sections(ix, h.has_lt13 != 0);
  CKL(cudaMemset(ix->d_cat, 0, nw * 16 + 64));
  size_t at = rec_bytes;
  for (const Section& s : secs) {
    if (s.bytes) CKL(cudaMemcpy(s.dev, buf.data() + at, s.bytes, cudaMemcpyHostToDevice));
    at += s.bytes;
  }
  std::vector<DevRecord> dr(nr);
  for (size_t i = 0; i < nr; ++i) {
    memset(&dr[i], 0, sizeof(DevRecord));
    dr[i].seq_off = ix->recs[i].seq_off;
    dr[i].cat_start = ix->recs[i].cat_start;
    dr[i].cat_len = ix->recs[i].cat_len;
    dr[i].bpl = ix->recs[i].bpl;
    dr[i].name_len = ix->recs[i].name_len;
    memcpy(dr[i].name, ix->recs[i].name, kNameMax);
    dr[i].regular = ix->recs[i].regular ? 1 : 0;
  }
  if (nr) CKL(cudaMemcpy(ix->d_recs, dr.data(), nr * sizeof(DevRecord), cudaMemcpyHostToDevice));
  // derived from the bases and postings, not stored
  launch_odd_bits(nullptr, ix->d_cat, (int64_t)nw, ix->d_odd);
  CKL(cudaGetLastError());
  if (index_global_positions(ix, nullptr) != SWIFT_OK) CKL(cudaErrorMemoryAllocation);
  CKL(cudaDeviceSynchronize());
#undef CKL
  ix->lt13_ready = h.has_lt13 != 0;
  *out = ix;
  return SWIFT_OK;
}

int swift_index_params(swift_ctx* ctx, const swift_index* ix, int32_t* seed_len,
                       int32_t* ignore_thres) {
  if (!ix) return fail(ctx, SWIFT_E_ARG, "null index");
  if (seed_len) *seed_len = ix->k;
  if (ignore_thres) *ignore_thres = ix->thres;
  return SWIFT_OK;
}

}  // extern "C"
