// Host-side structural parse of the reference FASTA (once per index), with
// the reference's reading rules: refMapCreate (src/refMap.cu:59-117) for
// name/sequence offsets and bases-per-line; lookupTable5Create
// (src/lookupTable5.cu:127-187) for the concatenated sequence its tuples come
// from.  The parse only records offsets; sequence bytes stay where they are
// and are copied to the device as one block.  (Reads are parsed on the
// device, parse.cu.)  Also the two batch schedules of the reference drivers.
#include <string.h>

#include <cmath>

#include "internal.h"

namespace swift {

namespace {

// Length of the chunk fgets(buf, MAX_LINE_LENGTH, f) returns at pos.
inline size_t chunk_at(const char* b, size_t n, size_t pos) {
  if (pos >= n) return 0;
  size_t lim = n - pos;
  if (lim > (size_t)kLineMax - 1) lim = (size_t)kLineMax - 1;
  const void* nl = memchr(b + pos, '\n', lim);
  return nl ? (size_t)((const char*)nl - (b + pos)) + 1 : lim;
}

// Rejects NUL bytes, bytes >= 128 and '>' anywhere but at a line start:
// the reference reads lines with strlen and indexes a 128-entry table with
// each byte, and treats any chunk starting with '>' as a header.
bool bytes_ok(const char* s, size_t len, bool header, std::string* err,
              const char* what, size_t off) {
  const unsigned char* u = (const unsigned char*)s;
  size_t i = 0;
  uint64_t acc_hi = 0;
  for (; i + 8 <= len; i += 8) {
    uint64_t w;
    memcpy(&w, u + i, 8);
    uint64_t zero = (w - 0x0101010101010101ull) & ~w & 0x8080808080808080ull;
    acc_hi |= (w & 0x8080808080808080ull) | zero;
  }
  for (; i < len; ++i) acc_hi |= (u[i] & 0x80) | (u[i] == 0 ? 0x80 : 0);
  if (acc_hi) {
    *err = std::string(what) + ": byte outside 7-bit text in the line at offset " +
           std::to_string(off);
    return false;
  }
  const void* gt = len > 1 ? memchr(s + 1, '>', len - 1) : nullptr;
  if (gt || (!header && len && s[0] == '>')) {
    *err = std::string(what) + ": '>' inside a line at offset " + std::to_string(off);
    return false;
  }
  return true;
}

// Records whose windows can be copied from the concatenation (see
// RefRecord::regular); the device computes offsets in 32 bits, so the
// record must also end below 4 GiB.
void mark_regular(HostRef* hr) {
  size_t li = 0;
  const size_t nl = hr->line_len.size();
  for (RefRecord& q : hr->recs) {
    const uint64_t end = q.cat_start + q.cat_len;
    size_t first = li;
    while (li < nl && hr->line_dst[li] < end) ++li;
    const size_t n = li - first;
    bool ok = q.seq_off + q.cat_len + (q.bpl ? q.cat_len / q.bpl : 0) + 1 < (1ull << 32);
    if (n == 0) {
      ok = false;
    } else if (q.bpl == 0) {
      ok = ok && n == 1 && hr->line_src[first] == q.seq_off;
    } else {
      for (size_t t = 0; ok && t < n; ++t) {
        ok = hr->line_src[first + t] == q.seq_off + t * (uint64_t)(q.bpl + 1) &&
             (t + 1 < n ? hr->line_len[first + t] == q.bpl : hr->line_len[first + t] <= q.bpl);
      }
    }
    q.regular = ok;
  }
}

}  // namespace

int parse_reference(const char* b, size_t n, HostRef* out, std::string* err) {
  HostRef& r = *out;
  r = HostRef();
  long prev_ll = 0, old_ll = 0;
  uint32_t pos_count = 0;
  int num_lines = 0;
  size_t pos = 0, c;
  auto finish = [&](RefRecord& p) {
    p.bpl = num_lines > 1 ? (uint32_t)(pos_count - (uint32_t)old_ll) / (uint32_t)(num_lines - 1)
                          : 0u;
  };
  while ((c = chunk_at(b, n, pos)) > 0) {
    long ll = (long)c - (b[pos + c - 1] == '\n');
    if (prev_ll > 0) old_ll = prev_ll;
    prev_ll = ll;
    if (ll == 0) {
      pos += c;
      continue;
    }
    if (b[pos] == '>') {
      if (!bytes_ok(b + pos, (size_t)ll, true, err, "reference", pos)) return SWIFT_E_INPUT;
      if (!r.recs.empty()) finish(r.recs.back());
      if ((int)r.recs.size() == kMaxRefs) {
        *err = "reference: more than 127 sequences (the reference keeps the "
               "sequence index in a char)";
        return SWIFT_E_LIMIT;
      }
      if (ll - 1 >= kNameMax) {
        *err = "reference: sequence name longer than 49 characters";
        return SWIFT_E_LIMIT;
      }
      RefRecord q;
      memset(&q, 0, sizeof(q));
      q.name_off = pos + c - (size_t)ll - 1;
      q.seq_off = pos + c;
      q.name_len = (uint32_t)(ll - 1);
      memcpy(q.name, b + pos + 1, (size_t)(ll - 1));
      q.cat_start = r.cat_len;
      r.recs.push_back(q);
      pos_count = 0;
      num_lines = 0;
    } else {
      if (r.recs.empty()) {
        *err = "reference: sequence before the first header";
        return SWIFT_E_INPUT;
      }
      if (!bytes_ok(b + pos, (size_t)ll, false, err, "reference", pos)) return SWIFT_E_INPUT;
      ++num_lines;
      pos_count += (uint32_t)ll;
      r.line_src.push_back(pos);
      r.line_dst.push_back(r.cat_len);
      r.line_len.push_back((uint32_t)ll);
      r.cat_len += (uint64_t)ll;
      r.recs.back().cat_len += (uint64_t)ll;
    }
    pos += c;
  }
  if (prev_ll > 0) old_ll = prev_ll;
  if (!r.recs.empty()) finish(r.recs.back());
  if (r.recs.empty()) {
    *err = "reference: no sequence header";
    return SWIFT_E_INPUT;
  }
  mark_regular(&r);
  return SWIFT_OK;
}

int parse_reads_host(const char* b, size_t n, int max_read, HostReads* out, std::string* err) {
  // The rules of the device parser (parse.cu) in one pass over the lines:
  // every failure is recorded with its offset and the first in file order
  // (offset, then code) is reported, as the device's atomicMin does.
  uint64_t worst = ~0ull;
  auto report = [&](uint64_t off, uint32_t code) {
    worst = std::min<uint64_t>(worst, (off << 8) | code);
  };
  HostReads r;
  int32_t mn = INT32_MAX, mx = 0;
  uint64_t line_start = 0, prev_start = 0;  // this line's and the previous line's start
  int64_t li = 0;
  const uint64_t n_nl = (uint64_t)std::count(b, b + n, '\n');
  const uint64_t n_lines = n_nl + ((n > 0 && b[n - 1] != '\n') ? 1 : 0);
  uint64_t pos = 0;
  while (li < (int64_t)n_lines) {
    const char* nlp = (const char*)memchr(b + pos, '\n', n - pos);
    const uint64_t end = nlp ? (uint64_t)(nlp - b) : n;
    // eight bytes at a time: a word with no NUL, no byte >= 128 and no '>'
    // (the line's first byte may be '>') needs no byte-wise look
    uint64_t i = pos + (pos < end ? 1 : 0);
    if (pos < end && ((uint8_t)b[pos] == 0 || (uint8_t)b[pos] >= 128))
      report(pos, kParseBadByte);
    for (; i + 8 <= end; i += 8) {
      uint64_t v;
      memcpy(&v, b + i, 8);
      const uint64_t k1 = 0x0101010101010101ull, k80 = 0x8080808080808080ull;
      const uint64_t gt = v ^ 0x3E3E3E3E3E3E3E3Eull;
      const uint64_t flags = (((v - k1) & ~v) | ((gt - k1) & ~gt) | v) & k80;
      if (flags) break;  // the byte loop below finds the offending offset
    }
    for (; i < end; ++i) {
      const uint8_t x = (uint8_t)b[i];
      if (x == 0 || x >= 128) report(i, kParseBadByte);
      if (x == '>') report(i, kParseGtInLine);  // not a line's first byte
    }
    line_start = pos;
    const uint64_t len = end - line_start;
    if (len == 0) {
      report(line_start, kParseEmptyLine);
    } else {
      const bool header = b[line_start] == '>';
      if ((li & 1) == 0) {
        if (!header) {
          report(line_start, li == 0 ? kParseSeqNoHeader : kParseMultiLine);
        } else {
          if (len - 1 > (uint64_t)(kNameMax - 2)) report(line_start, kParseNameLong);
          if ((uint64_t)li + 1 >= n_lines) report(line_start, kParseTrailingHeader);
        }
      } else if (header) {  // the line before has no sequence line
        report(li == 1 ? 0 : prev_start, kParseHeaderNoSeq);
      } else if (len > (uint64_t)max_read) {
        report(line_start, kParseReadLong);
      } else {
        DevRead d;
        d.name_off = prev_start;
        d.seq_off = line_start;
        d.len = (int32_t)len;
        d.name_len = (int32_t)(line_start - 1 - prev_start - 1);
        r.rd.push_back(d);
        mn = std::min(mn, (int32_t)len);
        mx = std::max(mx, (int32_t)len);
        if (li == 1) r.first_len = (int32_t)len - (end == n ? 1 : 0);  // strlen(line) - 1
      }
    }
    prev_start = line_start;
    pos = end + 1;
    ++li;
  }
  if (worst != ~0ull) return parse_error((uint32_t)(worst & 0xFF), worst >> 8, err, max_read);
  r.n = (int64_t)(n_lines / 2);
  r.n_gt = (int64_t)((n_lines + 1) / 2);
  r.min_len = r.n ? mn : 0;
  r.max_len = mx;
  *out = std::move(r);
  return SWIFT_OK;
}

std::vector<int32_t> phase1_stale_repeats(int64_t n_reads, int64_t n_gt) {
  // searchQueries3 (src/search.cu:325-357) calls qryGetNext2 in batches of
  // 16 while i < numQrs; a slot whose call finds the end of the file keeps
  // (and re-maps) the read it last held.  With well-formed input the first
  // n_reads calls return reads in order; the remaining calls of the last
  // batch repeat the slot's previous read.
  // Call c < n_reads takes read c into slot c % kP1Slots, so a later call c
  // repeats the last read r < n_reads with r % kP1Slots == c % kP1Slots.
  std::vector<int32_t> rep;
  if (n_gt <= 0) return rep;
  const int64_t calls = (n_gt + kP1Slots - 1) / kP1Slots * kP1Slots;
  for (int64_t call = std::max<int64_t>(n_reads, 0); call < calls; ++call) {
    const int64_t j = call % kP1Slots;
    if (n_reads - 1 >= j) rep.push_back((int32_t)(j + (n_reads - 1 - j) / kP1Slots * kP1Slots));
  }
  return rep;
}

int64_t phase2_batch(int64_t device_mem, int Q, int64_t nm) {
  int64_t per_iter;
  if (device_mem > 0) {
    int mem_pair = (kWin + 1) + (Q + 1) + 4 + 4 + 4 + 2 + 2 * (kWin + Q + 2);
    long gm = (long)(device_mem - 100000000LL);  // GLOBAL_MEM_MARGIN
    per_iter = (int)std::floor((float)gm / mem_pair);
    if (per_iter > 2147483647LL) per_iter = 2147483647LL;
  } else {
    per_iter = nm;
  }
  if (per_iter > nm) per_iter = nm;
  if (per_iter >= 2 && per_iter % 2 == 1) --per_iter;
  return per_iter;
}

int phase2_iterations(int64_t nm, int64_t per_iter) {
  if (per_iter <= 0) return 0;
  return (int)std::ceil((float)nm / (float)per_iter);
}

}  // namespace swift
