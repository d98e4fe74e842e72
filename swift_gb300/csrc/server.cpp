// Serving loop with continuous batching.  The reference and index stay
// resident on the device.  Requests (one reads FASTA each) are queued as
// they come; workers (a context and stream each) take
// the queued requests of neighbouring query-length classes (packed shapes at
// most twice as tall as each other), oldest first, up to a read cap and a
// device-memory budget, and run them as ONE merged wave:
// one seeding launch over all their reads, one set of Smith-Waterman
// launches over all their pairs, one formatting pass.  Requests that arrive
// while a wave runs join the next one; with two or more workers the next
// wave's host work and launches overlap the running one on the device.
//
// Each request keeps what is its own when it runs alone (query length,
// the stale-read tail of its 16-read loop, its Phase-2 batches), so its
// records are byte-identical to swift_align on that request alone.
// A wave runs the packed Smith-Waterman shapes of its tallest class; each
// pair's rows past its own query are all-mismatch rows, so a request of a
// shorter class gets its own results from them (at up to twice the rows).
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "handles.h"

using namespace swift;

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

enum : int { kQueued = 0, kRunning = 1, kDone = 2, kCancelled = 3 };

struct Request {
  int64_t ticket = 0;
  std::vector<char> reads;
  HostReads hr;              // its reads, parsed by the worker that takes it
  int32_t Q = 0;             // its query length
  int cls = 0;               // packed shape class of Q (a wave spans classes whose
                             // shapes are at most twice as tall as each other)
  std::vector<int32_t> repeats;
  int64_t est_bytes = 0;
  int64_t est_reads = 0;     // its '>' count, before it is parsed
  int64_t n_reads = 0;
  Clock::time_point submitted, started, finished;
  int state = kQueued;
  int status = SWIFT_OK;
  std::string error;
  char* out = nullptr;       // malloc'ed text, handed to the caller
  size_t out_len = 0;
  double device_ms = 0;      // its wave's device time
  double parse_ms = 0, wave_ms = 0;  // host times of its parse and its wave
  int64_t wave_requests = 0, wave_reads = 0;
};

// per worker: its context and pinned staging for the wave's bytes and text
struct Worker {
  swift_ctx* ctx = nullptr;
  char* pin_in = nullptr;
  size_t pin_in_cap = 0;
  char* pin_out = nullptr;
  size_t pin_out_cap = 0;
};

// Reads per wave at most: bounds a wave's device memory and latency.
constexpr int64_t kWaveMaxReads = 1 << 18;

}  // namespace

struct swift_server {
  int device = 0;
  const swift_index* idx = nullptr;
  swift_params params;
  int64_t budget = 0;      // device bytes for requests in flight
  int64_t in_flight = 0;
  std::vector<Worker> workers;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;
  std::map<int64_t, Request*> all;
  int64_t next_ticket = 1;
  bool stop = false;
};

namespace {

// Device memory a request may take at its peak: per read up to six records
// of pair buffers, results and formatting (about 1.6 KB each), a trace slot
// and seeding state (about 12 KB), the text and the input, plus fixed scan
// and list storage.
int64_t estimate_bytes(int64_t n_reads, size_t len) {
  return n_reads * (6 * 1600 + 12 * 1024) + 4 * (int64_t)len + (96ll << 20);
}

// Page-locked host buffer of at least n bytes (grown, never shrunk).
bool ensure_pinned(char** buf, size_t* cap, size_t n) {
  if (*cap >= n && *buf) return true;
  if (*buf) cudaFreeHost(*buf);
  *buf = nullptr;
  *cap = 0;
  const size_t want = n + n / 4 + (1 << 20);
  if (cudaHostAlloc((void**)buf, want, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    *buf = nullptr;
    return false;
  }
  *cap = want;
  return true;
}

// Runs the requests of one wave and fills their results (called without
// the server lock).
void run_requests(swift_server* s, Worker& w, const std::vector<Request*>& take) {
  size_t bytes = 0, n_reads = 0;
  for (const Request* r : take) {
    bytes += r->reads.size();
    n_reads += r->hr.rd.size();
  }
  std::vector<DevRead> rd;
  rd.reserve(n_reads);
  std::vector<WaveReq> wave(take.size());
  std::string err;
  int rc = SWIFT_OK;
  const char* src = nullptr;
  std::vector<char> host_bytes;  // if no pinned buffer could be had
  if (ensure_pinned(&w.pin_in, &w.pin_in_cap, bytes)) {
    src = w.pin_in;
  } else {
    host_bytes.resize(std::max<size_t>(bytes, 1));
    src = host_bytes.data();
  }
  char* dst = const_cast<char*>(src);
  uint64_t at = 0;
  for (size_t i = 0; i < take.size(); ++i) {
    const Request* r = take[i];
    if (!r->reads.empty()) memcpy(dst + at, r->reads.data(), r->reads.size());
    WaveReq& q = wave[i];
    q.read0 = (int64_t)rd.size();
    q.n = (int64_t)r->hr.rd.size();
    q.Q = r->Q;
    for (int32_t x : r->repeats) q.repeats.push_back((int32_t)(q.read0 + x));
    for (DevRead d : r->hr.rd) {
      d.name_off += at;
      d.seq_off += at;
      rd.push_back(d);
    }
    at += r->reads.size();
  }
  // the text: about the size of the last wave per read, else a first guess
  size_t out_len = 0;
  swift_stats st;
  memset(&st, 0, sizeof(st));
  const size_t guess = n_reads * 520 + (1 << 20);
  ensure_pinned(&w.pin_out, &w.pin_out_cap, std::max(guess, w.pin_out_cap));
  const auto t_wave = Clock::now();
  rc = run_wave(w.ctx, s->idx, &s->params, src, bytes, rd, &wave, w.pin_out,
                w.pin_out ? w.pin_out_cap : 0, &out_len, &st);
  const double wave_ms = ms_between(t_wave, Clock::now());
  if (rc != SWIFT_OK) err = swift_last_error(w.ctx);
  const char* text = nullptr;
  std::vector<char> fetched;
  if (rc == SWIFT_OK) {
    if (w.pin_out && out_len <= w.pin_out_cap) {
      text = w.pin_out;
    } else {  // larger than the staging buffer: fetch it from the device
      fetched.resize(std::max<size_t>(out_len, 1));
      rc = swift_fetch_output(w.ctx, fetched.data(), out_len);
      if (rc != SWIFT_OK) err = swift_last_error(w.ctx);
      text = fetched.data();
      ensure_pinned(&w.pin_out, &w.pin_out_cap, out_len);
    }
  }
  // each request's text out of the wave's (before taking the lock)
  for (size_t i = 0; i < take.size(); ++i) {
    Request* r = take[i];
    r->status = rc;
    if (rc == SWIFT_OK) {
      const size_t len = (size_t)(wave[i].text1 - wave[i].text0);
      r->out = (char*)malloc(len + 1);
      if (!r->out) {
        r->status = SWIFT_E_NOMEM;
        r->error = "host output buffer";
      } else {
        if (len) memcpy(r->out, text + wave[i].text0, len);
        r->out[len] = '\0';
        r->out_len = len;
      }
    } else {
      r->error = err;
    }
    r->reads.clear();
    r->reads.shrink_to_fit();
    r->hr = HostReads();
  }
  const auto now = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  for (size_t i = 0; i < take.size(); ++i) {
    Request* r = take[i];
    r->finished = now;
    r->device_ms = st.total_ms;
    r->wave_ms = wave_ms;
    r->wave_requests = (int64_t)take.size();
    r->wave_reads = (int64_t)n_reads;
    r->state = kDone;
    s->in_flight -= r->est_bytes;
  }
}

int admit(const swift_server* s, Request* r);

void worker(swift_server* s, int wi) {
  Worker& w = s->workers[wi];
  for (;;) {
    std::vector<Request*> take;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      // the oldest request decides the wave's class; it starts when it fits
      // the memory budget beside the waves in flight (a request larger than
      // the whole budget runs when nothing else is in flight)
      s->cv_work.wait(lk, [&] {
        if (s->stop && s->queue.empty()) return true;
        if (s->queue.empty()) return false;
        const Request* f = s->queue.front();
        return s->in_flight + f->est_bytes <= s->budget || s->in_flight == 0;
      });
      if (s->stop && s->queue.empty()) return;
      // requests of query-length classes whose packed shapes are at most
      // twice as tall as each other's share the wave: the wave runs the
      // tallest class's shapes, rows past a shorter query are the
      // all-mismatch rows those shapes compute anyway
      int lo = s->queue.front()->cls, hi = lo;
      int64_t reads = 0, est = 0;
      for (auto it = s->queue.begin(); it != s->queue.end();) {
        Request* r = *it;
        const bool first = take.empty();
        const int64_t nr = r->est_reads;
        const int nlo = std::min(lo, r->cls), nhi = std::max(hi, r->cls);
        if (packed_class_max_q(nhi) <= 2 * packed_class_max_q(nlo) &&
            (first || (reads + nr <= kWaveMaxReads &&
                       s->in_flight + est + r->est_bytes <= s->budget))) {
          take.push_back(r);
          reads += nr;
          est += r->est_bytes;
          lo = nlo;
          hi = nhi;
          it = s->queue.erase(it);
        } else {
          ++it;
        }
      }
      s->in_flight += est;
      const auto now = Clock::now();
      for (Request* r : take) {
        r->started = now;
        r->state = kRunning;
      }
    }
    // parse and check each request (outside the lock); one that fails is
    // done at once with its own error and leaves the wave
    std::vector<Request*> ok, failed;
    std::vector<int> failed_rc;
    for (Request* r : take) {
      const auto t0 = Clock::now();
      const int rc = admit(s, r);
      r->parse_ms = ms_between(t0, Clock::now());
      if (rc == SWIFT_OK) {
        ok.push_back(r);
      } else {
        failed.push_back(r);
        failed_rc.push_back(rc);
      }
    }
    if (!failed.empty()) {
      std::lock_guard<std::mutex> lk(s->mu);
      const auto now = Clock::now();
      for (size_t i = 0; i < failed.size(); ++i) {
        Request* r = failed[i];
        r->status = failed_rc[i];
        r->finished = now;
        r->reads.clear();
        r->reads.shrink_to_fit();
        r->state = kDone;
        s->in_flight -= r->est_bytes;
      }
    }
    if (!ok.empty()) run_requests(s, w, ok);
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
}

// At submission, without parsing: the query length the request will have
// if it is well formed (qry_len, else the first read's line length, one less
// when that line ends the input without a newline, as getSeqSize counts),
// its shape class and a memory estimate from its header count.
void classify(const swift_server* s, Request* r) {
  const char* b = r->reads.data();
  const size_t n = r->reads.size();
  int64_t q = 0;
  const char* nl = n ? (const char*)memchr(b, '\n', n) : nullptr;
  if (nl) {
    const size_t s1 = (size_t)(nl - b) + 1;
    const char* nl2 = s1 < n ? (const char*)memchr(b + s1, '\n', n - s1) : nullptr;
    q = nl2 ? (int64_t)(nl2 - (b + s1)) : (int64_t)(n - s1) - 1;
  }
  const swift_params& p = s->params;
  if (p.qry_len > 0) q = p.qry_len;
  const int c = q >= 1 && q <= kMaxQ ? packed_class((int)q) : 0;
  r->cls = c < 0 ? 0 : c;
  r->est_reads = (int64_t)std::count(b, b + n, '>');
  r->est_bytes = estimate_bytes(r->est_reads, n);
}

// The checks swift_align makes on a request alone, before its wave runs.
int admit(const swift_server* s, Request* r) {
  std::string err;
  const int limit = read_limit_of(&s->params);
  int rc = parse_reads_host(r->reads.data(), r->reads.size(), limit, &r->hr, &err);
  if (rc != SWIFT_OK) {
    r->error = err;
    return rc;
  }
  const swift_params& p = s->params;
  const int Q = p.qry_len > 0 ? p.qry_len : r->hr.first_len;
  if (Q < 1 || Q > kMaxQ) {
    r->error = "query length outside 1.." + std::to_string(kMaxQ);
    return SWIFT_E_LIMIT;
  }
  if (r->hr.n > 0 && r->hr.min_len < Q) {
    r->error = "a read is shorter than the query length; the reference aligns such reads "
               "against stale buffer contents";
    return SWIFT_E_INPUT;
  }
  if (p.seeder == 1 && r->hr.max_len > kReadMax) {
    r->error = "lt13 seeding takes reads of up to 199 bases";
    return SWIFT_E_LIMIT;
  }
  r->Q = Q;
  r->n_reads = r->hr.n;
  r->cls = packed_class(Q);
  if (p.seeder != 1) r->repeats = phase1_stale_repeats(r->hr.n, r->hr.n_gt);
  return SWIFT_OK;
}

}  // namespace

extern "C" {

int swift_server_create(int device, const swift_index* idx, const swift_params* p,
                        int32_t workers, int64_t mem_budget, swift_server** out) {
  if (!idx || !p || !out || workers < 1 || workers > 64) return SWIFT_E_ARG;
  if (p->seed_len != idx->k || p->ignore_thres != idx->thres || p->max_hits < 1 ||
      p->max_hits > 64 || (p->seeder != 0 && p->seeder != 1) || p->max_read_len < 0 ||
      p->max_read_len > kSeedReadMax)
    return SWIFT_E_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return SWIFT_E_CUDA;
  swift_server* s = new swift_server();
  s->device = device;
  s->idx = idx;
  s->params = *p;
  if (mem_budget <= 0) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
      delete s;
      return SWIFT_E_CUDA;
    }
    mem_budget = (int64_t)(fr / 2);
  }
  s->budget = mem_budget;
  s->workers.resize(workers);
  for (int w = 0; w < workers; ++w) {
    swift_ctx* c = nullptr;
    const int rc = swift_ctx_create(device, nullptr, &c);
    if (rc != SWIFT_OK) {
      for (Worker& x : s->workers)
        if (x.ctx) swift_ctx_destroy(x.ctx);
      delete s;
      return rc;
    }
    s->workers[w].ctx = c;
    // staging for a wave of up to kWaveMaxReads reads of 300 bases and
    // their records, pinned once here rather than grown while serving
    ensure_pinned(&s->workers[w].pin_in, &s->workers[w].pin_in_cap, 64ull << 20);
    ensure_pinned(&s->workers[w].pin_out, &s->workers[w].pin_out_cap, 160ull << 20);
  }
  for (int w = 0; w < workers; ++w) s->threads.emplace_back(worker, s, w);
  *out = s;
  return SWIFT_OK;
}

int swift_server_submit(swift_server* s, const char* reads, size_t len, int64_t* ticket) {
  if (!s || (!reads && len) || !ticket) return SWIFT_E_ARG;
  Request* r = new Request();
  r->reads.assign(reads, reads + len);
  r->submitted = Clock::now();
  classify(s, r);  // parsed by the worker that takes it
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
      delete r;
      return SWIFT_E_ARG;
    }
    r->ticket = s->next_ticket++;
    s->all[r->ticket] = r;
    *ticket = r->ticket;
    s->queue.push_back(r);
  }
  s->cv_work.notify_all();
  return SWIFT_OK;
}

int swift_server_poll(swift_server* s, int64_t ticket, int32_t* state) {
  if (!s || !state) return SWIFT_E_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(ticket);
  if (it == s->all.end()) return SWIFT_E_ARG;
  *state = it->second->state;
  return SWIFT_OK;
}

int swift_server_cancel(swift_server* s, int64_t ticket) {
  if (!s) return SWIFT_E_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return SWIFT_E_ARG;
    Request* r = it->second;
    if (r->state != kQueued) return SWIFT_E_LIMIT;  // running or done: too late
    for (auto q = s->queue.begin(); q != s->queue.end(); ++q)
      if (*q == r) {
        s->queue.erase(q);
        break;
      }
    r->state = kCancelled;
    r->status = SWIFT_E_CANCELLED;
    r->error = "request cancelled before it started";
    r->started = r->finished = Clock::now();
  }
  s->cv_done.notify_all();
  s->cv_work.notify_all();  // the queue's head may have changed
  return SWIFT_OK;
}

int swift_server_wait(swift_server* s, int64_t ticket, char** out, size_t* out_len,
                      swift_request_stats* st, char* err, size_t err_cap) {
  if (!s || !out || !out_len) return SWIFT_E_ARG;
  Request* r = nullptr;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return SWIFT_E_ARG;
    r = it->second;
    s->cv_done.wait(lk, [&] { return r->state == kDone || r->state == kCancelled; });
    s->all.erase(it);
  }
  *out = r->out;
  *out_len = r->out_len;
  if (st) {
    memset(st, 0, sizeof(*st));
    st->queue_ms = ms_between(r->submitted, r->started);
    st->run_ms = ms_between(r->started, r->finished);
    st->total_ms = ms_between(r->submitted, r->finished);
    st->reads = r->n_reads;
    st->out_bytes = (int64_t)r->out_len;
    st->device_ms = r->device_ms;
    st->wave_requests = r->wave_requests;
    st->wave_reads = r->wave_reads;
    st->parse_ms = r->parse_ms;
    st->wave_ms = r->wave_ms;
  }
  if (err && err_cap) {
    strncpy(err, r->error.c_str(), err_cap - 1);
    err[err_cap - 1] = '\0';
  }
  const int rc = r->status;
  delete r;
  return rc;
}

int swift_server_destroy(swift_server* s) {
  if (!s) return SWIFT_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (std::thread& t : s->threads) t.join();
  for (auto& kv : s->all) {
    free(kv.second->out);
    delete kv.second;
  }
  for (Worker& w : s->workers) {
    if (w.ctx) swift_ctx_destroy(w.ctx);
    if (w.pin_in) cudaFreeHost(w.pin_in);
    if (w.pin_out) cudaFreeHost(w.pin_out);
  }
  delete s;
  return SWIFT_OK;
}

}  // extern "C"
