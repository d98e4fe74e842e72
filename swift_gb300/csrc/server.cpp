// Serving loop: the reference and index stay resident on the device while
// requests (one reads FASTA each) queue up and run on several concurrent
// pipelines, each a context with its own stream, so a small request does not
// wait behind a large one and the device overlaps them.  A request is
// admitted to a pipeline while the estimated device memory of the requests
// in flight stays within a budget; results are per request and equal to
// what swift_align returns for that request alone.
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Request {
  int64_t ticket = 0;
  std::vector<char> reads;
  int64_t n_reads = 0;     // '>' count, for the memory estimate
  int64_t est_bytes = 0;
  Clock::time_point submitted, started, finished;
  bool done = false;
  int status = SWIFT_OK;
  std::string error;
  char* out = nullptr;     // malloc'ed text, handed to the caller
  size_t out_len = 0;
  swift_stats stats;
};

}  // namespace

struct swift_server {
  int device = 0;
  const swift_index* idx = nullptr;
  swift_params params;
  int64_t budget = 0;      // device bytes for requests in flight
  int64_t in_flight = 0;
  std::vector<swift_ctx*> ctxs;
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

void worker(swift_server* s, int w) {
  swift_ctx* ctx = s->ctxs[w];
  for (;;) {
    Request* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      // first request that fits the budget (a request larger than the
      // whole budget runs when nothing else is in flight)
      s->cv_work.wait(lk, [&] {
        if (s->stop && s->queue.empty()) return true;
        for (Request* q : s->queue)
          if (s->in_flight + q->est_bytes <= s->budget || s->in_flight == 0) return true;
        return false;
      });
      if (s->stop && s->queue.empty()) return;
      for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
        if (s->in_flight + (*it)->est_bytes <= s->budget || s->in_flight == 0) {
          r = *it;
          s->queue.erase(it);
          break;
        }
      }
      s->in_flight += r->est_bytes;
      r->started = Clock::now();
    }
    char* out = nullptr;
    size_t n = 0;
    swift_stats st;
    memset(&st, 0, sizeof(st));
    const int rc = swift_align(ctx, s->idx, r->reads.data(), r->reads.size(), &s->params, &out, &n, &st);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      r->finished = Clock::now();
      r->status = rc;
      if (rc != SWIFT_OK) r->error = swift_last_error(ctx);
      r->out = out;
      r->out_len = n;
      r->stats = st;
      r->done = true;
      r->reads.clear();
      r->reads.shrink_to_fit();
      s->in_flight -= r->est_bytes;
    }
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
}

}  // namespace

extern "C" {

int swift_server_create(int device, const swift_index* idx, const swift_params* p,
                        int32_t workers, int64_t mem_budget, swift_server** out) {
  if (!idx || !p || !out || workers < 1 || workers > 64) return SWIFT_E_ARG;
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
  for (int w = 0; w < workers; ++w) {
    swift_ctx* c = nullptr;
    const int rc = swift_ctx_create(device, nullptr, &c);
    if (rc != SWIFT_OK) {
      for (swift_ctx* x : s->ctxs) swift_ctx_destroy(x);
      delete s;
      return rc;
    }
    s->ctxs.push_back(c);
  }
  for (int w = 0; w < workers; ++w) s->threads.emplace_back(worker, s, w);
  *out = s;
  return SWIFT_OK;
}

int swift_server_submit(swift_server* s, const char* reads, size_t len, int64_t* ticket) {
  if (!s || (!reads && len) || !ticket) return SWIFT_E_ARG;
  Request* r = new Request();
  r->reads.assign(reads, reads + len);
  int64_t n = 0;
  for (size_t i = 0; i < len; ++i) n += reads[i] == '>';
  r->n_reads = n;
  r->est_bytes = estimate_bytes(n, len);
  r->submitted = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
      delete r;
      return SWIFT_E_ARG;
    }
    r->ticket = s->next_ticket++;
    s->all[r->ticket] = r;
    s->queue.push_back(r);
    *ticket = r->ticket;
  }
  s->cv_work.notify_one();
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
    s->cv_done.wait(lk, [&] { return r->done; });
    s->all.erase(it);
  }
  *out = r->out;
  *out_len = r->out_len;
  if (st) {
    memset(st, 0, sizeof(*st));
    st->queue_ms = ms_between(r->submitted, r->started);
    st->run_ms = ms_between(r->started, r->finished);
    st->total_ms = ms_between(r->submitted, r->finished);
    st->reads = r->stats.reads;
    st->out_bytes = (int64_t)r->out_len;
    st->device_ms = r->stats.total_ms;
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
  for (swift_ctx* c : s->ctxs) swift_ctx_destroy(c);
  delete s;
  return SWIFT_OK;
}

}  // extern "C"
