// Request loop over stc_query_batch (stc_server_* in include/stc.h): one
// thread answers submitted queries by continuous batching. Queries wait in
// arrival order; a batch takes them while its device footprint (records,
// counters and the output records reserved for queries that return
// contacts) stays within the configured budget, and the device output is
// bounded to that reservation, so a batch never holds more HBM than it was
// admitted with.
#include <time.h>

#include <algorithm>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "stc.h"

namespace stc {
void set_thread_error(const std::string &msg);
stc_status query_batch_limited(stc_ctx *c, const stc_query *queries, size_t nq, stc_contact *out, size_t cap,
                               uint64_t *offsets, uint64_t *counts, size_t device_limit);
}

namespace {

double mono_now() {
  timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + (double)ts.tv_nsec * 1e-9;
}

// device bytes a query takes in a batch besides its output: its record, its
// count, its offset and the box-query plan entries of one block
constexpr uint64_t QUERY_BYTES = sizeof(stc_query) + 3 * sizeof(uint64_t);
// device bytes of one output record (the contact and its query index)
constexpr uint64_t RECORD_BYTES = sizeof(stc_contact) + 8;

struct Pending {
  uint64_t ticket;
  stc_query q;
  double arrival;
};

struct Done {
  stc_answer a;
  std::vector<stc_contact> contacts;
};

}  // namespace

struct stc_server {
  stc_ctx *ctx = nullptr;
  stc_server_config cfg{};
  std::mutex mu;
  std::condition_variable cv_in, cv_out;
  std::deque<Pending> pending;
  std::deque<Done> done;
  std::thread th;
  bool stopping = false;
  uint64_t next_ticket = 1;
  stc_server_stats stats{};
};

static uint64_t footprint(const stc_server &s, const stc_query &q) {
  return QUERY_BYTES + ((q.kind & STC_QUERY_COUNT_ONLY) ? 0 : (uint64_t)s.cfg.result_cap * RECORD_BYTES);
}

static void serve(stc_server *s) {
  std::vector<Pending> take;
  std::vector<stc_query> qs;
  std::vector<stc_contact> out;
  std::vector<uint64_t> offsets, counts;
  uint32_t batch_no = 0;
  for (;;) {
    take.clear();
    uint64_t bytes = 0;
    bool cut = false;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_in.wait(lk, [&] { return s->stopping || !s->pending.empty(); });
      if (s->pending.empty()) break;  // stopping, and everything answered
      while (!s->pending.empty() && take.size() < s->cfg.max_batch) {
        const uint64_t f = footprint(*s, s->pending.front().q);
        if (!take.empty() && bytes + f > s->cfg.hbm_budget) {
          cut = true;
          break;
        }
        bytes += f;
        take.push_back(s->pending.front());
        s->pending.pop_front();
      }
    }
    const size_t n = take.size();
    size_t reserve = 0;
    qs.resize(n);
    for (size_t i = 0; i < n; i++) {
      qs[i] = take[i].q;
      if (!(qs[i].kind & STC_QUERY_COUNT_ONLY)) reserve += s->cfg.result_cap;
    }
    out.resize(std::max<size_t>(reserve, 1));
    offsets.assign(n + 1, 0);
    counts.assign(n, 0);
    const stc_status st = stc::query_batch_limited(s->ctx, qs.data(), n, out.data(), reserve, offsets.data(),
                                                   counts.data(), std::max<size_t>(reserve, 1));
    const double t_done = mono_now();
    const bool wrote = st == STC_OK && offsets[n] <= reserve;
    std::vector<Done> ready(n);
    for (size_t i = 0; i < n; i++) {
      Done &d = ready[i];
      d.a.ticket = take[i].ticket;
      d.a.count = st == STC_OK ? counts[i] : 0;
      d.a.contact_offset = 0;
      d.a.stored = 0;
      d.a.status = (uint32_t)st;
      d.a.latency_ms = (t_done - take[i].arrival) * 1e3;
      d.a.batch = batch_no;
      d.a.batch_size = (uint32_t)n;
      if (st == STC_OK && !(qs[i].kind & STC_QUERY_COUNT_ONLY)) {
        if (wrote) {
          d.contacts.assign(out.begin() + (ptrdiff_t)offsets[i], out.begin() + (ptrdiff_t)offsets[i + 1]);
          d.a.stored = (uint32_t)d.contacts.size();
        } else {
          d.a.status = STC_ERR_CAPACITY;  // the batch's matches exceed its reservation
        }
      }
    }
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (Done &d : ready) s->done.push_back(std::move(d));
      s->stats.answered += n;
      s->stats.batches++;
      s->stats.max_batch_queries = std::max<uint64_t>(s->stats.max_batch_queries, n);
      s->stats.max_batch_bytes = std::max<uint64_t>(s->stats.max_batch_bytes, bytes);
      if (cut) s->stats.budget_cuts++;
    }
    s->cv_out.notify_all();
    batch_no++;
  }
}

extern "C" stc_status stc_server_start(stc_ctx *ctx, const stc_server_config *cfg, stc_server **out) {
  if (out) *out = nullptr;
  if (!ctx || !out) {
    stc::set_thread_error("stc_server_start: null argument");
    return STC_ERR_INVALID_ARG;
  }
  stc_server *s = new (std::nothrow) stc_server();
  if (!s) {
    stc::set_thread_error("stc_server_start: out of host memory");
    return STC_ERR_CAPACITY;
  }
  s->ctx = ctx;
  if (cfg) s->cfg = *cfg;
  if (!s->cfg.max_batch) s->cfg.max_batch = 4096;
  if (!s->cfg.result_cap) s->cfg.result_cap = 1024;
  if (!s->cfg.hbm_budget) s->cfg.hbm_budget = 64ull << 20;
  try {
    s->th = std::thread(serve, s);
  } catch (...) {
    delete s;
    stc::set_thread_error("stc_server_start: cannot start the serving thread");
    return STC_ERR_STATE;
  }
  *out = s;
  return STC_OK;
}

extern "C" stc_status stc_server_submit(stc_server *s, const stc_query *queries, size_t nq, double arrival_s,
                                        uint64_t *first_ticket) {
  if (!s || (!queries && nq)) return STC_ERR_INVALID_ARG;
  const double arrival = arrival_s > 0 ? arrival_s : mono_now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) return STC_ERR_STATE;
    if (first_ticket) *first_ticket = s->next_ticket;
    for (size_t i = 0; i < nq; i++) s->pending.push_back(Pending{s->next_ticket++, queries[i], arrival});
    s->stats.submitted += nq;
  }
  s->cv_in.notify_one();
  return STC_OK;
}

extern "C" stc_status stc_server_poll(stc_server *s, stc_answer *out, size_t cap, stc_contact *contacts,
                                      size_t contacts_cap, size_t *n, int wait_ms) {
  if (!s || !n || (!out && cap) || (!contacts && contacts_cap)) return STC_ERR_INVALID_ARG;
  *n = 0;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->done.empty() && wait_ms > 0)
    s->cv_out.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->done.empty(); });
  size_t used = 0;
  while (*n < cap && !s->done.empty()) {
    Done &d = s->done.front();
    if (used + d.contacts.size() > contacts_cap) {
      if (*n) break;  // the rest on the next poll
      d.a.status = STC_ERR_CAPACITY;  // cannot ever fit this poll's buffer
      d.a.stored = 0;
      d.contacts.clear();
    }
    d.a.contact_offset = used;
    if (!d.contacts.empty()) std::copy(d.contacts.begin(), d.contacts.end(), contacts + used);
    used += d.contacts.size();
    out[(*n)++] = d.a;
    s->done.pop_front();
  }
  return STC_OK;
}

extern "C" stc_status stc_server_get_stats(const stc_server *s, stc_server_stats *out) {
  if (!s || !out) return STC_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(const_cast<stc_server *>(s)->mu);
  *out = s->stats;
  return STC_OK;
}

extern "C" stc_status stc_server_stop(stc_server *s) {
  if (!s) return STC_ERR_INVALID_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stopping = true;
  }
  s->cv_in.notify_all();
  if (s->th.joinable()) s->th.join();
  delete s;
  return STC_OK;
}
