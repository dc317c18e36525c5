// Request loop over stc_query_batch (stc_server_* in include/stc.h): worker
// threads answer submitted queries by continuous batching. Queries wait in
// arrival order; an idle worker takes what has arrived as its batch, while
// the device footprint of all batches in flight (records, counters and the
// output records reserved for queries that return contacts) stays within the
// configured budget, and runs it on its own query lane (stream and buffers).
// With QUERY_LANES workers, queries that arrive while a batch is on the GPU
// start at once on the other lane: batches overlap on the device instead of
// queueing behind one another. The device output of a batch is bounded to
// its reservation, so the batches in flight never hold more HBM than they
// were admitted with.
#include <time.h>

#include <algorithm>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "stc.h"

namespace stc {
void set_thread_error(const std::string &msg);
stc_status query_batch_limited(stc_ctx *c, int lane, const stc_query *queries, size_t nq, stc_contact *out,
                               size_t cap, uint64_t *offsets, uint64_t *counts, size_t device_limit,
                               float *gpu_ms);
size_t query_chunk(const stc_ctx *c);
void server_attach(stc_ctx *c, int d);
}

namespace {

constexpr int WORKERS = 2;  // one per query lane of the context (QUERY_LANES)

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
  size_t chunk = 1;                // queries one device pass takes
  std::mutex mu;
  std::condition_variable cv_in, cv_out;
  std::deque<Pending> pending;
  std::deque<Done> done;
  std::thread th[WORKERS];
  bool stopping = false;
  uint64_t next_ticket = 1;
  uint32_t next_batch = 0;
  uint64_t inflight_bytes = 0;     // admitted footprint of the batches on the GPU
  uint32_t busy = 0;               // workers running a batch
  stc_server_stats stats{};
};

static uint64_t footprint(const stc_server &s, const stc_query &q) {
  return QUERY_BYTES + ((q.kind & STC_QUERY_COUNT_ONLY) ? 0 : (uint64_t)s.cfg.result_cap * RECORD_BYTES);
}

// Runs queries qs[0..n) on `lane` with room for `reserve` contacts and fills
// their answers: a contact-returning query gets its contacts when it has at
// most result_cap of them, else STC_ERR_CAPACITY with its count. When the
// batch's matches exceed the reservation (some query is over its cap), the
// queries within their caps run once more on their own; their matches fit
// the reservation by construction.
// A worker's host buffer for a batch's contacts: allocated once to the
// largest reservation seen and never cleared (a batch's reservation runs to
// tens of MB; allocating and zeroing it per batch cost milliseconds).
struct ContactBuf {
  std::unique_ptr<stc_contact[]> p;
  size_t cap = 0;
  stc_contact *at_least(size_t n) {
    if (n > cap) {
      p.reset(new stc_contact[n]);  // default-initialised: no zeroing
      cap = n;
    }
    return p.get();
  }
};

static void answer(stc_server *s, int lane, const std::vector<stc_query> &qs, std::vector<Done> &ready,
                   ContactBuf &buf, float *gpu_ms) {
  const size_t n = qs.size();
  const uint64_t rcap = s->cfg.result_cap;
  size_t reserve = 0;
  for (const stc_query &q : qs)
    if (!(q.kind & STC_QUERY_COUNT_ONLY)) reserve += rcap;
  stc_contact *const out = buf.at_least(std::max<size_t>(reserve, 1));
  std::vector<uint64_t> offsets(n + 1, 0), counts(n, 0);
  stc_status st = stc::query_batch_limited(s->ctx, lane, qs.data(), n, out, reserve, offsets.data(),
                                           counts.data(), std::max<size_t>(reserve, 1), gpu_ms);
  bool wrote = st == STC_OK && offsets[n] <= reserve;
  std::vector<size_t> again;  // contact queries within their cap, when the batch's output was not written
  for (size_t i = 0; i < n; i++) {
    Done &d = ready[i];
    d.a.count = st == STC_OK ? counts[i] : 0;
    d.a.contact_offset = 0;
    d.a.stored = 0;
    d.a.status = (uint32_t)st;
    if (st != STC_OK || (qs[i].kind & STC_QUERY_COUNT_ONLY)) continue;
    if (counts[i] > rcap) {
      d.a.status = STC_ERR_CAPACITY;  // more contacts than its reservation
    } else if (wrote) {
      d.contacts.assign(out + offsets[i], out + offsets[i + 1]);
      d.a.stored = (uint32_t)d.contacts.size();
    } else {
      again.push_back(i);
    }
  }
  if (again.empty()) return;
  std::vector<stc_query> q2(again.size());
  for (size_t j = 0; j < again.size(); j++) q2[j] = qs[again[j]];
  offsets.assign(q2.size() + 1, 0);
  st = stc::query_batch_limited(s->ctx, lane, q2.data(), q2.size(), out, reserve, offsets.data(), nullptr,
                                std::max<size_t>(reserve, 1), nullptr);
  wrote = st == STC_OK && offsets[q2.size()] <= reserve;
  for (size_t j = 0; j < again.size(); j++) {
    Done &d = ready[again[j]];
    if (!wrote) {
      d.a.status = st != STC_OK ? (uint32_t)st : (uint32_t)STC_ERR_CAPACITY;  // the blocks changed meanwhile
      continue;
    }
    d.contacts.assign(out + offsets[j], out + offsets[j + 1]);
    d.a.stored = (uint32_t)d.contacts.size();
  }
}

static void serve(stc_server *s, int lane) {
  std::vector<Pending> take;
  std::vector<stc_query> qs;
  ContactBuf buf;
  for (;;) {
    take.clear();
    uint64_t bytes = 0;
    bool cut = false;
    uint32_t batch_no = 0;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      // work when queries wait and the first of them fits beside the
      // batches in flight (alone, it is always admitted)
      s->cv_in.wait(lk, [&] {
        if (s->pending.empty()) return s->stopping;
        return s->inflight_bytes == 0 ||
               s->inflight_bytes + footprint(*s, s->pending.front().q) <= s->cfg.hbm_budget;
      });
      if (s->pending.empty()) break;  // stopping, and everything answered
      const uint64_t room = s->cfg.hbm_budget > s->inflight_bytes ? s->cfg.hbm_budget - s->inflight_bytes : 0;
      const size_t most = std::min<size_t>(s->cfg.max_batch, s->chunk);
      while (!s->pending.empty() && take.size() < most) {
        const uint64_t f = footprint(*s, s->pending.front().q);
        if (!take.empty() && bytes + f > room) {
          cut = true;
          break;
        }
        bytes += f;
        take.push_back(s->pending.front());
        s->pending.pop_front();
      }
      s->inflight_bytes += bytes;
      if (++s->busy > 1) s->stats.overlapped_batches++;
      batch_no = s->next_batch++;
    }
    // the other worker may take what is left beside this batch
    s->cv_in.notify_one();
    const size_t n = take.size();
    qs.resize(n);
    for (size_t i = 0; i < n; i++) qs[i] = take[i].q;
    std::vector<Done> ready(n);
    const double t_start = mono_now();
    float gpu_ms = 0.f;
    answer(s, lane, qs, ready, buf, &gpu_ms);
    const double t_done = mono_now();
    for (size_t i = 0; i < n; i++) {
      ready[i].a.ticket = take[i].ticket;
      ready[i].a.latency_ms = (t_done - take[i].arrival) * 1e3;
      ready[i].a.batch = batch_no;
      ready[i].a.batch_size = (uint32_t)n;
    }
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (Done &d : ready) s->done.push_back(std::move(d));
      s->inflight_bytes -= bytes;
      s->stats.answered += n;
      s->stats.batches++;
      s->stats.max_batch_queries = std::max<uint64_t>(s->stats.max_batch_queries, n);
      s->stats.max_batch_bytes = std::max<uint64_t>(s->stats.max_batch_bytes, bytes);
      const uint64_t wall_us = (uint64_t)((t_done - t_start) * 1e6);
      if (wall_us > s->stats.slowest_batch_wall_us) {
        s->stats.slowest_batch_wall_us = wall_us;
        s->stats.slowest_batch_gpu_us = (uint64_t)(gpu_ms * 1e3f);
      }
      s->busy--;
      if (cut) s->stats.budget_cuts++;
    }
    s->cv_out.notify_all();
    s->cv_in.notify_all();  // memory freed: a waiting worker may admit now
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
  s->chunk = stc::query_chunk(ctx);
  int started = 0;
  try {
    for (; started < WORKERS; started++) s->th[started] = std::thread(serve, s, started);
  } catch (...) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stopping = true;
    }
    s->cv_in.notify_all();
    for (int i = 0; i < started; i++) s->th[i].join();
    delete s;
    stc::set_thread_error("stc_server_start: cannot start the serving threads");
    return STC_ERR_STATE;
  }
  stc::server_attach(ctx, 1);
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
      // the first answer alone does not fit: it stays queued for a poll
      // with a larger contacts buffer (result_cap contacts always suffice)
      return STC_ERR_CAPACITY;
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
  for (std::thread &t : s->th)
    if (t.joinable()) t.join();
  stc::server_attach(s->ctx, -1);
  delete s;
  return STC_OK;
}
