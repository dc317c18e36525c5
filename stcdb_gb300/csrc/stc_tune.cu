// Autotuner of the quadtree leaf capacity and the refinement's launch shape
// (stc_autotune). Every candidate runs the same steps from a fresh context,
// so candidates are compared on identical work; the score is the summed
// device time (stc_stats.step_ms) of the steps after the first two, which
// fill the meeting table.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "stc.h"

namespace stc {
void set_thread_error(const std::string &msg);
}

namespace {

constexpr uint32_t TUNE_WARM = 2;  // steps before the timed ones

// Device ms of the timed steps of cfg over xy, or a negative value on error
// (the message is left for stc_last_error(NULL)).
double run_candidate(const stc_config &cfg, const double mbr[4], const double *xy, uint32_t n, uint32_t steps) {
  stc_ctx *c = nullptr;
  if (stc_create(&cfg, mbr, xy, n, &c) != STC_OK) return -1.0;
  std::vector<stc_meeting> sink(1u << 20);  // drained meetings are not kept
  double ms = 0.0;
  for (uint32_t t = 0; t < steps; t++) {
    if (stc_step(c, xy + (size_t)t * n * 2, t) != STC_OK) {
      stc::set_thread_error(std::string("stc_autotune: ") + stc_last_error(c));
      stc_destroy(c);
      return -1.0;
    }
    stc_stats s;
    stc_get_stats(c, &s);
    if (t >= TUNE_WARM) ms += s.step_ms;
    size_t got = sink.size();
    while (got == sink.size())
      if (stc_drain_meetings(c, sink.data(), sink.size(), &got) != STC_OK) {
        stc::set_thread_error(std::string("stc_autotune: ") + stc_last_error(c));
        stc_destroy(c);
        return -1.0;
      }
  }
  stc_destroy(c);
  return ms;
}

}  // namespace

extern "C" stc_status stc_autotune(const stc_config *cfg, const double mbr[4], const double *xy, uint32_t n,
                                   uint32_t steps, const uint32_t *capacities, uint32_t n_capacities,
                                   stc_tune_result *out) {
  if (!cfg || !mbr || !xy || !out || steps < TUNE_WARM + 1 || (n_capacities && !capacities)) {
    stc::set_thread_error("stc_autotune: invalid arguments (steps must be at least 3)");
    return STC_ERR_INVALID_ARG;
  }
  stc_config base = *cfg;
  base.kv_restriction = 0;  // the memtable is not tuned
  base.kv_capacity = 0;
  base.flags = 0;
  std::vector<uint32_t> caps;
  if (n_capacities) caps.assign(capacities, capacities + n_capacities);
  else caps = {std::max<uint32_t>(cfg->grid_capacity / 2, 8u), cfg->grid_capacity, 2 * cfg->grid_capacity};
  // the configuration's own capacity is always a candidate (it gives base_step_ms)
  if (std::find(caps.begin(), caps.end(), cfg->grid_capacity) == caps.end()) caps.insert(caps.begin(), cfg->grid_capacity);
  stc_tune_result r;
  r.config = *cfg;
  r.trials = 0;
  r.reserved = 0;
  r.base_step_ms = 0.0f;
  r.best_step_ms = 0.0f;
  double best = -1.0;
  // 1. leaf capacity
  for (uint32_t cap : caps) {
    stc_config k = base;
    k.grid_capacity = cap;
    const double ms = run_candidate(k, mbr, xy, n, steps);
    r.trials++;
    if (ms < 0) {
      if (cap == cfg->grid_capacity) return STC_ERR_STATE;  // the configuration given must run
      continue;                                          // another capacity may not fit (leaf lists)
    }
    if (cap == cfg->grid_capacity) r.base_step_ms = (float)(ms / (steps - TUNE_WARM));
    if (best < 0 || ms < best) {
      best = ms;
      r.config.grid_capacity = cap;
    }
  }
  if (best < 0) return STC_ERR_STATE;
  // 2. launch shape, one field after the other (0 = the built-in default)
  stc_config k = base;
  k.grid_capacity = r.config.grid_capacity;
  k.job_chunk = cfg->job_chunk ? cfg->job_chunk : 8;  // 0 means these built-in values
  k.refine_chunk = cfg->refine_chunk;  // 0: the per-step automatic choice, itself a candidate
  k.refine_blocks_per_sm = cfg->refine_blocks_per_sm ? cfg->refine_blocks_per_sm : 8;
  k.hits_blocks_per_sm = cfg->hits_blocks_per_sm ? cfg->hits_blocks_per_sm : 16;
  const uint32_t job_chunks[] = {2, 4, 8, 16, 32}, refine_chunks[] = {64, 128, 256, 512},
                 refine_bps[] = {4, 8, 16}, hits_bps[] = {8, 16, 32};
  struct Field {
    uint32_t stc_config::*f;
    const uint32_t *vals;
    int n;
  } fields[] = {{&stc_config::job_chunk, job_chunks, 5},
                {&stc_config::refine_chunk, refine_chunks, 4},
                {&stc_config::refine_blocks_per_sm, refine_bps, 3},
                {&stc_config::hits_blocks_per_sm, hits_bps, 3}};
  for (const Field &fd : fields) {
    uint32_t keep = k.*(fd.f);
    for (int i = 0; i < fd.n; i++) {
      if (fd.vals[i] == k.*(fd.f)) continue;
      stc_config c2 = k;
      c2.*(fd.f) = fd.vals[i];
      const double ms = run_candidate(c2, mbr, xy, n, steps);
      r.trials++;
      if (ms >= 0 && ms < best) {
        best = ms;
        keep = fd.vals[i];
      }
    }
    k.*(fd.f) = keep;
  }
  r.config.job_chunk = k.job_chunk;
  r.config.refine_chunk = k.refine_chunk;
  r.config.refine_blocks_per_sm = k.refine_blocks_per_sm;
  r.config.hits_blocks_per_sm = k.hits_blocks_per_sm;
  r.best_step_ms = (float)(best / (steps - TUNE_WARM));
  *out = r;
  return STC_OK;
}
