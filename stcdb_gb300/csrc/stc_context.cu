// C ABI (include/stc.h): context lifetime and per-step orchestration.
//
// One context = one device, one stream, all state resident in HBM. A step
// launches only device-driven kernels (sizes that depend on the data are read
// from device memory inside the kernels), then copies the 128-byte control
// block back once to report counters and errors.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "stc_lsm.cuh"
#include "stc_pipeline.cuh"

using namespace stc;

namespace {

thread_local std::string g_create_error = "no error";

enum Phase { PH_START = 0, PH_COPY, PH_PART, PH_BORDER, PH_REFINE, PH_INSERT, PH_SWEEP, PH_APPEND, PH_SCHEMA,
             PH_FLUSH0, PH_FL_OBJECTS, PH_FL_SORT, PH_FL_META, PH_FL_ENCODE, PH_FLUSH1, PH_COUNT };

}  // namespace

namespace stc {
void set_thread_error(const std::string &msg) { g_create_error = msg; }
}  // namespace stc

static constexpr size_t DRAIN_CHUNK = (size_t)8 << 20;  // bytes per pinned staging chunk of a drain
static constexpr uint32_t PAIR_PARTS = 4;                // parts of the pair tests (more while serving)
// Input buffers of a pipelined window: the positions of step i + 3 are
// copied in as soon as step i (that buffer's last reader) has run, two steps
// before they are needed, so that a slow or uneven host link has slack.
static constexpr int WIN_BUFS = 3;

// A large host<->device copy of a step or drain as pieces of COPY_PIECE
// bytes: the copy engine takes them one by one, so that the small copies of
// a query batch on the query stream wait for one piece, not the whole copy.
static constexpr size_t COPY_PIECE = (size_t)16 << 20;
static cudaError_t copy_in_pieces(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  for (size_t off = 0; off < bytes && e == cudaSuccess; off += COPY_PIECE)
    e = cudaMemcpyAsync((uint8_t *)dst + off, (const uint8_t *)src + off, std::min(COPY_PIECE, bytes - off), kind, s);
  return e;
}

struct stc_ctx {
  std::atomic<int> servers{0};  // request loops (stc_server) attached to the context
  stc_config cfg;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;   // border units; the table update beside the pair tests
  cudaStream_t side2 = nullptr;  // the schema update, beside the table update and sweep
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr, fork2_ev = nullptr, join2_ev = nullptr, hits_ev = nullptr;
  cudaEvent_t part_ev[STC_MAX_PARTS] = {};  // end of each part of the pair tests
  cudaEvent_t ev[PH_COUNT] = {};
  std::string err;
  bool failed = false;
  bool stepped = false;
  PipeDev p;
  DevState *st_host = nullptr;   // pinned mirror
  // pinned staging of drained meetings: copies from pinned memory are plain
  // DMA, while copies into the caller's pageable memory go through the
  // driver's staging path, which other threads' copies (queries) wait on
  uint8_t *drain_stage[2] = {nullptr, nullptr};
  cudaEvent_t drain_ev[2] = {nullptr, nullptr};
  double2 *xy_own = nullptr;     // device copy target for host input (and every step of a window)
  // page-locked times of the steps being issued, one word per input buffer
  // (step_begin copies it): a window issues step i + 1 before step i has run
  uint32_t *t_pinned = nullptr;
  // pipelined windows (stc_step_window): per step parity, the state read
  // back after that step's memtable append and the step's events; per input
  // buffer, the end of the core that read it
  DevState *st_slot[2] = {nullptr, nullptr};
  cudaEvent_t st_ev[2] = {nullptr, nullptr};      // the state copy of the step of that parity has landed
  cudaEvent_t core_ev[WIN_BUFS] = {};             // end of the step's core: its input buffer is free
  cudaEvent_t wev[2][4] = {};                     // start of the core, start and end of the append,
                                                  // core's start once its positions are in
  cudaStream_t drain_stream = nullptr;            // meetings of a window go out here beside the next step
  cudaEvent_t drained_ev = nullptr;
  // the step's core captured as a CUDA graph, replayed by stc_step_window;
  // it holds the pipeline's arguments by value, so anything that changes
  // them (a flush, the slice count, a larger hit buffer) invalidates it; one
  // graph per input buffer
  cudaGraphExec_t graph[WIN_BUFS] = {};
  bool graph_valid[WIN_BUFS] = {};
  uint32_t graph_kernels = 0;
  double2 *xy_win[WIN_BUFS - 1] = {};  // a window's other input buffers (allocated on first use)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_ev[WIN_BUFS] = {};
  // start and end of each input copy (its duration in the window's
  // statistics), a ring of twice WIN_BUFS so that step i's are read before
  // step i + 2 * WIN_BUFS records them again
  cudaEvent_t copy_t0[2 * WIN_BUFS] = {}, copy_t1[2 * WIN_BUFS] = {};
  cudaEvent_t sweep_ev[2] = {};    // a window step's sweep start (its next inputs' copy waits for it)
  cudaEvent_t gate_ev = nullptr;   // recorded by issue_step before the insert and sweep, when set
  std::vector<void *> allocs;
  stc_stats stats;
  uint32_t last_t = 0;
  double map[4] = {0, 0, 0, 0};  // map box given at creation
  bool lsm_on = false;           // memtable and flush (kv_restriction > 0)
  LsmDev lsm;
  LsmHost lsmh;
};

static const char *error_name(uint32_t e) {
  switch (e) {
    case ERR_DESCENT: return "descent reached an invalid quadtree node";
    case ERR_UNITS: return "border checking units exceed refine_size * num_objects";
    case ERR_PROBE: return "meeting table probe exceeded the table size (table full)";
    case ERR_CAND: return "new-meeting candidate capacity exceeded";
    case ERR_DA: return "ordered insertion exceeded its iteration bound";
    case ERR_EMIT: return "emit buffer full: drain meetings more often or raise emit_capacity";
    case ERR_SCHEMA: return "quadtree schema or grid stack exhausted";
    case ERR_LOOKUP: return "border lookup stack overflow";
    case ERR_BUILD: return "initial quadtree exceeds schema capacity";
    case ERR_MEMTABLE: return "memtable full: raise kv_capacity";
    default: return "unknown device error";
  }
}

static stc_status status_of(uint32_t e) {
  switch (e) {
    case ERR_UNITS: case ERR_PROBE: case ERR_CAND: case ERR_EMIT: case ERR_SCHEMA: case ERR_LOOKUP: case ERR_BUILD:
    case ERR_MEMTABLE:
      return STC_ERR_CAPACITY;
    case ERR_DA: return STC_ERR_TIMEOUT;
    default: return STC_ERR_STATE;
  }
}

template <typename T>
static bool dalloc(stc_ctx *c, T **ptr, size_t count) {
  size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  void *v = nullptr;
  cudaError_t e = cudaMalloc(&v, bytes);
  if (e != cudaSuccess) {
    char buf[256];
    snprintf(buf, sizeof(buf), "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
    c->err = buf;
    *ptr = nullptr;
    return false;
  }
  c->allocs.push_back(v);
  *ptr = (T *)v;
  return true;
}

static stc_status fail(stc_ctx *c, stc_status s, const std::string &msg) {
  c->err = msg;
  if (s != STC_ERR_INVALID_ARG) c->failed = true;
  return s;
}

static stc_status cuda_fail(stc_ctx *c, cudaError_t e, const char *where) {
  char buf[256];
  snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
  return fail(c, STC_ERR_CUDA, buf);
}

static uint64_t next_pow2(uint64_t v) {
  uint64_t r = 1;
  while (r < v) r <<= 1;
  return r;
}

extern "C" void stc_config_default(stc_config *cfg, uint32_t n) {
  if (!cfg) return;
  memset(cfg, 0, sizeof(*cfg));
  cfg->num_objects = n;
  cfg->min_meet_time = 5;
  cfg->max_meet_time = 4096;
  cfg->grid_capacity = 50;
  cfg->grid_amplify = 2.0;
  cfg->reach_distance = 2.0;
  cfg->num_meeting_buckets = 2ULL * n;
  cfg->refine_size = 4;
  cfg->schema_update_delay = 1;
  cfg->dynamic_schema = 1;
  cfg->mbr_filter = 1;
}

static void destroy_all(stc_ctx *c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  lsm_release(c->lsmh);
  for (void *v : c->allocs) cudaFree(v);
  c->allocs.clear();
  if (c->drain_stream) cudaStreamSynchronize(c->drain_stream);
  if (c->st_host) cudaFreeHost(c->st_host);
  if (c->t_pinned) cudaFreeHost(c->t_pinned);
  for (int i = 0; i < 2; i++) {
    if (c->st_slot[i]) cudaFreeHost(c->st_slot[i]);
    if (c->st_ev[i]) cudaEventDestroy(c->st_ev[i]);
    for (cudaEvent_t ev : c->wev[i])
      if (ev) cudaEventDestroy(ev);
  }
  if (c->drained_ev) cudaEventDestroy(c->drained_ev);
  if (c->drain_stream) cudaStreamDestroy(c->drain_stream);
  for (int i = 0; i < WIN_BUFS; i++) {
    if (c->graph[i]) cudaGraphExecDestroy(c->graph[i]);
    if (c->copy_ev[i]) cudaEventDestroy(c->copy_ev[i]);
    if (c->core_ev[i]) cudaEventDestroy(c->core_ev[i]);
  }
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  for (cudaEvent_t ev : c->sweep_ev)
    if (ev) cudaEventDestroy(ev);
  for (int i = 0; i < 2 * WIN_BUFS; i++) {
    if (c->copy_t0[i]) cudaEventDestroy(c->copy_t0[i]);
    if (c->copy_t1[i]) cudaEventDestroy(c->copy_t1[i]);
  }
  for (int i = 0; i < 2; i++) {
    if (c->drain_stage[i]) cudaFreeHost(c->drain_stage[i]);
    if (c->drain_ev[i]) cudaEventDestroy(c->drain_ev[i]);
  }
  for (int i = 0; i < PH_COUNT; i++)
    if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  if (c->fork_ev) cudaEventDestroy(c->fork_ev);
  if (c->fork2_ev) cudaEventDestroy(c->fork2_ev);
  if (c->hits_ev) cudaEventDestroy(c->hits_ev);
  for (cudaEvent_t ev : c->part_ev)
    if (ev) cudaEventDestroy(ev);
  if (c->join2_ev) cudaEventDestroy(c->join2_ev);
  if (c->join_ev) cudaEventDestroy(c->join_ev);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->side2) cudaStreamDestroy(c->side2);
  if (c->stream) cudaStreamDestroy(c->stream);
}

extern "C" void stc_destroy(stc_ctx *c) {
  if (!c) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(c->device);
  destroy_all(c);
  cudaSetDevice(prev);
  delete c;
}

extern "C" const char *stc_last_error(const stc_ctx *c) {
  if (!c) return g_create_error.c_str();
  return c->err.empty() ? "no error" : c->err.c_str();
}

static stc_status read_state(stc_ctx *c, const char *where) {
  cudaError_t e = cudaMemcpyAsync(c->st_host, c->p.st, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, where);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(c, e, where);
  if (c->st_host->error) {
    char buf[320];
    snprintf(buf, sizeof(buf), "%s: %s (code %u, info %u)", where, error_name(c->st_host->error),
             c->st_host->error, c->st_host->error_info);
    return fail(c, status_of(c->st_host->error), buf);
  }
  return STC_OK;
}

// Creates a context; builds the quadtree from xy0 unless xy0 is null (a
// restore fills the schema from a checkpoint instead).
static stc_status create_ctx(const stc_config *cfg, const double mbr[4], const double *xy0, uint32_t n,
                             stc_ctx **out);

extern "C" stc_status stc_create(const stc_config *cfg, const double mbr[4], const double *xy0, uint32_t n,
                                 stc_ctx **out) {
  if (out) *out = nullptr;
  if (!xy0) {
    g_create_error = "stc_create: null argument";
    return STC_ERR_INVALID_ARG;
  }
  return create_ctx(cfg, mbr, xy0, n, out);
}

static stc_status create_ctx(const stc_config *cfg, const double mbr[4], const double *xy0, uint32_t n,
                             stc_ctx **out) {
  if (out) *out = nullptr;
  if (!cfg || !mbr || !out) {
    g_create_error = "stc_create: null argument";
    return STC_ERR_INVALID_ARG;
  }
  const stc_config &k = *cfg;
  double amp_cap = k.grid_amplify * k.grid_capacity;
  if (n == 0 || n != k.num_objects || n >= (1u << 31) || k.grid_capacity == 0 || !(k.reach_distance > 0) ||
      k.num_meeting_buckets < 2 || k.refine_size == 0 || k.schema_update_delay == 0 || !(amp_cap >= 1.0) ||
      amp_cap >= (double)STC_MAX_LEAF_CAP || !(mbr[2] > mbr[0]) || !(mbr[3] > mbr[1])) {
    g_create_error = "stc_create: invalid configuration";
    return STC_ERR_INVALID_ARG;
  }
  const uint32_t ctf_count = k.ctf_count ? k.ctf_count : 100;  // util/config.h:59
  const uint32_t split = (uint32_t)std::lround(std::sqrt((double)ctf_count));
  if (k.kv_restriction &&
      (split * split != ctf_count || ctf_count > 3969 || n >= (1u << 26) || k.max_meet_time == 0 ||
       k.area_restriction < 0 || (k.kv_capacity && k.kv_capacity <= k.kv_restriction) ||
       k.kv_restriction >= (1ull << 31) || k.kv_capacity >= (1ull << 31))) {
    g_create_error = "stc_create: invalid memtable configuration (ctf_count must be a square <= 3969, "
                     "num_objects < 2^26, kv_capacity > kv_restriction, both < 2^31)";
    return STC_ERR_INVALID_ARG;
  }
  if (k.refine_chunk % 32 || k.refine_chunk > 4096) {
    g_create_error = "stc_create: refine_chunk must be 0 (256) or a multiple of 32 up to 4096";
    return STC_ERR_INVALID_ARG;
  }
  if (k.bitmap_edge % 32 || k.bitmap_edge > 1024) {
    g_create_error = "stc_create: bitmap_edge must be 0 (256) or a multiple of 32 up to 1024";
    return STC_ERR_INVALID_ARG;
  }
  const uint32_t bm_edge = k.bitmap_edge ? k.bitmap_edge : 256;  // util/util.h:47
  stc_ctx *c = new (std::nothrow) stc_ctx();
  if (!c) {
    g_create_error = "stc_create: out of host memory";
    return STC_ERR_CAPACITY;
  }
  c->cfg = k;
  c->device = (int)k.device;
  for (int i = 0; i < 4; i++) c->map[i] = mbr[i];
  memset(&c->stats, 0, sizeof(c->stats));
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork2_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join2_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->hits_ev, cudaEventDisableTiming);
  for (uint32_t i = 0; i < STC_MAX_PARTS && e == cudaSuccess; i++)
    e = cudaEventCreateWithFlags(&c->part_ev[i], cudaEventDisableTiming);
  for (int i = 0; i < PH_COUNT && e == cudaSuccess; i++) e = cudaEventCreate(&c->ev[i]);
  if (e == cudaSuccess) e = cudaMallocHost(&c->st_host, sizeof(DevState));
  if (e == cudaSuccess) e = cudaMallocHost(&c->t_pinned, WIN_BUFS * sizeof(uint32_t));
  for (int i = 0; i < 2 && e == cudaSuccess; i++) {
    e = cudaMallocHost(&c->st_slot[i], sizeof(DevState));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->st_ev[i], cudaEventDisableTiming);
    for (int j = 0; j < 4 && e == cudaSuccess; j++) e = cudaEventCreate(&c->wev[i][j]);
  }
  for (int i = 0; i < WIN_BUFS && e == cudaSuccess; i++) e = cudaEventCreate(&c->core_ev[i]);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->drain_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->drained_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = schema_prepare();
  for (int i = 0; i < 2 && e == cudaSuccess; i++) {
    e = cudaMallocHost(&c->drain_stage[i], DRAIN_CHUNK);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->drain_ev[i], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    g_create_error = std::string("stc_create: ") + cudaGetErrorString(e);
    destroy_all(c);
    delete c;
    return STC_ERR_CUDA;
  }

  PipeDev &p = c->p;
  memset(&p, 0, sizeof(p));
  p.N = n;
  p.leaf_cap = (uint32_t)amp_cap;  // tracing/workbench.cpp:36
  uint32_t per = n / k.grid_capacity;
  p.G = 4 * std::max<uint32_t>(100000u, per);  // tracing/workbench.cpp:38
  p.S = (uint32_t)(1.6 * p.G);                 // tracing/workbench.cpp:41
  p.B = k.num_meeting_buckets;
  // only pairs found twice in one step (two border units targeting each
  // other's leaves) pass through the candidate set
  uint64_t cand_cap = k.candidate_capacity ? k.candidate_capacity
                                           : std::max<uint64_t>(1u << 20, std::min<uint64_t>(p.B / 2, 2ULL * n));
  p.cand_cap = cand_cap;
  p.C = next_pow2(2 * cand_cap);
  p.E = k.emit_capacity ? k.emit_capacity : std::max<uint64_t>(1u << 20, 4ULL * n);
  // hits beyond the buffer are applied inside the refinement instead
  p.hit_cap = k.hit_capacity ? k.hit_capacity : std::max<uint64_t>(1u << 22, 8ULL * n);
  p.U_cap = (uint64_t)k.refine_size * n - n;
  p.reach = k.reach_distance;
  p.x_buffer = k.reach_distance * stc_dpml_ref(mbr[1]);  // tracing/filter.cpp:30
  p.y_buffer = k.reach_distance * stc_dpm_lat();          // tracing/filter.cpp:31
  p.map_lo_x = mbr[0]; p.map_lo_y = mbr[1]; p.map_hi_x = mbr[2]; p.map_hi_y = mbr[3];
  {
    // for a float f and double D: f >= D <=> f >= (smallest float >= D), and
    // f <= D <=> f <= (largest float <= D)
    auto up = [](double d) { float f = (float)d; return (double)f < d ? nextafterf(f, INFINITY) : f; };
    auto down = [](double d) { float f = (float)d; return (double)f > d ? nextafterf(f, -INFINITY) : f; };
    p.fmap_lo_x = up(mbr[0]); p.fmap_lo_y = up(mbr[1]); p.fmap_hi_x = down(mbr[2]); p.fmap_hi_y = down(mbr[3]);
  }
  p.B_magic = (unsigned long long)(((unsigned __int128)1 << 64) / p.B + (((unsigned __int128)1 << 64) % p.B != 0));
  p.min_meet_time = k.min_meet_time;
  p.grid_capacity = k.grid_capacity;
  p.delay = k.schema_update_delay;
  p.mbr_filter = k.mbr_filter;
  p.slices = std::min<uint32_t>(std::max<uint32_t>(k.step_slices, 1u), 64u);
  p.job_chunk = k.job_chunk ? std::min<uint32_t>(k.job_chunk, 64u) : 8u;
  p.refine_chunk = k.refine_chunk ? k.refine_chunk : REFINE_CHUNK_DEFAULT;
  p.refine_bps = k.refine_blocks_per_sm ? std::min<uint32_t>(k.refine_blocks_per_sm, 32u) : 8u;
  p.hits_bps = k.hits_blocks_per_sm ? std::min<uint32_t>(k.hits_blocks_per_sm, 64u) : 16u;

  size_t nu = std::max<size_t>(n, p.U_cap);
  size_t scan_words = scan_tmp_words(std::max<size_t>({(size_t)n, (size_t)p.G + 1, (size_t)p.S,
                                                      radix_hist_words(nu)}));
  bool ok = dalloc(c, &p.st, 1) && dalloc(c, &c->xy_own, n) && dalloc(c, &p.sd.nodes, p.S) &&
            dalloc(c, &p.sd.meta, p.S) && dalloc(c, &p.sd.schema_stack, p.S) && dalloc(c, &p.sd.grids_stack, p.G) &&
            dalloc(c, &p.sd.gid_node, p.G) && dalloc(c, &p.sw.bnodes, p.S) && dalloc(c, &p.sw.bmeta, p.S) &&
            dalloc(c, &p.sw.bcount, p.S) && dalloc(c, &p.sw.bsub_nodes, p.S) &&
            dalloc(c, &p.sw.bsub_leaves, p.S) && dalloc(c, &p.sw.bpre, p.S) && dalloc(c, &p.sw.bleafbase, p.S) &&
            dalloc(c, &p.sw.node_of, n) && dalloc(c, &p.sw.ev_flag, p.S) && dalloc(c, &p.sw.ev_pos, p.S) &&
            dalloc(c, &p.sw.ev_list, p.S) && dalloc(c, &p.sw.old_under, p.S) && dalloc(c, &p.sw.heap, p.S) &&
            dalloc(c, &p.sw.ev_total, 2) && dalloc(c, &p.sw.par_scratch, 10 * 8192) && dalloc(c, &p.sw.queued, p.S) && dalloc(c, &p.leaf_gid, n) &&
            dalloc(c, &p.lastvalid, n) && dalloc(c, &p.iota, nu) && dalloc(c, &p.sorted_gid, n) &&
            dalloc(c, &p.sorted_pid, n) && dalloc(c, &p.sort_ktmp, nu) && dalloc(c, &p.sort_vtmp, nu) &&
            dalloc(c, &p.sort_hist, radix_hist_words(nu)) && dalloc(c, &p.grid_count, (size_t)p.G + 1) &&
            dalloc(c, &p.sort_ktmp2, nu) && dalloc(c, &p.sort_vtmp2, nu) &&
            dalloc(c, &p.hit_bounds, STC_MAX_PARTS + 1) &&
            dalloc(c, &p.sort_hist2, radix_hist_words(nu)) && dalloc(c, &p.scan_tmp2, scan_words) &&
            dalloc(c, &p.grid_start, (size_t)p.G + 1) && dalloc(c, &p.pts, n) && dalloc(c, &p.fxy, n) &&
            dalloc(c, &p.gfxy, n) && dalloc(c, &p.sfxy, n) &&
            dalloc(c, &p.spts, n) && dalloc(c, &p.sorig, n) && dalloc(c, &p.scand, n) &&
            dalloc(c, &p.lstrip, p.G) && dalloc(c, &p.cchunks, p.G) &&
            dalloc(c, &p.bcount, (size_t)n + 1) && dalloc(c, &p.boff, (size_t)n + 1) &&
            dalloc(c, &p.blist, n) && dalloc(c, &p.bres, 4 * (size_t)n) && dalloc(c, &p.sd.fbox, p.S) &&
            dalloc(c, &p.bu_gid, p.U_cap) && dalloc(c, &p.bu_pid, p.U_cap) && dalloc(c, &p.bu_sorted_gid, p.U_cap) &&
            dalloc(c, &p.bu_sorted_pos, p.U_cap) && dalloc(c, &p.bu_cnt, (size_t)p.G + 1) &&
            dalloc(c, &p.bu_start, (size_t)p.G + 1) && dalloc(c, &p.job_cnt, (size_t)p.G + 1) &&
            dalloc(c, &p.job_start, (size_t)p.G + 1) && dalloc(c, &p.slots, p.B) && dalloc(c, &p.hits, p.hit_cap) && dalloc(c, &p.cset, p.C) &&
            dalloc(c, &p.cand_list, p.cand_cap) && dalloc(c, &p.emit, p.E) && dalloc(c, &p.scan_tmp, scan_words) &&
            dalloc(c, &p.n_dev, 1);
  if (ok && k.kv_restriction) {
    LsmDev &L = c->lsm;
    memset(&L, 0, sizeof(L));
    c->lsm_on = true;
    L.N = n;
    L.max_meet = k.max_meet_time;
    L.F = ctf_count;
    L.split = split;
    L.end_time_min = k.start_time + k.min_meet_time;  // tracing/process.cpp:404
    L.area = k.area_restriction > 0 ? k.area_restriction : 100.0;  // process.cpp:408-411: 100 = no cut
    L.map[0] = mbr[0]; L.map[1] = mbr[1]; L.map[2] = mbr[2]; L.map[3] = mbr[3];
    L.edge = bm_edge;
    // a step adds at most two keys per emitted meeting, so the default never overflows
    L.cap = k.kv_capacity ? k.kv_capacity
                          : std::min<unsigned long long>(k.kv_restriction + 2 * p.E, (1ull << 31) - 1);
    size_t w = lsm_sort_words(L);
    size_t hw = radix_hist_words(w);
    ok = dalloc(c, &L.rec, L.cap) && dalloc(c, &L.box, L.cap) && dalloc(c, &L.brec, L.cap) &&
         dalloc(c, &L.bbox, L.cap) && dalloc(c, &L.over, L.cap) && dalloc(c, &L.hist, hw) &&
         dalloc(c, &L.scan, scan_tmp_words(hw)) && dalloc(c, &L.n_dev, 6) && dalloc(c, &L.cnt, n) &&
         dalloc(c, &L.obox, n) && dalloc(c, &L.sid, n) && dalloc(c, &L.bsid, n) && dalloc(c, &L.mid_lo, n) &&
         dalloc(c, &L.mid_hi, n) && dalloc(c, &L.ctf_cap, ctf_count) && dalloc(c, &L.ctf_first, ctf_count + 1) &&
         dalloc(c, &L.ctfs, ctf_count) && dalloc(c, &L.lim_box, ctf_count) && dalloc(c, &L.lim_time, ctf_count) &&
         dalloc(c, &L.bitmaps, (size_t)ctf_count * (STC_BITMAP_BYTES / 4)) &&
         dalloc(c, &L.obitmap, STC_MAP_BITMAP_BYTES(bm_edge) / 4) && dalloc(c, &L.kbytes, 16 * (size_t)L.cap);
    for (int i = 0; ok && i < 7; i++) ok = dalloc(c, &L.sk[i], w);
    L.st = p.st;
    LsmHost &H = c->lsmh;
    H.retain = k.ctb_retain ? k.ctb_retain : 8;
    H.edge = bm_edge;
    for (int i = 0; i < 4; i++) H.map[i] = mbr[i];
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    // query lanes (streams of the highest priority) and their buffers now:
    // allocating them later would wait for a step in flight
    std::string qerr;
    if (ok && lsm_query_reserve(H, 4096, ctf_count, greatest, qerr) != STC_OK) {
      c->err = qerr;
      ok = false;
    }
  }
  if (!ok) {
    g_create_error = "stc_create: " + c->err;
    destroy_all(c);
    delete c;
    return STC_ERR_CAPACITY;
  }
  p.sd.S = p.S;
  p.sd.G = p.G;
  p.sd.ox = mbr[0];
  p.sd.oy = mbr[1];
  {
    // fp32 band of the border lookup pre-filter: offsets from the map corner
    // are at most its extent W; each of the ~8 fp32 roundings on the path to
    // the degree distance adds <= u W, scaled to metres by <= 111.4 km/deg.
    const double u = 5.9604644775390625e-08;
    double ext_m = (mbr[2] - mbr[0]) * 111322.3 + (mbr[3] - mbr[1]) * 111322.3;
    p.border_delta = (float)(32.0 * u * ext_m + 64.0 * u * k.reach_distance + 1e-6 * k.reach_distance);
  }
  p.sw.scan_tmp = p.scan_tmp;
  cudaStream_t s = c->stream;
  cudaMemsetAsync(p.st, 0, sizeof(DevState), s);
  cudaMemsetAsync(p.sw.queued, 0, p.S, s);
  unsigned long long nn = n;
  cudaMemcpyAsync(p.n_dev, &nn, sizeof(nn), cudaMemcpyHostToDevice, s);
  iota_u32(p.iota, nu, s);
  init_tables(p, s);
  if (c->lsm_on) lsm_init(c->lsm, s);
  e = cudaSuccess;
  if (xy0) {
    e = cudaMemcpyAsync(c->xy_own, xy0, (size_t)n * sizeof(double2), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = build_schema(c->xy_own, n, mbr, k.reach_distance, k.grid_capacity, p.sd, p.sw, p.st, c->st_host, s);
  }
  stc_status rs = STC_OK;
  if (e != cudaSuccess) rs = cuda_fail(c, e, "stc_create");
  else rs = read_state(c, "stc_create");
  if (rs != STC_OK) {
    g_create_error = c->err;
    destroy_all(c);
    delete c;
    return rs;
  }
  c->stats.leaves = c->st_host->grids_stack_index;
  c->stats.schema_nodes = c->st_host->schema_stack_index;
  *out = c;
  return STC_OK;
}

static void invalidate_graphs(stc_ctx *c) {
  for (bool &v : c->graph_valid) v = false;
}

// Input buffer b of a window: the context's own copy target, then the
// buffers allocated for windows.
static double2 *window_buffer(stc_ctx *c, int b) { return b ? c->xy_win[b - 1] : c->xy_own; }

static stc_status flush_now(stc_ctx *c, uint32_t t) {
  invalidate_graphs(c);  // the memtable's arguments change
  cudaEventRecord(c->ev[PH_FLUSH0], c->stream);
  unsigned long long launches0 = tl_launches;
  std::string err;
  stc_status rs = lsm_flush(c->lsm, c->lsmh, t, c->stream, c->st_host, err, &c->ev[PH_FL_OBJECTS]);
  if (rs != STC_OK) return fail(c, rs, "stc flush: " + err);
  if (c->st_host->error) return read_state(c, "stc flush");
  rs = lsm_store_block(c->lsm, c->lsmh, c->stream, err);
  if (rs != STC_OK) return fail(c, rs, "stc flush: " + err);
  cudaEventRecord(c->ev[PH_FLUSH1], c->stream);
  cudaError_t e = cudaEventSynchronize(c->ev[PH_FLUSH1]);
  if (e != cudaSuccess) return cuda_fail(c, e, "stc flush");
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev[PH_FLUSH0], c->ev[PH_FLUSH1]);
  c->stats.flush_ms = ms;
  for (int i = 0; i < 5; i++) {
    float st = 0;
    cudaEventElapsedTime(&st, c->ev[PH_FLUSH0 + i], c->ev[PH_FLUSH0 + i + 1]);
    c->stats.flush_stage_ms[i] = st;
  }
  c->stats.flushes = c->lsmh.flushes;
  c->stats.memtable_keys = c->st_host->kv_count;
  c->stats.kernel_launches += (uint32_t)(tl_launches - launches0);
  return STC_OK;
}

// The step's device work, in stream order (phase events only when not being
// captured into a graph). `tword` is the page-locked word holding the step's
// time. The memtable append is part of it only when `append` is set: a
// pipelined window issues it separately, after the flush decision of the
// step before.
static void issue_step(stc_ctx *c, bool events, bool append, const uint32_t *tword) {
  PipeDev &p = c->p;
  cudaStream_t s = c->stream;
  step_begin(p, tword, s);
  if (events) cudaEventRecord(c->ev[PH_COPY], s);
  step_descend(p, s);
  // the border units (lookups, scan, sort by leaf) need the descent only:
  // they run on the side stream, with their own scratch, beside the
  // leaf-order sort and gather
  cudaEventRecord(c->fork2_ev, s);
  cudaStreamWaitEvent(c->side, c->fork2_ev, 0);
  step_border(p, c->side);
  cudaEventRecord(c->join2_ev, c->side);
  step_leaf_order(p, s);
  step_strips(p, s);
  if (events) cudaEventRecord(c->ev[PH_PART], s);
  cudaStreamWaitEvent(s, c->join2_ev, 0);
  step_jobs(p, s);
  if (events) cudaEventRecord(c->ev[PH_BORDER], s);
  // The pair tests run in parts; each part's hits are applied to the table
  // on the side stream while the next part's pairs are tested (the two
  // kernels are bound by different units; concurrent table updates are safe,
  // new meetings take their slots by priority).
  const uint32_t parts = std::min<uint32_t>(std::max<uint32_t>(p.slices, PAIR_PARTS), STC_MAX_PARTS);
  for (uint32_t part = 0; part < parts; part++) {
    step_pairs_part(p, part, parts, s);
    cudaEventRecord(c->part_ev[part], s);
    cudaStreamWaitEvent(c->side, c->part_ev[part], 0);
    step_hits_part(p, part, parts, c->side);
  }
  cudaEventRecord(c->hits_ev, c->side);
  // The schema update reads this step's leaf counts and rewrites quadtree
  // nodes, which only the pair tests read: once they are done it runs on a
  // third stream while the table update, insert, sweep and memtable append
  // run (none of them touches the schema or its scan scratch), and the step
  // ends when all have.
  const bool schema = c->cfg.dynamic_schema != 0;
  if (schema) {
    cudaStreamWaitEvent(c->side2, c->part_ev[parts - 1], 0);
    update_schema(p.sd, p.sw, p.grid_count, p.reach, p.grid_capacity, p.delay,
                  (c->cfg.flags & STC_FLAG_SERIAL_SCHEMA) != 0, p.st, c->side2);
    cudaEventRecord(c->join_ev, c->side2);
  }
  cudaStreamWaitEvent(s, c->hits_ev, 0);
  if (events) cudaEventRecord(c->ev[PH_REFINE], s);
  if (c->gate_ev) cudaEventRecord(c->gate_ev, s);
  step_insert(p, s);
  if (events) cudaEventRecord(c->ev[PH_INSERT], s);
  step_sweep(p, s);
  if (events) cudaEventRecord(c->ev[PH_SWEEP], s);
  if (append && c->lsm_on) lsm_append(p, c->lsm, s);
  if (events) cudaEventRecord(c->ev[PH_APPEND], s);
  if (schema) cudaStreamWaitEvent(s, c->join_ev, 0);
}

// Captures the step's core (without the memtable append) with positions in
// window input buffer b and its time in t_pinned[b] as a CUDA
// graph. Only this thread's work on the context's streams is captured: a
// serving thread's queries on other streams go on meanwhile.
static stc_status capture_step(stc_ctx *c, int b) {
  if (c->graph[b]) {
    cudaGraphExecDestroy(c->graph[b]);
    c->graph[b] = nullptr;
  }
  c->graph_valid[b] = false;
  c->p.xy = window_buffer(c, b);
  const unsigned long long l0 = tl_launches;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    issue_step(c, false, false, c->t_pinned + b);
    e = cudaStreamEndCapture(c->stream, &g);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&c->graph[b], g, 0);
  if (g) cudaGraphDestroy(g);
  c->graph_kernels = (uint32_t)(tl_launches - l0);
  tl_launches = l0;  // counted when replayed
  if (e != cudaSuccess) {
    c->graph[b] = nullptr;
    return cuda_fail(c, e, "capturing the step graph");
  }
  c->graph_valid[b] = true;
  return STC_OK;
}

// Counters of the step whose state is in c->st_host.
static void fill_stats(stc_ctx *c, uint32_t t, const float *phase, float step_ms, uint32_t launches) {
  const DevState &h = *c->st_host;
  const PipeDev &p = c->p;
  stc_stats &o = c->stats;
  o.step = t;
  o.leaves = h.grids_stack_index;
  o.schema_nodes = h.schema_stack_index;
  o.overflow_objects = h.overflow_objects;
  o.border_units = h.border_units;
  o.checking_units = h.border_units + p.N;
  o.pair_tests = h.tests;
  o.exact_tests = h.exact_tests;
  o.hits = h.hits;
  o.new_candidates = h.fast_claims;  // new meetings started by the step
  o.taken_buckets = h.taken;
  o.emitted = h.step_emitted;
  o.pending = std::min<unsigned long long>(h.emit_count, p.E);
  o.splits = h.splits;
  o.merges = h.merges;
  for (int i = 0; i < 8; i++) o.phase_ms[i] = phase ? phase[i] : 0.f;
  o.ambiguous_tests = (uint32_t)h.ambiguous;
  o.kernel_launches = launches;
  o.schema_path = h.schema_path;
  o.step_ms = step_ms;
  o.memtable_keys = h.kv_count;
  c->stepped = true;
  c->last_t = t;
}

// The reference flushes once a step leaves more keys than kv_restriction
// (cuda/geometry.cu:1752).
static bool flush_due(const stc_ctx *c) { return c->lsm_on && c->st_host->kv_count > c->cfg.kv_restriction; }

// With the automatic hit capacity (stc_config.hit_capacity 0) the hit buffer
// grows to the largest step seen: hits beyond it are applied inside the pair
// tests, which is correct but slow (they hold the pair-test warps on random
// table accesses). Called only with no step in flight; a failed allocation
// keeps the old buffer.
static void grow_hits(stc_ctx *c, unsigned long long need) {
  PipeDev &p = c->p;
  if (c->cfg.hit_capacity || need <= p.hit_cap) return;
  const unsigned long long cap = next_pow2(need + need / 4);
  void *h = nullptr;
  if (cudaMalloc(&h, cap * sizeof(HitRec)) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  for (void *&a : c->allocs)
    if (a == (void *)p.hits) {
      cudaFree(a);
      a = h;
    }
  p.hits = (HitRec *)h;
  p.hit_cap = cap;
  invalidate_graphs(c);  // the graphs hold the buffer by value
}

// How the pair tests hand over their hits: straight to the hit buffer when
// the last step found many hits per checking unit (dense leaves: hotspot-1M
// has about 17, its refinement 6.35 -> 5.94 ms a step that way), through a
// per-warp shared-memory queue otherwise (uniform-10M has about 6; the direct
// form's extra registers cost it 0.08 ms). Results do not depend on it.
static constexpr unsigned long long DIRECT_HITS_PER_UNIT = 12;
static void choose_hit_emission(stc_ctx *c) {
  PipeDev &p = c->p;
  uint32_t direct;
  if (c->cfg.flags & STC_FLAG_DIRECT_HITS) direct = 1;
  else if (c->cfg.flags & STC_FLAG_QUEUED_HITS) direct = 0;
  else {
    const DevState &st = *c->st_host;  // the last step's counters
    direct = st.hits > DIRECT_HITS_PER_UNIT * ((unsigned long long)p.N + st.border_units) ? 1u : 0u;
  }
  if (direct != p.direct_hits) {
    p.direct_hits = direct;
    invalidate_graphs(c);  // the captured steps launch the other kernel
  }
}

// Tile length of the refinement's jobs when stc_config.refine_chunk is 0:
// 64 candidates when the last step tested more than 16 candidates per
// checking unit (dense leaves have long candidate windows, and 256-long
// tiles left the tail of the pair tests to a few warps: hotspot-1M 8.46 ->
// 6.18 ms a step; hotspot-3M, bound by the table update, within 0.3%), else
// 256 (uniform-10M, 7.9 tests per unit: 64-long tiles cost 0.29 ms a step).
// Results do not depend on it.
static constexpr unsigned long long SHORT_TILE_TESTS_PER_UNIT = 16;
static void choose_refine_chunk(stc_ctx *c) {
  PipeDev &p = c->p;
  uint32_t chunk = c->cfg.refine_chunk;
  if (!chunk) {
    const DevState &st = *c->st_host;  // the last step's counters
    chunk = st.tests > SHORT_TILE_TESTS_PER_UNIT * ((unsigned long long)p.N + st.border_units) ? 64u
                                                                                           : REFINE_CHUNK_DEFAULT;
  }
  if (chunk != p.refine_chunk) {
    p.refine_chunk = chunk;
    invalidate_graphs(c);  // the captured steps carry the tile length
  }
}

static stc_status run_step(stc_ctx *c, const double2 *xy, uint32_t t, bool copied) {
  PipeDev &p = c->p;
  choose_hit_emission(c);
  choose_refine_chunk(c);
  cudaStream_t s = c->stream;
  p.xy = xy;
  c->t_pinned[0] = t;  // the previous step has been waited for: nothing reads it now
  unsigned long long launches0 = tl_launches;
  issue_step(c, true, true, c->t_pinned);
  cudaEventRecord(c->ev[PH_SCHEMA], s);
  stc_status rs = read_state(c, "stc_step");
  if (rs != STC_OK) return rs;
  float ms[PH_COUNT] = {0};
  for (int i = PH_COPY; i <= PH_SCHEMA; i++) cudaEventElapsedTime(&ms[i], c->ev[i - 1], c->ev[i]);
  const float phase[8] = {ms[PH_PART], ms[PH_BORDER], ms[PH_REFINE], ms[PH_INSERT],
                          ms[PH_SWEEP], ms[PH_SCHEMA], copied ? ms[PH_COPY] : 0.f, ms[PH_APPEND]};
  float tot = 0;
  cudaEventElapsedTime(&tot, c->ev[PH_START], c->ev[PH_SCHEMA]);
  fill_stats(c, t, phase, tot, (uint32_t)(tl_launches - launches0));
  grow_hits(c, c->st_host->hit_count);
  if (flush_due(c)) return flush_now(c, t);
  return STC_OK;
}

extern "C" stc_status stc_step(stc_ctx *c, const double *xy, uint32_t t) {
  if (!c) return STC_ERR_INVALID_ARG;
  if (!xy) return fail(c, STC_ERR_INVALID_ARG, "stc_step: null positions");
  if (c->failed) return STC_ERR_STATE;
  cudaSetDevice(c->device);
  cudaEventRecord(c->ev[PH_START], c->stream);
  cudaError_t e =
      copy_in_pieces(c->xy_own, xy, (size_t)c->p.N * sizeof(double2), cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "stc_step copy-in");
  return run_step(c, c->xy_own, t, true);
}

extern "C" stc_status stc_step_device(stc_ctx *c, const double *xy_device, uint32_t t) {
  if (!c) return STC_ERR_INVALID_ARG;
  if (!xy_device) return fail(c, STC_ERR_INVALID_ARG, "stc_step_device: null positions");
  if (c->failed) return STC_ERR_STATE;
  cudaSetDevice(c->device);
  cudaEventRecord(c->ev[PH_START], c->stream);
  return run_step(c, (const double2 *)xy_device, t, false);
}

// Copies emit records [from, from + k) to out on the drain stream once the
// state copy of the step in buffer b has landed (the records are complete
// then). Page-locked output takes direct copies; other memory goes through
// the two pinned chunks (the host waits for each, while the GPU runs on).
static cudaError_t drain_range(stc_ctx *c, int b, unsigned long long from, size_t k, stc_meeting *out,
                               bool pinned_out) {
  if (!k) return cudaSuccess;
  cudaStream_t ds = c->drain_stream;
  cudaError_t e = cudaStreamWaitEvent(ds, c->st_ev[b], 0);
  const size_t bytes = k * sizeof(stc_meeting);
  const uint8_t *src = (const uint8_t *)(c->p.emit + from);
  if (pinned_out) return e == cudaSuccess ? copy_in_pieces(out, src, bytes, cudaMemcpyDeviceToHost, ds) : e;
  const size_t nch = (bytes + DRAIN_CHUNK - 1) / DRAIN_CHUNK;
  for (size_t i = 0; e == cudaSuccess && i <= nch; i++) {
    if (i < nch) {
      const size_t off = i * DRAIN_CHUNK, len = std::min(DRAIN_CHUNK, bytes - off);
      e = cudaMemcpyAsync(c->drain_stage[i & 1], src + off, len, cudaMemcpyDeviceToHost, ds);
      if (e == cudaSuccess) e = cudaEventRecord(c->drain_ev[i & 1], ds);
    }
    if (e == cudaSuccess && i > 0) {
      const size_t j = i - 1, off = j * DRAIN_CHUNK, len = std::min(DRAIN_CHUNK, bytes - off);
      e = cudaEventSynchronize(c->drain_ev[j & 1]);
      if (e == cudaSuccess) memcpy((uint8_t *)out + off, c->drain_stage[j & 1], len);
    }
  }
  return e;
}

// Moves the emit records [from, count) to the front of the emit buffer and
// sets the device and host counts to count - from. Nothing may be writing
// the emit buffer (no step in flight).
static cudaError_t emit_keep_tail(stc_ctx *c, unsigned long long from, unsigned long long count) {
  PipeDev &p = c->p;
  cudaStream_t s = c->stream;
  cudaError_t e = cudaStreamSynchronize(c->drain_stream);  // copies out of [0, from) are done
  const unsigned long long left = count - from;
  for (unsigned long long src = from; e == cudaSuccess && from && src < count; src += from) {
    unsigned long long len = std::min<unsigned long long>(from, count - src);
    e = cudaMemcpyAsync(p.emit + (src - from), p.emit + src, len * sizeof(stc_meeting), cudaMemcpyDeviceToDevice, s);
  }
  c->st_host->emit_count = left;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&p.st->emit_count, &c->st_host->emit_count, sizeof(left), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  c->stats.pending = left;
  return e;
}

// A window of steps, pipelined one step deep: step i + 1 is queued on the
// GPU before the host waits for step i's state, so the GPU does not idle
// while the host reads a state, drains meetings or issues launches. The
// positions of step i + 3 are copied in once step i has run (three input
// buffers), two steps before they are needed.
//
// Device order per step i: core(i) (everything but the memtable append),
// then [flush after step i - 1, when due], append(i), state copy(i). The
// host issues core(i + 1) right after append(i), then waits for state(i)
// and decides step i's flush from it; the flush is queued behind core(i + 1)
// and before append(i + 1). The core of a step never touches the memtable,
// so the flush sees exactly the keys of steps <= i, as the reference's
// per-step rule does. Emitted meetings stay in place in the emit buffer for
// the whole window (nothing moves while a step is in flight) and go out on
// the drain stream beside the next step; past half the buffer the pipeline
// holds for one step so that the buffer can be emptied.
extern "C" stc_status stc_step_window(stc_ctx *c, const double *xy, int on_device, uint32_t steps, uint32_t t0,
                                      stc_meeting *out, size_t cap, size_t *n_out) {
  if (!c) return STC_ERR_INVALID_ARG;
  if (n_out) *n_out = 0;
  if (steps && !xy) return fail(c, STC_ERR_INVALID_ARG, "stc_step_window: null positions");
  if (out && !n_out) return fail(c, STC_ERR_INVALID_ARG, "stc_step_window: output without a count");
  if (c->failed) return STC_ERR_STATE;
  if (!steps) return STC_OK;
  cudaSetDevice(c->device);
  PipeDev &p = c->p;
  cudaStream_t s = c->stream;
  const size_t step_bytes = (size_t)p.N * sizeof(double2);
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (!c->xy_win[WIN_BUFS - 2] || !c->copy_stream) {
    cudaError_t e = cudaSuccess;
    for (int b = 0; b < WIN_BUFS - 1 && e == cudaSuccess; b++)
      if (!c->xy_win[b]) {
        e = cudaMalloc(&c->xy_win[b], step_bytes);
        if (e == cudaSuccess) c->allocs.push_back(c->xy_win[b]);
      }
    if (e == cudaSuccess && !c->copy_stream) e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
    for (int b = 0; b < WIN_BUFS && e == cudaSuccess; b++)
      if (!c->copy_ev[b]) e = cudaEventCreateWithFlags(&c->copy_ev[b], cudaEventDisableTiming);
    for (int b = 0; b < 2 * WIN_BUFS && e == cudaSuccess; b++) {
      if (!c->copy_t0[b]) e = cudaEventCreate(&c->copy_t0[b]);
      if (e == cudaSuccess && !c->copy_t1[b]) e = cudaEventCreate(&c->copy_t1[b]);
    }
    for (int b = 0; b < 2 && e == cudaSuccess; b++)
      if (!c->sweep_ev[b]) e = cudaEventCreateWithFlags(&c->sweep_ev[b], cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(c, e, "stc_step_window buffers");
  }
  // Automatic choice: graphs where launch costs show, i.e. for short steps.
  // The last step's device time decides when there is one (graphs below
  // 1.5 ms); a fresh context goes by its object count (2^18 or fewer). A
  // replayed graph ran long steps slower than direct launches (10M objects:
  // 15.75 against 14.33 ms; dense windows of 0.3-2M objects up to 14%).
  const float last_ms = c->stats.step_ms;
  const bool graphs_auto = last_ms > 0.f ? (last_ms < 1.5f && p.N <= (1u << 21)) : p.N <= (1u << 18);
  const bool graphs = c->cfg.window_graphs == 1 || (c->cfg.window_graphs == 0 && graphs_auto);
  bool pinned_out = false;
  if (out && cap) {
    cudaPointerAttributes pa;
    pinned_out = cudaPointerGetAttributes(&pa, out) == cudaSuccess && pa.type == cudaMemoryTypeHost;
    cudaGetLastError();  // pageable memory is not an error
  }
  unsigned long long launches[2] = {0, 0};
  double wait_ms = 0;  // device time of the window's steps spent waiting for their positions
  double copy_ms = 0;  // durations of the steps' input copies

  // Positions of step i into buffer i % WIN_BUFS on the copy stream, once
  // the core of step i - WIN_BUFS (the buffer's last reader) has run and the
  // step queued last (i - 2, or step 0 for steps 1 and 2, whose copies are
  // queued right after it) has reached its sweep: the copy then runs beside
  // the sweep, which streams the table with evict-first accesses, instead of
  // beside the pair tests and table update, whose leaf data and slots it
  // would push out of L2 (host input cost 0.4-0.6 ms a step at 10M objects
  // that way, 0.1-0.3 ms this way).
  // Device input without graphs is read where it lies (as stc_step_device
  // reads it): no copy beside the steps (a 160 MB device-to-device copy took
  // 1.5 ms beside a 10M-object step against 0.05 ms alone).
  const bool direct = on_device && !graphs;
  // Page-locked host input without graphs: the descent of each step reads
  // its positions from the host pages and writes the device copy the rest
  // of the step reads. A copy engine's 160 MB copy beside a 10M-object step
  // took 0.9 ms on some hosts and 3-9 ms on others (the same copy alone:
  // 0.8 ms); the descent's reads cost about 1 ms a step everywhere. Not
  // while a request loop is attached: its batches move their queries and
  // answers through mapped host memory too, and waited behind the descent's
  // reads (query p99 under ingest 2.5-4.7 against 1.8-1.9 ms). Both ends of
  // the range must lie in page-locked memory mapped for the device.
  const double2 *host_in = nullptr;
  if (!on_device && !graphs && !(c->cfg.flags & STC_FLAG_COPY_INPUT) && c->servers.load() == 0) {
    cudaPointerAttributes a0, a1;
    const uint8_t *last = (const uint8_t *)xy + (size_t)steps * step_bytes - 1;
    if (cudaPointerGetAttributes(&a0, xy) == cudaSuccess && cudaPointerGetAttributes(&a1, last) == cudaSuccess &&
        a0.type == cudaMemoryTypeHost && a1.type == cudaMemoryTypeHost && a0.devicePointer && a1.devicePointer &&
        (const uint8_t *)a1.devicePointer - (const uint8_t *)a0.devicePointer == last - (const uint8_t *)xy)
      host_in = (const double2 *)a0.devicePointer;
    cudaGetLastError();
  }
  auto fetch = [&](uint32_t i) -> cudaError_t {
    if (direct || host_in) return cudaSuccess;
    const int b = (int)(i % WIN_BUFS);
    cudaError_t e = i >= (uint32_t)WIN_BUFS ? cudaStreamWaitEvent(c->copy_stream, c->core_ev[b], 0) : cudaSuccess;
    // and runs beside the sweep of the step queued last (i - 2; step 0 for
    // the window's first inputs), not beside its pair tests and table update
    if (e == cudaSuccess && i >= 1 && !graphs)
      e = cudaStreamWaitEvent(c->copy_stream, c->sweep_ev[(i >= 2 ? i - 2 : 0) & 1], 0);
    if (e == cudaSuccess) e = cudaEventRecord(c->copy_t0[i % (2 * WIN_BUFS)], c->copy_stream);
    if (e == cudaSuccess)
      e = copy_in_pieces(window_buffer(c, b), (const uint8_t *)xy + (size_t)i * step_bytes, step_bytes, kind,
                         c->copy_stream);
    if (e == cudaSuccess) e = cudaEventRecord(c->copy_t1[i % (2 * WIN_BUFS)], c->copy_stream);
    return e == cudaSuccess ? cudaEventRecord(c->copy_ev[b], c->copy_stream) : e;
  };
  // (per step: events and state copy by parity i & 1, input buffer, its
  // copy event, time word and graph by i % WIN_BUFS)
  auto issue_core = [&](uint32_t i) -> stc_status {
    const int par = i & 1, b = (int)(i % WIN_BUFS);
    // launch forms by the density of the latest step whose state has been
    // taken (i - 2, or the step before the window): the hits' hand-over form
    // and the pair tests' tile length
    choose_hit_emission(c);
    choose_refine_chunk(c);
    c->t_pinned[b] = t0 + i;  // step i - WIN_BUFS, the word's last reader, has been waited for
    const unsigned long long l0 = tl_launches;
    cudaEventRecord(c->wev[par][0], s);
    cudaError_t e = (direct || host_in) ? cudaSuccess : cudaStreamWaitEvent(s, c->copy_ev[b], 0);
    if (e != cudaSuccess) return cuda_fail(c, e, "stc_step_window copy-in");
    cudaEventRecord(c->wev[par][3], s);
    if (graphs) {
      if (!c->graph_valid[b]) {
        stc_status gs = capture_step(c, b);
        if (gs != STC_OK) return gs;
      }
      e = cudaGraphLaunch(c->graph[b], s);
      if (e != cudaSuccess) return cuda_fail(c, e, "stc_step_window");
      tl_launches += c->graph_kernels;
    } else {
      p.xy = direct ? (const double2 *)((const uint8_t *)xy + (size_t)i * step_bytes) : window_buffer(c, b);
      p.xy_in = host_in ? (const double2 *)((const uint8_t *)host_in + (size_t)i * step_bytes) : nullptr;
      c->gate_ev = c->sweep_ev[par];
      issue_step(c, false, false, c->t_pinned + b);
      c->gate_ev = nullptr;
      p.xy_in = nullptr;
    }
    cudaEventRecord(c->core_ev[b], s);
    launches[par] = tl_launches - l0;
    return STC_OK;
  };
  auto issue_tail = [&](uint32_t i) -> stc_status {
    const int b = i & 1;
    const unsigned long long l0 = tl_launches;
    cudaEventRecord(c->wev[b][1], s);
    if (c->lsm_on) lsm_append(p, c->lsm, s);
    cudaEventRecord(c->wev[b][2], s);
    cudaError_t e = cudaMemcpyAsync(c->st_slot[b], p.st, sizeof(DevState), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaEventRecord(c->st_ev[b], s);
    launches[b] += tl_launches - l0;
    return e == cudaSuccess ? STC_OK : cuda_fail(c, e, "stc_step_window");
  };
  // Waits for the state of step i and takes it over as the context's state.
  auto take_state = [&](uint32_t i) -> stc_status {
    const int b = i & 1;
    cudaError_t e = cudaEventSynchronize(c->st_ev[b]);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "stc_step_window");
    *c->st_host = *c->st_slot[b];
    if (c->st_host->error) {
      char m[320];
      snprintf(m, sizeof(m), "stc_step_window: %s (code %u, info %u)", error_name(c->st_host->error),
               c->st_host->error, c->st_host->error_info);
      return fail(c, status_of(c->st_host->error), m);
    }
    float core = 0, app = 0, wait = 0;
    cudaEventElapsedTime(&core, c->wev[b][0], c->core_ev[i % WIN_BUFS]);
    cudaEventElapsedTime(&app, c->wev[b][1], c->wev[b][2]);
    cudaEventElapsedTime(&wait, c->wev[b][0], c->wev[b][3]);
    wait_ms += wait;
    // step i's copy ended before its core began, which has run
    float cp = 0;
    if (!direct && !host_in &&
        cudaEventElapsedTime(&cp, c->copy_t0[i % (2 * WIN_BUFS)], c->copy_t1[i % (2 * WIN_BUFS)]) == cudaSuccess)
      copy_ms += cp;
    cudaGetLastError();
    float phase[8] = {0, 0, 0, 0, 0, 0, 0, app};
    fill_stats(c, t0 + i, phase, core + app, (uint32_t)launches[b]);
    return STC_OK;
  };

  const auto wall0 = std::chrono::steady_clock::now();
  double busy_ms = 0;  // device time of the window's steps
  size_t n = 0;
  unsigned long long most_hits = 0;  // the window's largest step (hit buffer growth at its end)
  unsigned long long dpos = 0;  // emit records [0, dpos) are on their way to out
  bool out_full = false;
  stc_status rs = STC_OK;
  uint32_t ran = 0;             // steps whose state has been taken
  bool hold = false;            // empty the emit buffer before the next core
  cudaError_t e = fetch(0);
  if (e != cudaSuccess) return cuda_fail(c, e, "stc_step_window copy-in");
  rs = issue_core(0);
  for (uint32_t k = 1; rs == STC_OK && k < (uint32_t)WIN_BUFS && k < steps; k++) {
    e = fetch(k);
    if (e != cudaSuccess) rs = cuda_fail(c, e, "stc_step_window copy-in");
  }
  if (rs == STC_OK) rs = issue_tail(0);
  if (rs != STC_OK) {
    cudaStreamSynchronize(s);
    return rs;
  }
  for (uint32_t i = 0; i < steps; i++) {
    const bool ahead = i + 1 < steps && !hold;
    if (ahead) {
      rs = issue_core(i + 1);
      if (rs == STC_OK && i + WIN_BUFS < steps) {
        e = fetch(i + WIN_BUFS);
        if (e != cudaSuccess) rs = cuda_fail(c, e, "stc_step_window copy-in");
      }
    }
    if (rs == STC_OK) rs = take_state(i);
    if (rs == STC_OK) {
      ran = i + 1;
      busy_ms += c->stats.step_ms;
    }
    if (rs == STC_OK) most_hits = std::max(most_hits, c->st_host->hit_count);
    if (rs == STC_OK && out && !out_full) {
      const unsigned long long cnt = std::min<unsigned long long>(c->st_host->emit_count, p.E);
      const size_t k = (size_t)std::min<unsigned long long>(cnt - dpos, cap - n);
      e = drain_range(c, i & 1, dpos, k, out + n, pinned_out);
      if (e != cudaSuccess) rs = cuda_fail(c, e, "stc_step_window drain");
      dpos += k;
      n += k;
      *n_out = n;
      out_full = dpos < cnt;
    }
    if (rs == STC_OK && flush_due(c)) rs = flush_now(c, t0 + i);
    if (rs != STC_OK || out_full) {
      // the step already queued behind this one is finished and taken, its
      // meetings left pending; nothing is in flight when the call returns
      if (ahead && !c->failed) {
        stc_status r2 = issue_tail(i + 1);
        if (r2 == STC_OK) r2 = take_state(i + 1);
        if (r2 == STC_OK) ran = i + 2;
        if (r2 == STC_OK && flush_due(c)) r2 = flush_now(c, t0 + i + 1);
        if (rs == STC_OK) rs = r2;
      }
      cudaStreamSynchronize(s);
      cudaStreamSynchronize(c->copy_stream);
      cudaStreamSynchronize(c->drain_stream);
      if (!c->failed && out) {
        e = emit_keep_tail(c, dpos, std::min<unsigned long long>(c->st_host->emit_count, p.E));
        if (e != cudaSuccess && rs == STC_OK) rs = cuda_fail(c, e, "stc_step_window drain");
      }
      if (rs == STC_OK) {
        char m[160];
        snprintf(m, sizeof(m), "stc_step_window: the output buffer is full after step %u; %u of %u steps ran",
                 t0 + ran - 1, ran, steps);
        rs = fail(c, STC_ERR_CAPACITY, m);
        c->failed = false;  // a full output buffer leaves the context usable
      }
      return rs;
    }
    if (i + 1 < steps) {
      if (!ahead) {
        // held: nothing is in flight; every record emitted so far is drained
        // or on its way out, so the emit buffer can be emptied, and the hit
        // buffer can grow to the window's largest step
        if (out) {
          e = emit_keep_tail(c, dpos, std::min<unsigned long long>(c->st_host->emit_count, p.E));
          if (e != cudaSuccess) return cuda_fail(c, e, "stc_step_window drain");
          dpos = 0;
        }
        grow_hits(c, most_hits);
        hold = false;
        rs = issue_core(i + 1);
        if (rs == STC_OK && i + WIN_BUFS < steps) {
          e = fetch(i + WIN_BUFS);
          if (e != cudaSuccess) rs = cuda_fail(c, e, "stc_step_window copy-in");
        }
        if (rs != STC_OK) {
          cudaStreamSynchronize(s);
          return rs;
        }
      }
      rs = issue_tail(i + 1);
      if (rs != STC_OK) {
        cudaStreamSynchronize(s);
        return rs;
      }
      // step i + 1 adds its meetings behind step i's; past half of the
      // emit buffer, step i + 2 waits until the buffer has been emptied
      if (out && c->st_host->emit_count > p.E / 2) hold = true;
      // a step found more hits than the hit buffer holds (the rest were
      // applied inside its pair tests): grow it at the next step boundary
      if (!c->cfg.hit_capacity && most_hits > p.hit_cap) hold = true;
    }
  }
  cudaStreamSynchronize(c->copy_stream);
  if (out) {
    e = emit_keep_tail(c, dpos, std::min<unsigned long long>(c->st_host->emit_count, p.E));
    if (e != cudaSuccess) return cuda_fail(c, e, "stc_step_window drain");
  }
  cudaStreamSynchronize(s);
  grow_hits(c, most_hits);
  c->stats.window_device_ms = (float)busy_ms;
  c->stats.window_input_wait_ms = (float)wait_ms;
  c->stats.window_copy_ms = (float)copy_ms;
  c->stats.window_wall_ms =
      (float)std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
  return STC_OK;
}

extern "C" stc_status stc_get_stats(stc_ctx *c, stc_stats *out) {
  if (!c || !out) return STC_ERR_INVALID_ARG;
  *out = c->stats;
  return STC_OK;
}

extern "C" stc_status stc_drain_meetings(stc_ctx *c, stc_meeting *out, size_t cap, size_t *n) {
  if (!c || !n || (!out && cap)) return STC_ERR_INVALID_ARG;
  *n = 0;
  cudaSetDevice(c->device);
  PipeDev &p = c->p;
  unsigned long long pending = std::min<unsigned long long>(c->st_host->emit_count, p.E);
  size_t k = (size_t)std::min<unsigned long long>(pending, cap);
  cudaStream_t s = c->stream;
  cudaError_t e = cudaSuccess;
  // pinned (page-locked) output takes one direct copy; other memory gets the
  // k records through the two pinned chunks, the copy of chunk i + 1 running
  // while chunk i is moved to out
  const size_t bytes = k * sizeof(stc_meeting);
  cudaPointerAttributes pa;
  const bool pinned_out = k && cudaPointerGetAttributes(&pa, out) == cudaSuccess && pa.type == cudaMemoryTypeHost;
  cudaGetLastError();  // pageable memory is not an error
  if (pinned_out) e = copy_in_pieces(out, p.emit, bytes, cudaMemcpyDeviceToHost, s);
  const size_t nch = pinned_out ? 0 : (bytes + DRAIN_CHUNK - 1) / DRAIN_CHUNK;
  for (size_t i = 0; e == cudaSuccess && nch && i <= nch; i++) {
    if (i < nch) {
      const size_t off = i * DRAIN_CHUNK, len = std::min(DRAIN_CHUNK, bytes - off);
      e = cudaMemcpyAsync(c->drain_stage[i & 1], (const uint8_t *)p.emit + off, len, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaEventRecord(c->drain_ev[i & 1], s);
    }
    if (e == cudaSuccess && i > 0) {
      const size_t j = i - 1, off = j * DRAIN_CHUNK, len = std::min(DRAIN_CHUNK, bytes - off);
      e = cudaEventSynchronize(c->drain_ev[j & 1]);
      if (e == cudaSuccess) memcpy((uint8_t *)out + off, c->drain_stage[j & 1], len);
    }
  }
  // shift the rest down in non-overlapping chunks of k records
  for (size_t src = k; e == cudaSuccess && k && src < pending; src += k) {
    size_t len = std::min<size_t>(k, pending - src);
    e = cudaMemcpyAsync(p.emit + (src - k), p.emit + src, len * sizeof(stc_meeting), cudaMemcpyDeviceToDevice, s);
  }
  unsigned long long left = pending - k;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&p.st->emit_count, &(c->st_host->emit_count = left), sizeof(left), cudaMemcpyHostToDevice,
                        s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(c, e, "stc_drain_meetings");
  c->st_host->emit_count = left;
  c->stats.pending = left;
  *n = k;
  return STC_OK;
}

extern "C" stc_status stc_flush(stc_ctx *c, int *flushed) {
  if (!c) return STC_ERR_INVALID_ARG;
  if (flushed) *flushed = 0;
  if (c->failed) return STC_ERR_STATE;
  if (!c->lsm_on) return fail(c, STC_ERR_INVALID_ARG, "stc_flush: the memtable is off (kv_restriction 0)");
  cudaSetDevice(c->device);
  if (c->st_host->kv_count == 0) return STC_OK;
  stc_status rs = flush_now(c, c->last_t);
  if (rs == STC_OK && flushed) *flushed = 1;
  return rs;
}

extern "C" stc_status stc_get_ctb(stc_ctx *c, stc_ctb_info *info) {
  if (!c || !info) return STC_ERR_INVALID_ARG;
  if (!c->lsmh.has_block) {
    c->err = "stc_get_ctb: no block flushed yet";
    return STC_ERR_STATE;
  }
  *info = c->lsmh.info;
  return STC_OK;
}

extern "C" stc_status stc_read_ctb(stc_ctx *c, stc_ctf *ctfs, uint8_t *bitmaps, uint8_t *keys, uint16_t *sids,
                                   uint64_t *oversize_keys, float *oversize_boxes, uint8_t *oversize_bitmap) {
  if (!c) return STC_ERR_INVALID_ARG;
  if (!c->lsmh.has_block) {
    c->err = "stc_read_ctb: no block flushed yet";
    return STC_ERR_STATE;
  }
  cudaSetDevice(c->device);
  const stc_ctb_info &in = c->lsmh.info;
  const LsmDev &L = c->lsm;
  cudaStream_t s = c->stream;
  cudaError_t e = cudaSuccess;
  if (ctfs) memcpy(ctfs, c->lsmh.ctfs.data(), in.ctf_count * sizeof(stc_ctf));
  if (bitmaps)
    e = cudaMemcpyAsync(bitmaps, L.bitmaps, (size_t)in.ctf_count * STC_BITMAP_BYTES, cudaMemcpyDeviceToHost, s);
  if (keys && in.key_bytes && e == cudaSuccess)
    e = cudaMemcpyAsync(keys, L.kbytes, in.key_bytes, cudaMemcpyDeviceToHost, s);
  if (sids && e == cudaSuccess) e = cudaMemcpyAsync(sids, L.bsid, (size_t)L.N * 2, cudaMemcpyDeviceToHost, s);
  if (oversize_bitmap && e == cudaSuccess)
    e = cudaMemcpyAsync(oversize_bitmap, L.obitmap, STC_MAP_BITMAP_BYTES(L.edge), cudaMemcpyDeviceToHost, s);
  std::vector<uint4> orec;
  const size_t no = (size_t)in.oversize_kv_count;
  if (no && oversize_keys && e == cudaSuccess) {
    orec.resize(no);
    e = cudaMemcpyAsync(orec.data(), L.brec + in.ctf_kv_count, no * sizeof(uint4), cudaMemcpyDeviceToHost, s);
  }
  if (no && oversize_boxes && e == cudaSuccess)
    e = cudaMemcpyAsync(oversize_boxes, L.bbox + in.ctf_kv_count, no * sizeof(float4), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(c, e, "stc_read_ctb");
  // 128-bit oversize keys pid:26 | target:26 | duration:32 | end:32 (util/util.h:47-52)
  for (size_t i = 0; i < orec.size(); i++) {
    oversize_keys[2 * i] = ((uint64_t)orec[i].z << 32) | orec[i].w;
    oversize_keys[2 * i + 1] = ((uint64_t)orec[i].x << 26) | orec[i].y;
  }
  return STC_OK;
}

static stc_status query_checks(stc_ctx *c, const char *who) {
  if (!c) {
    g_create_error = std::string(who) + ": null context";
    return STC_ERR_INVALID_ARG;
  }
  if (!c->lsm_on) {
    g_create_error = std::string(who) + ": the memtable is off (kv_restriction 0), nothing to query";
    return STC_ERR_INVALID_ARG;
  }
  cudaSetDevice(c->device);
  return STC_OK;
}

namespace stc {
// stc_query_batch on query lane `lane` (-1: any free lane) with a bound on the
// match records held on the device at a time (the serving loop's
// admission); 0 = none.
stc_status query_batch_limited(stc_ctx *c, int lane, const stc_query *queries, size_t nq, stc_contact *out,
                               size_t cap, uint64_t *offsets, uint64_t *counts, size_t device_limit,
                               float *gpu_ms = nullptr);
// Queries one device pass takes (larger batches run as several passes).
size_t query_chunk(const stc_ctx *c);
// A request loop attaches (+1) to or detaches (-1) from the context.
void server_attach(stc_ctx *c, int d);
}

void stc::server_attach(stc_ctx *c, int d) {
  if (c) c->servers += d;
}

extern "C" stc_status stc_query_batch(stc_ctx *c, const stc_query *queries, size_t nq, stc_contact *out,
                                      size_t cap, uint64_t *offsets, uint64_t *counts) {
  return stc::query_batch_limited(c, -1, queries, nq, out, cap, offsets, counts, 0);
}

size_t stc::query_chunk(const stc_ctx *c) { return c && c->lsm_on ? lsm_query_chunk(c->lsmh) : 1; }

stc_status stc::query_batch_limited(stc_ctx *c, int lane, const stc_query *queries, size_t nq, stc_contact *out,
                                    size_t cap, uint64_t *offsets, uint64_t *counts, size_t device_limit,
                                    float *gpu_ms) {
  stc_status st = query_checks(c, "stc_query_batch");
  if (st != STC_OK) return st;
  if ((!queries && nq) || !offsets || (!out && cap)) {
    g_create_error = "stc_query_batch: null argument";
    return STC_ERR_INVALID_ARG;
  }
  for (size_t i = 0; i < nq; i++) {
    const stc_query &q = queries[i];
    const uint32_t kind = q.kind & ~STC_QUERY_COUNT_ONLY;
    if ((kind != STC_QUERY_OBJECT && kind != STC_QUERY_BOX) || (kind == STC_QUERY_OBJECT && q.pid >= c->p.N)) {
      g_create_error = "stc_query_batch: query " + std::to_string(i) + " has a bad kind or object id";
      return STC_ERR_INVALID_ARG;
    }
  }
  std::string err;
  const size_t chunk = lsm_query_chunk(c->lsmh);
  if (gpu_ms) *gpu_ms = 0.f;
  if (nq <= chunk) {
    st = lsm_query(c->lsmh, lane, queries, nq, out, cap, offsets, counts, err, device_limit, gpu_ms);
    if (st != STC_OK) g_create_error = "stc_query_batch: " + err;
    return st;
  }
  // queries x retained blocks must stay <= 65535 per device pass: the batch
  // runs as several passes; each writes its matches behind the previous
  // ones while the running total fits cap
  std::vector<uint64_t> off(chunk + 1);
  offsets[0] = 0;
  for (size_t a = 0; a < nq; a += chunk) {
    const size_t m = std::min(chunk, nq - a);
    const uint64_t done = offsets[a];
    const bool room = out && done <= cap;
    float ms = 0.f;
    st = lsm_query(c->lsmh, lane, queries + a, m, room ? out + done : nullptr, room ? cap - done : 0, off.data(),
                   counts ? counts + a : nullptr, err, device_limit, gpu_ms ? &ms : nullptr);
    if (gpu_ms) *gpu_ms += ms;
    if (st != STC_OK) {
      g_create_error = "stc_query_batch: " + err;
      return st;
    }
    for (size_t i = 0; i < m; i++) offsets[a + i + 1] = done + off[i + 1];
  }
  return STC_OK;
}

static stc_status query_one(stc_ctx *c, const stc_query &q, stc_contact *out, size_t cap, size_t *n,
                            const char *who) {
  if (!n || (!out && cap)) {
    g_create_error = std::string(who) + ": null argument";
    return STC_ERR_INVALID_ARG;
  }
  uint64_t off[2] = {0, 0};
  stc_status st = stc_query_batch(c, &q, 1, out, cap, off, nullptr);
  *n = (size_t)off[1];
  return st;
}

extern "C" stc_status stc_query_object(stc_ctx *c, uint32_t pid, uint32_t t_start, uint32_t t_end,
                                       stc_contact *out, size_t cap, size_t *n) {
  stc_query q{};
  q.kind = STC_QUERY_OBJECT;
  q.pid = pid;
  q.t_start = t_start;
  q.t_end = t_end;
  return query_one(c, q, out, cap, n, "stc_query_object");
}

extern "C" stc_status stc_query_box(stc_ctx *c, const double box[4], uint32_t t_start, uint32_t t_end,
                                    stc_contact *out, size_t cap, size_t *n) {
  if (!box) {
    g_create_error = "stc_query_box: null box";
    return STC_ERR_INVALID_ARG;
  }
  stc_query q{};
  q.kind = STC_QUERY_BOX;
  q.t_start = t_start;
  q.t_end = t_end;
  for (int i = 0; i < 4; i++) q.box[i] = box[i];
  return query_one(c, q, out, cap, n, "stc_query_box");
}

extern "C" stc_status stc_write_ctb(stc_ctx *c, uint32_t index, const char *dir, const char *prefix) {
  if (!c) return STC_ERR_INVALID_ARG;
  if (!dir || !prefix) return fail(c, STC_ERR_INVALID_ARG, "stc_write_ctb: null path");
  if (!c->lsm_on) return fail(c, STC_ERR_INVALID_ARG, "stc_write_ctb: the memtable is off (kv_restriction 0)");
  cudaSetDevice(c->device);
  std::string err;
  stc_status st = lsm_write_block(c->lsmh, index, c->p.N, dir, prefix, err);
  if (st != STC_OK) c->err = "stc_write_ctb: " + err;
  return st;
}

extern "C" stc_status stc_get_block(stc_ctx *c, uint32_t index, stc_ctb_info *info) {
  if (!c) return STC_ERR_INVALID_ARG;
  if (!info) return fail(c, STC_ERR_INVALID_ARG, "stc_get_block: null info");
  std::string err;
  stc_status st = lsm_block_info(c->lsmh, index, info, err);
  if (st != STC_OK) c->err = "stc_get_block: " + err;
  return st;
}

extern "C" stc_status stc_read_block(stc_ctx *c, uint32_t index, stc_ctf *ctfs, uint8_t *bitmaps, uint8_t *keys,
                                     uint16_t *sids, uint64_t *oversize_keys, float *oversize_boxes,
                                     uint8_t *oversize_bitmap) {
  if (!c) return STC_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  std::string err;
  stc_status st = lsm_read_block(c->lsmh, index, c->p.N, ctfs, bitmaps, keys, sids, oversize_keys, oversize_boxes,
                                 oversize_bitmap, err);
  if (st != STC_OK) c->err = "stc_read_block: " + err;
  return st;
}

extern "C" stc_status stc_set_step_slices(stc_ctx *c, uint32_t slices) {
  if (!c) return STC_ERR_INVALID_ARG;
  c->cfg.step_slices = slices;
  c->p.slices = std::min<uint32_t>(std::max<uint32_t>(slices, 1u), 64u);
  invalidate_graphs(c);
  return STC_OK;
}

extern "C" stc_status stc_compact(stc_ctx *c, uint32_t first_index, uint32_t count, uint32_t split,
                                  uint32_t *new_index, float *device_ms) {
  if (!c) return STC_ERR_INVALID_ARG;
  if (!c->lsm_on) return fail(c, STC_ERR_INVALID_ARG, "stc_compact: the memtable is off (kv_restriction 0)");
  if (c->failed) return STC_ERR_STATE;
  cudaSetDevice(c->device);
  std::string err;
  float ms = 0.0f;
  const uint32_t idx = c->lsmh.next_index;
  stc_status st = lsm_compact(c->lsm, c->lsmh, first_index, count, split, idx, c->stream, &ms, err,
                              c->stats.compact_stage_ms);
  if (st != STC_OK) {
    c->err = "stc_compact: " + err;
    return st;
  }
  c->lsmh.next_index++;
  if (new_index) *new_index = idx;
  if (device_ms) *device_ms = ms;
  return STC_OK;
}

extern "C" stc_status stc_load_ctb(stc_ctx *c, uint32_t index, const char *dir, const char *prefix) {
  if (!c) return STC_ERR_INVALID_ARG;
  if (!dir || !prefix) return fail(c, STC_ERR_INVALID_ARG, "stc_load_ctb: null path");
  if (!c->lsm_on) return fail(c, STC_ERR_INVALID_ARG, "stc_load_ctb: the memtable is off (kv_restriction 0)");
  if (c->failed) return STC_ERR_STATE;
  cudaSetDevice(c->device);
  invalidate_graphs(c);
  std::string err;
  stc_status st = lsm_load_block(c->lsm, c->lsmh, index, dir, prefix, c->stream, err);
  if (st != STC_OK) c->err = "stc_load_ctb: " + err;
  return st;
}

// ---- Checkpoint / restore ------------------------------------------------------
//
// A versioned replacement for the reference's raw workbench dumps
// (tracing/workbench.cpp:574-694): a header (magic, version, the sizes of the
// structs it embeds, configuration, map box, counters) then length-prefixed
// sections holding every piece of device state that lives from one step to
// the next, and a 64-bit checksum of the section bytes.

namespace {

const char CKPT_MAGIC[8] = {'S', 'T', 'C', 'C', 'K', 'P', 'T', '1'};
constexpr uint32_t CKPT_VERSION = 1;
constexpr size_t CKPT_CHUNK = 64u << 20;

struct CkptHeader {
  char magic[8];
  uint32_t version, header_bytes;
  uint32_t config_bytes, stats_bytes, state_bytes, node_bytes, meta_bytes, pad0;
  stc_config cfg;
  double map[4];
  uint32_t N, S, G, F;
  unsigned long long B, E, lsm_cap;
  uint32_t last_t, stepped, lsm_on, lsm_end_time_min, lsm_flushes, lsm_next_index;
  stc_stats stats;
  DevState st;
};

struct Section {
  void *dev;
  unsigned long long bytes;
};

unsigned long long mix_words(unsigned long long h, const uint8_t *p, size_t n) {
  size_t i = 0;
  for (; i + 8 <= n; i += 8) {
    unsigned long long w;
    memcpy(&w, p + i, 8);
    h = (h ^ w) * 0x100000001B3ull;
  }
  for (; i < n; i++) h = (h ^ p[i]) * 0x100000001B3ull;
  return h;
}

std::vector<Section> sections(stc_ctx *c, const DevState &st) {
  PipeDev &p = c->p;
  std::vector<Section> v = {
      {p.sd.nodes, (unsigned long long)p.S * sizeof(Node)},
      {p.sd.meta, (unsigned long long)p.S * sizeof(NodeMeta)},
      {p.sd.schema_stack, (unsigned long long)p.S * 4},
      {p.sd.grids_stack, (unsigned long long)p.G * 4},
      {p.sd.gid_node, (unsigned long long)p.G * 4},
      {p.sd.fbox, (unsigned long long)p.S * sizeof(float4)},
      {p.sw.queued, (unsigned long long)p.S},
      {p.slots, p.B * sizeof(Slot)},
      {p.emit, std::min<unsigned long long>(st.emit_count, p.E) * sizeof(stc_meeting)},
  };
  if (c->lsm_on) {
    LsmDev &L = c->lsm;
    unsigned long long kv = std::min<unsigned long long>(st.kv_count, L.cap);
    v.push_back({L.rec, kv * sizeof(uint4)});
    v.push_back({L.box, kv * sizeof(float4)});
    v.push_back({L.cnt, (unsigned long long)L.N * 4});
    v.push_back({L.obox, (unsigned long long)L.N * sizeof(uint4)});
    v.push_back({L.sid, (unsigned long long)L.N * 2});
  }
  return v;
}

}  // namespace

extern "C" stc_status stc_checkpoint(stc_ctx *c, const char *path) {
  if (!c) return STC_ERR_INVALID_ARG;
  if (!path) return fail(c, STC_ERR_INVALID_ARG, "stc_checkpoint: null path");
  if (c->failed) return STC_ERR_STATE;
  cudaSetDevice(c->device);
  stc_status rs = read_state(c, "stc_checkpoint");
  if (rs != STC_OK) return rs;
  CkptHeader h;
  memset(&h, 0, sizeof(h));
  memcpy(h.magic, CKPT_MAGIC, 8);
  h.version = CKPT_VERSION;
  h.header_bytes = sizeof(CkptHeader);
  h.config_bytes = sizeof(stc_config);
  h.stats_bytes = sizeof(stc_stats);
  h.state_bytes = sizeof(DevState);
  h.node_bytes = sizeof(Node);
  h.meta_bytes = sizeof(NodeMeta);
  h.cfg = c->cfg;
  for (int i = 0; i < 4; i++) h.map[i] = c->map[i];
  h.N = c->p.N;
  h.S = c->p.S;
  h.G = c->p.G;
  h.F = c->lsm_on ? c->lsm.F : 0;
  h.B = c->p.B;
  h.E = c->p.E;
  h.lsm_cap = c->lsm_on ? c->lsm.cap : 0;
  h.last_t = c->last_t;
  h.stepped = c->stepped;
  h.lsm_on = c->lsm_on;
  h.lsm_end_time_min = c->lsm_on ? c->lsm.end_time_min : 0;
  h.lsm_flushes = c->lsmh.flushes;
  h.lsm_next_index = c->lsmh.next_index;
  h.stats = c->stats;
  h.st = *c->st_host;
  FILE *f = fopen(path, "wb");
  if (!f) return fail(c, STC_ERR_INVALID_ARG, std::string("stc_checkpoint: cannot create ") + path);
  uint8_t *stage = nullptr;
  cudaError_t e = cudaMallocHost(&stage, CKPT_CHUNK);
  bool io = e == cudaSuccess && fwrite(&h, sizeof(h), 1, f) == 1;
  unsigned long long hash = 0xcbf29ce484222325ull;
  for (const Section &sec : sections(c, h.st)) {
    io = io && fwrite(&sec.bytes, 8, 1, f) == 1;
    for (unsigned long long off = 0; io && off < sec.bytes; off += CKPT_CHUNK) {
      size_t n = (size_t)std::min<unsigned long long>(CKPT_CHUNK, sec.bytes - off);
      e = cudaMemcpy(stage, (const uint8_t *)sec.dev + off, n, cudaMemcpyDeviceToHost);
      io = e == cudaSuccess && fwrite(stage, 1, n, f) == n;
      if (io) hash = mix_words(hash, stage, n);
    }
  }
  io = io && fwrite(&hash, 8, 1, f) == 1;
  if (stage) cudaFreeHost(stage);
  io = (fclose(f) == 0) && io;
  if (e != cudaSuccess) return cuda_fail(c, e, "stc_checkpoint");
  if (!io) return fail(c, STC_ERR_INVALID_ARG, std::string("stc_checkpoint: writing ") + path + " failed");
  return STC_OK;
}

extern "C" stc_status stc_restore(const char *path, uint32_t device, stc_ctx **out) {
  if (out) *out = nullptr;
  if (!path || !out) {
    g_create_error = "stc_restore: null argument";
    return STC_ERR_INVALID_ARG;
  }
  FILE *f = fopen(path, "rb");
  if (!f) {
    g_create_error = std::string("stc_restore: cannot open ") + path;
    return STC_ERR_INVALID_ARG;
  }
  CkptHeader h;
  if (fread(&h, sizeof(h), 1, f) != 1 || memcmp(h.magic, CKPT_MAGIC, 8) != 0 || h.version != CKPT_VERSION ||
      h.header_bytes != sizeof(CkptHeader) || h.config_bytes != sizeof(stc_config) ||
      h.stats_bytes != sizeof(stc_stats) || h.state_bytes != sizeof(DevState) || h.node_bytes != sizeof(Node) ||
      h.meta_bytes != sizeof(NodeMeta)) {
    fclose(f);
    g_create_error = std::string("stc_restore: ") + path + " is not a checkpoint of this library version";
    return STC_ERR_INVALID_ARG;
  }
  stc_config cfg = h.cfg;
  cfg.device = device;
  stc_ctx *c = nullptr;
  stc_status rs = create_ctx(&cfg, h.map, nullptr, h.N, &c);
  if (rs != STC_OK) {
    fclose(f);
    return rs;
  }
  auto bail = [&](stc_status st, const std::string &msg) {
    fclose(f);
    g_create_error = "stc_restore: " + msg;
    stc_destroy(c);
    return st;
  };
  if (c->p.S != h.S || c->p.G != h.G || c->p.B != h.B || c->p.E != h.E || (c->lsm_on ? 1u : 0u) != h.lsm_on ||
      (c->lsm_on && (c->lsm.cap != h.lsm_cap || c->lsm.F != h.F)))
    return bail(STC_ERR_INVALID_ARG, "the checkpoint's sizes do not match its configuration");
  uint8_t *stage = nullptr;
  cudaError_t e = cudaMallocHost(&stage, CKPT_CHUNK);
  if (e != cudaSuccess) return bail(STC_ERR_CUDA, cudaGetErrorString(e));
  unsigned long long hash = 0xcbf29ce484222325ull;
  std::string bad;
  for (const Section &sec : sections(c, h.st)) {
    unsigned long long bytes = 0;
    if (fread(&bytes, 8, 1, f) != 1 || bytes != sec.bytes) {
      bad = "a section's size does not match";
      break;
    }
    for (unsigned long long off = 0; off < bytes && bad.empty(); off += CKPT_CHUNK) {
      size_t n = (size_t)std::min<unsigned long long>(CKPT_CHUNK, bytes - off);
      if (fread(stage, 1, n, f) != n) {
        bad = "the file is truncated";
        break;
      }
      hash = mix_words(hash, stage, n);
      e = cudaMemcpy((uint8_t *)sec.dev + off, stage, n, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) bad = cudaGetErrorString(e);
    }
    if (!bad.empty()) break;
  }
  unsigned long long want = 0;
  if (bad.empty() && (fread(&want, 8, 1, f) != 1 || want != hash)) bad = "checksum mismatch";
  cudaFreeHost(stage);
  if (!bad.empty()) return bail(STC_ERR_INVALID_ARG, bad);
  fclose(f);
  e = cudaMemcpy(c->p.st, &h.st, sizeof(DevState), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    g_create_error = std::string("stc_restore: ") + cudaGetErrorString(e);
    stc_destroy(c);
    return STC_ERR_CUDA;
  }
  *c->st_host = h.st;
  c->stats = h.stats;
  c->last_t = h.last_t;
  c->stepped = h.stepped != 0;
  if (c->lsm_on) {
    c->lsm.end_time_min = h.lsm_end_time_min;
    c->lsmh.flushes = h.lsm_flushes;
    c->lsmh.next_index = std::max(h.lsm_flushes, h.lsm_next_index);
  }
  *out = c;
  return STC_OK;
}

extern "C" stc_status stc_get_config(const stc_ctx *c, stc_config *cfg) {
  if (!c || !cfg) return STC_ERR_INVALID_ARG;
  *cfg = c->cfg;
  return STC_OK;
}
