/*
 * Device-side seeded trace generator (include/stc_trace.h).
 *
 * Stands in for the reference's road-network walker (Map::navigate,
 * geometry/Map.cpp:483-589, driven from tracing/generator.cpp:387-406) as
 * the source of synthetic positions, so a benchmark or a simulation feeds
 * stc_step_device without generating on the host and copying 16 bytes per
 * object per step over the host link.
 *
 * Layout in device memory:
 *   node_x, node_y  f64[G*G]      street nodes (G = 200: 640 KB, L2-resident)
 *   hot_x, hot_y, hot_cdf  f64[H] hotspot centres and cumulative weights
 *   u, v, turns     u32[N]        walker state, one array per field
 *   along, len, speed  f64[N]
 * A call writing S steps runs one thread per object: it loads the object's
 * state once, keeps it in registers across the S steps, writes each step's
 * (lon, lat) as one 16-byte store (a warp writes 512 contiguous bytes), and
 * stores the state back once. Per object and call that is 40 bytes of state
 * read, 40 written and 16*S of positions; the street-node reads hit L2.
 * The arithmetic is FP64 (a division per position, a square root per turn).
 *
 * The per-object code is tracegen_walk.h, shared with the host generator
 * (tracegen.c); the device side uses round-to-nearest intrinsics for every
 * operation, so positions are bit-identical to the host generator's.
 */
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

#include "stc_common.cuh"
#include "stc_trace.h"
#include "tracegen_walk.h"

struct stc_trace_dev {
  stc_trace_config cfg;
  int device = 0;
  tg_world w;                 /* device pointers */
  double *tab = nullptr;      /* node_x | node_y | hot_x | hot_y | hot_cdf */
  uint32_t *u = nullptr, *v = nullptr, *turns = nullptr;
  double *along = nullptr, *len = nullptr, *speed = nullptr;
  uint32_t step = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.0f;
};

namespace {

constexpr int TG_THREADS = 256;

__global__ void k_tg_nodes(uint64_t seed, int32_t G, double spacing, double jitter_m, uint32_t nn,
                           double *node_x, double *node_y) {
  uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= nn) return;
  double x, y;
  tg_node_xy(seed, G, spacing, jitter_m, id, &x, &y);
  node_x[id] = x;
  node_y[id] = y;
}

__global__ void __launch_bounds__(TG_THREADS) k_tg_place(tg_world w, uint32_t n, uint32_t *u, uint32_t *v,
                                                         uint32_t *turns, double *along, double *len,
                                                         double *speed) {
  uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n) return;
  tg_obj ob;
  tg_place(&w, o, &ob);
  u[o] = ob.u;
  v[o] = ob.v;
  turns[o] = ob.turns;
  along[o] = ob.along;
  len[o] = ob.len;
  speed[o] = ob.speed;
}

/* Steps first_step .. first_step + steps - 1 of every object; step k's
 * positions go to xy + 2 * n * k. The walker advances before every step but
 * step 0 (the start positions). */
__global__ void __launch_bounds__(TG_THREADS) k_tg_steps(tg_world w, uint32_t n, uint32_t first_step,
                                                         uint32_t steps, uint32_t *u, uint32_t *v,
                                                         uint32_t *turns, double *along, double *len,
                                                         const double *speed, double2 *xy) {
  uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n) return;
  tg_obj ob;
  ob.u = u[o];
  ob.v = v[o];
  ob.turns = turns[o];
  ob.along = along[o];
  ob.len = len[o];
  ob.speed = speed[o];
  const uint32_t turns0 = ob.turns;
  for (uint32_t k = 0; k < steps; k++) {
    if (first_step + k > 0) tg_advance(&w, o, &ob);
    double lon, lat;
    tg_lonlat(&w, &ob, &lon, &lat);
    xy[(size_t)n * k + o] = make_double2(lon, lat);
  }
  along[o] = ob.along;
  if (ob.turns != turns0) {
    u[o] = ob.u;
    v[o] = ob.v;
    turns[o] = ob.turns;
    len[o] = ob.len;
  }
}

template <typename T>
bool dev_alloc(T **p, size_t count) {
  void *v = nullptr;
  if (cudaMalloc(&v, count * sizeof(T) > 0 ? count * sizeof(T) : 16) != cudaSuccess) return false;
  *p = (T *)v;
  return true;
}

void release(stc_trace_dev *g) {
  if (g->stream) cudaStreamSynchronize(g->stream);
  cudaFree(g->tab);
  cudaFree(g->u);
  cudaFree(g->v);
  cudaFree(g->turns);
  cudaFree(g->along);
  cudaFree(g->len);
  cudaFree(g->speed);
  if (g->ev0) cudaEventDestroy(g->ev0);
  if (g->ev1) cudaEventDestroy(g->ev1);
  if (g->stream) cudaStreamDestroy(g->stream);
}

struct DeviceScope {
  int prev = 0;
  explicit DeviceScope(int d) {
    cudaGetDevice(&prev);
    cudaSetDevice(d);
  }
  ~DeviceScope() { cudaSetDevice(prev); }
};

uint32_t blocks_for(uint32_t n) { return (n + TG_THREADS - 1) / TG_THREADS; }

}  // namespace

extern "C" stc_status stc_trace_dev_create(const stc_trace_config *cfg, int device, stc_trace_dev **out) {
  if (!out) return STC_ERR_INVALID_ARG;
  *out = nullptr;
  if (!cfg || cfg->num_objects == 0 || cfg->grid_n < 2 || cfg->box_m <= 0.0 || cfg->n_hotspots < 0 ||
      (uint64_t)cfg->grid_n * (uint64_t)cfg->grid_n > 0xFFFFFFFFull)
    return STC_ERR_INVALID_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return STC_ERR_INVALID_ARG;
  DeviceScope scope(device);
  stc_trace_dev *g = new stc_trace_dev();
  g->cfg = *cfg;
  g->device = device;
  const int32_t G = cfg->grid_n, H = cfg->n_hotspots;
  const uint32_t nn = (uint32_t)G * (uint32_t)G, n = cfg->num_objects;
  const size_t tab = 2 * (size_t)nn + 3 * (size_t)(H > 0 ? H : 1);
  bool ok = dev_alloc(&g->tab, tab) && dev_alloc(&g->u, n) && dev_alloc(&g->v, n) && dev_alloc(&g->turns, n) &&
            dev_alloc(&g->along, n) && dev_alloc(&g->len, n) && dev_alloc(&g->speed, n) &&
            cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreate(&g->ev0) == cudaSuccess && cudaEventCreate(&g->ev1) == cudaSuccess;
  if (!ok) {
    release(g);
    delete g;
    return STC_ERR_CUDA;
  }
  tg_world &w = g->w;
  double *node_x = g->tab, *node_y = g->tab + nn;
  double *hot = g->tab + 2 * (size_t)nn;
  w.node_x = node_x;
  w.node_y = node_y;
  w.hot_x = hot;
  w.hot_y = hot + (H > 0 ? H : 1);
  w.hot_cdf = hot + 2 * (H > 0 ? H : 1);
  w.grid_n = G;
  w.n_hotspots = H;
  w.spacing = cfg->box_m / (double)(G - 1);
  w.box_m = cfg->box_m;
  w.sigma_m = cfg->sigma_m;
  w.hot_frac = cfg->hot_frac;
  w.speed_lo = cfg->speed_lo;
  w.speed_hi = cfg->speed_hi;
  w.seed = cfg->seed;
  cudaError_t e = cudaSuccess;
  if (H > 0) {
    /* The hotspot table is a few thousand FP64 series terms: computed here
     * with the same operations as the host generator and copied. */
    double *hx = (double *)malloc(3 * (size_t)H * sizeof(double));
    if (!hx) {
      release(g);
      delete g;
      return STC_ERR_CUDA;
    }
    double *hy = hx + H, *hc = hx + 2 * (size_t)H, total = 0.0;
    for (int k = 0; k < H; k++) {
      double wk;
      tg_hotspot(cfg->seed, cfg->box_m, cfg->zipf_s, k, &hx[k], &hy[k], &wk);
      total = total + wk;
      hc[k] = total;
    }
    for (int k = 0; k < H; k++) hc[k] = hc[k] / total;
    hc[H - 1] = 1.0;
    e = cudaMemcpyAsync(hot, hx, 3 * (size_t)H * sizeof(double), cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    free(hx);
  }
  if (e == cudaSuccess) {
    k_tg_nodes<<<(nn + TG_THREADS - 1) / TG_THREADS, TG_THREADS, 0, g->stream>>>(
        cfg->seed, G, w.spacing, cfg->jitter_m, nn, node_x, node_y);
    k_tg_place<<<blocks_for(n), TG_THREADS, 0, g->stream>>>(w, n, g->u, g->v, g->turns, g->along, g->len,
                                                           g->speed);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  }
  if (e != cudaSuccess) {
    release(g);
    delete g;
    return STC_ERR_CUDA;
  }
  *out = g;
  return STC_OK;
}

extern "C" stc_status stc_trace_dev_next(stc_trace_dev *g, double *xy_device, uint32_t steps) {
  if (!g || !xy_device || ((uintptr_t)xy_device & 15) != 0) return STC_ERR_INVALID_ARG;
  if (steps == 0) return STC_OK;
  DeviceScope scope(g->device);
  const uint32_t n = g->cfg.num_objects;
  cudaEventRecord(g->ev0, g->stream);
  k_tg_steps<<<blocks_for(n), TG_THREADS, 0, g->stream>>>(g->w, n, g->step, steps, g->u, g->v, g->turns,
                                                         g->along, g->len, g->speed, (double2 *)xy_device);
  cudaError_t e = cudaGetLastError();
  cudaEventRecord(g->ev1, g->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  if (e != cudaSuccess) return STC_ERR_CUDA;
  cudaEventElapsedTime(&g->last_ms, g->ev0, g->ev1);
  g->step += steps;
  return STC_OK;
}

extern "C" uint32_t stc_trace_dev_step(const stc_trace_dev *g) { return g ? g->step : 0; }

extern "C" stc_status stc_trace_dev_map_box(const stc_trace_dev *g, double pad_m, double mbr[4]) {
  if (!g || !mbr) return STC_ERR_INVALID_ARG;
  tg_map_box(g->cfg.box_m, g->cfg.jitter_m, pad_m, mbr);
  return STC_OK;
}

extern "C" float stc_trace_dev_last_ms(const stc_trace_dev *g) { return g ? g->last_ms : 0.0f; }

extern "C" void stc_trace_dev_destroy(stc_trace_dev *g) {
  if (!g) return;
  DeviceScope scope(g->device);
  release(g);
  delete g;
}
