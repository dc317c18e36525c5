/*
 * Seeded synthetic object traces for the co-occurrence pipeline.
 *
 * The reference generates positions with an unseeded road-network walker
 * (tracing/generator.cpp:387-406, srand(time(NULL)) at :388) over Chicago
 * data files; its trace files are not available. This generator stands in
 * for them with a deterministic grid-graph walker:
 *   - a G x G grid of street nodes spanning a square box, every node jittered
 *     uniformly by +-jitter metres, 4-neighbour edges;
 *   - each object starts on an edge (uniform edge, or projected from a
 *     Gaussian hotspot sample) and moves along edges at a constant speed
 *     drawn from U[speed_lo, speed_hi] m/s, one second per step, choosing a
 *     uniformly random incident edge at every node it reaches;
 *   - hotspot weights follow a Zipf law k^-s over the hotspot ranks.
 * Positions are converted from metres to lon/lat degrees at the reference
 * map's south-west corner (data/streets.map), because the reference's
 * distance arithmetic works on degrees (util/util.h:57-66).
 *
 * Determinism across hosts: every random draw comes from a counter-based
 * hash (splitmix64 finaliser) keyed by (seed, stream, counter); the only
 * floating-point operations are IEEE +, -, *, / and sqrt, compiled with
 * -ffp-contract=off, so x86-64 and aarch64 produce identical bits. The two
 * transcendental constants are fixed bit patterns, and the Zipf weights use
 * the series below instead of libm pow().
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#include "tracegen.h"

/* Reference map corner (data/streets.map) and degree scales. */
static const double LON0 = -0x1.5fc2a607825b0p+6;          /* -87.94008647664191 */
static const double LAT0 = 0x1.4d281bab9fff8p+5;           /*  41.644584027118924 */
/* 360/(sin((90-|LAT0|)*3.14159265/180)*40076*1000): degrees of longitude per
 * metre at LAT0, evaluated once with the reference's formula (util/util.h:59-66). */
static const double DPML0 = 0x1.935a0c55da44bp-17;
/* 360/(40076*1000): degrees of latitude per metre (util/util.h:57). */
static const double DPM_LAT = 0x1.2d6acd5025901p-17;

static inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

static inline uint64_t rnd(uint64_t seed, uint64_t stream, uint64_t ctr) {
  return mix64(mix64(seed ^ mix64(stream * 0xD1B54A32D192ED03ULL)) ^ ctr);
}

/* Uniform double in [0, 1). */
static inline double unif(uint64_t seed, uint64_t stream, uint64_t ctr) {
  return (double)(rnd(seed, stream, ctr) >> 11) * 0x1.0p-53;
}

enum { ST_NODE = 1, ST_OBJ = 2, ST_HOT = 3, ST_TURN = 4, ST_INIT = 5 };

/* ln(x) for x >= 1 from the atanh series: x = m 2^e, ln m = 2 atanh((m-1)/(m+1)). */
static double portable_log(double x) {
  int e = 0;
  while (x >= 2.0) { x *= 0.5; e++; }
  double z = (x - 1.0) / (x + 1.0), z2 = z * z, term = z, sum = 0.0;
  for (int k = 1; k < 80; k += 2) { sum = sum + term / (double)k; term = term * z2; }
  const double LN2 = 0x1.62e42fefa39efp-1;
  return 2.0 * sum + (double)e * LN2;
}

/* exp(x) for x <= 0 by argument halving and a Taylor series. */
static double portable_exp(double x) {
  int h = 0;
  while (x < -0.25) { x *= 0.5; h++; }
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 30; k++) { term = term * x / (double)k; sum = sum + term; }
  for (int i = 0; i < h; i++) sum = sum * sum;
  return sum;
}

struct stc_tracegen {
  stc_trace_config cfg;
  double spacing;
  double *node_x, *node_y;          /* metres, G*G */
  double *hot_x, *hot_y, *hot_cdf;  /* hotspots */
  uint32_t *u, *v, *turns;
  double *along, *len, *speed;
  uint32_t step;
};

static inline uint32_t node_id(const stc_tracegen *g, int i, int j) {
  return (uint32_t)j * (uint32_t)g->cfg.grid_n + (uint32_t)i;
}

static inline double edge_len(const stc_tracegen *g, uint32_t a, uint32_t b) {
  double dx = g->node_x[b] - g->node_x[a], dy = g->node_y[b] - g->node_y[a];
  return sqrt(dx * dx + dy * dy);
}

/* Neighbours of node n in a fixed order: +x, -x, +y, -y. */
static int neighbours(const stc_tracegen *g, uint32_t n, uint32_t out[4]) {
  int G = g->cfg.grid_n, i = (int)(n % (uint32_t)G), j = (int)(n / (uint32_t)G), c = 0;
  if (i + 1 < G) out[c++] = node_id(g, i + 1, j);
  if (i > 0) out[c++] = node_id(g, i - 1, j);
  if (j + 1 < G) out[c++] = node_id(g, i, j + 1);
  if (j > 0) out[c++] = node_id(g, i, j - 1);
  return c;
}

static void place_uniform(stc_tracegen *g, uint32_t o) {
  uint64_t s = g->cfg.seed;
  uint32_t nn = (uint32_t)g->cfg.grid_n * (uint32_t)g->cfg.grid_n;
  uint32_t a = (uint32_t)(unif(s, ST_INIT, 4ull * o) * nn);
  if (a >= nn) a = nn - 1;
  uint32_t nb[4];
  int c = neighbours(g, a, nb);
  int k = (int)(unif(s, ST_INIT, 4ull * o + 1) * c);
  if (k >= c) k = c - 1;
  g->u[o] = a;
  g->v[o] = nb[k];
  g->len[o] = edge_len(g, a, nb[k]);
  g->along[o] = unif(s, ST_INIT, 4ull * o + 2) * g->len[o];
}

static void place_hotspot(stc_tracegen *g, uint32_t o) {
  uint64_t s = g->cfg.seed;
  double r = unif(s, ST_INIT, 4ull * o + 3);
  int lo = 0, hi = g->cfg.n_hotspots - 1;
  while (lo < hi) {  /* first hotspot with cdf > r */
    int mid = (lo + hi) / 2;
    if (g->hot_cdf[mid] > r) hi = mid; else lo = mid + 1;
  }
  /* Irwin-Hall approximation of a standard normal: sum of 12 uniforms - 6. */
  double gx = -6.0, gy = -6.0;
  for (int k = 0; k < 12; k++) {
    gx = gx + unif(s, ST_OBJ, 32ull * o + (uint64_t)k);
    gy = gy + unif(s, ST_OBJ, 32ull * o + 12u + (uint64_t)k);
  }
  double box = g->cfg.box_m;
  double px = g->hot_x[lo] + gx * g->cfg.sigma_m, py = g->hot_y[lo] + gy * g->cfg.sigma_m;
  if (px < 0.0) px = 0.0;
  if (px > box) px = box;
  if (py < 0.0) py = 0.0;
  if (py > box) py = box;
  int G = g->cfg.grid_n;
  int i = (int)(px / g->spacing + 0.5), j = (int)(py / g->spacing + 0.5);
  if (i >= G) i = G - 1;
  if (j >= G) j = G - 1;
  uint32_t a = node_id(g, i, j);
  double dx = px - g->node_x[a], dy = py - g->node_y[a];
  int ni = i, nj = j;
  if (fabs(dx) >= fabs(dy)) {
    ni = dx >= 0.0 ? i + 1 : i - 1;
    if (ni < 0 || ni >= G) ni = dx >= 0.0 ? i - 1 : i + 1;
  } else {
    nj = dy >= 0.0 ? j + 1 : j - 1;
    if (nj < 0 || nj >= G) nj = dy >= 0.0 ? j - 1 : j + 1;
  }
  uint32_t b = node_id(g, ni, nj);
  double L = edge_len(g, a, b);
  double ex = (g->node_x[b] - g->node_x[a]) / L, ey = (g->node_y[b] - g->node_y[a]) / L;
  double t = dx * ex + dy * ey;
  if (t < 0.0) t = 0.0;
  if (t >= L) t = L * 0.999;
  g->u[o] = a;
  g->v[o] = b;
  g->len[o] = L;
  g->along[o] = t;
}

stc_tracegen *stc_tracegen_create(const stc_trace_config *cfg) {
  if (!cfg || cfg->num_objects == 0 || cfg->grid_n < 2 || cfg->box_m <= 0.0) return NULL;
  stc_tracegen *g = (stc_tracegen *)calloc(1, sizeof(stc_tracegen));
  if (!g) return NULL;
  g->cfg = *cfg;
  int G = cfg->grid_n;
  size_t nn = (size_t)G * G, n = cfg->num_objects;
  g->spacing = cfg->box_m / (double)(G - 1);
  g->node_x = (double *)malloc(nn * sizeof(double));
  g->node_y = (double *)malloc(nn * sizeof(double));
  g->u = (uint32_t *)malloc(n * 4);
  g->v = (uint32_t *)malloc(n * 4);
  g->turns = (uint32_t *)calloc(n, 4);
  g->along = (double *)malloc(n * 8);
  g->len = (double *)malloc(n * 8);
  g->speed = (double *)malloc(n * 8);
  int H = cfg->n_hotspots > 0 ? cfg->n_hotspots : 1;
  g->hot_x = (double *)malloc(H * sizeof(double));
  g->hot_y = (double *)malloc(H * sizeof(double));
  g->hot_cdf = (double *)malloc(H * sizeof(double));
  if (!g->node_x || !g->node_y || !g->u || !g->v || !g->turns || !g->along || !g->len ||
      !g->speed || !g->hot_x || !g->hot_y || !g->hot_cdf) {
    stc_tracegen_destroy(g);
    return NULL;
  }
  uint64_t s = cfg->seed;
  for (int j = 0; j < G; j++)
    for (int i = 0; i < G; i++) {
      uint32_t id = node_id(g, i, j);
      double jx = (2.0 * unif(s, ST_NODE, 2ull * id) - 1.0) * cfg->jitter_m;
      double jy = (2.0 * unif(s, ST_NODE, 2ull * id + 1) - 1.0) * cfg->jitter_m;
      g->node_x[id] = (double)i * g->spacing + jx;
      g->node_y[id] = (double)j * g->spacing + jy;
    }
  if (cfg->n_hotspots > 0) {
    double total = 0.0;
    for (int k = 0; k < cfg->n_hotspots; k++) {
      g->hot_x[k] = (0.05 + 0.9 * unif(s, ST_HOT, 2ull * k)) * cfg->box_m;
      g->hot_y[k] = (0.05 + 0.9 * unif(s, ST_HOT, 2ull * k + 1)) * cfg->box_m;
      double w = portable_exp(-cfg->zipf_s * portable_log((double)(k + 1)));
      total = total + w;
      g->hot_cdf[k] = total;
    }
    for (int k = 0; k < cfg->n_hotspots; k++) g->hot_cdf[k] = g->hot_cdf[k] / total;
    g->hot_cdf[cfg->n_hotspots - 1] = 1.0;
  }
  long long N = (long long)n;
#pragma omp parallel for schedule(static)
  for (long long oo = 0; oo < N; oo++) {
    uint32_t o = (uint32_t)oo;
    int hot = cfg->n_hotspots > 0 && unif(s, ST_OBJ, 32ull * o + 30) < cfg->hot_frac;
    if (hot) place_hotspot(g, o); else place_uniform(g, o);
    g->speed[o] = cfg->speed_lo + (cfg->speed_hi - cfg->speed_lo) * unif(s, ST_OBJ, 32ull * o + 31);
  }
  g->step = 0;
  return g;
}

void stc_tracegen_destroy(stc_tracegen *g) {
  if (!g) return;
  free(g->node_x); free(g->node_y); free(g->hot_x); free(g->hot_y); free(g->hot_cdf);
  free(g->u); free(g->v); free(g->turns); free(g->along); free(g->len); free(g->speed);
  free(g);
}

static void write_positions(const stc_tracegen *g, double *xy) {
  long long N = (long long)g->cfg.num_objects;
#pragma omp parallel for schedule(static)
  for (long long oo = 0; oo < N; oo++) {
    uint32_t o = (uint32_t)oo;
    uint32_t a = g->u[o], b = g->v[o];
    double f = g->along[o] / g->len[o];
    double mx = g->node_x[a] + (g->node_x[b] - g->node_x[a]) * f;
    double my = g->node_y[a] + (g->node_y[b] - g->node_y[a]) * f;
    xy[2 * (size_t)o] = LON0 + mx * DPML0;
    xy[2 * (size_t)o + 1] = LAT0 + my * DPM_LAT;
  }
}

int stc_tracegen_next(stc_tracegen *g, double *xy) {
  if (!g || !xy) return -1;
  if (g->step > 0) {
    long long N = (long long)g->cfg.num_objects;
    uint64_t s = g->cfg.seed;
#pragma omp parallel for schedule(static)
    for (long long oo = 0; oo < N; oo++) {
      uint32_t o = (uint32_t)oo;
      double a = g->along[o] + g->speed[o];
      int guard = 0;
      while (a >= g->len[o] && guard++ < 64) {
        a = a - g->len[o];
        uint32_t nb[4];
        uint32_t cur = g->v[o];
        int c = neighbours(g, cur, nb);
        int k = (int)(unif(s, ST_TURN, ((uint64_t)o << 24) ^ (uint64_t)g->turns[o]) * c);
        if (k >= c) k = c - 1;
        g->turns[o]++;
        g->u[o] = cur;
        g->v[o] = nb[k];
        g->len[o] = edge_len(g, cur, nb[k]);
      }
      g->along[o] = a;
    }
  }
  write_positions(g, xy);
  g->step++;
  return 0;
}

void stc_tracegen_map_box(const stc_tracegen *g, double pad_m, double mbr[4]) {
  double lo = -g->cfg.jitter_m - pad_m, hi = g->cfg.box_m + g->cfg.jitter_m + pad_m;
  mbr[0] = LON0 + lo * DPML0;
  mbr[1] = LAT0 + lo * DPM_LAT;
  mbr[2] = LON0 + hi * DPML0;
  mbr[3] = LAT0 + hi * DPM_LAT;
}

uint32_t stc_tracegen_step(const stc_tracegen *g) { return g ? g->step : 0; }
