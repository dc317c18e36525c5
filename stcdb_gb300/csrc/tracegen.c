/*
 * Seeded synthetic object traces for the co-occurrence pipeline (host side).
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
 * The per-object arithmetic lives in tracegen_walk.h, shared with the device
 * generator (stc_tracegen.cu). Determinism across hosts: every random draw
 * comes from a counter-based hash; the only floating-point operations are
 * IEEE +, -, *, / and sqrt, compiled with -ffp-contract=off, so x86-64 and
 * aarch64 (and the device) produce identical bits. The Zipf weights use the
 * series in tracegen_walk.h instead of libm pow().
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "tracegen.h"
#include "tracegen_walk.h"

struct stc_tracegen {
  stc_trace_config cfg;
  tg_world w;
  double *node_x, *node_y;          /* metres, G*G */
  double *hot_x, *hot_y, *hot_cdf;  /* hotspots */
  tg_obj *obj;
  uint32_t step;
};

stc_tracegen *stc_tracegen_create(const stc_trace_config *cfg) {
  if (!cfg || cfg->num_objects == 0 || cfg->grid_n < 2 || cfg->box_m <= 0.0) return NULL;
  stc_tracegen *g = (stc_tracegen *)calloc(1, sizeof(stc_tracegen));
  if (!g) return NULL;
  g->cfg = *cfg;
  int G = cfg->grid_n;
  size_t nn = (size_t)G * G, n = cfg->num_objects;
  g->node_x = (double *)malloc(nn * sizeof(double));
  g->node_y = (double *)malloc(nn * sizeof(double));
  g->obj = (tg_obj *)malloc(n * sizeof(tg_obj));
  int H = cfg->n_hotspots > 0 ? cfg->n_hotspots : 1;
  g->hot_x = (double *)malloc(H * sizeof(double));
  g->hot_y = (double *)malloc(H * sizeof(double));
  g->hot_cdf = (double *)malloc(H * sizeof(double));
  if (!g->node_x || !g->node_y || !g->obj || !g->hot_x || !g->hot_y || !g->hot_cdf) {
    stc_tracegen_destroy(g);
    return NULL;
  }
  uint64_t s = cfg->seed;
  tg_world *w = &g->w;
  w->node_x = g->node_x;
  w->node_y = g->node_y;
  w->hot_x = g->hot_x;
  w->hot_y = g->hot_y;
  w->hot_cdf = g->hot_cdf;
  w->grid_n = G;
  w->n_hotspots = cfg->n_hotspots;
  w->spacing = cfg->box_m / (double)(G - 1);
  w->box_m = cfg->box_m;
  w->sigma_m = cfg->sigma_m;
  w->hot_frac = cfg->hot_frac;
  w->speed_lo = cfg->speed_lo;
  w->speed_hi = cfg->speed_hi;
  w->seed = s;
  for (uint32_t id = 0; id < (uint32_t)nn; id++)
    tg_node_xy(s, G, w->spacing, cfg->jitter_m, id, &g->node_x[id], &g->node_y[id]);
  if (cfg->n_hotspots > 0) {
    double total = 0.0;
    for (int k = 0; k < cfg->n_hotspots; k++) {
      double wk;
      tg_hotspot(s, cfg->box_m, cfg->zipf_s, k, &g->hot_x[k], &g->hot_y[k], &wk);
      total = total + wk;
      g->hot_cdf[k] = total;
    }
    for (int k = 0; k < cfg->n_hotspots; k++) g->hot_cdf[k] = g->hot_cdf[k] / total;
    g->hot_cdf[cfg->n_hotspots - 1] = 1.0;
  }
  long long N = (long long)n;
#pragma omp parallel for schedule(static)
  for (long long oo = 0; oo < N; oo++) tg_place(w, (uint32_t)oo, &g->obj[oo]);
  g->step = 0;
  return g;
}

void stc_tracegen_destroy(stc_tracegen *g) {
  if (!g) return;
  free(g->node_x); free(g->node_y); free(g->hot_x); free(g->hot_y); free(g->hot_cdf);
  free(g->obj);
  free(g);
}

int stc_tracegen_next(stc_tracegen *g, double *xy) {
  if (!g || !xy) return -1;
  long long N = (long long)g->cfg.num_objects;
  int advance = g->step > 0;
#pragma omp parallel for schedule(static)
  for (long long oo = 0; oo < N; oo++) {
    tg_obj *ob = &g->obj[oo];
    if (advance) tg_advance(&g->w, (uint32_t)oo, ob);
    tg_lonlat(&g->w, ob, &xy[2 * (size_t)oo], &xy[2 * (size_t)oo + 1]);
  }
  g->step++;
  return 0;
}

void stc_tracegen_map_box(const stc_tracegen *g, double pad_m, double mbr[4]) {
  tg_map_box(g->cfg.box_m, g->cfg.jitter_m, pad_m, mbr);
}

uint32_t stc_tracegen_step(const stc_tracegen *g) { return g ? g->step : 0; }
