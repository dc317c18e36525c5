/*
 * Per-object arithmetic of the seeded grid-graph walker, shared by the host
 * generator (tracegen.c, gcc -ffp-contract=off) and the device generator
 * (stc_tracegen.cu).
 *
 * Every floating-point operation goes through TG_ADD, TG_SUB, TG_MUL, TG_DIV
 * and TG_SQRT: the plain IEEE operators on the host, the round-to-nearest
 * intrinsics on the device, where the compiler would otherwise fuse a
 * multiply and an add into one rounding. Conversions are exact or truncate
 * the same way on both sides, so the two produce the same bits.
 *
 * Random draws come from a counter-based hash (the splitmix64 finaliser)
 * keyed by (seed, stream, counter): an object's draws do not depend on how
 * many threads run or in which order.
 */
#ifndef STC_TRACEGEN_WALK_H
#define STC_TRACEGEN_WALK_H

#include <stdint.h>

#if defined(__CUDACC__)
#define TG_FN static inline __host__ __device__
#else
#define TG_FN static inline
#endif

#if defined(__CUDA_ARCH__)
#define TG_ADD(a, b) __dadd_rn((a), (b))
#define TG_SUB(a, b) __dsub_rn((a), (b))
#define TG_MUL(a, b) __dmul_rn((a), (b))
#define TG_DIV(a, b) __ddiv_rn((a), (b))
#define TG_SQRT(a) __dsqrt_rn(a)
#else
#include <math.h>
#define TG_ADD(a, b) ((a) + (b))
#define TG_SUB(a, b) ((a) - (b))
#define TG_MUL(a, b) ((a) * (b))
#define TG_DIV(a, b) ((a) / (b))
#define TG_SQRT(a) sqrt(a)
#endif

/* Reference map corner (data/streets.map) and degree scales. */
#define TG_LON0 (-0x1.5fc2a607825b0p+6)   /* -87.94008647664191 */
#define TG_LAT0 (0x1.4d281bab9fff8p+5)    /*  41.644584027118924 */
/* 360/(sin((90-|LAT0|)*3.14159265/180)*40076*1000): degrees of longitude per
 * metre at LAT0, evaluated once with the reference's formula (util/util.h:59-66). */
#define TG_DPML0 (0x1.935a0c55da44bp-17)
/* 360/(40076*1000): degrees of latitude per metre (util/util.h:57). */
#define TG_DPM_LAT (0x1.2d6acd5025901p-17)

enum { TG_ST_NODE = 1, TG_ST_OBJ = 2, TG_ST_HOT = 3, TG_ST_TURN = 4, TG_ST_INIT = 5 };
enum { TG_MAX_TURNS_PER_STEP = 64 };

/* The read-only world an object walks in. Arrays live on the side that runs
 * the walker (host memory for tracegen.c, device memory for the kernels). */
typedef struct tg_world {
  const double *node_x, *node_y;            /* metres, grid_n * grid_n, id = j * G + i */
  const double *hot_x, *hot_y, *hot_cdf;    /* n_hotspots entries */
  int32_t grid_n, n_hotspots;
  double spacing, box_m, sigma_m, hot_frac, speed_lo, speed_hi;
  uint64_t seed;
} tg_world;

/* One object's walker state: on the edge u -> v of length len, `along`
 * metres from u. */
typedef struct tg_obj {
  uint32_t u, v, turns;
  double along, len, speed;
} tg_obj;

TG_FN uint64_t tg_mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

TG_FN uint64_t tg_rnd(uint64_t seed, uint64_t stream, uint64_t ctr) {
  return tg_mix64(tg_mix64(seed ^ tg_mix64(stream * 0xD1B54A32D192ED03ULL)) ^ ctr);
}

/* Uniform double in [0, 1): the top 53 bits, scaled exactly. */
TG_FN double tg_unif(uint64_t seed, uint64_t stream, uint64_t ctr) {
  return (double)(tg_rnd(seed, stream, ctr) >> 11) * 0x1.0p-53;
}

/* ln(x) for x >= 1 from the atanh series: x = m 2^e, ln m = 2 atanh((m-1)/(m+1)). */
TG_FN double tg_log(double x) {
  int e = 0;
  while (x >= 2.0) { x = TG_MUL(x, 0.5); e++; }
  double z = TG_DIV(TG_SUB(x, 1.0), TG_ADD(x, 1.0)), z2 = TG_MUL(z, z), term = z, sum = 0.0;
  for (int k = 1; k < 80; k += 2) {
    sum = TG_ADD(sum, TG_DIV(term, (double)k));
    term = TG_MUL(term, z2);
  }
  const double LN2 = 0x1.62e42fefa39efp-1;
  return TG_ADD(TG_MUL(2.0, sum), TG_MUL((double)e, LN2));
}

/* exp(x) for x <= 0 by argument halving and a Taylor series. */
TG_FN double tg_exp(double x) {
  int h = 0;
  while (x < -0.25) { x = TG_MUL(x, 0.5); h++; }
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 30; k++) {
    term = TG_DIV(TG_MUL(term, x), (double)k);
    sum = TG_ADD(sum, term);
  }
  for (int i = 0; i < h; i++) sum = TG_MUL(sum, sum);
  return sum;
}

TG_FN uint32_t tg_node_id(int32_t G, int i, int j) { return (uint32_t)j * (uint32_t)G + (uint32_t)i; }

/* Node id's position: the grid point (i, j) * spacing, jittered by +-jitter_m. */
TG_FN void tg_node_xy(uint64_t seed, int32_t G, double spacing, double jitter_m, uint32_t id,
                      double *x, double *y) {
  int i = (int)(id % (uint32_t)G), j = (int)(id / (uint32_t)G);
  double jx = TG_MUL(TG_SUB(TG_MUL(2.0, tg_unif(seed, TG_ST_NODE, 2ull * id)), 1.0), jitter_m);
  double jy = TG_MUL(TG_SUB(TG_MUL(2.0, tg_unif(seed, TG_ST_NODE, 2ull * id + 1)), 1.0), jitter_m);
  *x = TG_ADD(TG_MUL((double)i, spacing), jx);
  *y = TG_ADD(TG_MUL((double)j, spacing), jy);
}

/* Hotspot k's centre and its Zipf weight (k+1)^-zipf_s. */
TG_FN void tg_hotspot(uint64_t seed, double box_m, double zipf_s, int k, double *x, double *y,
                      double *w) {
  *x = TG_MUL(TG_ADD(0.05, TG_MUL(0.9, tg_unif(seed, TG_ST_HOT, 2ull * k))), box_m);
  *y = TG_MUL(TG_ADD(0.05, TG_MUL(0.9, tg_unif(seed, TG_ST_HOT, 2ull * k + 1))), box_m);
  *w = tg_exp(TG_MUL(-zipf_s, tg_log((double)(k + 1))));
}

TG_FN double tg_edge_len(const tg_world *w, uint32_t a, uint32_t b) {
  double dx = TG_SUB(w->node_x[b], w->node_x[a]), dy = TG_SUB(w->node_y[b], w->node_y[a]);
  return TG_SQRT(TG_ADD(TG_MUL(dx, dx), TG_MUL(dy, dy)));
}

/* Neighbours of node n in a fixed order: +x, -x, +y, -y. */
TG_FN int tg_neighbours(int32_t G, uint32_t n, uint32_t out[4]) {
  int i = (int)(n % (uint32_t)G), j = (int)(n / (uint32_t)G), c = 0;
  if (i + 1 < G) out[c++] = tg_node_id(G, i + 1, j);
  if (i > 0) out[c++] = tg_node_id(G, i - 1, j);
  if (j + 1 < G) out[c++] = tg_node_id(G, i, j + 1);
  if (j > 0) out[c++] = tg_node_id(G, i, j - 1);
  return c;
}

/* A uniformly drawn edge and a uniform point on it. */
TG_FN void tg_place_uniform(const tg_world *w, uint32_t o, tg_obj *ob) {
  uint64_t s = w->seed;
  uint32_t nn = (uint32_t)w->grid_n * (uint32_t)w->grid_n;
  uint32_t a = (uint32_t)TG_MUL(tg_unif(s, TG_ST_INIT, 4ull * o), (double)nn);
  if (a >= nn) a = nn - 1;
  uint32_t nb[4];
  int c = tg_neighbours(w->grid_n, a, nb);
  int k = (int)TG_MUL(tg_unif(s, TG_ST_INIT, 4ull * o + 1), (double)c);
  if (k >= c) k = c - 1;
  ob->u = a;
  ob->v = nb[k];
  ob->len = tg_edge_len(w, a, nb[k]);
  ob->along = TG_MUL(tg_unif(s, TG_ST_INIT, 4ull * o + 2), ob->len);
}

/* A Gaussian sample around a Zipf-drawn hotspot, projected onto the edge
 * from its nearest grid node towards the sample. */
TG_FN void tg_place_hotspot(const tg_world *w, uint32_t o, tg_obj *ob) {
  uint64_t s = w->seed;
  double r = tg_unif(s, TG_ST_INIT, 4ull * o + 3);
  int lo = 0, hi = w->n_hotspots - 1;
  while (lo < hi) {  /* first hotspot with cdf > r */
    int mid = (lo + hi) / 2;
    if (w->hot_cdf[mid] > r) hi = mid; else lo = mid + 1;
  }
  /* Irwin-Hall approximation of a standard normal: sum of 12 uniforms - 6. */
  double gx = -6.0, gy = -6.0;
  for (int k = 0; k < 12; k++) {
    gx = TG_ADD(gx, tg_unif(s, TG_ST_OBJ, 32ull * o + (uint64_t)k));
    gy = TG_ADD(gy, tg_unif(s, TG_ST_OBJ, 32ull * o + 12u + (uint64_t)k));
  }
  double box = w->box_m;
  double px = TG_ADD(w->hot_x[lo], TG_MUL(gx, w->sigma_m));
  double py = TG_ADD(w->hot_y[lo], TG_MUL(gy, w->sigma_m));
  if (px < 0.0) px = 0.0;
  if (px > box) px = box;
  if (py < 0.0) py = 0.0;
  if (py > box) py = box;
  int G = w->grid_n;
  int i = (int)TG_ADD(TG_DIV(px, w->spacing), 0.5), j = (int)TG_ADD(TG_DIV(py, w->spacing), 0.5);
  if (i >= G) i = G - 1;
  if (j >= G) j = G - 1;
  uint32_t a = tg_node_id(G, i, j);
  double dx = TG_SUB(px, w->node_x[a]), dy = TG_SUB(py, w->node_y[a]);
  int ni = i, nj = j;
  if (fabs(dx) >= fabs(dy)) {
    ni = dx >= 0.0 ? i + 1 : i - 1;
    if (ni < 0 || ni >= G) ni = dx >= 0.0 ? i - 1 : i + 1;
  } else {
    nj = dy >= 0.0 ? j + 1 : j - 1;
    if (nj < 0 || nj >= G) nj = dy >= 0.0 ? j - 1 : j + 1;
  }
  uint32_t b = tg_node_id(G, ni, nj);
  double L = tg_edge_len(w, a, b);
  double ex = TG_DIV(TG_SUB(w->node_x[b], w->node_x[a]), L);
  double ey = TG_DIV(TG_SUB(w->node_y[b], w->node_y[a]), L);
  double t = TG_ADD(TG_MUL(dx, ex), TG_MUL(dy, ey));
  if (t < 0.0) t = 0.0;
  if (t >= L) t = TG_MUL(L, 0.999);
  ob->u = a;
  ob->v = b;
  ob->len = L;
  ob->along = t;
}

/* Step-0 state of object o: a hotspot start with probability hot_frac, else
 * a uniform one; a speed from U[speed_lo, speed_hi]. */
TG_FN void tg_place(const tg_world *w, uint32_t o, tg_obj *ob) {
  uint64_t s = w->seed;
  int hot = w->n_hotspots > 0 && tg_unif(s, TG_ST_OBJ, 32ull * o + 30) < w->hot_frac;
  if (hot) tg_place_hotspot(w, o, ob); else tg_place_uniform(w, o, ob);
  ob->turns = 0;
  ob->speed = TG_ADD(w->speed_lo,
                     TG_MUL(TG_SUB(w->speed_hi, w->speed_lo), tg_unif(s, TG_ST_OBJ, 32ull * o + 31)));
}

/* One second of movement: `speed` metres along the edges, a uniformly drawn
 * incident edge at every node reached (at most TG_MAX_TURNS_PER_STEP). */
TG_FN void tg_advance(const tg_world *w, uint32_t o, tg_obj *ob) {
  double a = TG_ADD(ob->along, ob->speed);
  int guard = 0;
  while (a >= ob->len && guard++ < TG_MAX_TURNS_PER_STEP) {
    a = TG_SUB(a, ob->len);
    uint32_t nb[4];
    uint32_t cur = ob->v;
    int c = tg_neighbours(w->grid_n, cur, nb);
    int k = (int)TG_MUL(tg_unif(w->seed, TG_ST_TURN, ((uint64_t)o << 24) ^ (uint64_t)ob->turns), (double)c);
    if (k >= c) k = c - 1;
    ob->turns++;
    ob->u = cur;
    ob->v = nb[k];
    ob->len = tg_edge_len(w, cur, nb[k]);
  }
  ob->along = a;
}

/* The object's position in degrees at the reference map's corner. */
TG_FN void tg_lonlat(const tg_world *w, const tg_obj *ob, double *lon, double *lat) {
  uint32_t a = ob->u, b = ob->v;
  double f = TG_DIV(ob->along, ob->len);
  double mx = TG_ADD(w->node_x[a], TG_MUL(TG_SUB(w->node_x[b], w->node_x[a]), f));
  double my = TG_ADD(w->node_y[a], TG_MUL(TG_SUB(w->node_y[b], w->node_y[a]), f));
  *lon = TG_ADD(TG_LON0, TG_MUL(mx, TG_DPML0));
  *lat = TG_ADD(TG_LAT0, TG_MUL(my, TG_DPM_LAT));
}

/* Map box around the street grid padded by pad_m metres. */
TG_FN void tg_map_box(double box_m, double jitter_m, double pad_m, double mbr[4]) {
  double lo = TG_SUB(-jitter_m, pad_m), hi = TG_ADD(TG_ADD(box_m, jitter_m), pad_m);
  mbr[0] = TG_ADD(TG_LON0, TG_MUL(lo, TG_DPML0));
  mbr[1] = TG_ADD(TG_LAT0, TG_MUL(lo, TG_DPM_LAT));
  mbr[2] = TG_ADD(TG_LON0, TG_MUL(hi, TG_DPML0));
  mbr[3] = TG_ADD(TG_LAT0, TG_MUL(hi, TG_DPM_LAT));
}

#endif
