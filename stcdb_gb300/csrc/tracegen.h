/* Seeded synthetic grid-graph traces (host code). See tracegen.c. */
#ifndef STC_TRACEGEN_H
#define STC_TRACEGEN_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct stc_trace_config {
  uint32_t num_objects;
  int32_t grid_n;       /* street nodes per side */
  double box_m;         /* side of the square box, metres */
  double jitter_m;      /* node jitter, +- metres */
  double speed_lo, speed_hi;  /* m/s, uniform */
  int32_t n_hotspots;   /* 0: all objects start uniformly on edges */
  double hot_frac;      /* fraction of objects drawn from hotspots */
  double sigma_m;       /* hotspot Gaussian sigma, metres */
  double zipf_s;        /* hotspot weight exponent */
  uint64_t seed;
} stc_trace_config;

typedef struct stc_tracegen stc_tracegen;

stc_tracegen *stc_tracegen_create(const stc_trace_config *cfg);
void stc_tracegen_destroy(stc_tracegen *g);
/* Writes the positions of the current step as num_objects (lon, lat) f64
 * pairs and advances the walker by one second. The first call returns the
 * start positions. */
int stc_tracegen_next(stc_tracegen *g, double *xy);
/* Map box around the street grid padded by pad_m metres: lon/lat degrees
 * (low x, low y, high x, high y). */
void stc_tracegen_map_box(const stc_tracegen *g, double pad_m, double mbr[4]);
uint32_t stc_tracegen_step(const stc_tracegen *g);

#ifdef __cplusplus
}
#endif
#endif
