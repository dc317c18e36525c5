/*
 * stc_trace.h -- seeded synthetic object traces, generated on the device.
 *
 * The reference produces its traces with an unseeded road-network walker
 * (Map::navigate, geometry/Map.cpp:483-589, driven from
 * tracing/generator.cpp:387-406) over Chicago street data that is not part
 * of the checkout. This library stands in for it with a seeded grid-graph
 * walker: a G x G grid of jittered street nodes, objects moving along edges
 * at a constant speed and turning onto a random incident edge at every node,
 * a Zipf-weighted set of Gaussian hotspots for the starting points.
 *
 * Two implementations share one per-object arithmetic:
 *   libstctrace.so  host C (stc_tracegen_* in the package's tracegen.h)
 *   libstc.so       the stc_trace_dev_* calls below: walker state resident in
 *                   device memory, one thread per object, positions written
 *                   straight into a device buffer that stc_step_device reads.
 * Both write bit-identical (lon, lat) f64 positions for the same
 * configuration and step.
 */
#ifndef STC_TRACE_H
#define STC_TRACE_H

#include <stdint.h>

#include "stc.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct stc_trace_config {
  uint32_t num_objects;
  int32_t grid_n;             /* street nodes per side, >= 2 */
  double box_m;               /* side of the square box, metres */
  double jitter_m;            /* node jitter, +- metres */
  double speed_lo, speed_hi;  /* m/s, uniform */
  int32_t n_hotspots;         /* 0: all objects start uniformly on edges */
  double hot_frac;            /* fraction of objects drawn from hotspots */
  double sigma_m;             /* hotspot Gaussian sigma, metres */
  double zipf_s;              /* hotspot weight exponent */
  uint64_t seed;
} stc_trace_config;

typedef struct stc_trace_dev stc_trace_dev;

/* Places every object on the device of the given ordinal (step 0).
 * STC_ERR_INVALID_ARG for an empty or degenerate configuration. */
stc_status stc_trace_dev_create(const stc_trace_config *cfg, int device, stc_trace_dev **out);

/* Writes `steps` consecutive steps of positions, step k at
 * xy_device + 2 * num_objects * k, as (lon, lat) f64 pairs indexed by object,
 * and advances the walker by one second after each; the first step written
 * by a fresh generator is the start positions. Returns after the positions
 * are in device memory. */
stc_status stc_trace_dev_next(stc_trace_dev *g, double *xy_device, uint32_t steps);

/* Number of steps written so far. */
uint32_t stc_trace_dev_step(const stc_trace_dev *g);

/* Map box around the street grid padded by pad_m metres: lon/lat degrees
 * (low x, low y, high x, high y); the same box as the host generator's. */
stc_status stc_trace_dev_map_box(const stc_trace_dev *g, double pad_m, double mbr[4]);

/* Milliseconds of device time of the last stc_trace_dev_next call. */
float stc_trace_dev_last_ms(const stc_trace_dev *g);

void stc_trace_dev_destroy(stc_trace_dev *g);

#ifdef __cplusplus
}
#endif
#endif
