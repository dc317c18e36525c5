/*
 * CPU restatement of the reference's co-occurrence path -- TEST
 * INFRASTRUCTURE ONLY. Tests, the smoke check and the benchmark's CPU
 * baseline use it as the checker; the product library never links it.
 *
 * Parity: pinned. The (pid_lo, pid_hi, start, end) tuples are checked
 * against the reference's own CPU implementation compiled from its sources
 * (oracle/build_ref.sh + oracle/ref_driver.cpp) on seeded workloads, and
 * against the fixtures under tests/golden/ generated that way. The meeting
 * MBR and the map-box filter restate the reference's GPU semantics
 * (cuda/geometry.cu:461-489, :665-670); the reference's CPU path does not
 * compute them, so that part is pinned only by this restatement.
 */
#ifndef STC_ORACLE_H
#define STC_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#include "stc.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_ctx oracle_ctx;

/* threads <= 1: deterministic single-threaded order (the golden order).
 * threads > 1: OpenMP-parallel filter/refine/sweep with atomic inserts, for
 * timing only (its output depends on thread interleaving, like the
 * reference's pthread path). */
oracle_ctx *oracle_create(const stc_config *cfg, const double mbr[4], const double *xy0, uint32_t n,
                          int threads);
/* 0 on success; negative on error (see oracle_error). */
int oracle_step(oracle_ctx *c, const double *xy, uint32_t t);
/* Meetings emitted by the last step, in bucket order. */
size_t oracle_emitted(oracle_ctx *c, const stc_meeting **out);
void oracle_stats(oracle_ctx *c, stc_stats *s);
const char *oracle_error(oracle_ctx *c);
void oracle_destroy(oracle_ctx *c);

/* Copies the current schema (node type, grid id, children, boxes) for
 * inspection in tests: arrays sized by oracle_schema_size. */
uint32_t oracle_schema_size(oracle_ctx *c);
void oracle_schema_dump(oracle_ctx *c, int16_t *type, uint32_t *grid_id, uint32_t *children,
                        double *boxes);
uint32_t oracle_schema_stack_index(oracle_ctx *c);
uint32_t oracle_grids_stack_index(oracle_ctx *c);

/* The reference's degree_per_meter_longitude (util/util.h:59-66), exported
 * so tests can compare the device implementation against host libm. */
double oracle_dpml(double latitude);

#ifdef __cplusplus
}
#endif
#endif
