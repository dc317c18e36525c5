/* Seeded synthetic grid-graph traces (host code). See tracegen.c. */
#ifndef STC_TRACEGEN_H
#define STC_TRACEGEN_H
#include <stdint.h>

#include "stc_trace.h" /* stc_trace_config */

#ifdef __cplusplus
extern "C" {
#endif

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
