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

/* ---- memtable and flush (oracle/stc_lsm.c) ----------------------------
 * Feed each step's emitted meetings with lsm_append; flush when
 * lsm_kv_count exceeds the restriction (or to end a run). Read-out layout is
 * that of stc_read_ctb. */
typedef struct lsm_oracle lsm_oracle;
lsm_oracle *lsm_create(uint32_t n, uint32_t max_meet_time, uint32_t ctf_count, double area_restriction,
                       uint32_t first_end_time_min, const double map[4], uint64_t capacity);
void lsm_destroy(lsm_oracle *o);
const char *lsm_error(const lsm_oracle *o);
int lsm_append(lsm_oracle *o, const stc_meeting *m, size_t count);
uint64_t lsm_kv_count(const lsm_oracle *o);
int lsm_flush(lsm_oracle *o, uint32_t cur_time);
int lsm_get_ctb(const lsm_oracle *o, stc_ctb_info *info);
int lsm_read_ctb(const lsm_oracle *o, stc_ctf *ctfs, uint8_t *bitmaps, uint8_t *keys, uint16_t *sids,
                 uint64_t *okeys, float *oboxes, uint8_t *obitmap);
/* single routines, pinned against the reference's host code */
int lsm_ctf_bits(const float mbr[4], const double map[4], uint32_t num_objects, uint32_t max_meet_time,
                 stc_ctf *c);
uint64_t lsm_serialize_mbr(const float b[4], const stc_ctf *c);
void lsm_pack_key(uint64_t pid_field, uint64_t target, uint64_t duration, uint64_t end, uint64_t value_mbr,
                  const stc_ctf *c, uint8_t *out);
void lsm_o_bitmap(const float b[4], const double map[4], uint8_t *bitmap);  /* edge 256 */
void lsm_o_bitmap_edge(const float b[4], const double map[4], uint32_t edge, uint8_t *bitmap);
/* map bitmap edge of the blocks flushed from now on (default 256) */
int lsm_set_bitmap_edge(lsm_oracle *o, uint32_t edge);
void lsm_decode_key(const uint8_t *key, const stc_ctf *c, uint32_t *oid, uint32_t *target, uint32_t *duration,
                    uint32_t *end, uint64_t *value_mbr, double box[4]);
/* queries on one block read out as stc_read_ctb lays it out; n: matches so
 * far (results go to out[n..cap)); returns the new count */
size_t lsm_query_object_block(const stc_ctb_info *in, const stc_ctf *ctfs, const uint8_t *keys,
                              const uint16_t *sids, const uint64_t *okeys, const float *oboxes, uint32_t pid,
                              uint32_t t1, uint32_t t2, stc_contact *out, size_t cap, size_t n);
size_t lsm_query_box_block(const stc_ctb_info *in, const stc_ctf *ctfs, const uint8_t *keys, const uint64_t *okeys,
                           const float *oboxes, const double q[4], uint32_t t1, uint32_t t2, stc_contact *out,
                           size_t cap, size_t n);

/* Compaction (stc_compact.cpp): merges m blocks, each read out as
 * stc_read_ctb lays it out, into one block of split x split CTFs. */
typedef struct cmp_block {
  stc_ctb_info info;
  const stc_ctf *ctfs;
  const uint8_t *keys;
  const uint16_t *sids;
  const uint64_t *okeys;
  const float *oboxes;
  const uint8_t *obitmap;
} cmp_block;
typedef struct cmp_result cmp_result;
/* reference_mode: follow merge_dump literally where its output is pinned
 * (see stc_compact.cpp). NULL on error (message in err). */
cmp_result *cmp_compact(const cmp_block *blocks, uint32_t m, uint32_t num_objects, uint32_t split,
                        uint32_t max_meet_time, const double map[4], uint32_t new_index, int reference_mode,
                        char *err, size_t errlen);
int cmp_get(const cmp_result *r, stc_ctb_info *info);
int cmp_read(const cmp_result *r, stc_ctf *ctfs, uint8_t *bitmaps, uint8_t *keys, uint16_t *sids, uint64_t *okeys,
             float *oboxes, uint8_t *obitmap);
void cmp_free(cmp_result *r);

#ifdef __cplusplus
}
#endif
#endif
