/* CPU restatement of the reference's memtable and flush (the LSM layer of the
 * co-occurrence path) -- TEST INFRASTRUCTURE ONLY: the checker for the GPU
 * flush in stcdb_gb300/csrc/stc_lsm.cu, never linked into the product.
 *
 * The reference builds its memtable in cuda_identify_meetings
 * (cuda/geometry.cu:701-737) and flushes it in process_with_gpu
 * (cuda/geometry.cu:1752-2138). Everything here is sequential and
 * deterministic; the reference's thrust sorts are stated as the stable sorts
 * they are (radix sort on integer keys), and its 128-bit key sort has no ties
 * (a directed pair has at most one meeting ending at a given step).
 *
 * Pinned against the reference's own host code (tests/golden/ctf_pin.npz,
 * made by tests/golden/make_ctf_pin.py through oracle/ref_ctf.cpp):
 * lsm_ctf_bits = CTF::get_ctf_bits, lsm_serialize_mbr = CTF::serial_mbr,
 * lsm_pack_key = CTF::serial_key, lsm_o_bitmap = oversize_buffer::write_o_buffer
 * (tracing/step_merge.cpp:41-63, 140-186, 284-310). The object ordering
 * (set_oid, STR slabs, make_sid) and the per-CTF reductions exist only as GPU
 * kernels in the reference and are restated here from cuda/geometry.cu:
 * 739-1107; those parts are unpinned.
 *
 * Float conversions follow the GPU's cvt.rzi rules: NaN -> 0, negative -> 0,
 * too large -> the maximum (the reference's host casts are undefined there;
 * they occur only for empty or zero-width CTFs). */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "stc_oracle.h"

typedef unsigned __int128 u128;

static uint32_t f2u32(float x) {
  if (!(x > 0.0f)) return 0;
  if (x >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)x;
}
static uint64_t f2u64(float x) {
  if (!(x > 0.0f)) return 0;
  if (x >= 18446744073709551616.0f) return ~0ull;
  return (uint64_t)x;
}
static uint32_t d2u32(double x) {
  if (!(x > 0.0)) return 0;
  if (x >= 4294967296.0) return 0xFFFFFFFFu;
  return (uint32_t)x;
}
static int32_t d2i32(double x) {
  if (x != x) return 0;
  if (x <= -2147483648.0) return INT32_MIN;
  if (x >= 2147483647.0) return INT32_MAX;
  return (int32_t)x;
}

/* util/util.h:528-533 */
static uint32_t min_bits_to_store(uint32_t v) {
  if (v == 0) return 1;
  return (uint32_t)log2((double)v) + 1;
}

/* cuda/cuda_util.cuh:116-125 */
static uint32_t float_to_uint(float xy) {
  float t = xy + 180.0f;
  return f2u32(t * 100000.0f);
}
static float uint_to_float(uint32_t f) { return (float)f / 100000.0f - 180.0f; }

/* CTF::get_ctf_bits (tracing/step_merge.cpp:140-186). mbr: the CTF's float
 * box; map: the map box (double). Returns 0, or -1 if the key would need
 * more than 64 box bits or 128 key bits (the reference asserts). */
int lsm_ctf_bits(const float mbr[4], const double map[4], uint32_t num_objects, uint32_t max_meet_time,
                 stc_ctf *c) {
  c->id_bit = (uint16_t)min_bits_to_store(num_objects);
  c->duration_bit = (uint16_t)min_bits_to_store(max_meet_time - 1);
  c->end_bit = c->duration_bit;
  double map_x_grid_length = (map[2] - map[0]) / 3000;
  double map_y_grid_length = (map[3] - map[1]) / 4200;
  float wx = mbr[2] - mbr[0], wy = mbr[3] - mbr[1];
  uint32_t low_x_grid = d2u32((double)wx / map_x_grid_length);
  uint32_t low_y_grid = d2u32((double)wy / map_y_grid_length);
  c->low_x_bit = (uint16_t)min_bits_to_store((low_x_grid > 1 ? low_x_grid : 1) - 1);
  c->low_y_bit = (uint16_t)min_bits_to_store((low_y_grid > 1 ? low_y_grid : 1) - 1);
  c->edge_bit = c->low_x_bit > c->low_y_bit ? c->low_x_bit : c->low_y_bit;
  c->mbr_bit = (uint16_t)(c->low_x_bit + c->low_y_bit + 2 * c->edge_bit);
  uint32_t temp_bit = 2u * c->id_bit + c->duration_bit + c->end_bit + c->mbr_bit;
  c->key_bit = (uint16_t)((temp_bit + 7) / 8 * 8);  /* CTF::eight_parallel */
  int32_t old_width_grid = d2i32((double)wx / (map[2] - map[0]) * 300);
  int32_t old_high_grid = d2i32((double)wy / (map[3] - map[1]) * 420);
  int32_t xg = old_width_grid + 1 > 32 ? old_width_grid + 1 : 32;
  int32_t yg = old_high_grid + 1 > 32 ? old_high_grid + 1 : 32;
  if (xg >= 256 || yg >= 256) {
    xg = old_width_grid + 1 < 255 ? old_width_grid + 1 : 255;
    yg = old_high_grid + 1 < 255 ? old_high_grid + 1 : 255;
  }
  c->x_grid = (uint16_t)xg;
  c->y_grid = (uint16_t)yg;
  c->bitmap_bytes = ((uint32_t)c->x_grid * c->y_grid + 7) / 8;
  return (c->mbr_bit > 64 || temp_bit > 128) ? -1 : 0;
}

/* serialize_mbr (cuda/geometry.cu:161-171) = CTF::serial_mbr
 * (tracing/step_merge.cpp:290-310): box corner relative to the CTF box in
 * low_x/low_y bits, extent relative to the CTF's longer edge in edge bits. */
uint64_t lsm_serialize_mbr(const float b[4], const stc_ctf *c) {
  const float *m = c->mbr;
  float wx = m[2] - m[0], wy = m[3] - m[1];
  float longer_edge = wx > wy ? wx : wy;
  uint64_t low0 = f2u64((b[0] - m[0]) / wx * (float)((1ull << c->low_x_bit) - 1));
  uint64_t low1 = f2u64((b[1] - m[1]) / wy * (float)((1ull << c->low_y_bit) - 1));
  uint64_t x = f2u64((b[2] - b[0]) / longer_edge * (float)((1ull << c->edge_bit) - 1));
  uint64_t y = f2u64((b[3] - b[1]) / longer_edge * (float)((1ull << c->edge_bit) - 1));
  return (low0 << (c->low_y_bit + c->edge_bit + c->edge_bit)) + (low1 << (c->edge_bit + c->edge_bit)) +
         (x << c->edge_bit) + y;
}

/* write_key_and_mbr (cuda/geometry.cu:1062-1098) / CTF::serial_key
 * (tracing/step_merge.cpp:284-288): pid carries the bits above it in the
 * 128-bit memtable key (extract_fields, cuda/cuda_util.cuh:164-169, does not
 * mask them), i.e. the sid. Fields are added, not or-ed. Writes the low
 * key_bit/8 bytes little-endian. */
void lsm_pack_key(uint64_t pid_field, uint64_t target, uint64_t duration, uint64_t end, uint64_t value_mbr,
                  const stc_ctf *c, uint8_t *out) {
  u128 k = ((u128)pid_field << (c->id_bit + c->duration_bit + c->end_bit + c->mbr_bit)) +
           ((u128)target << (c->duration_bit + c->end_bit + c->mbr_bit)) +
           ((u128)duration << (c->end_bit + c->mbr_bit)) + ((u128)end << c->mbr_bit) + (u128)value_mbr;
  for (uint32_t i = 0; i < c->key_bit / 8u; i++) out[i] = (uint8_t)(k >> (8 * i));
}

/* cuda_write_o_bitmap (cuda/geometry.cu:904-923): cells of a box on the
 * edge x edge map grid (edge = DEFAULT_bitmap_edge, util/util.h:47, 256 in
 * the reference), in double. The GPU kernel has no bound on the cell index;
 * cells past the last bit of the bitmap are skipped here. */
void lsm_o_bitmap_edge(const float b[4], const double map[4], uint32_t edge, uint8_t *bitmap) {
  const uint64_t bits = (uint64_t)edge * edge;
  uint32_t low0 = d2u32((b[0] - map[0]) / (map[2] - map[0]) * edge);
  uint32_t low1 = d2u32((b[1] - map[1]) / (map[3] - map[1]) * edge);
  uint32_t high0 = d2u32((b[2] - map[0]) / (map[2] - map[0]) * edge);
  uint32_t high1 = d2u32((b[3] - map[1]) / (map[3] - map[1]) * edge);
  /* (i, j) past either bound gives a bit past the bitmap */
  if (high0 > bits - 1) high0 = (uint32_t)(bits - 1);
  if (high1 > edge - 1) high1 = edge - 1;
  for (uint64_t i = low0; i <= high0; i++)
    for (uint64_t j = low1; j <= high1; j++) {
      uint64_t bit = i + j * edge;
      if (bit < bits) bitmap[bit / 8] |= (uint8_t)(1u << (bit % 8));
    }
}

void lsm_o_bitmap(const float b[4], const double map[4], uint8_t *bitmap) { lsm_o_bitmap_edge(b, map, 256, bitmap); }

/* ---- memtable and flush ------------------------------------------------ */

typedef struct {
  uint32_t pid, target, dur, end;
  float box[4];
  uint8_t over;  /* oversize at partition time */
} okey;

struct lsm_oracle {
  uint32_t n, max_meet, F, split;
  double area, map[4];
  uint32_t end_time_min;
  uint64_t kv, cap;
  okey *keys;
  uint32_t *cnt;
  uint32_t (*obox)[4];  /* uint_box: low0, low1, high0, high1 */
  uint16_t *sid;
  uint32_t sid_count, over_count;
  /* last block */
  int has_block;
  stc_ctb_info info;
  stc_ctf *ctfs;
  uint8_t *bitmaps, *kbytes, *obitmap;
  uint32_t edge;  /* map bitmap edge */
  uint16_t *bsids;
  okey *bkeys;  /* sorted: CTF keys, then oversize keys */
  char err[160];
};

static void reset_memtable(lsm_oracle *o) {
  o->kv = 0;
  memset(o->cnt, 0, o->n * sizeof(uint32_t));
  memset(o->sid, 0, o->n * sizeof(uint16_t));
  for (uint32_t i = 0; i < o->n; i++) {
    o->obox[i][0] = o->obox[i][1] = 100000000u;
    o->obox[i][2] = o->obox[i][3] = 0u;
  }
  o->sid_count = o->over_count = 0;
}

lsm_oracle *lsm_create(uint32_t n, uint32_t max_meet_time, uint32_t ctf_count, double area_restriction,
                       uint32_t first_end_time_min, const double map[4], uint64_t capacity) {
  lsm_oracle *o = (lsm_oracle *)calloc(1, sizeof(lsm_oracle));
  if (!o) return NULL;
  o->n = n;
  o->max_meet = max_meet_time;
  o->F = ctf_count;
  o->split = (uint32_t)sqrt((double)ctf_count);
  o->area = area_restriction;
  memcpy(o->map, map, sizeof(o->map));
  o->end_time_min = first_end_time_min;
  o->cap = capacity;
  o->keys = (okey *)malloc(capacity * sizeof(okey));
  o->bkeys = (okey *)malloc(capacity * sizeof(okey));
  o->cnt = (uint32_t *)malloc(n * sizeof(uint32_t));
  o->obox = malloc(n * sizeof(*o->obox));
  o->sid = (uint16_t *)malloc(n * sizeof(uint16_t));
  o->bsids = (uint16_t *)calloc(n, sizeof(uint16_t));
  o->ctfs = (stc_ctf *)calloc(ctf_count, sizeof(stc_ctf));
  o->bitmaps = (uint8_t *)calloc((size_t)ctf_count, 8192);
  o->kbytes = (uint8_t *)malloc(capacity * 16 + 16);
  o->edge = 256;
  o->obitmap = (uint8_t *)calloc(8192, 1);
  if (!o->keys || !o->bkeys || !o->cnt || !o->obox || !o->sid || !o->bsids || !o->ctfs || !o->bitmaps ||
      !o->kbytes || !o->obitmap) {
    lsm_destroy(o);
    return NULL;
  }
  reset_memtable(o);
  strcpy(o->err, "no error");
  return o;
}

void lsm_destroy(lsm_oracle *o) {
  if (!o) return;
  free(o->keys); free(o->bkeys); free(o->cnt); free(o->obox); free(o->sid); free(o->bsids);
  free(o->ctfs); free(o->bitmaps); free(o->kbytes); free(o->obitmap);
  free(o);
}

int lsm_set_bitmap_edge(lsm_oracle *o, uint32_t edge) {
  if (edge == 0 || edge % 32 || edge > 1024) return -1;
  uint8_t *bm = (uint8_t *)calloc((size_t)edge * edge / 8, 1);
  if (!bm) return -1;
  free(o->obitmap);
  o->obitmap = bm;
  o->edge = edge;
  return 0;
}

const char *lsm_error(const lsm_oracle *o) { return o->err; }
uint64_t lsm_kv_count(const lsm_oracle *o) { return o->kv; }

/* cuda_identify_meetings, emission branch (cuda/geometry.cu:701-737). */
int lsm_append(lsm_oracle *o, const stc_meeting *m, size_t count) {
  for (size_t i = 0; i < count; i++) {
    uint32_t dur = m[i].end - m[i].start;
    uint32_t a = m[i].pid_lo, b = m[i].pid_hi;
    if (dur > o->max_meet) {
      o->over_count++;
      o->sid[a] = 1;
      o->sid[b] = 1;
    }
    if (o->kv + 2 > o->cap) {
      strcpy(o->err, "memtable full");
      return -1;
    }
    for (int k = 0; k < 2; k++) {
      uint32_t pid = k ? b : a, target = k ? a : b;
      okey *e = &o->keys[o->kv++];
      e->pid = pid;
      e->target = target;
      e->dur = dur;
      e->end = m[i].end - o->end_time_min;
      memcpy(e->box, m[i].mbr, sizeof(e->box));
      e->over = 0;
      if (o->cnt[pid]++ == 0) o->sid_count++;
      uint32_t lo0 = float_to_uint(m[i].mbr[0]), lo1 = float_to_uint(m[i].mbr[1]);
      uint32_t hi0 = float_to_uint(m[i].mbr[2]), hi1 = float_to_uint(m[i].mbr[3]);
      if (lo0 < o->obox[pid][0]) o->obox[pid][0] = lo0;
      if (hi0 > o->obox[pid][2]) o->obox[pid][2] = hi0;
      if (lo1 < o->obox[pid][1]) o->obox[pid][1] = lo1;
      if (hi1 > o->obox[pid][3]) o->obox[pid][3] = hi1;
    }
  }
  return 0;
}

typedef struct {
  uint64_t key;
  uint32_t id;
} kv64;

static int cmp_kv64(const void *x, const void *y) {
  const kv64 *a = (const kv64 *)x, *b = (const kv64 *)y;
  if (a->key != b->key) return a->key < b->key ? -1 : 1;
  return a->id < b->id ? -1 : (a->id > b->id);  /* stable */
}

static const uint16_t *g_sid;  /* qsort context */

static int cmp_okey(const void *x, const void *y) {
  const okey *a = (const okey *)x, *b = (const okey *)y;
  if (a->over != b->over) return a->over < b->over ? -1 : 1;
  uint32_t sa = a->over ? 0 : g_sid[a->pid], sb = b->over ? 0 : g_sid[b->pid];
  if (sa != sb) return sa < sb ? -1 : 1;
  if (a->pid != b->pid) return a->pid < b->pid ? -1 : 1;
  if (a->target != b->target) return a->target < b->target ? -1 : 1;
  if (a->dur != b->dur) return a->dur < b->dur ? -1 : 1;
  if (a->end != b->end) return a->end < b->end ? -1 : 1;
  return 0;
}

/* The flush of cuda/geometry.cu:1752-2138 at step cur_time. */
int lsm_flush(lsm_oracle *o, uint32_t cur_time) {
  const uint32_t N = o->n, S = o->split, F = o->F;
  /* set_oid (cuda/geometry.cu:740-767) */
  kv64 *ord = (kv64 *)malloc((size_t)N * sizeof(kv64));
  if (!ord) return -1;
  for (uint32_t id = 0; id < N; id++) {
    ord[id].id = id;
    ord[id].key = 0;
    if (o->cnt[id] >= 1) {
      float low0 = uint_to_float(o->obox[id][0]), high0 = uint_to_float(o->obox[id][2]);
      float low1 = uint_to_float(o->obox[id][1]), high1 = uint_to_float(o->obox[id][3]);
      float area = (high1 - low1) * (high0 - low0);
      if ((double)area > o->area) {
        o->over_count++;
        o->sid[id] = 1;
        continue;
      }
      uint32_t ave_mid0 = o->obox[id][0] / 2 + o->obox[id][2] / 2;
      uint32_t ave_mid1 = o->obox[id][3] / 2 + o->obox[id][3] / 2;  /* high y twice, as the reference */
      ord[id].key = ((uint64_t)ave_mid0 << 32) + ave_mid1;
    }
  }
  /* partition (cuda/geometry.cu:1779-1796): keys of sid-1 objects go last */
  for (uint64_t i = 0; i < o->kv; i++) o->keys[i].over = o->sid[o->keys[i].pid] == 1;
  /* STR: sort by (x, y) midpoint, then each x slab by y (:1858-1891) */
  qsort(ord, N, sizeof(kv64), cmp_kv64);
  uint64_t z = (uint64_t)(uint32_t)((N - o->sid_count) + o->over_count);
  uint32_t xcap = (o->sid_count - o->over_count) / S + 1;
  uint32_t ycap = xcap / S + 1;
  if (z < N) {
    for (uint64_t p = z; p < N; p++) {
      ord[p].key &= 0xFFFFFFFFull;                      /* narrow_xy_to_y */
    }
    /* stable per-slab sort by y: carry the original position as the tie-break */
    kv64 *tmp = (kv64 *)malloc((size_t)(N - z) * sizeof(kv64));
    uint32_t *oid_at = (uint32_t *)malloc((size_t)(N - z) * sizeof(uint32_t));
    if (!tmp || !oid_at) { free(tmp); free(oid_at); free(ord); return -1; }
    for (uint64_t p = z; p < N; p++) oid_at[p - z] = ord[p].id;
    for (uint32_t s = 0; s < S; s++) {
      uint64_t lo = z + (uint64_t)xcap * s, hi = s + 1 < S ? z + (uint64_t)xcap * (s + 1) : N;
      if (lo > N) lo = N;
      if (hi > N) hi = N;
      for (uint64_t p = lo; p < hi; p++) {
        tmp[p - lo].key = ord[p].key;
        tmp[p - lo].id = (uint32_t)(p - z);
      }
      if (hi > lo) qsort(tmp, hi - lo, sizeof(kv64), cmp_kv64);
      for (uint64_t p = lo; p < hi; p++) ord[p] = (kv64){tmp[p - lo].key, oid_at[tmp[p - lo].id]};
    }
    free(tmp);
    free(oid_at);
    /* make_sid (:780-796) */
    for (uint64_t p = z; p < N; p++) {
      uint32_t x_index = (uint32_t)(p - z) / xcap;
      uint32_t y_index = ((uint32_t)(p - z) - x_index * xcap) / ycap;
      o->sid[ord[p].id] = (uint16_t)(x_index * S + y_index + 2);
    }
  }
  /* sort the keys: CTF keys by (sid, pid, target, duration, end), then the
   * oversize keys by (pid, target, duration, end) (:1800, 1904) */
  g_sid = o->sid;
  memcpy(o->bkeys, o->keys, o->kv * sizeof(okey));
  qsort(o->bkeys, o->kv, sizeof(okey), cmp_okey);
  uint64_t n_over = 0;
  for (uint64_t i = 0; i < o->kv; i++) n_over += o->keys[i].over;
  uint64_t slim = o->kv - n_over;
  /* get_CTF_capacity (:808-818) */
  uint32_t *cap = (uint32_t *)calloc(F, sizeof(uint32_t));
  uint64_t *first = (uint64_t *)calloc((size_t)F + 1, sizeof(uint64_t));
  if (!cap || !first) { free(cap); free(first); free(ord); return -1; }
  for (uint64_t p = z; p < N; p++) {
    uint32_t oid = ord[p].id;
    uint32_t c = (uint32_t)o->sid[oid] - 2;
    if (c < F) cap[c] += o->cnt[oid];
  }
  for (uint32_t c = 0; c < F; c++) first[c + 1] = first[c] + cap[c];
  /* cuda_get_limit (:820-891) and the host's get_ctf_bits (:1960-1963) */
  memset(o->bitmaps, 0, (size_t)F * 8192);
  uint64_t key_off = 0;
  int bad = 0;
  for (uint32_t c = 0; c < F; c++) {
    stc_ctf *t = &o->ctfs[c];
    memset(t, 0, sizeof(*t));
    float lo0 = 100000.0f, lo1 = 100000.0f, hi0 = -100000.0f, hi1 = -100000.0f;
    uint32_t smin = 1u << 30, smax = 0;
    /* ranges index the whole sorted array: when an object partitioned as
     * oversize later gets a CTF sid (a meeting longer than max_meet_time
     * with a small box), the capacities run past the CTF keys into the
     * oversize keys, as in the reference. The capacities never exceed kv. */
    uint64_t a = first[c], b = first[c + 1];
    for (uint64_t k = a; k < b; k++) {
      const okey *e = &o->bkeys[k];
      lo0 = fminf(lo0, e->box[0]); lo1 = fminf(lo1, e->box[1]);
      hi0 = fmaxf(hi0, e->box[2]); hi1 = fmaxf(hi1, e->box[3]);
      uint32_t st = e->end + o->end_time_min - e->dur;
      if (st < smin) smin = st;
      if (st > smax) smax = st;
    }
    t->mbr[0] = lo0; t->mbr[1] = lo1; t->mbr[2] = hi0; t->mbr[3] = hi1;
    t->kv_count = cap[c];
    t->start_time_min = smin;
    t->start_time_max = smax;
    t->end_time_min = o->end_time_min;
    t->end_time_max = cur_time;
    if (lsm_ctf_bits(t->mbr, o->map, N, o->max_meet, t) != 0) bad = 1;
    t->first_key = first[c];
    t->key_offset = key_off;
    key_off += (uint64_t)cap[c] * (t->key_bit / 8u);
    /* cuda_write_bitmap (:957-987) and write_key_and_mbr (:1062-1098) */
    uint8_t *bm = o->bitmaps + (size_t)c * 8192;
    for (uint64_t k = a; k < b; k++) {
      const okey *e = &o->bkeys[k];
      float wx = t->mbr[2] - t->mbr[0], wy = t->mbr[3] - t->mbr[1];
      uint32_t l0 = f2u32((e->box[0] - t->mbr[0]) / wx * (float)t->x_grid);
      uint32_t l1 = f2u32((e->box[1] - t->mbr[1]) / wy * (float)t->y_grid);
      uint32_t h0 = f2u32((e->box[2] - t->mbr[0]) / wx * (float)t->x_grid);
      uint32_t h1 = f2u32((e->box[3] - t->mbr[1]) / wy * (float)t->y_grid);
      for (uint64_t i = l0; i <= h0; i++)
        for (uint64_t j = l1; j <= h1; j++) {
          uint64_t bit = i + j * t->x_grid;
          if (bit < 65536) bm[bit / 8] |= (uint8_t)(1u << (bit % 8));
        }
      /* write_sid_in_key ran on the CTF keys only (cuda/geometry.cu:799-806) */
      uint64_t pid_field = e->over ? e->pid : (((uint64_t)o->sid[e->pid] << 26) | e->pid);
      lsm_pack_key(pid_field, e->target, e->dur, e->end, lsm_serialize_mbr(e->box, t), t,
                   o->kbytes + t->key_offset + (k - first[c]) * (t->key_bit / 8u));
    }
  }
  /* oversize buffer: time limits (get_o_limit, :957-1010) and map bitmap */
  memset(o->obitmap, 0, (size_t)o->edge * o->edge / 8);
  uint32_t osmin = 1u << 30, osmax = 0;
  for (uint64_t k = slim; k < o->kv; k++) {
    const okey *e = &o->bkeys[k];
    uint32_t st = e->end + o->end_time_min - e->dur;
    if (st < osmin) osmin = st;
    if (st > osmax) osmax = st;
    lsm_o_bitmap_edge(e->box, o->map, o->edge, o->obitmap);
  }
  memcpy(o->bsids, o->sid, N * sizeof(uint16_t));
  stc_ctb_info *in = &o->info;
  in->index = o->has_block ? in->index + 1 : 0;
  in->ctf_count = F;
  in->flush_time = cur_time;
  in->end_time_min = o->end_time_min;
  in->kv_count = o->kv;
  in->ctf_kv_count = slim;
  in->oversize_kv_count = n_over;
  in->key_bytes = key_off;
  in->sid_count = o->sid_count;
  in->oversize_oid_count = o->over_count;
  in->o_start_time_min = osmin;
  in->o_start_time_max = osmax;
  in->o_end_time_min = o->end_time_min;
  in->o_end_time_max = cur_time;
  in->bitmap_edge = o->edge;
  o->has_block = 1;
  free(cap);
  free(first);
  free(ord);
  o->end_time_min = cur_time;  /* straight_dump (process.cpp:271) */
  reset_memtable(o);
  if (bad) {
    strcpy(o->err, "CTF key exceeds 128 bits");
    return -1;
  }
  return 0;
}

int lsm_get_ctb(const lsm_oracle *o, stc_ctb_info *info) {
  if (!o->has_block) return -1;
  *info = o->info;
  return 0;
}

/* Same layout as stc_read_ctb. */
int lsm_read_ctb(const lsm_oracle *o, stc_ctf *ctfs, uint8_t *bitmaps, uint8_t *keys, uint16_t *sids,
                 uint64_t *okeys, float *oboxes, uint8_t *obitmap) {
  if (!o->has_block) return -1;
  const stc_ctb_info *in = &o->info;
  if (ctfs) memcpy(ctfs, o->ctfs, in->ctf_count * sizeof(stc_ctf));
  if (bitmaps) memcpy(bitmaps, o->bitmaps, (size_t)in->ctf_count * 8192);
  if (keys) memcpy(keys, o->kbytes, in->key_bytes);
  if (sids) memcpy(sids, o->bsids, o->n * sizeof(uint16_t));
  for (uint64_t i = 0; i < in->oversize_kv_count; i++) {
    const okey *e = &o->bkeys[in->ctf_kv_count + i];
    if (okeys) {
      okeys[2 * i] = ((uint64_t)e->dur << 32) | e->end;
      okeys[2 * i + 1] = ((uint64_t)e->pid << 26) | e->target;
    }
    if (oboxes) memcpy(oboxes + 4 * i, e->box, 4 * sizeof(float));
  }
  if (obitmap) memcpy(obitmap, o->obitmap, (size_t)o->edge * o->edge / 8);
  return 0;
}

/* ---- queries over a block ------------------------------------------------
 * The reference's lookups (workbench::id_search_in_CTB, CTF::binary_search,
 * CTF::search_SSTable, oversize_buffer::search_buffer, mbr_search_in_disk;
 * tracing/workbench.cpp:413-460, 495-572, tracing/step_merge.cpp:65-110,
 * 518-570) with the time window applied as its time_query states
 * (util/query_context.h:95-105: key start < t_end and t_start < key end)
 * and without the fixed test box of search_SSTable (step_merge.cpp:549). */

static u128 load_key(const uint8_t *p, uint32_t kb) {
  u128 k = 0;
  for (uint32_t i = 0; i < kb; i++) k |= (u128)p[i] << (8 * i);
  return k;
}

static uint64_t mask64(uint32_t bits) { return bits >= 64 ? ~0ull : (1ull << bits) - 1; }

/* CTF::ctf_get_key_oid, CTF::parse_key and CTF::new_parse_mbr
 * (tracing/step_merge.cpp:329-379): fields masked to their widths, the box
 * decoded in double from the CTF box. */
void lsm_decode_key(const uint8_t *key, const stc_ctf *c, uint32_t *oid, uint32_t *target, uint32_t *duration,
                    uint32_t *end, uint64_t *value_mbr, double box[4]) {
  u128 k = load_key(key, c->key_bit / 8u);
  *oid = (uint32_t)((k >> (c->id_bit + c->duration_bit + c->end_bit + c->mbr_bit)) & mask64(c->id_bit));
  uint64_t vm = (uint64_t)(k & (u128)mask64(c->mbr_bit));
  k >>= c->mbr_bit;
  *end = (uint32_t)(k & mask64(c->end_bit));
  k >>= c->end_bit;
  *duration = (uint32_t)(k & mask64(c->duration_bit));
  k >>= c->duration_bit;
  *target = (uint32_t)(k & mask64(c->id_bit));
  *value_mbr = vm;
  uint64_t me = mask64(c->edge_bit), my = mask64(c->low_y_bit), mx = mask64(c->low_x_bit);
  uint64_t y = vm & me;
  vm >>= c->edge_bit;
  uint64_t x = vm & me;
  vm >>= c->edge_bit;
  uint64_t low1 = vm & my;
  vm >>= c->low_y_bit;
  uint64_t low0 = vm & mx;
  float wx = c->mbr[2] - c->mbr[0], wy = c->mbr[3] - c->mbr[1];
  float longer_edge = wx > wy ? wx : wy;
  box[0] = c->mbr[0] + (double)low0 / mx * wx;
  box[1] = c->mbr[1] + (double)low1 / my * wy;
  box[2] = box[0] + (double)x / me * longer_edge;
  box[3] = box[1] + (double)y / me * longer_edge;
}

static int time_ok(uint32_t start, uint32_t end, uint32_t t1, uint32_t t2) { return start < t2 && t1 < end; }

static int box_hits(const double a[4], const double q[4]) {  /* box::intersect (geometry/geometry.h:128-133) */
  return !(q[0] > a[2] || q[2] < a[0] || q[1] > a[3] || q[3] < a[1]);
}

static size_t put(stc_contact *out, size_t cap, size_t n, uint32_t pid, uint32_t target, uint32_t start,
                  uint32_t end, const double box[4], uint32_t block, uint32_t ctf) {
  if (n < cap) {
    stc_contact *r = &out[n];
    r->pid = pid; r->target = target; r->start = start; r->end = end;
    memcpy(r->mbr, box, sizeof(r->mbr));
    r->block = block;
    r->ctf = ctf;
  }
  return n + 1;
}

static void oversize_fields(const uint64_t *ok, uint32_t *pid, uint32_t *target, uint32_t *dur, uint32_t *end) {
  *pid = (uint32_t)(ok[1] >> 26) & ((1u << 26) - 1);
  *target = (uint32_t)ok[1] & ((1u << 26) - 1);
  *dur = (uint32_t)(ok[0] >> 32);
  *end = (uint32_t)ok[0];
}

/* Object query on one block: its sid picks the oversize buffer or one CTF,
 * binary search for the first key of pid, scan while the pid matches.
 * Returns the number of matches (only the first cap are written). */
size_t lsm_query_object_block(const stc_ctb_info *in, const stc_ctf *ctfs, const uint8_t *keys,
                              const uint16_t *sids, const uint64_t *okeys, const float *oboxes, uint32_t pid,
                              uint32_t t1, uint32_t t2, stc_contact *out, size_t cap, size_t n) {
  uint16_t sid = sids[pid];
  if (sid == 0) return n;
  if (sid == 1) {
    int64_t low = 0, high = (int64_t)in->oversize_kv_count - 1, find = -1;
    while (low <= high) {
      int64_t mid = (low + high) / 2;
      uint32_t p, tg, d, e;
      oversize_fields(okeys + 2 * mid, &p, &tg, &d, &e);
      if (p == pid) { find = mid; high = mid - 1; }
      else if (p > pid) high = mid - 1;
      else low = mid + 1;
    }
    if (find < 0) return n;
    for (uint64_t i = (uint64_t)find; i < in->oversize_kv_count; i++) {
      uint32_t p, tg, d, e;
      oversize_fields(okeys + 2 * i, &p, &tg, &d, &e);
      if (p != pid) break;
      uint32_t end_abs = e + in->o_end_time_min, start = end_abs - d;
      if (!time_ok(start, end_abs, t1, t2)) continue;
      double b[4] = {oboxes[4 * i], oboxes[4 * i + 1], oboxes[4 * i + 2], oboxes[4 * i + 3]};
      n = put(out, cap, n, pid, tg, start, end_abs, b, in->index, in->ctf_count);
    }
    return n;
  }
  uint32_t c = (uint32_t)sid - 2;
  if (c >= in->ctf_count) return n;
  const stc_ctf *t = &ctfs[c];
  const uint32_t kb = t->key_bit / 8u;
  const uint8_t *base = keys + t->key_offset;
  /* CTF::binary_search (tracing/step_merge.cpp:496-521): unsigned bounds */
  uint32_t low = 0, high = t->kv_count - 1;
  int64_t find = -1;
  while (low <= high) {
    uint64_t mid = low + (uint64_t)(high - low) / 2;
    if (mid >= t->kv_count) break;
    uint32_t oid, tg, d, e;
    uint64_t vm;
    double b[4];
    lsm_decode_key(base + mid * kb, t, &oid, &tg, &d, &e, &vm, b);
    if (oid == pid) {
      find = (int64_t)mid;
      if (mid == 0) break;
      high = (uint32_t)mid - 1;
    } else if (oid < pid) {
      low = (uint32_t)mid + 1;
    } else {
      if (mid == 0) break;
      high = (uint32_t)mid - 1;
    }
  }
  if (find < 0) return n;
  for (uint64_t i = (uint64_t)find; i < t->kv_count; i++) {
    uint32_t oid, tg, d, e;
    uint64_t vm;
    double b[4];
    lsm_decode_key(base + i * kb, t, &oid, &tg, &d, &e, &vm, b);
    if (oid != pid) break;
    uint32_t end_abs = e + t->end_time_min, start = end_abs - d;
    if (!time_ok(start, end_abs, t1, t2)) continue;
    n = put(out, cap, n, pid, tg, start, end_abs, b, in->index, c);
  }
  return n;
}

/* Box query on one block: every CTF key whose decoded box intersects q and
 * every oversize key whose box does, inside the time window. The oracle
 * scans every key; the GPU prunes CTFs by box, times and bitmap first. */
size_t lsm_query_box_block(const stc_ctb_info *in, const stc_ctf *ctfs, const uint8_t *keys, const uint64_t *okeys,
                           const float *oboxes, const double q[4], uint32_t t1, uint32_t t2, stc_contact *out,
                           size_t cap, size_t n) {
  for (uint32_t c = 0; c < in->ctf_count; c++) {
    const stc_ctf *t = &ctfs[c];
    const uint32_t kb = t->key_bit / 8u;
    for (uint64_t i = 0; i < t->kv_count; i++) {
      uint32_t oid, tg, d, e;
      uint64_t vm;
      double b[4];
      lsm_decode_key(keys + t->key_offset + i * kb, t, &oid, &tg, &d, &e, &vm, b);
      uint32_t end_abs = e + t->end_time_min, start = end_abs - d;
      if (time_ok(start, end_abs, t1, t2) && box_hits(b, q)) n = put(out, cap, n, oid, tg, start, end_abs, b, in->index, c);
    }
  }
  for (uint64_t i = 0; i < in->oversize_kv_count; i++) {
    uint32_t p, tg, d, e;
    oversize_fields(okeys + 2 * i, &p, &tg, &d, &e);
    uint32_t end_abs = e + in->o_end_time_min, start = end_abs - d;
    double b[4] = {oboxes[4 * i], oboxes[4 * i + 1], oboxes[4 * i + 2], oboxes[4 * i + 3]};
    if (time_ok(start, end_abs, t1, t2) && box_hits(b, q)) n = put(out, cap, n, p, tg, start, end_abs, b, in->index, in->ctf_count);
  }
  return n;
}
