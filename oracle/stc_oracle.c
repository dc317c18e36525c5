/*
 * CPU restatement of the reference's co-occurrence path -- TEST
 * INFRASTRUCTURE ONLY (the checker; never linked into the product).
 *
 * Every function names the reference lines it restates. Paths are inside the
 * tengdj/STCDB checkout. Single-threaded mode reproduces the reference CPU
 * path run with one thread, which is the only deterministic configuration of
 * the reference (its multi-threaded insert at tracing/refinement.cpp:43-52 is
 * racy). Meeting MBRs and the map-box filter follow the reference's GPU
 * kernels (cuda/geometry.cu:461-489, :665-670).
 *
 * Compile with -ffp-contract=off: the reference's x86-64 build evaluates
 * every expression below without fused multiply-add.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "stc_oracle.h"

/* util/util.h:38-39, :57 */
#define REF_PI 3.14159265
#define EMPTY_KEY (1ULL << 62)
static const double DPM_LAT = 360.0 / (40076.0 * 1000.0);

enum { INVALID = 0, BRANCH = 1, LEAF = 2 }; /* index/QTree.h:43-47 */

/* util/util.h:59-66 */
double oracle_dpml(double latitude) {
  double absla = fabs(latitude);
  if (absla == 90) absla = 89;
  return 360.0 / (sin((90 - absla) * REF_PI / 180) * 40076.0 * 1000.0);
}

typedef struct { double lo[2], hi[2]; } obox;

/* geometry/geometry.h:140-145 */
static int box_contain_pt(const obox *b, double x, double y) {
  return x >= b->lo[0] && x <= b->hi[0] && y >= b->lo[1] && y <= b->hi[1];
}

/* geometry/geometry.h:174-185 (box::distance with geography = true) */
static double box_distance(const obox *b, double x, double y) {
  if (box_contain_pt(b, x, y)) return 0;
  double dx = fabs(x - (b->lo[0] + b->hi[0]) / 2) - (b->hi[0] - b->lo[0]) / 2;
  double dy = fabs(y - (b->lo[1] + b->hi[1]) / 2) - (b->hi[1] - b->lo[1]) / 2;
  if (dx < 0.0) dx = 0.0;
  if (dy < 0.0) dy = 0.0;
  dy = dy / DPM_LAT;
  dx = dx / oracle_dpml(y);
  return sqrt(dx * dx + dy * dy);
}

/* geometry/geometry.h:166-172 (box::width with geography = true) */
static double box_width_geo(const obox *b) {
  return (b->hi[0] - b->lo[0]) / oracle_dpml(b->lo[1]);
}

/* geometry/geometry.h:40-48 (Point::distance with geography = true; p1 is
 * `this`, so the longitude scale is taken at p1's latitude) */
static double point_distance(double x1, double y1, double x2, double y2) {
  double dx = x1 - x2;
  double dy = y1 - y2;
  dy = dy / DPM_LAT;
  dx = dx / oracle_dpml(y1);
  return sqrt(dx * dx + dy * dy);
}

/* util/util.h:68-70 */
static uint64_t cantor(uint32_t a, uint32_t b) {
  uint64_t s = (uint64_t)(uint32_t)(a + b);
  return s * (uint64_t)(uint32_t)(a + b + 1) / 2 + b;
}

static uint64_t isqrt64(uint64_t v) {
  uint64_t r = (uint64_t)sqrt((double)v);
  while (r > 0 && r * r > v) r--;
  while ((r + 1) * (r + 1) <= v) r++;
  return r;
}

/* exact integer inverse of cantor() */
static void cantor_decode(uint64_t z, uint32_t *a, uint32_t *b) {
  uint64_t w = (isqrt64(8 * z + 1) - 1) / 2;
  uint64_t t = (w * w + w) / 2;
  *b = (uint32_t)(z - t);
  *a = (uint32_t)(w - (z - t));
}

/* ---------------- quadtree build: index/QTree.h:65-312 ---------------- */

typedef struct qt_node {
  obox mbr;
  double mid_x, mid_y;
  int isleaf;
  short level;
  int child[4];
  uint32_t *objs;
  int nobj, cap;
  uint32_t node_id;
} qt_node;

typedef struct {
  qt_node *nodes;
  int n, cap;
  const double *xy;
  uint32_t grid_capacity;
  double reach;
  int failed;
} qt_tree;

static int qt_new(qt_tree *t, double lx, double ly, double hx, double hy, short level) {
  if (t->n == t->cap) {
    int nc = t->cap ? 2 * t->cap : 1024;
    qt_node *nn = (qt_node *)realloc(t->nodes, (size_t)nc * sizeof(qt_node));
    if (!nn) { t->failed = 1; return -1; }
    t->nodes = nn;
    t->cap = nc;
  }
  qt_node *q = &t->nodes[t->n];
  memset(q, 0, sizeof(*q));
  q->mbr.lo[0] = lx; q->mbr.lo[1] = ly; q->mbr.hi[0] = hx; q->mbr.hi[1] = hy;
  q->mid_x = (q->mbr.hi[0] + q->mbr.lo[0]) / 2;  /* QTree.h:103-104 */
  q->mid_y = (q->mbr.hi[1] + q->mbr.lo[1]) / 2;
  q->isleaf = 1;
  q->level = level;
  q->cap = (int)t->grid_capacity;
  q->objs = (uint32_t *)malloc((size_t)q->cap * sizeof(uint32_t));
  if (!q->objs) t->failed = 1;
  for (int i = 0; i < 4; i++) q->child[i] = -1;
  return t->n++;
}

static int quadrant(double mid_x, double mid_y, double x, double y) {
  return (y > mid_y) * 2 + (x > mid_x);
}

/* QTree.h:157-185 */
static void qt_split(qt_tree *t, int id) {
  qt_node *q = &t->nodes[id];
  int should = q->nobj >= (int)t->grid_capacity && box_width_geo(&q->mbr) / 2 > t->reach;
  if (!should || t->failed) return;
  double lx = q->mbr.lo[0], ly = q->mbr.lo[1], hx = q->mbr.hi[0], hy = q->mbr.hi[1];
  double mx = q->mid_x, my = q->mid_y;
  short lv = (short)(q->level + 1);
  int c0 = qt_new(t, lx, ly, mx, my, lv);
  int c1 = qt_new(t, mx, ly, hx, my, lv);
  int c2 = qt_new(t, lx, my, mx, hy, lv);
  int c3 = qt_new(t, mx, my, hx, hy, lv);
  if (t->failed) return;
  q = &t->nodes[id];
  q->child[0] = c0; q->child[1] = c1; q->child[2] = c2; q->child[3] = c3;
  for (int i = 0; i < q->nobj; i++) {
    uint32_t pid = q->objs[i];
    int loc = quadrant(q->mid_x, q->mid_y, t->xy[2 * (size_t)pid], t->xy[2 * (size_t)pid + 1]);
    qt_node *c = &t->nodes[q->child[loc]];
    c->objs[c->nobj++] = pid;  /* a fresh child holds at most grid_capacity objects */
  }
  for (int i = 0; i < 4; i++) qt_split(t, t->nodes[id].child[i]);
  q = &t->nodes[id];
  free(q->objs);
  q->objs = NULL;
  q->nobj = 0;
  q->isleaf = 0;
}

/* QTree.h:187-214 (single-threaded) */
static void qt_insert(qt_tree *t, uint32_t pid) {
  int id = 0;
  double x = t->xy[2 * (size_t)pid], y = t->xy[2 * (size_t)pid + 1];
  while (!t->nodes[id].isleaf) {
    qt_node *q = &t->nodes[id];
    id = q->child[quadrant(q->mid_x, q->mid_y, x, y)];
  }
  qt_node *q = &t->nodes[id];
  if (q->nobj == q->cap) {
    int nc = q->cap + (int)t->grid_capacity;
    uint32_t *no = (uint32_t *)realloc(q->objs, (size_t)nc * sizeof(uint32_t));
    if (!no) { t->failed = 1; return; }
    q->objs = no;
    q->cap = nc;
  }
  q->objs[q->nobj++] = pid;
  qt_split(t, id);
}

/* ---------------- workbench state ---------------- */

typedef struct {
  uint32_t grid_id;
  short level, type, overflow_count, underflow_count;
  double mid_x, mid_y;
  obox mbr;
  uint32_t children[4];
} oschema; /* index/QTree.h:49-62 */

typedef struct {
  uint32_t pid, gid;
  uint16_t offset, inside;
} ounit; /* tracing/workbench.h:55-60 */

typedef struct {
  uint64_t key;
  uint32_t start, end;
  float lo[2], hi[2];
} obucket; /* tracing/workbench.h:62-83 plus the f_box of cuda/geometry.cu */

struct oracle_ctx {
  stc_config cfg;
  int threads;
  obox map;
  double x_buffer, y_buffer;
  uint32_t N, leaf_cap, G, S;
  uint32_t *grids, *grid_counter, *grids_stack, *schema_stack;
  uint32_t grids_stack_index, schema_stack_index;
  oschema *schema;
  ounit *units;
  uint64_t unit_cap, unit_count;
  obucket *buckets;
  stc_meeting *emitted;
  size_t emitted_count, emitted_cap;
  const double *xy;
  uint32_t cur_time;
  stc_stats stats;
  char err[256];
};

static void set_err(oracle_ctx *c, const char *msg) {
  snprintf(c->err, sizeof(c->err), "%s", msg);
}

const char *oracle_error(oracle_ctx *c) { return c ? c->err : "null context"; }

/* QTree.h:301-311 (create_schema, preorder offsets) */
static void qt_create_schema(qt_tree *t, int id, oschema *schema, uint32_t *offset) {
  uint32_t cur = (*offset)++;
  qt_node *q = &t->nodes[id];
  oschema *s = &schema[cur];
  s->mid_x = q->mid_x;
  s->mid_y = q->mid_y;
  s->level = q->level;
  s->grid_id = q->node_id;
  s->type = q->isleaf ? LEAF : BRANCH;
  s->overflow_count = 0;
  s->underflow_count = 0;
  s->mbr = q->mbr;
  if (!q->isleaf) {
    for (int i = 0; i < 4; i++) {
      s->children[i] = *offset;
      qt_create_schema(t, q->child[i], schema, offset);
    }
  }
}

/* QTree.h:88-96 (leaf ids in depth-first order) */
static void qt_set_id(qt_tree *t, int id, uint32_t *next) {
  qt_node *q = &t->nodes[id];
  if (q->isleaf) { q->node_id = (*next)++; return; }
  for (int i = 0; i < 4; i++) qt_set_id(t, q->child[i], next);
}

oracle_ctx *oracle_create(const stc_config *cfg, const double mbr[4], const double *xy0, uint32_t n,
                          int threads) {
  oracle_ctx *c = (oracle_ctx *)calloc(1, sizeof(oracle_ctx));
  if (!c) return NULL;
  c->cfg = *cfg;
  c->threads = threads < 1 ? 1 : threads;
  c->N = n;
  c->map.lo[0] = mbr[0]; c->map.lo[1] = mbr[1]; c->map.hi[0] = mbr[2]; c->map.hi[1] = mbr[3];
  if (n != cfg->num_objects || cfg->grid_capacity == 0 || cfg->num_meeting_buckets == 0) {
    set_err(c, "invalid configuration");
    return c;
  }
  /* tracing/filter.cpp:30-31 */
  c->x_buffer = cfg->reach_distance * oracle_dpml(c->map.lo[1]);
  c->y_buffer = cfg->reach_distance * DPM_LAT;
  /* tracing/workbench.cpp:36-47 */
  c->leaf_cap = (uint32_t)(cfg->grid_amplify * cfg->grid_capacity);
  uint32_t per = n / cfg->grid_capacity;
  c->G = 4 * (per > 100000u ? per : 100000u);
  c->S = (uint32_t)(1.6 * c->G);
  c->unit_cap = (uint64_t)cfg->refine_size * n;

  /* tracing/filter.cpp:34-47: build the quadtree from step-0 positions */
  qt_tree t;
  memset(&t, 0, sizeof(t));
  t.xy = xy0;
  t.grid_capacity = cfg->grid_capacity;
  t.reach = cfg->reach_distance;
  qt_new(&t, mbr[0], mbr[1], mbr[2], mbr[3], 0);
  for (uint32_t pid = 0; pid < n && !t.failed; pid++) qt_insert(&t, pid);
  uint32_t leaves = 0;
  if (!t.failed) qt_set_id(&t, 0, &leaves);

  /* tracing/workbench.cpp:84-130 (claim_space) */
  c->grids = (uint32_t *)malloc((size_t)c->leaf_cap * c->G * sizeof(uint32_t));
  c->grid_counter = (uint32_t *)calloc(c->G, sizeof(uint32_t));
  c->grids_stack = (uint32_t *)malloc((size_t)c->G * sizeof(uint32_t));
  c->schema = (oschema *)calloc(c->S, sizeof(oschema));
  c->schema_stack = (uint32_t *)malloc((size_t)c->S * sizeof(uint32_t));
  c->units = (ounit *)malloc((size_t)c->unit_cap * sizeof(ounit));
  c->buckets = (obucket *)malloc((size_t)cfg->num_meeting_buckets * sizeof(obucket));
  c->emitted_cap = 1024;
  c->emitted = (stc_meeting *)malloc(c->emitted_cap * sizeof(stc_meeting));
  if (t.failed || !c->grids || !c->grid_counter || !c->grids_stack || !c->schema ||
      !c->schema_stack || !c->units || !c->buckets || !c->emitted) {
    set_err(c, "out of host memory");
    for (int i = 0; i < t.n; i++) free(t.nodes[i].objs);
    free(t.nodes);
    return c;
  }
  for (uint32_t i = 0; i < c->G; i++) c->grids_stack[i] = i;
  for (uint32_t i = 0; i < c->S; i++) { c->schema_stack[i] = i; c->schema[i].type = INVALID; }
  for (uint64_t i = 0; i < cfg->num_meeting_buckets; i++) c->buckets[i].key = EMPTY_KEY;

  /* tracing/filter.cpp:81-88 */
  uint32_t nodes = (uint32_t)t.n;
  if (nodes >= c->S || leaves >= c->G) {
    set_err(c, "schema capacity exceeded at build");
  } else {
    c->schema_stack_index = nodes;
    c->grids_stack_index = leaves;
    uint32_t off = 0;
    qt_create_schema(&t, 0, c->schema, &off);
  }
  for (int i = 0; i < t.n; i++) free(t.nodes[i].objs);
  free(t.nodes);
  return c;
}

void oracle_destroy(oracle_ctx *c) {
  if (!c) return;
  free(c->grids); free(c->grid_counter); free(c->grids_stack); free(c->schema);
  free(c->schema_stack); free(c->units); free(c->buckets); free(c->emitted);
  free(c);
}

/* tracing/filter.cpp:130-152 (lookup_rec, query_all = false) */
static int lookup_rec(const oracle_ctx *c, double x, double y, uint32_t cur, uint32_t *out, int n,
                      int cap) {
  for (int i = 0; i < 4; i++) {
    uint32_t ch = c->schema[cur].children[i];
    const oschema *s = &c->schema[ch];
    double dist = box_distance(&s->mbr, x, y);
    if (dist <= c->cfg.reach_distance) {
      if (s->type == LEAF) {
        if (y < s->mbr.lo[1] || (y < s->mbr.hi[1] && x < s->mbr.lo[0])) {
          if (n < cap) out[n] = ch;
          n++;
        }
      } else {
        n = lookup_rec(c, x, y, ch, out, n, cap);
      }
    }
  }
  return n;
}

/* tracing/filter.cpp:228-243: phased descent; returns the leaf, sets last_valid */
static uint32_t descend(const oracle_ctx *c, double x, double y, uint32_t *last_valid, int *bad) {
  uint32_t cur = 0, lv = 0;
  for (int depth = 0; depth < 200; depth++) {
    const oschema *s = &c->schema[cur];
    int child = (y > s->mid_y) * 2 + (x > s->mid_x);
    cur = s->children[child];
    const oschema *d = &c->schema[cur];
    if (d->type == INVALID) { *bad = 1; return cur; }
    if (x + c->x_buffer < d->mbr.hi[0] && y + c->y_buffer < d->mbr.hi[1]) lv = cur;
    if (d->type == LEAF) { *last_valid = lv; return cur; }
  }
  *bad = 1;
  return cur;
}

static void mbr_update(obucket *b, double x, double y) { /* cuda/geometry.cu:82-96 */
  if ((double)b->lo[0] > x) b->lo[0] = (float)x;
  if ((double)b->hi[0] < x) b->hi[0] = (float)x;
  if ((double)b->lo[1] > y) b->lo[1] = (float)y;
  if ((double)b->hi[1] < y) b->hi[1] = (float)y;
}

/* tracing/filter.cpp:95-111 + 210-313 (single-threaded) */
static int filter_st(oracle_ctx *c) {
  const double *xy = c->xy;
  uint32_t N = c->N;
  uint64_t count = N;  /* grid_check_counter = num_objects (filter.cpp:303) */
  uint32_t nodes[64];
  for (uint32_t pid = 0; pid < N; pid++) {
    double x = xy[2 * (size_t)pid], y = xy[2 * (size_t)pid + 1];
    uint32_t lv = 0;
    int bad = 0;
    uint32_t leaf = descend(c, x, y, &lv, &bad);
    if (bad) { set_err(c, "descent reached an invalid schema node"); return -1; }
    uint32_t gid = c->schema[leaf].grid_id;
    uint32_t cur = c->grid_counter[gid]++;
    if (cur < c->leaf_cap) c->grids[(size_t)c->leaf_cap * gid + cur] = pid;
    c->units[pid].pid = pid;
    c->units[pid].gid = gid;
    c->units[pid].offset = 0;
    c->units[pid].inside = 1;
    if (lv != leaf) {
      int k = lookup_rec(c, x, y, lv, nodes, 0, 64);
      if (k > 64) { set_err(c, "border lookup overflow"); return -1; }
      for (int i = 0; i < k; i++) {
        if (count + 1 >= c->unit_cap) { set_err(c, "checking unit capacity exceeded"); return -1; }
        c->units[count].pid = pid;
        c->units[count].gid = c->schema[nodes[i]].grid_id;
        c->units[count].offset = 0;
        c->units[count].inside = 0;
        count++;
      }
    }
  }
  c->unit_count = count;
  return 0;
}

static int filter_mt(oracle_ctx *c) {
  const double *xy = c->xy;
  long long N = c->N;
  uint64_t count = c->N;
  int fail = 0;
#pragma omp parallel num_threads(c->threads)
  {
    uint32_t nodes[64];
#pragma omp for schedule(dynamic, 4096)
    for (long long pp = 0; pp < N; pp++) {
      uint32_t pid = (uint32_t)pp;
      double x = xy[2 * (size_t)pid], y = xy[2 * (size_t)pid + 1];
      uint32_t lv = 0;
      int bad = 0;
      uint32_t leaf = descend(c, x, y, &lv, &bad);
      if (bad) { fail = 1; continue; }
      uint32_t gid = c->schema[leaf].grid_id;
      uint32_t cur = __atomic_fetch_add(&c->grid_counter[gid], 1u, __ATOMIC_RELAXED);
      if (cur < c->leaf_cap) c->grids[(size_t)c->leaf_cap * gid + cur] = pid;
      c->units[pid].pid = pid;
      c->units[pid].gid = gid;
      c->units[pid].offset = 0;
      c->units[pid].inside = 1;
      if (lv != leaf) {
        int k = lookup_rec(c, x, y, lv, nodes, 0, 64);
        if (k > 64) { fail = 1; continue; }
        uint64_t at = __atomic_fetch_add(&count, (uint64_t)k, __ATOMIC_RELAXED);
        if (at + k >= c->unit_cap) { fail = 1; continue; }
        for (int i = 0; i < k; i++) {
          c->units[at + i].pid = pid;
          c->units[at + i].gid = c->schema[nodes[i]].grid_id;
          c->units[at + i].offset = 0;
          c->units[at + i].inside = 0;
        }
      }
    }
  }
  if (fail) { set_err(c, "filter failed (invalid node, lookup or unit overflow)"); return -1; }
  c->unit_count = count;
  return 0;
}

/* tracing/refinement.cpp:19-60 with the MBR of cuda/geometry.cu:474-490 */
static int refine_unit(oracle_ctx *c, uint64_t u, int atomic_insert, uint64_t *tests, uint64_t *hits) {
  const double *xy = c->xy;
  uint32_t pid = c->units[u].pid, gid = c->units[u].gid;
  uint32_t size = c->grid_counter[gid] < c->leaf_cap ? c->grid_counter[gid] : c->leaf_cap;
  const uint32_t *members = c->grids + (size_t)c->leaf_cap * gid;
  double x1 = xy[2 * (size_t)pid], y1 = xy[2 * (size_t)pid + 1];
  uint64_t B = c->cfg.num_meeting_buckets;
  for (uint32_t i = 0; i < size; i++) {
    uint32_t q = members[i];
    if (!(pid < q || !c->units[u].inside)) continue;
    (*tests)++;
    double x2 = xy[2 * (size_t)q], y2 = xy[2 * (size_t)q + 1];
    if (!(point_distance(x1, y1, x2, y2) <= c->cfg.reach_distance)) continue;
    (*hits)++;
    uint32_t p1 = pid < q ? pid : q, p2 = pid < q ? q : pid;
    uint64_t key = cantor(p1, p2);
    uint64_t slot = key % B;
    uint64_t probes = 0;
    while (1) {
      obucket *b = &c->buckets[slot];
      uint64_t k = atomic_insert ? __atomic_load_n(&b->key, __ATOMIC_RELAXED) : b->key;
      if (k == key) {
        b->end = c->cur_time;
        mbr_update(b, x1, y1);
        mbr_update(b, x2, y2);
        break;
      } else if (k == EMPTY_KEY) {
        int ok = 1;
        if (atomic_insert) {
          uint64_t exp = EMPTY_KEY;
          ok = __atomic_compare_exchange_n(&b->key, &exp, key, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED);
          if (!ok && exp == key) { b->end = c->cur_time; break; }
        } else {
          b->key = key;
        }
        if (ok) {
          b->start = c->cur_time;
          b->end = c->cur_time;
          b->lo[0] = 100000.0f; b->lo[1] = 100000.0f;
          b->hi[0] = -100000.0f; b->hi[1] = -100000.0f;
          mbr_update(b, x1, y1);
          mbr_update(b, x2, y2);
          break;
        }
        continue;
      }
      slot = (slot + 1) % B;
      if (++probes > B || probes > (1u << 16)) return -1;  /* table full */
    }
  }
  return 0;
}

static int reachability(oracle_ctx *c) {
  uint64_t tests = 0, hits = 0;
  if (c->threads <= 1) {
    for (uint64_t u = 0; u < c->unit_count; u++)
      if (refine_unit(c, u, 0, &tests, &hits)) { set_err(c, "meeting table full"); return -1; }
  } else {
    int fail = 0;
    long long U = (long long)c->unit_count;
#pragma omp parallel for num_threads(c->threads) schedule(dynamic, 256) reduction(+ : tests, hits)
    for (long long u = 0; u < U; u++)
      if (refine_unit(c, (uint64_t)u, 1, &tests, &hits)) fail = 1;
    if (fail) { set_err(c, "meeting table full"); return -1; }
  }
  c->stats.pair_tests = tests;
  c->stats.hits = hits;
  return 0;
}

static int emit(oracle_ctx *c, const obucket *b) {
  if (c->emitted_count == c->emitted_cap) {
    size_t nc = c->emitted_cap * 2;
    stc_meeting *ne = (stc_meeting *)realloc(c->emitted, nc * sizeof(stc_meeting));
    if (!ne) return -1;
    c->emitted = ne;
    c->emitted_cap = nc;
  }
  stc_meeting *m = &c->emitted[c->emitted_count++];
  cantor_decode(b->key, &m->pid_lo, &m->pid_hi);
  m->start = b->start;
  m->end = b->end;
  m->mbr[0] = b->lo[0]; m->mbr[1] = b->lo[1]; m->mbr[2] = b->hi[0]; m->mbr[3] = b->hi[1];
  return 0;
}

/* cuda/geometry.cu:53-58 (box_contain of a double box and a float box) */
static int map_contains(const obox *m, const obucket *b) {
  return (double)b->lo[0] >= m->lo[0] && (double)b->hi[0] <= m->hi[0] &&
         (double)b->lo[1] >= m->lo[1] && (double)b->hi[1] <= m->hi[1];
}

/* tracing/meeting.cpp:32-76 (plus the map-box filter of cuda/geometry.cu:667-670) */
static int update_meetings(oracle_ctx *c) {
  uint64_t B = c->cfg.num_meeting_buckets;
  uint64_t taken = 0;
  c->emitted_count = 0;
  for (uint64_t bid = 0; bid < B; bid++) {
    obucket *b = &c->buckets[bid];
    if (b->key == EMPTY_KEY) continue;
    if (b->end == c->cur_time) { taken++; continue; }
    if (c->cur_time - b->start >= c->cfg.min_meet_time + 1) {
      if (!c->cfg.mbr_filter || map_contains(&c->map, b))
        if (emit(c, b)) { set_err(c, "out of host memory"); return -1; }
    }
    b->key = EMPTY_KEY;
  }
  c->stats.taken_buckets = taken;
  c->stats.emitted = c->emitted_count;
  return 0;
}

/* tracing/filter.cpp:316-336 */
static void merge_node(oracle_ctx *c, uint32_t cur) {
  for (int i = 0; i < 4; i++) {
    uint32_t ch = c->schema[cur].children[i];
    c->schema[ch].type = INVALID;
    c->schema_stack[--c->schema_stack_index] = ch;
    c->grids_stack[--c->grids_stack_index] = c->schema[ch].grid_id;
    c->grid_counter[c->schema[ch].grid_id] = 0;
  }
  c->schema[cur].type = LEAF;
  c->schema[cur].grid_id = c->grids_stack[c->grids_stack_index++];
}

/* tracing/filter.cpp:338-375 */
static int split_node(oracle_ctx *c, uint32_t cur) {
  oschema *s = &c->schema[cur];
  s->type = BRANCH;
  if (c->grids_stack_index == 0) return -1;
  c->grids_stack[--c->grids_stack_index] = s->grid_id;
  double xhalf = s->mid_x - s->mbr.lo[0];
  double yhalf = s->mid_y - s->mbr.lo[1];
  for (int i = 0; i < 4; i++) {
    if (c->schema_stack_index >= c->S || c->grids_stack_index >= c->G) return -1;
    uint32_t child = c->schema_stack[c->schema_stack_index++];
    s->children[i] = child;
    oschema *d = &c->schema[child];
    d->grid_id = c->grids_stack[c->grids_stack_index++];
    c->grid_counter[d->grid_id] = 0;
    d->level = (short)(s->level + 1);
    d->type = LEAF;
    d->overflow_count = 0;
    d->underflow_count = 0;
    d->mbr.lo[0] = s->mbr.lo[0] + (i % 2 == 1) * xhalf;
    d->mbr.lo[1] = s->mbr.lo[1] + (i / 2 == 1) * yhalf;
    d->mbr.hi[0] = s->mid_x + (i % 2 == 1) * xhalf;
    d->mbr.hi[1] = s->mid_y + (i / 2 == 1) * yhalf;
    d->mid_x = (d->mbr.lo[0] + d->mbr.hi[0]) / 2;
    d->mid_y = (d->mbr.lo[1] + d->mbr.hi[1]) / 2;
  }
  return 0;
}

/* tracing/filter.cpp:377-424 (visited in node order, single-threaded) */
static int update_schema(oracle_ctx *c) {
  uint32_t splits = 0, merges = 0;
  double reach = c->cfg.reach_distance;
  uint32_t cap = c->cfg.grid_capacity;
  for (uint32_t cur = 0; cur < c->S; cur++) {
    oschema *s = &c->schema[cur];
    if (s->type == LEAF) {
      if (box_width_geo(&s->mbr) > reach * 2 && c->grid_counter[s->grid_id] > cap) {
        s->overflow_count++;
        if ((uint32_t)s->overflow_count >= c->cfg.schema_update_delay) {
          if (split_node(c, cur)) { set_err(c, "schema capacity exceeded"); return -1; }
          c->schema[cur].overflow_count = 0;
          splits++;
        }
      } else {
        s->overflow_count = 0;
      }
    } else if (s->type == BRANCH) {
      int leafchild = 0;
      int ncounter = 0;
      for (int i = 0; i < 4; i++) {
        uint32_t ch = s->children[i];
        if (c->schema[ch].type == LEAF) {
          leafchild++;
          ncounter += (int)c->grid_counter[c->schema[ch].grid_id];
        }
      }
      if (leafchild == 4 && ncounter < (int)cap) {
        s->underflow_count++;
        if ((uint32_t)s->underflow_count >= c->cfg.schema_update_delay) {
          merge_node(c, cur);
          c->schema[cur].underflow_count = 0;
          merges++;
        }
      } else {
        s->underflow_count = 0;
      }
    }
  }
  c->stats.splits = splits;
  c->stats.merges = merges;
  return 0;
}

int oracle_step(oracle_ctx *c, const double *xy, uint32_t t) {
  if (!c || c->err[0]) return -1;
  c->xy = xy;
  c->cur_time = t;
  memset(&c->stats, 0, sizeof(c->stats));
  /* workbench::reset (tracing/workbench.h:323-329) */
  memset(c->grid_counter, 0, (size_t)c->G * sizeof(uint32_t));
  c->unit_count = 0;
  int rc = c->threads <= 1 ? filter_st(c) : filter_mt(c);
  if (rc) return -1;
  uint32_t overflow = 0;
  for (uint32_t g = 0; g < c->G; g++)
    if (c->grid_counter[g] > c->leaf_cap) overflow += c->grid_counter[g] - c->leaf_cap;
  if (reachability(c)) return -1;
  if (update_meetings(c)) return -1;
  c->stats.step = t;
  c->stats.checking_units = c->unit_count;
  c->stats.border_units = c->unit_count - c->N;
  c->stats.overflow_objects = overflow;
  if (c->cfg.dynamic_schema) {
    if (update_schema(c)) return -1;
  }
  c->stats.leaves = c->grids_stack_index;
  c->stats.schema_nodes = c->schema_stack_index;
  return 0;
}

size_t oracle_emitted(oracle_ctx *c, const stc_meeting **out) {
  *out = c->emitted;
  return c->emitted_count;
}

void oracle_stats(oracle_ctx *c, stc_stats *s) { *s = c->stats; }

uint32_t oracle_schema_size(oracle_ctx *c) { return c->S; }
uint32_t oracle_schema_stack_index(oracle_ctx *c) { return c->schema_stack_index; }
uint32_t oracle_grids_stack_index(oracle_ctx *c) { return c->grids_stack_index; }

void oracle_schema_dump(oracle_ctx *c, int16_t *type, uint32_t *grid_id, uint32_t *children,
                        double *boxes) {
  for (uint32_t i = 0; i < c->S; i++) {
    type[i] = c->schema[i].type;
    grid_id[i] = c->schema[i].grid_id;
    for (int k = 0; k < 4; k++) children[4 * (size_t)i + k] = c->schema[i].children[k];
    boxes[4 * (size_t)i + 0] = c->schema[i].mbr.lo[0];
    boxes[4 * (size_t)i + 1] = c->schema[i].mbr.lo[1];
    boxes[4 * (size_t)i + 2] = c->schema[i].mbr.hi[0];
    boxes[4 * (size_t)i + 3] = c->schema[i].mbr.hi[1];
  }
}
