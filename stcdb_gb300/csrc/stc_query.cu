// Queries over the retained flushed blocks (the reference's disk searches,
// with the time window of its time_query; semantics in include/stc.h).
//
// Object queries get one CTA per (block, query): the object's sid picks the
// oversize buffer or a CTF, one thread runs the reference's binary search for
// the first key of the pid and the CTA scans on while the pid matches. Box
// queries are planned per (query, block, CTF) and run as rows of the blocks'
// cell indexes, one warp per row (k_box_plan, k_box_rows). Matches are
// appended to one device buffer tagged with their query; the host groups
// them by query.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "stc_lsm.cuh"

namespace stc {

namespace {

constexpr uint32_t QOBJ_THREADS = 128;
constexpr uint32_t QBOX_THREADS = 128;

struct Key {
  uint32_t oid, target, duration, end;
  double box[4];
};

__host__ __device__ __forceinline__ unsigned long long mask64(uint32_t bits) {
  return bits >= 64 ? ~0ull : (1ull << bits) - 1;
}

// The low key_bit/8 bytes at p, little-endian, from three aligned words (the
// key buffers carry 32 bytes of padding).
__device__ __forceinline__ unsigned __int128 load_key(const uint8_t *p, uint32_t kb) {
  uintptr_t a = (uintptr_t)p;
  const unsigned long long *w = (const unsigned long long *)(a & ~(uintptr_t)7);
  uint32_t sh = (uint32_t)(a & 7) * 8;
  unsigned __int128 lo = ((unsigned __int128)__ldg(w + 1) << 64) | __ldg(w);
  unsigned __int128 k = lo >> sh;
  if (sh) k |= (unsigned __int128)__ldg(w + 2) << (128 - sh);
  if (kb < 16) k &= (((unsigned __int128)1) << (8 * kb)) - 1;
  return k;
}

// CTF::ctf_get_key_oid, CTF::parse_key, CTF::new_parse_mbr
// (tracing/step_merge.cpp:329-379), the box in double from the CTF box.
__device__ __forceinline__ uint32_t key_oid(unsigned __int128 k, const stc_ctf &c) {
  return (uint32_t)((k >> (c.id_bit + c.duration_bit + c.end_bit + c.mbr_bit)) & mask64(c.id_bit));
}

// The packed box fields of value_mbr in CTF c, decoded (CTF::new_parse_mbr).
__device__ void exact_box(unsigned long long vm, const stc_ctf &c, double box[4]) {
  unsigned long long me = mask64(c.edge_bit), my = mask64(c.low_y_bit), mx = mask64(c.low_x_bit);
  unsigned long long y = vm & me;
  vm >>= c.edge_bit;
  unsigned long long x = vm & me;
  vm >>= c.edge_bit;
  unsigned long long low1 = vm & my;
  vm >>= c.low_y_bit;
  unsigned long long low0 = vm & mx;
  float wx = __fsub_rn(c.mbr[2], c.mbr[0]), wy = __fsub_rn(c.mbr[3], c.mbr[1]);
  double le = (double)fmaxf(wx, wy);
  box[0] = __dadd_rn((double)c.mbr[0], __dmul_rn(__ddiv_rn(__ull2double_rn(low0), __ull2double_rn(mx)), (double)wx));
  box[1] = __dadd_rn((double)c.mbr[1], __dmul_rn(__ddiv_rn(__ull2double_rn(low1), __ull2double_rn(my)), (double)wy));
  box[2] = __dadd_rn(box[0], __dmul_rn(__ddiv_rn(__ull2double_rn(x), __ull2double_rn(me)), le));
  box[3] = __dadd_rn(box[1], __dmul_rn(__ddiv_rn(__ull2double_rn(y), __ull2double_rn(me)), le));
}

// The integer fields of a packed key (CTF::parse_key with the oid masked).
__device__ __forceinline__ unsigned long long key_fields(unsigned __int128 k, const stc_ctf &c, Key &o) {
  o.oid = key_oid(k, c);
  unsigned long long vm = (unsigned long long)(k & (unsigned __int128)mask64(c.mbr_bit));
  k >>= c.mbr_bit;
  o.end = (uint32_t)(k & mask64(c.end_bit));
  k >>= c.end_bit;
  o.duration = (uint32_t)(k & mask64(c.duration_bit));
  k >>= c.duration_bit;
  o.target = (uint32_t)(k & mask64(c.id_bit));
  return vm;
}

// Screening of the box test without decode_key's four correctly rounded
// divisions: the decoded corners computed with reciprocals differ from the
// exact ones by a few ulp of coordinates below 2^8 degrees (< 1e-12), so a
// key whose approximate box clears every query edge by BOX_EPS is decided;
// box_screen returns 1 (meets the query), 0 (misses it) or -1 (decode it).
constexpr double BOX_EPS = 1e-10;
struct BoxRecip {
  double m0, m1, wx, wy, le, rx, ry, re;
};

__device__ __forceinline__ BoxRecip box_recip(const stc_ctf &c) {
  BoxRecip r;
  const float wx = __fsub_rn(c.mbr[2], c.mbr[0]), wy = __fsub_rn(c.mbr[3], c.mbr[1]);
  r.m0 = c.mbr[0];
  r.m1 = c.mbr[1];
  r.wx = wx;
  r.wy = wy;
  r.le = (double)fmaxf(wx, wy);
  r.rx = 1.0 / (double)mask64(c.low_x_bit);
  r.ry = 1.0 / (double)mask64(c.low_y_bit);
  r.re = 1.0 / (double)mask64(c.edge_bit);
  return r;
}

__device__ __forceinline__ int box_screen(unsigned long long vm, const stc_ctf &c, const BoxRecip &r, const double *q) {
  const unsigned long long y = vm & mask64(c.edge_bit);
  vm >>= c.edge_bit;
  const unsigned long long x = vm & mask64(c.edge_bit);
  vm >>= c.edge_bit;
  const unsigned long long low1 = vm & mask64(c.low_y_bit);
  vm >>= c.low_y_bit;
  const unsigned long long low0 = vm & mask64(c.low_x_bit);
  const double b0 = r.m0 + (double)low0 * r.rx * r.wx, b1 = r.m1 + (double)low1 * r.ry * r.wy;
  const double b2 = b0 + (double)x * r.re * r.le, b3 = b1 + (double)y * r.re * r.le;
  // box::intersect (geometry/geometry.h:128-133) on closed intervals
  if (b0 > q[2] + BOX_EPS || b2 < q[0] - BOX_EPS || b1 > q[3] + BOX_EPS || b3 < q[1] - BOX_EPS) return 0;
  if (b0 < q[2] - BOX_EPS && b2 > q[0] + BOX_EPS && b1 < q[3] - BOX_EPS && b3 > q[1] + BOX_EPS) return 1;
  return -1;
}

__device__ void decode_key(unsigned __int128 k, const stc_ctf &c, Key &o) {
  exact_box(key_fields(k, c, o), c, o.box);
}

__device__ __forceinline__ bool time_ok(uint32_t start, uint32_t end, uint32_t t1, uint32_t t2) {
  return start < t2 && t1 < end;  // util/query_context.h:100-103
}

__device__ __forceinline__ bool box_hits(const double *a, const double *q) {  // geometry/geometry.h:128-133
  return !(q[0] > a[2] || q[2] < a[0] || q[1] > a[3] || q[3] < a[1]);
}

__device__ __forceinline__ void emit(QueryRec *out, unsigned long long cap, unsigned long long *count, uint32_t q,
                                     uint32_t pid, uint32_t target, uint32_t start, uint32_t end, const double *b,
                                     uint32_t block, uint32_t ctf) {
  unsigned long long i = agg_inc(count);
  if (i >= cap) return;  // counted; the host re-runs with a larger buffer
  QueryRec r;
  r.c.pid = pid;
  r.c.target = target;
  r.c.start = start;
  r.c.end = end;
  r.c.mbr[0] = b[0]; r.c.mbr[1] = b[1]; r.c.mbr[2] = b[2]; r.c.mbr[3] = b[3];
  r.c.block = block;
  r.c.ctf = ctf;
  r.q = q;
  r.pad = 0;
  out[i] = r;
}

// Adds the CTA's per-thread match counts to the query's total.
__device__ __forceinline__ void add_count(unsigned long long *qcounts, uint32_t q, uint32_t mine) {
  __shared__ unsigned int s_n;
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  if (mine) atomicAdd(&s_n, mine);
  __syncthreads();
  if (threadIdx.x == 0 && s_n) atomicAdd(&qcounts[q], (unsigned long long)s_n);
}

__device__ __forceinline__ void oversize_key(const QBlock &b, unsigned long long i, uint32_t &pid, uint32_t &target,
                                             uint32_t &start, uint32_t &end) {
  uint4 r = b.orec[i];
  pid = r.x;
  target = r.y;
  end = r.w + b.o_end_time_min;
  start = end - r.z;
}

// ---- object queries ----------------------------------------------------------

__global__ void __launch_bounds__(QOBJ_THREADS) k_query_object(const QBlock *qb, const stc_query *qs,
                                                              QueryRec *out, unsigned long long cap,
                                                              unsigned long long *count,
                                                              unsigned long long *qcounts) {
  const QBlock &b = qb[blockIdx.x];
  const stc_query q = qs[blockIdx.y];
  if ((q.kind & 0xFFu) != STC_QUERY_OBJECT) return;
  const bool count_only = (q.kind & STC_QUERY_COUNT_ONLY) != 0;
  uint32_t mine = 0;
  __shared__ long long s_find;
  __shared__ unsigned long long s_lim, s_bad;
  __shared__ uint32_t s_ctf;
  const uint32_t pid = q.pid;
  if (threadIdx.x == 0) {
    s_find = -1;
    s_lim = 0;
    s_ctf = b.F;
    uint16_t sid = b.sids[pid];
    if (sid == 1) {
      // oversize_buffer::search_buffer (tracing/step_merge.cpp:65-110)
      long long low = 0, high = (long long)b.n_over - 1;
      while (low <= high) {
        long long mid = (low + high) / 2;
        uint32_t p = b.orec[mid].x;
        if (p == pid) { s_find = mid; high = mid - 1; }
        else if (p > pid) high = mid - 1;
        else low = mid + 1;
      }
      s_lim = b.n_over;
    } else if (sid >= 2 && (uint32_t)sid - 2 < b.F) {
      // CTF::binary_search (tracing/step_merge.cpp:496-521)
      const uint32_t c = sid - 2;
      const stc_ctf &t = b.ctfs[c];
      const uint32_t kb = t.key_bit / 8u;
      const uint8_t *base = b.keys + t.key_offset;
      uint32_t low = 0, high = t.kv_count - 1;
      while (low <= high) {
        unsigned long long mid = low + (unsigned long long)(high - low) / 2;
        if (mid >= t.kv_count) break;
        uint32_t oid = key_oid(load_key(base + mid * kb, kb), t);
        if (oid == pid) {
          s_find = (long long)mid;
          if (mid == 0) break;
          high = (uint32_t)mid - 1;
        } else if (oid < pid) {
          low = (uint32_t)mid + 1;
        } else {
          if (mid == 0) break;
          high = (uint32_t)mid - 1;
        }
      }
      s_lim = t.kv_count;
      s_ctf = c;
    }
  }
  __syncthreads();
  if (s_find < 0) return;  // uniform: no count to add
  const uint32_t c = s_ctf;
  const unsigned long long lim = s_lim;
  // scan on while the pid matches (search_SSTable, step_merge.cpp:530-568)
  for (unsigned long long base = (unsigned long long)s_find;; base += blockDim.x) {
    if (threadIdx.x == 0) s_bad = ~0ull;
    __syncthreads();
    unsigned long long i = base + threadIdx.x;
    bool match = false;
    uint32_t target = 0, start = 0, end = 0;
    double box[4];
    if (i < lim) {
      if (c == b.F) {
        uint32_t p;
        oversize_key(b, i, p, target, start, end);
        match = p == pid;
        float4 fb = b.obox[i];
        box[0] = fb.x; box[1] = fb.y; box[2] = fb.z; box[3] = fb.w;
      } else {
        const stc_ctf &t = b.ctfs[c];
        Key k;
        decode_key(load_key(b.keys + t.key_offset + i * (t.key_bit / 8u), t.key_bit / 8u), t, k);
        match = k.oid == pid;
        target = k.target;
        end = k.end + t.end_time_min;
        start = end - k.duration;
        box[0] = k.box[0]; box[1] = k.box[1]; box[2] = k.box[2]; box[3] = k.box[3];
      }
    }
    if (!match) atomicMin(&s_bad, i);
    __syncthreads();
    const unsigned long long bad = s_bad;
    if (match && i < bad && time_ok(start, end, q.t_start, q.t_end)) {
      mine++;
      if (!count_only) emit(out, cap, count, blockIdx.y, pid, target, start, end, box, b.index, c);
    }
    if (bad != ~0ull) break;  // uniform
    __syncthreads();
  }
  add_count(qcounts, blockIdx.y, mine);
}

// ---- box queries ---------------------------------------------------------------

// Position of v on a grid of n cells over [m0, m1], in cells (monotone in v;
// the cell index and the query windows both use it).
__device__ __forceinline__ double grid_coord(double v, double m0, double m1, uint32_t n) {
  double w = __dsub_rn(m1, m0);
  return __dmul_rn(__ddiv_rn(__dsub_rn(v, m0), w), (double)n);
}

// Cell range [lo, hi] of the interval [a, b] on a grid of n cells over
// [m0, m1], one cell of slack either side, clamped to [0, n].
__device__ __forceinline__ void cell_range(double a, double b, double m0, double m1, uint32_t n, int &lo, int &hi) {
  const bool ok = m1 > m0;
  double fa = ok ? grid_coord(a, m0, m1, n) : 0.0, fb = ok ? grid_coord(b, m0, m1, n) : (double)n;
  fa = fmax(fmin(fa, (double)n + 2), -2.0);
  fb = fmax(fmin(fb, (double)n + 2), -2.0);
  lo = max((int)floor(fa) - 1, 0);
  hi = min((int)floor(fb) + 1, (int)n);
}

// Position of v in level-0 cells of a CTF's index: (v - m0) times the CTF's
// stored cells per degree. Monotone in v, and the same function files keys
// and bounds queries, which is all the index's exactness needs.
__device__ __forceinline__ double index_coord(double v, double m0, double scale) {
  return __dmul_rn(__dsub_rn(v, m0), scale);
}

// cell_range on the index grid: [lo, hi] of [a, b], one cell of slack either
// side, clamped to [0, n]; scale 0 (a degenerate CTF box) takes every cell.
__device__ __forceinline__ void index_range(double a, double b, double m0, double scale, uint32_t n, int &lo,
                                            int &hi) {
  const bool ok = scale > 0.0;
  double fa = ok ? index_coord(a, m0, scale) : 0.0, fb = ok ? index_coord(b, m0, scale) : (double)n;
  fa = fmax(fmin(fa, (double)n + 2), -2.0);
  fb = fmax(fmin(fb, (double)n + 2), -2.0);
  lo = max((int)floor(fa) - 1, 0);
  hi = min((int)floor(fb) + 1, (int)n);
}

// ---- cell index of a block ------------------------------------------------------

constexpr uint32_t MAX_CTF = 3969;

// Dense cell id of each CTF key in its CTF's loose grid (stc_lsm.cuh): the
// level whose cells cover the extent of its decoded box, the cell of the box's
// low corner there; or the CTF's wide slot.
//
// The cell depends on the decoded box only through floor() of its four corner
// coordinates in level-0 cells. These are first computed in float from the
// key's integer fields (cells per field unit, ixf); a corner whose float value
// lies within its error margin of an integer could floor the other way, and
// only keys with such a corner take the exact decode (four correctly rounded
// FP64 divisions, which the key's filing must agree with).
struct IndexFile {
  uint32_t l0, l1;  // floor of the low corner, level-0 cells
  float ext;        // extent in level-0 cells: max over x, y of floor(high) - floor(low)
  bool inside;      // low corner in [0, g + 1) on both axes
};

__device__ __forceinline__ uint32_t index_cell_of(const IndexFile &f, uint32_t g, uint32_t levels) {
  if (!f.inside) return 0xFFFFFFFFu;
  uint32_t lv = 0, off = 0;
  while (lv + 1 < levels && f.ext > (float)(1u << lv)) {
    uint32_t side = index_level_side(g, lv);
    off += side * side;
    lv++;
  }
  if (f.ext > (float)(1u << lv)) return 0xFFFFFFFFu;
  return off + (f.l1 >> lv) * index_level_side(g, lv) + (f.l0 >> lv);
}

// floor(v) when every value within d of v has the same floor; else false.
__device__ __forceinline__ bool sure_floor(float v, float d, float &fl) {
  fl = floorf(v - d);
  return fl == floorf(v + d);
}

__device__ __forceinline__ bool index_file_fast(unsigned long long vm, const stc_ctf &c, const float4 &ax,
                                                const float4 &ay, uint32_t g, IndexFile &f) {
  if (ax.w == 0.0f || ay.w == 0.0f) return false;
  const unsigned long long y = vm & mask64(c.edge_bit);
  vm >>= c.edge_bit;
  const unsigned long long x = vm & mask64(c.edge_bit);
  vm >>= c.edge_bit;
  const unsigned long long low1 = vm & mask64(c.low_y_bit);
  vm >>= c.low_y_bit;
  const unsigned long long low0 = vm & mask64(c.low_x_bit);
  const float fx0 = __ull2float_rn(low0) * ax.x, fy0 = __ull2float_rn(low1) * ay.x;
  const float fx1 = fx0 + __ull2float_rn(x) * ax.y, fy1 = fy0 + __ull2float_rn(y) * ay.y;
  float a, b, p, q;
  if (!sure_floor(fx0, fmaf(fx0, 1e-6f, ax.z), a) || !sure_floor(fy0, fmaf(fy0, 1e-6f, ay.z), b) ||
      !sure_floor(fx1, fmaf(fx1, 1e-6f, ax.z), p) || !sure_floor(fy1, fmaf(fy1, 1e-6f, ay.z), q))
    return false;
  f.inside = a >= 0.0f && b >= 0.0f && a <= (float)g && b <= (float)g;
  f.l0 = f.inside ? (uint32_t)a : 0u;
  f.l1 = f.inside ? (uint32_t)b : 0u;
  f.ext = fmaxf(p - a, q - b);
  return true;
}

__device__ __forceinline__ void index_file_exact(unsigned long long vm, const stc_ctf &c, const double2 sc,
                                                 uint32_t g, IndexFile &f) {
  double box[4];
  exact_box(vm, c, box);
  const double fx0 = index_coord(box[0], c.mbr[0], sc.x), fx1 = index_coord(box[2], c.mbr[0], sc.x);
  const double fy0 = index_coord(box[1], c.mbr[1], sc.y), fy1 = index_coord(box[3], c.mbr[1], sc.y);
  f.inside = fx0 >= 0 && fy0 >= 0 && fx0 < g + 1 && fy0 < g + 1 && fx1 >= fx0 && fy1 >= fy0;
  f.l0 = f.inside ? (uint32_t)floor(fx0) : 0u;
  f.l1 = f.inside ? (uint32_t)floor(fy0) : 0u;
  f.ext = f.inside ? (float)fmax(floor(fx1) - f.l0, floor(fy1) - f.l1) : 0.0f;
}

__global__ void k_index_cells(const uint8_t *keys, const stc_ctf *ctfs, uint32_t F, const uint32_t *cbase,
                              const uint4 *ixg, const double2 *ixs, const float4 *ixf, unsigned long long total,
                              uint32_t *cells, uint32_t *pos, uint32_t *endo, unsigned long long *max_end) {
  __shared__ unsigned long long s_first[MAX_CTF + 1];
  __shared__ uint32_t s_max;
  if (threadIdx.x == 0) s_max = 0;
  uint32_t my_max = 0;
  for (uint32_t c = threadIdx.x; c < F; c += blockDim.x) s_first[c] = ctfs[c].first_key;
  __syncthreads();
  for (unsigned long long kid = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; kid < total;
       kid += (unsigned long long)gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = F - 1;
    while (lo < hi) {
      uint32_t mid = (lo + hi + 1) >> 1;
      if (s_first[mid] <= kid) lo = mid;
      else hi = mid - 1;
    }
    const stc_ctf &t = ctfs[lo];
    const uint32_t kb = t.key_bit / 8u;
    Key k;
    const unsigned long long vm = key_fields(load_key(keys + t.key_offset + (kid - s_first[lo]) * kb, kb), t, k);
    const uint32_t g = ixg[lo].x, levels = ixg[lo].y;
    const double2 sc = ixs[lo];
    uint32_t cell = 0xFFFFFFFFu;  // the wide slot, after every level
    if (sc.x > 0.0 && sc.y > 0.0) {
      IndexFile f;
      if (!index_file_fast(vm, t, ixf[2 * lo], ixf[2 * lo + 1], g, f)) index_file_exact(vm, t, sc, g, f);
      cell = index_cell_of(f, g, levels);
    }
    if (cell == 0xFFFFFFFFu) cell = cbase[lo + 1] - cbase[lo] - 1;
    cells[kid] = cbase[lo] + cell;
    pos[kid] = (uint32_t)kid;
    endo[kid] = min(k.end, 65535u);
    my_max = max(my_max, min(k.end, 65535u));
  }
  __syncthreads();
  atomicMax(&s_max, my_max);
  __syncthreads();
  if (threadIdx.x == 0 && s_max) atomicMax(max_end, (unsigned long long)s_max);
}

// Sort keys of the one-pass index order: cell above the end offset.
__global__ void k_index_keys(const uint32_t *cells, const uint32_t *endo, uint32_t eb, unsigned long long n,
                             uint32_t *keys) {
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x)
    keys[i] = (cells[i] << eb) | endo[i];
}

__global__ void k_index_ends(const uint32_t *sorted, uint32_t eb, unsigned long long n, uint16_t *pend) {
  const uint32_t mask = (1u << eb) - 1u;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x)
    pend[i] = (uint16_t)(sorted[i] & mask);
}

__global__ void k_gather_cells(const uint32_t *src, const uint32_t *idx, uint32_t *dst, unsigned long long n) {
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x)
    dst[i] = src[idx[i]];
}

__global__ void k_gather_ends(const uint32_t *endo, const uint32_t *perm, uint16_t *pend, unsigned long long n) {
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x)
    pend[i] = (uint16_t)endo[perm[i]];
}

// cstart[k] = first position of the sorted cell ids (sorted >> shift)
// holding an id >= k.
__global__ void k_cell_starts(const uint32_t *sorted, uint32_t shift, unsigned long long total, uint32_t ncells,
                              uint32_t *cstart) {
  for (unsigned long long k = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; k <= ncells;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    unsigned long long lo = 0, hi = total;
    while (lo < hi) {
      unsigned long long mid = (lo + hi) >> 1;
      if ((sorted[mid] >> shift) < k) lo = mid + 1;
      else hi = mid;
    }
    cstart[k] = (uint32_t)lo;
  }
}

__global__ void k_set_one(unsigned long long *p, unsigned long long v) { *p = v; }

// ---- box queries: plan, then rows --------------------------------------------
//
// A batch's box queries run in three launches. k_box_plan gives every
// (query, block, CTF or oversize buffer) pair one thread: it prunes by the CTF
// box and bitmap (widened so that no key whose decoded box meets the query is
// lost), counts whole CTFs a counting query holds, and writes how many work
// items the pair needs: one per row of every index level plus the wide list
// (CTFs), or one per OV_CHUNK oversize keys. An exclusive scan turns the
// counts into the items' first numbers, and k_box_rows gives each work item
// one warp, so that big and small queries alike spread over the whole GPU.

constexpr uint32_t OV_CHUNK = 2048;       // oversize keys per work item
constexpr uint32_t SEQ_BITMAP_CELLS = 1024;  // larger windows skip the per-thread bitmap test

// Any set bit in cells [i0, i1] x [j0, j1] (one thread); windows of more than
// SEQ_BITMAP_CELLS cells are taken as hit (the bitmap only prunes).
// Bits past `nbits` (the bitmap's size) read as clear.
__device__ bool any_bit_seq(const uint32_t *bm, int i0, int i1, int j0, int j1, uint32_t xg, long long nbits) {
  long long ni = (long long)i1 - i0 + 1, nj = (long long)j1 - j0 + 1;
  if (ni <= 0 || nj <= 0) return false;
  if (ni * nj > SEQ_BITMAP_CELLS) return true;
  for (long long j = j0; j <= j1; j++)
    for (long long i = i0; i <= i1; i++) {
      long long bit = i + j * (long long)xg;
      if (bit >= 0 && bit < nbits && ((__ldg(&bm[bit >> 5]) >> (bit & 31)) & 1u)) return true;
    }
  return false;
}

// What a box query needs to know about one CTF.
struct BoxCtx {
  double wide[4];
  double qx, qy;
  bool all_starts, all_ends;
  uint32_t ts;                 // end offsets above ts pass t_start < end
  uint32_t g, levels;          // the CTF's index
  int i0, i1, j0, j1;          // query window in level-0 cells, one cell of slack
  int ii0, ii1, jj0, jj1;      // interior level-0 cells (counting queries), empty if ii0 > ii1
};

// Fills x for CTF t and query q; false when the CTF box misses the widened query.
__device__ bool box_ctx(const stc_ctf &t, const uint4 &ix, const double2 &sc, const stc_query &q, BoxCtx &x) {
  // A decoded box differs from the key's exact box (which set the CTF box
  // and the bitmap) by less than one corner quantum plus one edge quantum on
  // either side (float conversions truncate, and may round up first): widen
  // the query by that much for the box and bitmap tests.
  const double *qbox = q.box;
  const float fwx = __fsub_rn(t.mbr[2], t.mbr[0]), fwy = __fsub_rn(t.mbr[3], t.mbr[1]);
  const double le = (double)fmaxf(fwx, fwy), me = (double)mask64(t.edge_bit);
  x.qx = (double)fwx / (double)mask64(t.low_x_bit) + le / me + 1e-9;
  x.qy = (double)fwy / (double)mask64(t.low_y_bit) + le / me + 1e-9;
  x.wide[0] = qbox[0] - x.qx;
  x.wide[1] = qbox[1] - x.qy;
  x.wide[2] = qbox[2] + x.qx;
  x.wide[3] = qbox[3] + x.qy;
  const double ctfb[4] = {t.mbr[0], t.mbr[1], t.mbr[2], t.mbr[3]};
  if (!box_hits(ctfb, x.wide)) return false;
  // Time conditions that hold for every key of the CTF: no time field can
  // have outgrown its bit width (decoded = stored times), and then every
  // start is below t_end, or every end above t_start (ends are >= the
  // block's base).
  const bool fits = (unsigned long long)(t.end_time_max - t.end_time_min) <= mask64(t.end_bit) &&
                    (unsigned long long)(t.end_time_max - t.start_time_min) <= mask64(t.duration_bit) &&
                    t.start_time_min <= t.end_time_max && t.end_time_min <= t.end_time_max;
  x.all_starts = fits && t.start_time_max < q.t_end;
  x.all_ends = fits && q.t_start < t.end_time_min;
  // the saturated end offsets of the index order them exactly below 65535
  x.ts = x.all_ends ? 0u : q.t_start - t.end_time_min;
  x.g = ix.x;
  x.levels = ix.y;
  index_range(x.wide[0], x.wide[2], t.mbr[0], sc.x, x.g, x.i0, x.i1);
  index_range(x.wide[1], x.wide[3], t.mbr[1], sc.y, x.g, x.j0, x.j1);
  // Interior cells (counting only, every start passing): level-0 cells whose
  // every decoded low corner lies in the query box. A key's box meets the
  // query when its low corner is inside it; index_coord is monotone, so a
  // corner in cell i (gc in [i, i + 1)) lies in [q_lo, q_hi] when
  // i > gc(q_lo) and i + 1 <= gc(q_hi).
  x.ii0 = x.jj0 = 1;
  x.ii1 = x.jj1 = 0;
  const bool count_only = (q.kind & STC_QUERY_COUNT_ONLY) != 0;
  if (count_only && x.all_starts && (x.all_ends || x.ts < 65535u) && sc.x > 0.0 && sc.y > 0.0) {
    auto interior = [](double g0, double g1, uint32_t n, int &lo, int &hi) {
      g0 = fmax(fmin(g0, (double)n + 2), -2.0);
      g1 = fmax(fmin(g1, (double)n + 2), -2.0);
      lo = max((int)floor(g0) + 1, 0);
      hi = min((int)floor(g1) - 1, (int)n);
    };
    interior(index_coord(qbox[0], t.mbr[0], sc.x), index_coord(qbox[2], t.mbr[0], sc.x), x.g, x.ii0, x.ii1);
    interior(index_coord(qbox[1], t.mbr[1], sc.y), index_coord(qbox[3], t.mbr[1], sc.y), x.g, x.jj0, x.jj1);
  }
  return true;
}

// Rows of level lv in the window: a key filed at level lv under cell
// (cx, cy) whose box meets the widened query has cy in
// [(j0 >> lv) - 1, j1 >> lv] (its box ends at most one cell above cy), and
// likewise cx.
__device__ __forceinline__ int level_rows(const BoxCtx &x, uint32_t lv, int &cj0) {
  const int side = (int)index_level_side(x.g, lv);
  cj0 = max((x.j0 >> lv) - 1, 0);
  return max(min(x.j1 >> lv, side - 1) - cj0 + 1, 0);
}

__global__ void k_box_plan(const QBlock *qb, uint32_t nb, const stc_query *qs, uint32_t nq, uint32_t F1,
                           double m0x, double m0y, double m1x, double m1y, uint32_t *items,
                           unsigned long long *qcounts) {
  const uint32_t P = nq * nb * F1;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const uint32_t c = p % F1, bi = (p / F1) % nb, qi = p / F1 / nb;
    const stc_query &q = qs[qi];
    const QBlock &b = qb[bi];
    uint32_t n = 0;
    if ((q.kind & 0xFFu) == STC_QUERY_BOX && c <= b.F) {
      if (c == b.F) {  // oversize buffer: the map bitmap prunes
        if (b.n_over) {
          int i0, i1, j0, j1;
          cell_range(q.box[0], q.box[2], m0x, m1x, b.edge, i0, i1);
          cell_range(q.box[1], q.box[3], m0y, m1y, b.edge, j0, j1);
          if (any_bit_seq(b.obitmap, i0, i1, j0, j1, b.edge, (long long)b.edge * b.edge))
            n = (uint32_t)((b.n_over + OV_CHUNK - 1) / OV_CHUNK);
        }
      } else {
        const stc_ctf &t = b.ctfs[c];
        BoxCtx x;
        if (t.kv_count && box_ctx(t, b.ixg[c], b.ixs[c], q, x)) {
          const double *qbox = q.box;
          const bool count_only = (q.kind & STC_QUERY_COUNT_ONLY) != 0;
          if (count_only && x.all_starts && x.all_ends && qbox[0] <= t.mbr[0] - x.qx && qbox[1] <= t.mbr[1] - x.qy &&
              qbox[2] >= t.mbr[2] + x.qx && qbox[3] >= t.mbr[3] + x.qy) {
            // Every key matches -- count the CTF without decoding it, as the
            // reference's box search does (workbench.cpp:525-528).
            atomicAdd(&qcounts[qi], (unsigned long long)t.kv_count);
          } else {
            int bi0, bi1, bj0, bj1;  // the bitmap's cells
            cell_range(x.wide[0], x.wide[2], t.mbr[0], t.mbr[2], t.x_grid, bi0, bi1);
            cell_range(x.wide[1], x.wide[3], t.mbr[1], t.mbr[3], t.y_grid, bj0, bj1);
            if (any_bit_seq(b.bitmaps + (size_t)c * (STC_BITMAP_BYTES / 4), bi0, bi1, bj0, bj1, t.x_grid,
                            8ll * STC_BITMAP_BYTES)) {
              n = 1;  // the wide list
              for (uint32_t lv = 0; lv < x.levels; lv++) {
                int cj0;
                n += (uint32_t)level_rows(x, lv, cj0);
              }
            }
          }
        }
      }
    }
    items[p] = n;
  }
}

// One warp per work item; item numbers come from the exclusive scan of the
// plan's counts (items[P] = all items).
__global__ void __launch_bounds__(QBOX_THREADS) k_box_rows(const QBlock *qb, uint32_t nb, const stc_query *qs,
                                                          uint32_t nq, uint32_t F1, const uint32_t *first,
                                                          QueryRec *out, unsigned long long cap,
                                                          unsigned long long *count, unsigned long long *qcounts) {
  const uint32_t P = nq * nb * F1;
  const uint32_t total = first[P];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t item = gw; item < total; item += nw) {
    uint32_t lo = 0, hi = P - 1;  // the pair: largest p with first[p] <= item
    while (lo < hi) {
      uint32_t mid = (lo + hi + 1) >> 1;
      if (__ldg(&first[mid]) <= item) lo = mid;
      else hi = mid - 1;
    }
    const uint32_t p = lo, r = item - first[p];
    const uint32_t c = p % F1, bi = (p / F1) % nb, qi = p / F1 / nb;
    const stc_query q = qs[qi];
    const QBlock &b = qb[bi];
    const bool count_only = (q.kind & STC_QUERY_COUNT_ONLY) != 0;
    const double *qbox = q.box;
    uint32_t mine = 0;
    if (c == b.F) {  // oversize keys [r * OV_CHUNK, ...): float boxes decide
      const unsigned long long k1 = min((unsigned long long)(r + 1) * OV_CHUNK, b.n_over);
      for (unsigned long long i = (unsigned long long)r * OV_CHUNK + lane; i < k1; i += 32) {
        float4 fb = b.obox[i];
        double box[4] = {fb.x, fb.y, fb.z, fb.w};
        uint32_t pid, target, start, end;
        oversize_key(b, i, pid, target, start, end);
        if (time_ok(start, end, q.t_start, q.t_end) && box_hits(box, qbox)) {
          mine++;
          if (!count_only) emit(out, cap, count, qi, pid, target, start, end, box, b.index, c);
        }
      }
    } else {
      const stc_ctf &t = b.ctfs[c];
      BoxCtx x;
      box_ctx(t, b.ixg[c], b.ixs[c], q, x);  // the plan saw it pass
      const uint32_t cb = b.cbase[c], wide_slot = b.cbase[c + 1] - 1u;
      uint32_t a, e, ma, me2;  // scan [a, ma) and [me2, e); [ma, me2) is counted
      int clo = 1, chi = 0;    // counted cells of this row
      uint32_t row_base = 0;
      uint32_t rr = r, lv = 0, off = 0;
      int cj0 = 0, n = 0;
      for (; lv < x.levels; lv++) {
        n = level_rows(x, lv, cj0);
        if (rr < (uint32_t)n) break;
        rr -= (uint32_t)n;
        const uint32_t side = index_level_side(x.g, lv);
        off += side * side;
      }
      if (lv < x.levels) {  // row cj0 + rr of level lv
        const int side = (int)index_level_side(x.g, lv);
        const int jr = cj0 + (int)rr;
        const int ci0 = max((x.i0 >> lv) - 1, 0), ci1 = min(x.i1 >> lv, side - 1);
        row_base = cb + off + (uint32_t)(jr * side);
        a = b.cstart[row_base + (uint32_t)ci0];
        e = ci1 >= ci0 ? b.cstart[row_base + (uint32_t)ci1 + 1] : a;
        ma = me2 = a;
        // interior at this level: cell C covers level-0 cells [C 2^lv, (C + 1) 2^lv - 1]
        const int s2 = 1 << lv;
        const bool row_in = x.ii0 <= x.ii1 && x.jj0 <= x.jj1 && jr * s2 >= x.jj0 && (jr + 1) * s2 - 1 <= x.jj1;
        if (row_in) {
          clo = max((x.ii0 + s2 - 1) >> lv, ci0);
          chi = min(((x.ii1 + 1) >> lv) - 1, ci1);
        }
        if (clo <= chi) {
          ma = b.cstart[row_base + (uint32_t)clo];
          me2 = b.cstart[row_base + (uint32_t)chi + 1];
          if (x.all_ends) {
            if (lane == 0) mine += me2 - ma;
          } else {
            // the counted cells' end offsets lie side by side: one coalesced pass
            for (uint32_t pp = ma + lane; pp < me2; pp += 32) mine += __ldg(&b.pend[pp]) > x.ts;
          }
        }
      } else {  // the wide list
        a = b.cstart[wide_slot];
        e = b.cstart[wide_slot + 1];
        ma = me2 = a;
      }
      const uint32_t kb = t.key_bit / 8u;
      const uint8_t *base = b.keys + t.key_offset;
      const BoxRecip rc = box_recip(t);
      for (int seg = 0; seg < 2; seg++) {
        for (uint32_t pp = (seg ? me2 : a) + lane, pe = seg ? e : ma; pp < pe; pp += 32) {
          const unsigned long long local = (unsigned long long)b.perm[pp] - t.first_key;
          Key k;
          const unsigned long long vm = key_fields(load_key(base + local * kb, kb), t, k);
          uint32_t end = k.end + t.end_time_min, start = end - k.duration;
          if (!time_ok(start, end, q.t_start, q.t_end)) continue;
          const int sc = box_screen(vm, t, rc, qbox);
          if (sc == 0) continue;
          if (sc < 0 || !count_only) exact_box(vm, t, k.box);
          if (sc > 0 || box_hits(k.box, qbox)) {
            mine++;
            if (!count_only) emit(out, cap, count, qi, k.oid, k.target, start, end, k.box, b.index, c);
          }
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
    if (lane == 0 && mine) atomicAdd(&qcounts[qi], (unsigned long long)mine);
  }
}

// Mapped pinned host buffer of at least `need` elements (contents not kept):
// *p is its host address, *m the address kernels use.
template <typename T>
cudaError_t grow_mapped(T **p, T **m, size_t *cap, size_t need) {
  if (*cap >= need) return cudaSuccess;
  size_t n = std::max<size_t>(need, 2 * *cap);
  if (*p) cudaFreeHost(*p);
  *p = *m = nullptr;
  cudaError_t e = cudaHostAlloc((void **)p, n * sizeof(T), cudaHostAllocMapped | cudaHostAllocPortable);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)m, *p, 0);
  if (e != cudaSuccess && *p) {
    cudaFreeHost(*p);
    *p = *m = nullptr;
  }
  *cap = e == cudaSuccess ? n : 0;
  return e;
}

// Copies `words` 8-byte words between device memory and mapped host memory
// with ordinary loads and stores, which cross the host link without a copy
// engine.
__global__ void k_link_copy(unsigned long long *__restrict__ dst, const unsigned long long *__restrict__ src,
                            size_t words) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

// A batch's per-query match counts, then its total, into mapped host memory.
__global__ void k_counts_out(unsigned long long *__restrict__ dst, const unsigned long long *__restrict__ qcounts,
                             size_t nq, const unsigned long long *__restrict__ total) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i <= nq; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = i < nq ? qcounts[i] : *total;
}

constexpr unsigned LINK_THREADS = 256;

unsigned link_blocks(size_t words) {
  return (unsigned)std::min<size_t>(std::max<size_t>((words + LINK_THREADS - 1) / LINK_THREADS, 1),
                                    (size_t)num_sms() * 4);
}

// Stream-ordered copy of `bytes` (a multiple of 8) between device memory and
// mapped host memory.
template <typename T>
cudaError_t link_copy(T *dst, const T *src, size_t bytes, cudaStream_t s) {
  static_assert(sizeof(T) % 8 == 0, "link copies move 8-byte words");
  const size_t words = bytes / 8;
  if (words == 0) return cudaSuccess;
  k_link_copy<<<link_blocks(words), LINK_THREADS, 0, s>>>((unsigned long long *)dst,
                                                          (const unsigned long long *)src, words);
  return cudaGetLastError();
}

template <typename T>
cudaError_t grow(T **p, size_t *cap, size_t need) {
  if (*cap >= need) return cudaSuccess;
  size_t n = std::max<size_t>(need, 2 * *cap);
  if (*p) cudaFree(*p);
  *p = nullptr;
  cudaError_t e = cudaMalloc(p, n * sizeof(T));
  *cap = e == cudaSuccess ? n : 0;
  return e;
}

}  // namespace

void free_block(CtbBlock &B) {
  for (void *v : {(void *)B.keys, (void *)B.d_ctfs, (void *)B.bitmaps, (void *)B.sids, (void *)B.orec,
                  (void *)B.obox, (void *)B.obitmap, (void *)B.perm, (void *)B.cstart, (void *)B.cbase,
                  (void *)B.ixg, (void *)B.ixs, (void *)B.ixf, (void *)B.pend})
    if (v) cudaFree(v);
  B.ixf = nullptr;
  B.ixg = nullptr;
  B.ixs = nullptr;
  B.pend = nullptr;
  B.keys = nullptr;
  B.d_ctfs = nullptr;
  B.bitmaps = nullptr;
  B.sids = nullptr;
  B.orec = nullptr;
  B.obox = nullptr;
  B.obitmap = nullptr;
  B.perm = nullptr;
  B.cstart = nullptr;
  B.cbase = nullptr;
}

static void retain_block(LsmHost &H, CtbBlock &&B);

// Float filing coefficients of one axis of CTF t (k_index_cells): level-0
// cells per unit of the low field and of the edge field, the absolute error
// margin of the exact filing in cells, and 1 when the float filing applies.
// The exact corner differs from its real value by a few units of 2^-52 of the
// largest coordinate (one division, one product, two sums and a difference,
// each correctly rounded); the margin is 2^6 times that.
static float4 index_file_coeffs(const stc_ctf &t, double scale, bool x_axis) {
  const float wx = t.mbr[2] - t.mbr[0], wy = t.mbr[3] - t.mbr[1];
  const double w = x_axis ? wx : wy, le = std::max(wx, wy);
  const double lowmax = (double)mask64(x_axis ? t.low_x_bit : t.low_y_bit), edgemax = (double)mask64(t.edge_bit);
  double m = 0.0;
  for (int i = 0; i < 4; i++) m = std::max(m, std::fabs((double)t.mbr[i]));
  m += le + 1.0;
  const double a = scale * w / lowmax, b = scale * le / edgemax, d = scale * m * std::ldexp(1.0, -46);
  const bool ok = scale > 0.0 && w > 0.0 && le > 0.0 && lowmax > 0.0 && edgemax > 0.0 && std::isfinite(a) &&
                  std::isfinite(b) && std::isfinite(d) && a < 1e30 && b < 1e30 && d < 1e30;
  return ok ? make_float4((float)a, (float)b, (float)d + 1e-9f, 1.0f) : make_float4(0.f, 0.f, 0.f, 0.f);
}

cudaError_t build_index(const LsmDev &L, CtbBlock &B, cudaStream_t s) {
  const uint32_t F = (uint32_t)B.ctfs.size();
  std::vector<uint32_t> cbase(F + 1, 0);
  std::vector<uint4> ixg(F);
  std::vector<double2> ixs(F);
  std::vector<float4> ixf(2 * (size_t)F);
  unsigned long long total = 0;
  for (uint32_t c = 0; c < F; c++) {
    const stc_ctf &t = B.ctfs[c];
    const double want = std::sqrt((double)t.kv_count / LSM_INDEX_KEYS_PER_CELL);
    uint32_t g = LSM_INDEX_MIN_GRID, levels = 1, cells = 1;  // the wide slot
    while (g < LSM_INDEX_MAX_GRID && g < want) g *= 2;
    while ((1u << (levels - 1)) < g) levels++;  // down to one cell of the whole box
    for (uint32_t lv = 0; lv < levels; lv++) cells += index_level_side(g, lv) * index_level_side(g, lv);
    ixg[c] = make_uint4(g, levels, 0u, 0u);
    const double wx = (double)t.mbr[2] - (double)t.mbr[0], wy = (double)t.mbr[3] - (double)t.mbr[1];
    ixs[c] = make_double2(t.mbr[2] > t.mbr[0] && t.mbr[3] > t.mbr[1] ? (double)g / wx : 0.0,
                          t.mbr[2] > t.mbr[0] && t.mbr[3] > t.mbr[1] ? (double)g / wy : 0.0);
    ixf[2 * c] = index_file_coeffs(t, ixs[c].x, true);
    ixf[2 * c + 1] = index_file_coeffs(t, ixs[c].y, false);
    cbase[c + 1] = cbase[c] + cells;
    total = std::max<unsigned long long>(total, t.first_key + t.kv_count);
  }
  const uint32_t ncells = cbase[F];
  if (total > lsm_sort_words(L)) return cudaErrorInvalidValue;  // more keys than the sort scratch holds
  cudaError_t e = cudaMalloc(&B.perm, std::max<unsigned long long>(total, 1) * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&B.cstart, ((size_t)ncells + 1) * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&B.cbase, (F + 1) * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&B.ixg, std::max<size_t>(F, 1) * sizeof(uint4));
  if (e == cudaSuccess) e = cudaMalloc(&B.ixs, std::max<size_t>(F, 1) * sizeof(double2));
  if (e == cudaSuccess) e = cudaMalloc(&B.ixf, std::max<size_t>(2 * (size_t)F, 1) * sizeof(float4));
  if (e == cudaSuccess) e = cudaMemcpyAsync(B.ixs, ixs.data(), F * sizeof(double2), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B.ixf, ixf.data(), 2 * (size_t)F * sizeof(float4), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B.cbase, cbase.data(), (F + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B.ixg, ixg.data(), F * sizeof(uint4), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  if (e == cudaSuccess) e = cudaMalloc(&B.pend, std::max<unsigned long long>(total, 1) * sizeof(uint16_t));
  if (e != cudaSuccess) return e;
  uint32_t *const *sk = L.sk;
  uint32_t shift = 0;  // of the cell ids in the sorted keys (sk[2])
  if (total) {
    int bits = 1;
    while (bits < 32 && ((unsigned long long)ncells >> bits)) bits++;
    // keys by (cell, end offset)
    STC_KL k_set_one<<<1, 1, 0, s>>>(L.n_dev + 3, total);
    e = cudaMemsetAsync(L.n_dev + 4, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    STC_KL k_index_cells<<<num_sms() * 8, 256, 0, s>>>(B.keys, B.d_ctfs, F, B.cbase, B.ixg, B.ixs, B.ixf, total,
                                                         sk[0], sk[1], sk[6], L.n_dev + 4);  // tables copied above
    unsigned long long max_end = 65535;
    e = cudaMemcpyAsync(&max_end, L.n_dev + 4, sizeof(max_end), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    int eb = 1;
    while (eb < 16 && (max_end >> eb)) eb++;
    if (bits + eb <= 32) {
      // one sort of (cell << eb | end offset); the end offsets are the sorted keys' low bits
      STC_KL k_index_keys<<<num_sms() * 8, 256, 0, s>>>(sk[0], sk[6], (uint32_t)eb, total, sk[4]);
      radix_sort_u32(sk[4], sk[1], sk[2], B.perm, sk[0], sk[5], L.n_dev + 3, (size_t)total, bits + eb, L.hist,
                     L.scan, s);
      STC_KL k_index_ends<<<num_sms() * 8, 256, 0, s>>>(sk[2], (uint32_t)eb, total, B.pend);
      shift = (uint32_t)eb;
    } else {
      // stable sorts by end, then by cell
      radix_sort_u32(sk[6], sk[1], sk[2], sk[3], sk[4], sk[5], L.n_dev + 3, (size_t)total, 16, L.hist, L.scan, s);
      STC_KL k_gather_cells<<<num_sms() * 8, 256, 0, s>>>(sk[0], sk[3], sk[4], total);
      radix_sort_u32(sk[4], sk[3], sk[2], B.perm, sk[0], sk[5], L.n_dev + 3, (size_t)total, bits, L.hist, L.scan,
                     s);
      STC_KL k_gather_ends<<<num_sms() * 8, 256, 0, s>>>(sk[6], B.perm, B.pend, total);
    }
  }
  STC_KL k_cell_starts<<<num_sms() * 8, 256, 0, s>>>(sk[2], shift, total, ncells, B.cstart);
  e = cudaStreamSynchronize(s);  // the copies of cbase, ixg and ixs read this stack frame
  return e == cudaSuccess ? cudaGetLastError() : e;
}

stc_status lsm_store_block(const LsmDev &L, LsmHost &H, cudaStream_t s, std::string &err) {
  CtbBlock B;
  B.info = H.info;
  B.ctfs = H.ctfs;
  const size_t F = L.F, no = (size_t)H.info.oversize_kv_count;
  cudaError_t e = cudaMalloc(&B.keys, H.info.key_bytes + 32);
  if (e == cudaSuccess) e = cudaMalloc(&B.d_ctfs, F * sizeof(stc_ctf));
  if (e == cudaSuccess) e = cudaMalloc(&B.bitmaps, F * STC_BITMAP_BYTES);
  if (e == cudaSuccess) e = cudaMalloc(&B.sids, (size_t)L.N * sizeof(uint16_t));
  if (e == cudaSuccess) e = cudaMalloc(&B.orec, std::max<size_t>(no, 1) * sizeof(uint4));
  if (e == cudaSuccess) e = cudaMalloc(&B.obox, std::max<size_t>(no, 1) * sizeof(float4));
  if (e == cudaSuccess) e = cudaMalloc(&B.obitmap, STC_MAP_BITMAP_BYTES(L.edge));
  if (e == cudaSuccess) e = cudaMemsetAsync(B.keys + H.info.key_bytes, 0, 32, s);
  if (e == cudaSuccess && H.info.key_bytes)
    e = cudaMemcpyAsync(B.keys, L.kbytes, H.info.key_bytes, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B.d_ctfs, L.ctfs, F * sizeof(stc_ctf), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B.bitmaps, L.bitmaps, F * STC_BITMAP_BYTES, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B.sids, L.bsid, (size_t)L.N * 2, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && no)
    e = cudaMemcpyAsync(B.orec, L.brec + H.info.ctf_kv_count, no * sizeof(uint4), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && no)
    e = cudaMemcpyAsync(B.obox, L.bbox + H.info.ctf_kv_count, no * sizeof(float4), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(B.obitmap, L.obitmap, STC_MAP_BITMAP_BYTES(L.edge), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = build_index(L, B, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    free_block(B);
    err = std::string("keeping the flushed block for queries: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? STC_ERR_CAPACITY : STC_ERR_CUDA;
  }
  retain_block(H, std::move(B));
  return STC_OK;
}

static void retain_block(LsmHost &H, CtbBlock &&B) {
  std::unique_lock<std::shared_mutex> lock(H.blocks_mu);
  H.blocks.push_back(std::move(B));
  while (H.blocks.size() > H.retain) {
    free_block(H.blocks.front());
    H.blocks.pop_front();
  }
}

void lsm_release(LsmHost &H) {
  std::unique_lock<std::shared_mutex> lock(H.blocks_mu);
  for (CtbBlock &o : H.blocks) free_block(o);
  H.blocks.clear();
  for (QueryLane &Q : H.lanes) {
    std::lock_guard<std::mutex> ql(Q.mu);
    if (Q.stream) cudaStreamSynchronize(Q.stream);
    for (void *v : {(void *)Q.d_qb, (void *)Q.d_q, (void *)Q.d_out, (void *)Q.d_count, (void *)Q.d_qcounts,
                    (void *)Q.d_items, (void *)Q.d_iscan})
      if (v) cudaFree(v);
    for (void *v : {(void *)Q.h_qb, (void *)Q.h_q, (void *)Q.h_counts, (void *)Q.h_recs})
      if (v) cudaFreeHost(v);
    if (Q.stream) cudaStreamDestroy(Q.stream);
    if (Q.ev0) cudaEventDestroy(Q.ev0);
    if (Q.ev1) cudaEventDestroy(Q.ev1);
    Q.ev0 = Q.ev1 = nullptr;
    Q.d_qb = nullptr;
    Q.d_q = nullptr;
    Q.d_out = nullptr;
    Q.d_count = Q.d_qcounts = nullptr;
    Q.d_items = Q.d_iscan = nullptr;
    Q.h_qb = Q.m_qb = nullptr;
    Q.h_q = Q.m_q = nullptr;
    Q.h_counts = Q.m_counts = nullptr;
    Q.h_recs = Q.m_recs = nullptr;
    Q.stream = nullptr;
    Q.q_cap = Q.out_cap = Q.qc_cap = Q.items_cap = Q.iscan_cap = Q.hq_cap = Q.hrecs_cap = 0;
  }
}

// Device and pinned buffers of a batch of up to nq queries over H.retain
// blocks of up to F CTFs on lane Q. Allocations synchronise with the device
// (a step in flight), so they are made once, before any step runs; batches
// that need more grow them.
static cudaError_t query_buffers(const LsmHost &H, QueryLane &Q, size_t nq, uint32_t F) {
  cudaError_t e = cudaSuccess;
  const size_t nb = std::max<uint32_t>(H.retain, 1);
  if (!Q.d_qb) e = cudaMalloc(&Q.d_qb, nb * sizeof(QBlock));
  size_t cap_qb = Q.h_qb ? nb : 0;
  if (e == cudaSuccess) e = grow_mapped(&Q.h_qb, &Q.m_qb, &cap_qb, nb);
  if (e == cudaSuccess && !Q.d_count) e = cudaMalloc(&Q.d_count, sizeof(unsigned long long));
  if (e == cudaSuccess && Q.hq_cap < nq) {
    size_t cap_q = Q.hq_cap;
    e = grow_mapped(&Q.h_q, &Q.m_q, &Q.hq_cap, nq);
    if (e == cudaSuccess) e = grow_mapped(&Q.h_counts, &Q.m_counts, &cap_q, Q.hq_cap + 1);
  }
  if (e == cudaSuccess) e = grow(&Q.d_q, &Q.q_cap, nq);
  if (e == cudaSuccess) e = grow(&Q.d_qcounts, &Q.qc_cap, nq);
  if (e == cudaSuccess) e = grow(&Q.d_out, &Q.out_cap, std::max<size_t>(1 << 16, Q.out_cap));
  // size the plan for the retained-block limit, not today's count
  const size_t npairs = nq * nb * ((size_t)F + 1) + 1;
  if (e == cudaSuccess) e = grow(&Q.d_items, &Q.items_cap, npairs);
  if (e == cudaSuccess) e = grow(&Q.d_iscan, &Q.iscan_cap, scan_tmp_words(npairs));
  if (e == cudaSuccess) e = grow_mapped(&Q.h_recs, &Q.m_recs, &Q.hrecs_cap, 1 << 16);
  return e;
}

stc_status lsm_query_reserve(LsmHost &H, size_t nq, uint32_t F, int priority, std::string &err) {
  cudaError_t e = cudaSuccess;
  for (QueryLane &Q : H.lanes) {
    std::lock_guard<std::mutex> ql(Q.mu);
    if (e == cudaSuccess && !Q.stream) e = cudaStreamCreateWithPriority(&Q.stream, cudaStreamNonBlocking, priority);
    if (e == cudaSuccess && !Q.ev0) e = cudaEventCreate(&Q.ev0);
    if (e == cudaSuccess && !Q.ev1) e = cudaEventCreate(&Q.ev1);
    if (e == cudaSuccess) e = query_buffers(H, Q, nq, F);
  }
  // load the query kernels now: with lazy module loading their first launch
  // would load them then, which waits for a step in flight
  cudaFuncAttributes fa;
  for (const void *k : {(const void *)k_query_object, (const void *)k_box_plan, (const void *)k_box_rows,
                        (const void *)k_link_copy, (const void *)k_counts_out})
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k);
  if (e != cudaSuccess) {
    err = std::string("query buffers: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? STC_ERR_CAPACITY : STC_ERR_CUDA;
  }
  return STC_OK;
}

size_t lsm_query_chunk(const LsmHost &H) { return std::max<size_t>(1, 65535 / std::max<uint32_t>(H.retain, 1)); }

// The lane a batch runs on: `lane` when given, else the first lane no batch
// holds, else lane 0 once it frees.
static std::unique_lock<std::mutex> take_lane(LsmHost &H, int lane, QueryLane **out) {
  if (lane >= 0 && lane < QUERY_LANES) {
    *out = &H.lanes[lane];
    return std::unique_lock<std::mutex>(H.lanes[lane].mu);
  }
  for (QueryLane &Q : H.lanes) {
    std::unique_lock<std::mutex> l(Q.mu, std::try_to_lock);
    if (l.owns_lock()) {
      *out = &Q;
      return l;
    }
  }
  *out = &H.lanes[0];
  return std::unique_lock<std::mutex>(H.lanes[0].mu);
}

stc_status lsm_query(LsmHost &H, int lane, const stc_query *qs, size_t nq, stc_contact *out, size_t cap,
                     uint64_t *offsets, uint64_t *counts, std::string &err, size_t device_limit, float *gpu_ms) {
  QueryLane *Qp = nullptr;
  std::unique_lock<std::mutex> qlock = take_lane(H, lane, &Qp);
  QueryLane &Q = *Qp;
  std::shared_lock<std::shared_mutex> lock(H.blocks_mu);
  const uint32_t nb = (uint32_t)H.blocks.size();
  for (size_t i = 0; i <= nq; i++) offsets[i] = 0;
  if (counts)
    for (size_t i = 0; i < nq; i++) counts[i] = 0;
  if (nq == 0 || nb == 0) return STC_OK;
  if (nq * nb > 65535) {
    err = "query batch too large: queries x retained blocks must be <= 65535";
    return STC_ERR_INVALID_ARG;
  }
  cudaStream_t s = Q.stream;
  uint32_t maxF = 0;
  for (uint32_t i = 0; i < nb; i++) maxF = std::max(maxF, H.blocks[i].info.ctf_count);
  // box-query plan: one count per (query, block, CTF or oversize buffer), then their exclusive scan
  if (nq * nb * ((size_t)maxF + 1) + 1 > 0xFFFFFFFFull) {
    err = "query batch too large for the box-query plan";
    return STC_ERR_INVALID_ARG;
  }
  cudaError_t e = query_buffers(H, Q, nq, maxF);
  if (e != cudaSuccess) {
    err = std::string("query buffers: ") + cudaGetErrorString(e);
    return STC_ERR_CUDA;
  }
  QBlock *qb = Q.h_qb;
  for (uint32_t i = 0; i < nb; i++) {
    const CtbBlock &B = H.blocks[i];
    qb[i] = QBlock{B.keys, B.d_ctfs, B.sids, B.orec, B.obox, B.bitmaps, B.obitmap, B.perm, B.cstart, B.cbase, B.ixg,
                   B.ixs, B.pend,
                   (unsigned long long)B.info.oversize_kv_count, B.info.ctf_count, B.info.index,
                   B.info.o_end_time_min, B.info.bitmap_edge ? B.info.bitmap_edge : 256u};
  }
  bool has_obj = false, has_box = false;
  for (size_t i = 0; i < nq; i++) ((qs[i].kind & 0xFFu) == STC_QUERY_BOX ? has_box : has_obj) = true;
  memcpy(Q.h_q, qs, nq * sizeof(stc_query));
  if (gpu_ms) cudaEventRecord(Q.ev0, s);
  e = link_copy(Q.d_qb, Q.m_qb, nb * sizeof(QBlock), s);
  if (e == cudaSuccess) e = link_copy(Q.d_q, Q.m_q, nq * sizeof(stc_query), s);
  unsigned long long total = 0;
  bool over = false;  // more matches than device_limit: counted only
  for (int attempt = 0; attempt < 2 && e == cudaSuccess; attempt++) {
    e = cudaMemsetAsync(Q.d_count, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(Q.d_qcounts, 0, nq * sizeof(unsigned long long), s);
    if (e != cudaSuccess) break;
    if (has_obj)
      STC_KL k_query_object<<<dim3(nb, (unsigned)nq), QOBJ_THREADS, 0, s>>>(Q.d_qb, Q.d_q, Q.d_out, Q.out_cap,
                                                                           Q.d_count, Q.d_qcounts);
    if (has_box) {
      const uint32_t F1 = maxF + 1, P = (uint32_t)nq * nb * F1;
      STC_KL k_box_plan<<<(P + 255) / 256, 256, 0, s>>>(Q.d_qb, nb, Q.d_q, (uint32_t)nq, F1, H.map[0], H.map[1],
                                                        H.map[2], H.map[3], Q.d_items, Q.d_qcounts);
      exclusive_scan_u32(Q.d_items, Q.d_items, (size_t)P + 1, nullptr, Q.d_iscan, s);
      STC_KL k_box_rows<<<num_sms() * 16, QBOX_THREADS, 0, s>>>(Q.d_qb, nb, Q.d_q, (uint32_t)nq, F1, Q.d_items,
                                                                Q.d_out, Q.out_cap, Q.d_count, Q.d_qcounts);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) {
      k_counts_out<<<link_blocks(nq + 1), LINK_THREADS, 0, s>>>(Q.m_counts, Q.d_qcounts, nq, Q.d_count);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    total = Q.h_counts[nq];
    if (e == cudaSuccess && counts) memcpy(counts, Q.h_counts, nq * sizeof(unsigned long long));
    if (e != cudaSuccess || total <= Q.out_cap) break;
    if (device_limit && total > device_limit) {
      over = true;
      break;
    }
    e = grow(&Q.d_out, &Q.out_cap, (size_t)total);  // too many matches: once more with room for all
  }
  if (e != cudaSuccess) {
    err = std::string("query: ") + cudaGetErrorString(e);
    return STC_ERR_CUDA;
  }
  // the span up to the counts' read-back (the contacts' copy follows)
  if (gpu_ms) {
    cudaEventRecord(Q.ev1, s);
    cudaEventSynchronize(Q.ev1);
    *gpu_ms = 0.f;
    cudaEventElapsedTime(gpu_ms, Q.ev0, Q.ev1);
  }
  if (over) {
    for (size_t i = 0; i < nq; i++) offsets[i + 1] = offsets[i] + Q.h_counts[i];
    return STC_OK;
  }
  if (total) {
    e = grow_mapped(&Q.h_recs, &Q.m_recs, &Q.hrecs_cap, (size_t)total);
    if (e == cudaSuccess) e = link_copy(Q.m_recs, Q.d_out, total * sizeof(QueryRec), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      err = std::string("query read-back: ") + cudaGetErrorString(e);
      return STC_ERR_CUDA;
    }
  }
  // group by query (counting sort)
  const QueryRec *recs = Q.h_recs;
  for (unsigned long long i = 0; i < total; i++) offsets[recs[i].q + 1]++;
  for (size_t i = 0; i < nq; i++) offsets[i + 1] += offsets[i];
  if (total <= cap && out) {
    std::vector<uint64_t> pos(offsets, offsets + nq);
    for (unsigned long long i = 0; i < total; i++) out[pos[recs[i].q]++] = recs[i].c;
  }
  return STC_OK;
}


// ---- the reference's block files --------------------------------------------------
//
// straight_dump (tracing/process.cpp:254-348) writes a block as
//   <prefix>_SSTable_<ctb>-<ctf>  the packed keys of each CTF,
//   <prefix>_CTB<ctb>             the CTB object, sids, oversize keys (128-bit),
//                                 boxes (f_box) and map bitmap (workbench::dump_CTB_meta),
//   <prefix>_STcL<ctb>-<ctf>      the CTF object and its bitmap (CTF::dump_meta),
// with the objects written raw. Their byte layout on LP64 (little-endian):
//   CTF (80 B): ctf_mbr f32[4] @0, keys ptr @16, bitmap ptr @24, CTF_kv_capacity @32,
//     start_time_min/max @36/40, end_time_min/max @44/48, ctf_bitmap_size @52,
//     key_bit, id_bit, duration_bit, end_bit, low_x_bit, low_y_bit, edge_bit, mbr_bit,
//     x_grid, y_grid u16 @56..74 (tracing/step_merge.h:64-87);
//   CTB (128 B): ctfs ptr @0, CTF_count @8, start/end times @12..24, pointers @32..64,
//     o_buffer @72 { oversize_kv_count @+0, pointers @+8..+24, start_time_min/max @+32/36,
//     end_time_min/max @+40/44 }, box_rtree ptr @120 (step_merge.h:33-61, 111-131).
// Pointers and padding are written as 0 (the reference's loaders replace the
// pointers, workbench.cpp:639-694). straight_dump leaves CTF_count and the CTB's
// own times at 0; so does this writer. The reference spreads the key files over
// two RAID directories by CTF parity; here they all go to one directory.

namespace {

constexpr size_t REF_CTF_BYTES = 80, REF_CTB_BYTES = 128, REF_OBUF = 72;

inline void put32(uint8_t *b, size_t off, uint32_t v) { memcpy(b + off, &v, 4); }
inline void put16(uint8_t *b, size_t off, uint16_t v) { memcpy(b + off, &v, 2); }
inline uint32_t get32(const uint8_t *b, size_t off) { uint32_t v; memcpy(&v, b + off, 4); return v; }
inline uint16_t get16(const uint8_t *b, size_t off) { uint16_t v; memcpy(&v, b + off, 2); return v; }

// Bytes of a block's map bitmap.
size_t map_bitmap_bytes(const stc_ctb_info &in) { return STC_MAP_BITMAP_BYTES(in.bitmap_edge ? in.bitmap_edge : 256); }

std::string ctb_path(const std::string &dir, const std::string &prefix, const char *kind, uint32_t ctb, long ctf) {
  std::string p = dir + "/" + prefix + kind + std::to_string(ctb);
  if (ctf >= 0) p += "-" + std::to_string(ctf);
  return p;
}

bool write_file(const std::string &path, const void *a, size_t na, const void *b, size_t nb) {
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) return false;
  bool ok = (na == 0 || fwrite(a, 1, na, f) == na) && (nb == 0 || fwrite(b, 1, nb, f) == nb);
  return fclose(f) == 0 && ok;
}

bool read_file(const std::string &path, std::vector<uint8_t> &out) {
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) return false;
  out.clear();
  uint8_t buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + n);
  bool ok = !ferror(f);
  fclose(f);
  return ok;
}

void ctf_to_bytes(const stc_ctf &c, uint8_t *b) {
  memset(b, 0, REF_CTF_BYTES);
  memcpy(b, c.mbr, 16);
  put32(b, 32, c.kv_count);
  put32(b, 36, c.start_time_min);
  put32(b, 40, c.start_time_max);
  put32(b, 44, c.end_time_min);
  put32(b, 48, c.end_time_max);
  put32(b, 52, c.bitmap_bytes);
  const uint16_t f[10] = {c.key_bit, c.id_bit, c.duration_bit, c.end_bit, c.low_x_bit,
                          c.low_y_bit, c.edge_bit, c.mbr_bit, c.x_grid, c.y_grid};
  for (int i = 0; i < 10; i++) put16(b, 56 + 2 * i, f[i]);
}

void ctf_from_bytes(const uint8_t *b, stc_ctf &c) {
  memset(&c, 0, sizeof(c));
  memcpy(c.mbr, b, 16);
  c.kv_count = get32(b, 32);
  c.start_time_min = get32(b, 36);
  c.start_time_max = get32(b, 40);
  c.end_time_min = get32(b, 44);
  c.end_time_max = get32(b, 48);
  c.bitmap_bytes = get32(b, 52);
  uint16_t *f[10] = {&c.key_bit, &c.id_bit, &c.duration_bit, &c.end_bit, &c.low_x_bit,
                     &c.low_y_bit, &c.edge_bit, &c.mbr_bit, &c.x_grid, &c.y_grid};
  for (int i = 0; i < 10; i++) *f[i] = get16(b, 56 + 2 * i);
}

}  // namespace

stc_status lsm_write_block(LsmHost &H, uint32_t index, uint32_t N, const std::string &dir, const std::string &prefix,
                           std::string &err) {
  std::shared_lock<std::shared_mutex> lock(H.blocks_mu);
  const CtbBlock *B = nullptr;
  for (const CtbBlock &b : H.blocks)
    if (b.info.index == index) B = &b;
  if (!B) {
    err = "block " + std::to_string(index) + " is not retained";
    return STC_ERR_INVALID_ARG;
  }
  const stc_ctb_info &in = B->info;
  const uint32_t F = in.ctf_count;
  const size_t no = (size_t)in.oversize_kv_count;
  std::vector<uint8_t> keys(in.key_bytes), bitmaps((size_t)F * STC_BITMAP_BYTES), obitmap(map_bitmap_bytes(in));
  std::vector<uint16_t> sids(N);
  std::vector<uint4> orec(no);
  std::vector<float4> obox(no);
  cudaError_t e = cudaSuccess;
  if (in.key_bytes) e = cudaMemcpy(keys.data(), B->keys, in.key_bytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(bitmaps.data(), B->bitmaps, bitmaps.size(), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(sids.data(), B->sids, (size_t)N * 2, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && no) e = cudaMemcpy(orec.data(), B->orec, no * sizeof(uint4), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && no) e = cudaMemcpy(obox.data(), B->obox, no * sizeof(float4), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(obitmap.data(), B->obitmap, obitmap.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    err = std::string("reading the block: ") + cudaGetErrorString(e);
    return STC_ERR_CUDA;
  }
  for (uint32_t c = 0; c < F; c++) {
    const stc_ctf &t = B->ctfs[c];
    uint8_t hdr[REF_CTF_BYTES];
    ctf_to_bytes(t, hdr);
    const size_t kb = t.key_bit / 8u, nbytes = (size_t)t.kv_count * kb;
    std::string pm = ctb_path(dir, prefix, "_STcL", index, c), pk = ctb_path(dir, prefix, "_SSTable_", index, c);
    if (!write_file(pm, hdr, REF_CTF_BYTES, bitmaps.data() + (size_t)c * STC_BITMAP_BYTES, t.bitmap_bytes) ||
        !write_file(pk, keys.data() + t.key_offset, nbytes, nullptr, 0)) {
      err = "cannot write " + pm + " or " + pk;
      return STC_ERR_INVALID_ARG;
    }
  }
  std::vector<uint8_t> ctb(REF_CTB_BYTES + (size_t)N * 2 + no * 32 + obitmap.size(), 0);
  uint8_t *h = ctb.data();
  put32(h, REF_OBUF + 0, (uint32_t)no);
  put32(h, REF_OBUF + 32, in.o_start_time_min);
  put32(h, REF_OBUF + 36, in.o_start_time_max);
  put32(h, REF_OBUF + 40, in.o_end_time_min);
  put32(h, REF_OBUF + 44, in.o_end_time_max);
  size_t off = REF_CTB_BYTES;
  memcpy(h + off, sids.data(), (size_t)N * 2);
  off += (size_t)N * 2;
  for (size_t i = 0; i < no; i++) {  // 128-bit keys pid:26 | target:26 | duration:32 | end:32 (util/util.h:47-52)
    uint64_t lo = ((uint64_t)orec[i].z << 32) | orec[i].w, hi = ((uint64_t)orec[i].x << 26) | orec[i].y;
    memcpy(h + off + 16 * i, &lo, 8);
    memcpy(h + off + 16 * i + 8, &hi, 8);
  }
  off += no * 16;
  memcpy(h + off, obox.data(), no * 16);
  off += no * 16;
  memcpy(h + off, obitmap.data(), obitmap.size());
  std::string pc = ctb_path(dir, prefix, "_CTB", index, -1);
  if (!write_file(pc, ctb.data(), ctb.size(), nullptr, 0)) {
    err = "cannot write " + pc;
    return STC_ERR_INVALID_ARG;
  }
  return STC_OK;
}

stc_status lsm_block_info(LsmHost &H, uint32_t index, stc_ctb_info *info, std::string &err) {
  std::shared_lock<std::shared_mutex> lock(H.blocks_mu);
  for (const CtbBlock &b : H.blocks)
    if (b.info.index == index) {
      *info = b.info;
      return STC_OK;
    }
  err = "block " + std::to_string(index) + " is not retained";
  return STC_ERR_INVALID_ARG;
}

stc_status lsm_read_block(LsmHost &H, uint32_t index, uint32_t N, stc_ctf *ctfs, uint8_t *bitmaps, uint8_t *keys,
                          uint16_t *sids, uint64_t *okeys, float *oboxes, uint8_t *obitmap, std::string &err) {
  std::shared_lock<std::shared_mutex> lock(H.blocks_mu);
  const CtbBlock *B = nullptr;
  for (const CtbBlock &b : H.blocks)
    if (b.info.index == index) B = &b;
  if (!B) {
    err = "block " + std::to_string(index) + " is not retained";
    return STC_ERR_INVALID_ARG;
  }
  const stc_ctb_info &in = B->info;
  const size_t no = (size_t)in.oversize_kv_count;
  if (ctfs) memcpy(ctfs, B->ctfs.data(), B->ctfs.size() * sizeof(stc_ctf));
  cudaError_t e = cudaSuccess;
  if (bitmaps) e = cudaMemcpy(bitmaps, B->bitmaps, (size_t)in.ctf_count * STC_BITMAP_BYTES, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && keys && in.key_bytes) e = cudaMemcpy(keys, B->keys, in.key_bytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && sids) e = cudaMemcpy(sids, B->sids, (size_t)N * 2, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && obitmap) e = cudaMemcpy(obitmap, B->obitmap, map_bitmap_bytes(in), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && oboxes && no) e = cudaMemcpy(oboxes, B->obox, no * sizeof(float4), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && okeys && no) {
    std::vector<uint4> orec(no);
    e = cudaMemcpy(orec.data(), B->orec, no * sizeof(uint4), cudaMemcpyDeviceToHost);
    for (size_t i = 0; e == cudaSuccess && i < no; i++) {
      okeys[2 * i] = ((uint64_t)orec[i].z << 32) | orec[i].w;
      okeys[2 * i + 1] = ((uint64_t)orec[i].x << 26) | orec[i].y;
    }
  }
  if (e != cudaSuccess) {
    err = std::string("reading the block: ") + cudaGetErrorString(e);
    return STC_ERR_CUDA;
  }
  return STC_OK;
}

stc_status lsm_load_block(const LsmDev &L, LsmHost &H, uint32_t index, const std::string &dir,
                          const std::string &prefix, cudaStream_t s, std::string &err) {
  const uint32_t N = L.N;
  // the block's CTFs: the consecutive CTF meta files from CTF 0
  uint32_t F = 0;
  while (F < 3969u) {
    FILE *f = fopen(ctb_path(dir, prefix, "_STcL", index, F).c_str(), "rb");
    if (!f) break;
    fclose(f);
    F++;
  }
  if (F == 0) {
    err = "no CTF files " + ctb_path(dir, prefix, "_STcL", index, 0);
    return STC_ERR_INVALID_ARG;
  }
  std::vector<uint8_t> ctb;
  std::string pc = ctb_path(dir, prefix, "_CTB", index, -1);
  if (!read_file(pc, ctb) || ctb.size() < REF_CTB_BYTES) {
    err = "cannot read " + pc;
    return STC_ERR_INVALID_ARG;
  }
  const size_t no = get32(ctb.data(), REF_OBUF);
  const size_t obm_bytes = STC_MAP_BITMAP_BYTES(H.edge);  // the file does not record the edge
  if (ctb.size() != REF_CTB_BYTES + (size_t)N * 2 + no * 32 + obm_bytes) {
    err = pc + ": size does not match " + std::to_string(N) + " objects, " + std::to_string(no) +
          " oversize keys and a map bitmap of edge " + std::to_string(H.edge);
    return STC_ERR_INVALID_ARG;
  }
  CtbBlock B;
  B.ctfs.resize(F);
  std::vector<uint8_t> keys, bitmaps((size_t)F * STC_BITMAP_BYTES, 0), meta, part;
  unsigned long long first = 0;
  for (uint32_t c = 0; c < F; c++) {
    std::string pm = ctb_path(dir, prefix, "_STcL", index, c), pk = ctb_path(dir, prefix, "_SSTable_", index, c);
    if (!read_file(pm, meta) || meta.size() < REF_CTF_BYTES) {
      err = "cannot read " + pm;
      return STC_ERR_INVALID_ARG;
    }
    stc_ctf &t = B.ctfs[c];
    ctf_from_bytes(meta.data(), t);
    if (t.key_bit % 8 || t.key_bit > 128 || t.bitmap_bytes > STC_BITMAP_BYTES ||
        meta.size() != REF_CTF_BYTES + t.bitmap_bytes) {
      err = pm + ": not a CTF meta file of this layout";
      return STC_ERR_INVALID_ARG;
    }
    memcpy(bitmaps.data() + (size_t)c * STC_BITMAP_BYTES, meta.data() + REF_CTF_BYTES, t.bitmap_bytes);
    if (!read_file(pk, part) || part.size() != (size_t)t.kv_count * (t.key_bit / 8u)) {
      err = "cannot read " + std::to_string((size_t)t.kv_count * (t.key_bit / 8u)) + " key bytes from " + pk;
      return STC_ERR_INVALID_ARG;
    }
    t.first_key = first;
    t.key_offset = keys.size();
    first += t.kv_count;
    keys.insert(keys.end(), part.begin(), part.end());
  }
  if (first > lsm_sort_words(L)) {
    err = "the block holds " + std::to_string(first) + " CTF keys, more than this context's sort scratch (" +
          std::to_string(lsm_sort_words(L)) + "); raise kv_capacity";
    return STC_ERR_CAPACITY;
  }
  const uint8_t *h = ctb.data();
  std::vector<uint16_t> sids(N);
  memcpy(sids.data(), h + REF_CTB_BYTES, (size_t)N * 2);
  std::vector<uint4> orec(no);
  std::vector<float4> obox(no);
  const uint8_t *ok = h + REF_CTB_BYTES + (size_t)N * 2;
  for (size_t i = 0; i < no; i++) {
    uint64_t lo, hi;
    memcpy(&lo, ok + 16 * i, 8);
    memcpy(&hi, ok + 16 * i + 8, 8);
    orec[i] = make_uint4((uint32_t)(hi >> 26) & ((1u << 26) - 1), (uint32_t)hi & ((1u << 26) - 1),
                         (uint32_t)(lo >> 32), (uint32_t)lo);
  }
  memcpy(obox.data(), ok + no * 16, no * 16);
  const uint8_t *obm = ok + no * 32;
  stc_ctb_info &in = B.info;
  in.index = index;
  in.ctf_count = F;
  in.flush_time = F ? B.ctfs[0].end_time_max : 0;
  in.end_time_min = F ? B.ctfs[0].end_time_min : 0;
  in.ctf_kv_count = first;
  in.oversize_kv_count = no;
  in.kv_count = first + no;
  in.key_bytes = keys.size();
  for (uint16_t v : sids) in.sid_count += v != 0;
  in.o_start_time_min = get32(h, REF_OBUF + 32);
  in.o_start_time_max = get32(h, REF_OBUF + 36);
  in.o_end_time_min = get32(h, REF_OBUF + 40);
  in.o_end_time_max = get32(h, REF_OBUF + 44);
  in.bitmap_edge = H.edge;
  cudaError_t e = cudaMalloc(&B.keys, keys.size() + 32);
  if (e == cudaSuccess) e = cudaMalloc(&B.d_ctfs, F * sizeof(stc_ctf));
  if (e == cudaSuccess) e = cudaMalloc(&B.bitmaps, bitmaps.size());
  if (e == cudaSuccess) e = cudaMalloc(&B.sids, (size_t)N * 2);
  if (e == cudaSuccess) e = cudaMalloc(&B.orec, std::max<size_t>(no, 1) * sizeof(uint4));
  if (e == cudaSuccess) e = cudaMalloc(&B.obox, std::max<size_t>(no, 1) * sizeof(float4));
  if (e == cudaSuccess) e = cudaMalloc(&B.obitmap, obm_bytes);
  if (e == cudaSuccess) e = cudaMemsetAsync(B.keys + keys.size(), 0, 32, s);
  if (e == cudaSuccess && !keys.empty()) e = cudaMemcpyAsync(B.keys, keys.data(), keys.size(), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B.d_ctfs, B.ctfs.data(), F * sizeof(stc_ctf), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B.bitmaps, bitmaps.data(), bitmaps.size(), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B.sids, sids.data(), (size_t)N * 2, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && no) e = cudaMemcpyAsync(B.orec, orec.data(), no * sizeof(uint4), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && no) e = cudaMemcpyAsync(B.obox, obox.data(), no * sizeof(float4), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B.obitmap, obm, obm_bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = build_index(L, B, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    free_block(B);
    err = std::string("loading the block: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? STC_ERR_CAPACITY : STC_ERR_CUDA;
  }
  retain_block(H, std::move(B));
  H.next_index = std::max(H.next_index, index + 1);
  return STC_OK;
}

}  // namespace stc
