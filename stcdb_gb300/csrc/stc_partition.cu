// Step kernels (a): quadtree partitioning of one step's positions.
//
//   k_descend   phased descent of every point to its leaf, tracking the
//               deepest ancestor whose box keeps the point away from its top
//               and right border (tracing/filter.cpp:228-243); leaf histogram
//   sort        stable radix sort of pids by leaf id: leaf member lists in pid
//               order, exactly the order the reference's single-threaded
//               insert fills grids[] (tracing/filter.cpp:95-111)
//   k_gather    leaf-ordered copy of the points as fp32 offsets from the leaf
//               corner (for the refinement pre-filter) and fp32 lon/lat (MBR)
//   k_strip_order  each leaf's kept members again in strip order (strips at
//               least reach tall), the refinement's candidate ranges
//   k_border    depth-first lookup of the top/right leaves within reach of a
//               border point (tracing/filter.cpp:130-152), counted then filled
//               in the reference's unit order (pid, then DFS order)
//   k_jobs      per-leaf refinement jobs (32 rows x one chunk of candidates)
#include "stc_pipeline.cuh"

namespace stc {

static inline unsigned nblk(size_t n, unsigned t = 256) { return (unsigned)((n + t - 1) / t); }

__device__ __forceinline__ double dpml_fast_d(double lat) {
  double absla = fabs(lat);
  if (absla == 90) absla = 89;
  double arg = RN_DIV(RN_MUL(RN_SUB(90.0, absla), STC_REF_PI), 180.0);
  return RN_DIV(360.0, RN_MUL(RN_MUL(sin(arg), 40076.0), 1000.0));
}

__global__ void k_descend(PipeDev p) {
  uint32_t pid = blockIdx.x * blockDim.x + threadIdx.x;
  if (pid >= p.N) return;
  double2 q;
  if (p.xy_in) {
    q = p.xy_in[pid];
    const_cast<double2 *>(p.xy)[pid] = q;
  } else {
    q = p.xy[pid];
  }
  uint32_t cur = 0, lv = 0;
  NodeMeta m = p.sd.meta[0];
  if (m.type != NODE_LEAF) {
    int d = 0;
    for (; d < STC_MAX_DEPTH; d++) {
      const Node *n = &p.sd.nodes[cur];
      int child = (q.y > n->mid_y) * 2 + (q.x > n->mid_x);
      cur = n->child[child];
      m = p.sd.meta[cur];
      if (m.type == NODE_INVALID) {
        stc_set_error(p.st, ERR_DESCENT, pid);
        return;
      }
      const Node *c = &p.sd.nodes[cur];
      if (RN_ADD(q.x, p.x_buffer) < c->hi_x && RN_ADD(q.y, p.y_buffer) < c->hi_y) lv = cur;
      if (m.type == NODE_LEAF) break;
    }
    if (d == STC_MAX_DEPTH) {
      stc_set_error(p.st, ERR_DESCENT, pid);
      return;
    }
  }
  p.leaf_gid[pid] = m.grid_id;
  p.lastvalid[pid] = lv != cur ? lv : STC_NONE;
  atomicAdd(&p.grid_count[m.grid_id], 1u);
  if (lv != cur) p.blist[agg_inc(&p.st->border_points)] = pid;
}

__global__ void k_gather(PipeDev p) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.N) return;
  uint32_t pid = p.sorted_pid[i];
  uint32_t g = p.sorted_gid[i];
  const Node *o = &p.sd.nodes[p.sd.gid_node[g]];
  double2 q = p.xy[pid];
  float lx = __double2float_rn(RN_SUB(q.x, o->lo_x));
  float ly = __double2float_rn(RN_SUB(q.y, o->lo_y));
  float2 f = make_float2(__double2float_rn(q.x), __double2float_rn(q.y));
  p.pts[i] = make_float4(lx, ly, metres_per_deg_lon_f(q.y), __uint_as_float(pid));
  p.gfxy[i] = f;
  p.fxy[pid] = f;
}

// Strip order of each leaf's kept members, for the refinement's candidate
// ranges. The leaf is cut into H horizontal strips (H <= STRIPS_MAX) at
// least s_min metres tall, s_min a little above reach. The reference's
// distance takes dy / dpm_lat, a constant scale, so two members within reach
// lie at most one strip apart. Within a strip of at most XSORT_MAX members
// the members are ordered by longitude offset; |dx| * (metres per degree at
// the first point's latitude) <= reach bounds |dx| by wx degrees, wx taken at
// the leaf's smallest scale, so the partners of a member in an ordered strip
// form one window of it, found by binary search. A larger strip (dense
// hotspot leaves at the minimum width, where most pairs are within reach
// anyway) keeps its members unordered and is taken whole.
// Candidates of member i (own rows): the members after it in its strip up
// to its window's end, and its window in the next strip; every pair at most
// a strip apart and within wx is thereby tested once, by its member earlier
// in (strip, longitude) order. Strip and window bounds are computed in fp32
// from the members' leaf offsets; s_min and wx cover their rounding (u times
// the leaf extent) and the scale's with wide margins (2e-4 relative plus 1e-6
// of the leaf extent plus 1-2 mm).
// One warp per leaf: a counting sort by strip in shared memory, then a rank
// sort by longitude of each small strip with shuffles (the order within a
// strip only decides which member of a pair tests it; each hit's priority
// comes from the pid-order index).
static constexpr uint32_t STRIPS_MAX = 64;
static constexpr uint32_t XSORT_MAX = 128;

__device__ __forceinline__ uint32_t member_strip(float ly, float inv, uint32_t H) {
  float c = floorf(ly * inv);
  c = fminf(fmaxf(c, 0.0f), (float)(H - 1));
  return (uint32_t)c;
}

// First index in [lo, hi) of a longitude-ordered strip whose offset is
// greater than x (upper = true) or not below x (upper = false).
__device__ __forceinline__ uint32_t x_bound(const float4 *pts, uint32_t lo, uint32_t hi, float x, bool upper) {
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    const float v = pts[mid].x;
    if (upper ? v <= x : v < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(256) k_strip_order(PipeDev p) {
  __shared__ uint32_t hist_all[8][STRIPS_MAX + 1];
  const uint32_t lane = lane_id(), wid = threadIdx.x >> 5;
  uint32_t *hist = hist_all[wid];
  uint32_t *tmp = p.sort_ktmp;  // (strip << 16 | rank within strip) per member in pid order
  const uint32_t nw = gridDim.x * 8;
  for (uint32_t g = blockIdx.x * 8 + wid; g < p.G; g += nw) {
    const uint32_t cnt = p.grid_count[g];
    const uint32_t n = cnt < p.leaf_cap ? cnt : p.leaf_cap;
    if (n == 0) continue;
    const uint32_t base = p.grid_start[g];
    const Node *o = &p.sd.nodes[p.sd.gid_node[g]];
    const double h_deg = RN_SUB(o->hi_y, o->lo_y), w_deg = RN_SUB(o->hi_x, o->lo_x);
    const float h_m = (float)h_deg * STC_SLAT_F, w_m = (float)w_deg * STC_SMAX_F;
    const float s_min = (float)p.reach * 1.0001f + 1e-6f * h_m + 1e-3f;
    float hf = floorf(h_m / s_min);
    const uint32_t H = hf < 1.0f ? 1u : (hf > (float)STRIPS_MAX ? STRIPS_MAX : (uint32_t)hf);
    const float inv = H > 1 ? (float)H / (float)h_deg : 0.0f;  // strips per degree from the low edge
    // smallest metres per degree of longitude of any first point of a pair
    // (the leaf's latitudes, widened by 1e-3 degrees for border points)
    const double lat = fmax(fabs(o->lo_y), fabs(o->hi_y)) + 1e-3;
    const float s_lon = metres_per_deg_lon_f(lat < 89.0 ? lat : 89.0) * (1.0f - 1e-5f);
    const float wx = ((float)p.reach * 1.0002f + 1e-6f * (w_m + h_m) + 2e-3f) / s_lon;
    for (uint32_t k = lane; k <= STRIPS_MAX; k += 32) hist[k] = 0;
    __syncwarp();
    for (uint32_t i = lane; i < n; i += 32) {
      const uint32_t sidx = member_strip(p.pts[base + i].y, inv, H);
      tmp[base + i] = sidx << 16 | atomicAdd(&hist[sidx], 1u);
    }
    __syncwarp();
    // exclusive scan of the H <= 64 strip counts, two per lane
    const uint32_t v0 = hist[2 * lane], v1 = hist[2 * lane + 1];
    uint32_t x = v0 + v1;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
      if ((int)lane >= d) x += y;
    }
    x -= v0 + v1;
    __syncwarp();
    hist[2 * lane] = x;
    hist[2 * lane + 1] = x + v0;
    __syncwarp();
    if (lane == 0) hist[H] = n;
    __syncwarp();
    for (uint32_t i = lane; i < n; i += 32) {
      const uint32_t u = tmp[base + i], sidx = u >> 16;
      const uint32_t k = hist[sidx] + (u & 0xFFFFu);
      p.spts[base + k] = p.pts[base + i];
      p.sfxy[base + k] = p.gfxy[base + i];
      p.sorig[base + k] = i | sidx << 16;
    }
    __syncwarp();
    // small strips in longitude order: each member's rank among the strip's
    // (offset, position) pairs, its elements in four slots of 32 lanes
    for (uint32_t sidx = 0; sidx < H; sidx++) {
      const uint32_t st = hist[sidx], L = hist[sidx + 1] - st;
      if (L > XSORT_MAX || L < 2) continue;  // one member: in order already
      if (L <= 32) {
        // one member per lane (most strips)
        const float4 v = lane < L ? p.spts[base + st + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float2 f = lane < L ? p.sfxy[base + st + lane] : make_float2(0.f, 0.f);
        const uint32_t og = lane < L ? p.sorig[base + st + lane] : 0u;
        uint32_t rk = 0;
        for (uint32_t b = 0; b < L; b++) {
          const float xb = __shfl_sync(0xffffffffu, v.x, b);
          rk += (xb < v.x || (xb == v.x && b < lane)) ? 1u : 0u;
        }
        __syncwarp();
        if (lane < L) {
          p.spts[base + st + rk] = v;
          p.sfxy[base + st + rk] = f;
          p.sorig[base + st + rk] = og | STRIP_XSORTED;
        }
        __syncwarp();
        continue;
      }
      const uint32_t slots = (L + 31) / 32;
      float4 v[4];
      float2 f[4];
      uint32_t og[4], rk[4] = {0, 0, 0, 0};
#pragma unroll
      for (int m = 0; m < 4; m++) {
        const uint32_t e = lane + 32u * m;
        v[m] = e < L ? p.spts[base + st + e] : make_float4(0.f, 0.f, 0.f, 0.f);
        f[m] = e < L ? p.sfxy[base + st + e] : make_float2(0.f, 0.f);
        og[m] = e < L ? p.sorig[base + st + e] : 0u;
      }
#pragma unroll
      for (int m2 = 0; m2 < 4; m2++) {
        if ((uint32_t)m2 >= slots) break;
        for (uint32_t src = 0; src < 32; src++) {
          const float xb = __shfl_sync(0xffffffffu, v[m2].x, src);
          const uint32_t b = src + 32u * m2;
          if (b >= L) break;
#pragma unroll
          for (int m = 0; m < 4; m++) {
            const uint32_t a = lane + 32u * m;
            rk[m] += (xb < v[m].x || (xb == v[m].x && b < a)) ? 1u : 0u;
          }
        }
      }
      __syncwarp();
#pragma unroll
      for (int m = 0; m < 4; m++) {
        const uint32_t e = lane + 32u * m;
        if (e < L) {
          p.spts[base + st + rk[m]] = v[m];
          p.sfxy[base + st + rk[m]] = f[m];
          p.sorig[base + st + rk[m]] = og[m] | STRIP_XSORTED;
        }
      }
      __syncwarp();
    }
    // candidate ranges of every member (positions within the leaf); the
    // longest range of any 32-member row block sets the leaf's candidate
    // chunks per row block (k_jobs)
    const float4 *lp = p.spts + base;
    uint32_t longest = 0;
    for (uint32_t i0 = 0; i0 < n; i0 += 32) {
      const uint32_t i = i0 + lane;
      uint32_t len = 0;
      if (i < n) {
        const uint32_t sidx = (p.sorig[base + i] >> 16) & 63u;
        const float xi = lp[i].x;
        const uint32_t en = hist[sidx + 1];
        const bool xs = en - hist[sidx] <= XSORT_MAX;
        const uint32_t e1 = xs ? x_bound(lp, i + 1, en, xi + wx, true) : en;
        uint32_t a2 = 0, b2 = 0;
        if (sidx + 1 < H) {
          const uint32_t st2 = hist[sidx + 1], en2 = hist[sidx + 2];
          if (en2 - st2 <= XSORT_MAX) {
            a2 = x_bound(lp, st2, en2, xi - wx, false);
            b2 = x_bound(lp, a2, en2, xi + wx, true);
          } else {
            a2 = st2;
            b2 = en2;
          }
        }
        p.scand[base + i] = make_uint2(e1 | a2 << 16, b2);
        len = (e1 - (i + 1)) + (b2 - a2);
      }
      longest = max(longest, __reduce_max_sync(0xffffffffu, len));
    }
    if (lane == 0) p.cchunks[g] = max(1u, (longest + p.refine_chunk - 1) / p.refine_chunk);
    if (lane == 0) p.lstrip[g] = make_float4(inv, (float)H, wx, 0.0f);
    __syncwarp();
  }
}

// box::distance(p, geography=true) <= reach (geometry/geometry.h:174-185),
// decided exactly: fp64 containment and degree offsets as in the reference,
// then the metric step in fp32 with a +-64 u relative band (u = 2^-24), then
// the reference's fp64 division and square root, and within 1e-12 of reach
// the correctly rounded sine.
__device__ bool box_within_exact(const Node &c, double x, double y, double reach, float reach_f, float s_lon,
                                 double &dp_fast) {
  if (x >= c.lo_x && x <= c.hi_x && y >= c.lo_y && y <= c.hi_y) return true;  // distance 0
  double dx = RN_SUB(fabs(RN_SUB(x, RN_MUL(RN_ADD(c.lo_x, c.hi_x), 0.5))), RN_MUL(RN_SUB(c.hi_x, c.lo_x), 0.5));
  double dy = RN_SUB(fabs(RN_SUB(y, RN_MUL(RN_ADD(c.lo_y, c.hi_y), 0.5))), RN_MUL(RN_SUB(c.hi_y, c.lo_y), 0.5));
  if (dx < 0.0) dx = 0.0;
  if (dy < 0.0) dy = 0.0;
  float fx = __double2float_rn(dx) * s_lon, fy = __double2float_rn(dy) * STC_SLAT_F;
  float d2 = fx * fx + fy * fy;
  const float lo = reach_f * (1.0f - 64.0f * 5.9604645e-08f), hi = reach_f * (1.0f + 64.0f * 5.9604645e-08f);
  if (d2 <= lo * lo) return true;
  if (d2 >= hi * hi) return false;
  if (dp_fast == 0.0) dp_fast = dpml_fast_d(y);
  double d = stc_box_distance_ref(c.lo_x, c.lo_y, c.hi_x, c.hi_y, x, y, dp_fast);
  if (fabs(d - reach) > 1e-12 * reach) return d <= reach;
  return stc_box_distance_ref(c.lo_x, c.lo_y, c.hi_x, c.hi_y, x, y, stc_dpml_ref(y)) <= reach;
}

// Lookup of one border point (tracing/filter.cpp:130-152): depth-first from
// last_valid over children 0..3, collecting the leaves within reach that lie
// above the point or to its right. Node distances are first classified in
// fp32 from map-relative float boxes; the band of width border_delta around
// reach (bounding the fp32 rounding of the offsets, see stc_create) goes to
// box_within_exact. Writes the first `keep` leaf ids to out; returns the
// count, or 0xFFFFFFFF on stack overflow.
#define LOOKUP_STACK 64
__device__ uint32_t border_lookup(const PipeDev &p, uint32_t pid, uint32_t lv, uint32_t *out, uint32_t keep) {
  double2 q = p.xy[pid];
  float px = __double2float_rn(RN_SUB(q.x, p.sd.ox)), py = __double2float_rn(RN_SUB(q.y, p.sd.oy));
  float s_lon = metres_per_deg_lon_f(q.y);
  float reach_f = (float)p.reach;
  float rlo = fmaxf(reach_f - p.border_delta, 0.0f), rhi = reach_f + p.border_delta;
  float rlo2 = rlo * rlo, rhi2 = rhi * rhi;
  // the fp32 band only covers points inside the map box (offsets bounded by its extent)
  bool fast_ok = q.x >= p.map_lo_x && q.x <= p.map_hi_x && q.y >= p.map_lo_y && q.y <= p.map_hi_y;
  double dpf = 0.0;
  uint32_t stk[LOOKUP_STACK];
  uint8_t nxt[LOOKUP_STACK];
  int sp = 1;
  stk[0] = lv;
  nxt[0] = 0;
  uint32_t cnt = 0;
  while (sp > 0) {
    int i = nxt[sp - 1];
    if (i == 4) {
      sp--;
      continue;
    }
    nxt[sp - 1] = (uint8_t)(i + 1);
    uint32_t ch = p.sd.nodes[stk[sp - 1]].child[i];
    int decided = 0;  // 1 within, -1 outside, 0 undecided
    if (fast_ok) {
      float4 fb = p.sd.fbox[ch];
      float cx = (fb.x + fb.z) * 0.5f, hwx = (fb.z - fb.x) * 0.5f;
      float cy = (fb.y + fb.w) * 0.5f, hwy = (fb.w - fb.y) * 0.5f;
      float dx = fmaxf(fabsf(px - cx) - hwx, 0.0f) * s_lon;
      float dy = fmaxf(fabsf(py - cy) - hwy, 0.0f) * STC_SLAT_F;
      float d2 = dx * dx + dy * dy;
      decided = d2 <= rlo2 ? 1 : (d2 >= rhi2 ? -1 : 0);
    }
    if (decided < 0) continue;
    NodeMeta cm = p.sd.meta[ch];
    if (cm.type == NODE_LEAF) {
      // leaf test needs the exact box; fetch it only for leaves
      Node c = p.sd.nodes[ch];
      if (decided == 0 && !box_within_exact(c, q.x, q.y, p.reach, reach_f, s_lon, dpf)) continue;
      // the leaf lies above, or to the right within the point's row
      if (q.y < c.lo_y || (q.y < c.hi_y && q.x < c.lo_x)) {
        if (cnt < keep) out[cnt] = cm.grid_id;
        cnt++;
      }
    } else {
      if (decided == 0) {
        Node c = p.sd.nodes[ch];
        if (!box_within_exact(c, q.x, q.y, p.reach, reach_f, s_lon, dpf)) continue;
      }
      if (sp == LOOKUP_STACK) return 0xFFFFFFFFu;
      stk[sp] = ch;
      nxt[sp] = 0;
      sp++;
    }
  }
  return cnt;
}

#define BORDER_KEEP 4

__global__ void k_border_count(PipeDev p) {
  const unsigned long long nb = p.st->border_points;
  for (unsigned long long b = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; b < nb;
       b += (unsigned long long)gridDim.x * blockDim.x) {
    uint32_t pid = p.blist[b];
    uint32_t c = border_lookup(p, pid, p.lastvalid[pid], p.bres + BORDER_KEEP * b, BORDER_KEEP);
    if (c == 0xFFFFFFFFu) {
      stc_set_error(p.st, ERR_LOOKUP, pid);
      c = 0;
    }
    p.bcount[pid] = c;
  }
}

__global__ void k_border_fill(PipeDev p) {
  const unsigned long long nb = p.st->border_points;
  for (unsigned long long b = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; b < nb;
       b += (unsigned long long)gridDim.x * blockDim.x) {
    uint32_t pid = p.blist[b];
    uint32_t c = p.bcount[pid];
    unsigned long long base = p.boff[pid];
    if (base + c > p.U_cap) continue;  // reported by k_check_units
    const uint32_t *src = p.bres + BORDER_KEEP * b;
    if (c > BORDER_KEEP) {
      // rare: more leaves than kept by the counting pass; walk again into place
      border_lookup(p, pid, p.lastvalid[pid], p.bu_gid + base, c);
      src = p.bu_gid + base;
    }
    for (uint32_t k = 0; k < c; k++) {
      uint32_t gid = src[k];
      p.bu_gid[base + k] = gid;
      p.bu_pid[base + k] = pid;
      atomicAdd(&p.bu_cnt[gid], 1u);
    }
  }
}

__global__ void k_check_units(PipeDev p) {
  if (p.st->border_units >= p.U_cap) stc_set_error(p.st, ERR_UNITS, (uint32_t)p.st->border_units);
}

__global__ void k_jobs(PipeDev p) {
  uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g > p.G) return;
  if (g == p.G) {
    p.job_cnt[g] = 0;
    return;
  }
  uint32_t cnt = p.grid_count[g];
  uint32_t n = cnt < p.leaf_cap ? cnt : p.leaf_cap;
  if (cnt > p.leaf_cap) atomicAdd(&p.st->overflow_objects, cnt - p.leaf_cap);
  uint32_t m = p.bu_cnt[g];
  // one job: 32 members (strip order) or 32 border units against one chunk
  // of refine_chunk positions of their candidate ranges (a border unit's
  // ranges hold at most n members)
  uint32_t jobs = n ? (n + 31) / 32 * p.cchunks[g] + (m + 31) / 32 * ((n + p.refine_chunk - 1) / p.refine_chunk) : 0;
  p.job_cnt[g] = jobs;
}

void step_descend(PipeDev &p, cudaStream_t s) {
  cudaMemsetAsync(p.grid_count, 0, (size_t)(p.G + 1) * sizeof(uint32_t), s);
  cudaMemsetAsync(p.bcount, 0, (size_t)p.N * sizeof(uint32_t), s);
  STC_KL k_descend<<<nblk(p.N), 256, 0, s>>>(p);
}

void step_leaf_order(PipeDev &p, cudaStream_t s) {
  int bits = 1;
  while ((1u << bits) < p.G && bits < 32) bits++;
  radix_sort_u32(p.leaf_gid, p.iota, p.sorted_gid, p.sorted_pid, p.sort_ktmp, p.sort_vtmp, p.n_dev, p.N, bits,
                 p.sort_hist, p.scan_tmp, s);
  exclusive_scan_u32(p.grid_count, p.grid_start, (size_t)p.G + 1, nullptr, p.scan_tmp, s);
  STC_KL k_gather<<<nblk(p.N), 256, 0, s>>>(p);
}

void step_strips(PipeDev &p, cudaStream_t s) {
  STC_KL k_strip_order<<<num_sms() * 8, 256, 0, s>>>(p);
}

void step_border(PipeDev &p, cudaStream_t s) {
  cudaMemsetAsync(p.bu_cnt, 0, (size_t)(p.G + 1) * sizeof(uint32_t), s);
  STC_KL k_border_count<<<num_sms() * 16, 128, 0, s>>>(p);
  exclusive_scan_u32(p.bcount, p.boff, p.N, &p.st->border_units, p.scan_tmp2, s);
  STC_KL k_check_units<<<1, 1, 0, s>>>(p);
  STC_KL k_border_fill<<<num_sms() * 16, 128, 0, s>>>(p);
  int bits = 1;
  while ((1u << bits) < p.G && bits < 32) bits++;
  radix_sort_u32(p.bu_gid, p.iota, p.bu_sorted_gid, p.bu_sorted_pos, p.sort_ktmp2, p.sort_vtmp2,
                 &p.st->border_units, p.U_cap, bits, p.sort_hist2, p.scan_tmp2, s);
  exclusive_scan_u32(p.bu_cnt, p.bu_start, (size_t)p.G + 1, nullptr, p.scan_tmp2, s);
}

void step_jobs(PipeDev &p, cudaStream_t s) {
  STC_KL k_jobs<<<nblk((size_t)p.G + 1), 256, 0, s>>>(p);
  exclusive_scan_u32(p.job_cnt, p.job_start, (size_t)p.G + 1, &p.st->jobs_total, p.scan_tmp, s);
}

}  // namespace stc
