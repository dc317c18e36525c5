// Step kernel (b): proximity refinement fused with the first pass of the
// meeting-table insert.
//
// Work tiles: for every leaf with n kept members (the first leaf_cap in pid
// order, tracing/filter.cpp:100-104) the own-leaf pairs i < j form the upper
// triangle of a 32 x 32 tiling, and the border units that target the leaf
// (pid outside the leaf, tracing/filter.cpp:248-259) form extra row tiles
// against all members. One warp runs one tile: rows in lanes, the 32 column
// points broadcast with shuffles.
//
// Distance decisions equal the reference's fp64 test
// `p1->distance(p2, true) <= reach` (tracing/refinement.cpp:30-33,
// geometry/geometry.h:40-48). Each pair is first classified in fp32 from the
// points' offsets to the leaf corner; the classification is conservative by
// construction (error bound below), and only pairs inside the uncertainty
// band are recomputed with the reference's exact fp64 expression.
//
// Error bound of the fp32 estimate d_f of the reference distance d, with
// u = 2^-24, X = |x - corner| <= mx (degrees lon), Y <= my (degrees lat):
//   offsets round with |err| <= u X, so dx picks up <= 2 u mx degrees and dy
//   <= 2 u my; the rest (subtraction, scale factor from sinf, products, sum)
//   is relative and below 30 u. Hence
//     |d_f - d| <= 30 u d + 2.1 u (2 mx SMAX + 2 my SLAT) = 30 u d + E.
//   A pair is accepted when d_f^2 <= (r - delta)^2 and rejected when
//   d_f^2 >= (r + delta)^2 with delta = 4E + 64 u r + 1e-6 r, which leaves
//   slack for the rounding of the squared thresholds themselves.
//
// Hits (tracing/refinement.cpp:34-55) probe the meeting table from
// key % B. A key found before the first empty slot is extended in place
// (end = t, MBR); every other key becomes a candidate for the ordered insert
// of stc_meetings.cu, keyed with its first position in the reference's
// sequential processing order: unit rank << 24 | member index.
#include "stc_insert.cuh"

namespace stc {

static constexpr int REFINE_THREADS = 256;

__device__ __forceinline__ double dpml_fast_r(double lat) {
  double absla = fabs(lat);
  if (absla == 90) absla = 89;
  double arg = RN_DIV(RN_MUL(RN_SUB(90.0, absla), STC_REF_PI), 180.0);
  return RN_DIV(360.0, RN_MUL(RN_MUL(sin(arg), 40076.0), 1000.0));
}

// Reference distance decision for p1 (whose latitude sets the scale) and p2.
__device__ bool exact_within(const PipeDev &p, uint32_t pid1, uint32_t pid2, uint32_t &amb) {
  double2 a = p.xy[pid1], b = p.xy[pid2];
  double d = stc_distance_ref(a.x, a.y, b.x, b.y, dpml_fast_r(a.y));
  if (fabs(d - p.reach) > 1e-12 * p.reach) return d <= p.reach;
  d = stc_distance_ref(a.x, a.y, b.x, b.y, stc_dpml_ref(a.y));
  // within a few ulp of reach the decision depends on the last bit of sin()
  if (fabs(d - p.reach) <= 8.0 * 2.220446049250313e-16 * p.reach) amb++;
  return d <= p.reach;
}

// Merges one instance of a key that may occur twice in this step into the
// candidate set (minimum priority); the candidate pass walks it afterwards.
__device__ void cand_insert(const PipeDev &p, unsigned long long key, unsigned long long order) {
  unsigned long long h = mix64(key) & (p.C - 1);
  for (unsigned long long probe = 0; probe < STC_PROBE_LIMIT; probe++) {
    Cand *c = &p.cset[h];
    unsigned long long k = *(volatile unsigned long long *)&c->key;
    if (k == STC_EMPTY_KEY) {
      // the list bounds the set's load factor at cand_cap / C <= 1/2
      if (*(volatile unsigned long long *)&p.st->cand_count >= p.cand_cap) {
        stc_set_error(p.st, ERR_CAND, 0u);
        return;
      }
      k = atomicCAS(&c->key, STC_EMPTY_KEY, key);
      if (k == STC_EMPTY_KEY) {
        unsigned long long n = agg_inc(&p.st->cand_count);
        if (n < p.cand_cap) p.cand_list[n] = (uint32_t)h;
        else stc_set_error(p.st, ERR_CAND, (uint32_t)n);
        k = key;
      }
    }
    if (k == key) {
      atomicMin(&c->order, order);
      return;
    }
    h = (h + 1) & (p.C - 1);
  }
  stc_set_error(p.st, ERR_CAND, 0xFFFFFFFFu);
}


static constexpr int QCAP = 64;  // per-warp queue; flushed 32 at a time
#define DUP_BIT (1ULL << 63)

// Applies one hit (key = cantor(h.a, h.b)) to the table. kv/mbr: the slot
// at key % B, already loaded.
__device__ void process_hit_at(const PipeDev &p, const HitRec &h, unsigned long long key, uint32_t t,
                               unsigned long long slot, U128 kv, float4 mbr) {
  for (unsigned long long probe = 0; probe < STC_PROBE_LIMIT && probe < p.B; probe++) {
    Slot *s = &p.slots[slot];
    if (kv.lo == key) {  // tracing/refinement.cpp:40-42 (+ MBR, cuda/geometry.cu:474-478)
      s->end = t;
      // both objects' float positions this step; the MBR only grows during a
      // step, so a stale read can only cause an extra atomic
      const float2 fa = p.fxy[h.a], fb = p.fxy[h.b];
      const float lx = fminf(fa.x, fb.x), ly = fminf(fa.y, fb.y), hx = fmaxf(fa.x, fb.x), hy = fmaxf(fa.y, fb.y);
      if (lx < mbr.x) atomic_min_f(&s->lo_x, lx);
      if (ly < mbr.y) atomic_min_f(&s->lo_y, ly);
      if (hx > mbr.z) atomic_max_f(&s->hi_x, hx);
      if (hy > mbr.w) atomic_max_f(&s->hi_y, hy);
      return;
    }
    if (kv.lo == STC_EMPTY_KEY || (kv.lo & STC_CLAIM_BIT)) {  // empty before this step: a new key
      if (h.order & DUP_BIT) {
        cand_insert(p, key, h.order & ~DUP_BIT);
      } else {
        if (!ordered_walk(p, key, h.order, slot, t, &kv)) stc_set_error(p.st, ERR_DA, (uint32_t)slot);
      }
      return;
    }
    slot = slot + 1 == p.B ? 0 : slot + 1;
    kv = load_slot_pair(&p.slots[slot]);
    mbr = __ldcg((const float4 *)&p.slots[slot].lo_x);
  }
  stc_set_error(p.st, ERR_PROBE, (uint32_t)slot);
}

__device__ __forceinline__ void process_hit(const PipeDev &p, const HitRec &h, uint32_t t) {
  const unsigned long long key = stc_cantor(h.a, h.b);
  unsigned long long slot = fast_mod(key, p.B, p.B_magic);
  process_hit_at(p, h, key, t, slot, load_slot_pair(&p.slots[slot]), __ldcg((const float4 *)&p.slots[slot].lo_x));
}

// Per-warp window of the step's hit buffer, reserved HIT_CHUNK entries at a
// time so that the shared counter sees one atomic per HIT_CHUNK hits.
static constexpr uint32_t HIT_CHUNK = 256;
struct HitWindow {
  unsigned long long next, end;  // warp-uniform
};

// Moves the first `n` (<= 32) queued hits to the step's hit buffer, which
// k_hits processes with one thread per hit; hits that do not fit are
// processed here, one per lane.
__device__ __forceinline__ void flush_queue(const PipeDev &p, HitRec *q, uint32_t n, uint32_t t, HitWindow &w) {
  __syncwarp();
  uint32_t lane = lane_id();
  if (w.end - w.next < n) {
    // pad the rest of the old window with empty records, then reserve a new one
    for (unsigned long long i = w.next + lane; i < w.end; i += 32)
      if (i < p.hit_cap) p.hits[i].a = STC_NONE;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&p.st->hit_count, (unsigned long long)HIT_CHUNK);
    base = __shfl_sync(0xffffffffu, base, 0);
    w.next = base;
    w.end = base + HIT_CHUNK;
  }
  if (lane < n) {
    HitRec h = q[lane];
    unsigned long long pos = w.next + lane;
    if (pos < p.hit_cap) p.hits[pos] = h;
    else process_hit(p, h, t);
  }
  w.next += n;
  __syncwarp();
}

__device__ __forceinline__ HitRec load_hit(const HitRec *r) {
  // streamed once: evict-first loads keep L2 for the table and positions
  ulonglong2 v = __ldcs((const ulonglong2 *)r);
  HitRec h;
  h.a = (uint32_t)v.x;
  h.b = (uint32_t)(v.x >> 32);
  h.order = v.y;
  return h;
}

// One thread per hit, two hits in flight per thread: both records and both
// home slots are requested before either is used.
// Slice `part` of `parts` covers hits [nh * part / parts, nh * (part + 1) / parts).
// Part `part` applies the hits the pair tests' part `part` appended:
// [hit_bounds[part], hit_bounds[part + 1]).
__global__ void __launch_bounds__(256) k_hits(PipeDev p, uint32_t part, uint32_t parts) {
  const uint32_t t = p.st->step_t;
  (void)parts;
  const unsigned long long h0i = p.hit_bounds[part], nh = p.hit_bounds[part + 1];
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = h0i + (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < nh;
       i += 2 * stride) {
    unsigned long long i2 = i + stride;
    HitRec h0 = load_hit(&p.hits[i]);
    HitRec h1;
    h1.a = STC_NONE;
    if (i2 < nh) h1 = load_hit(&p.hits[i2]);
    const bool v0 = h0.a != STC_NONE, v1 = h1.a != STC_NONE;
    const unsigned long long k0 = v0 ? stc_cantor(h0.a, h0.b) : 0, k1 = v1 ? stc_cantor(h1.a, h1.b) : 0;
    unsigned long long s0 = fast_mod(k0, p.B, p.B_magic), s1 = fast_mod(k1, p.B, p.B_magic);
    U128 kv0 = {0, 0}, kv1 = {0, 0};
    float4 m0 = make_float4(0.f, 0.f, 0.f, 0.f), m1 = m0;
    if (v0) {
      kv0 = load_slot_pair(&p.slots[s0]);
      m0 = __ldcg((const float4 *)&p.slots[s0].lo_x);
    }
    if (v1) {
      kv1 = load_slot_pair(&p.slots[s1]);
      m1 = __ldcg((const float4 *)&p.slots[s1].lo_x);
    }
    if (v0) process_hit_at(p, h0, k0, t, s0, kv0, m0);
    if (v1) process_hit_at(p, h1, k1, t, s1, kv1, m1);
  }
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

struct Counters {
  uint32_t tests, exact, hits, amb;  // per thread; summed into 64-bit totals per warp
};

// One 32x32 tile. Rows: own members (own=true) or border units.
// A tile's 32 column points, staged per warp in shared memory: the test loop
// reads one broadcast (x, y) per column; pid and border data on a hit only.
struct ColTile {
  float2 xy[32];     // leaf-relative fp32 offsets
  uint32_t pid[32];
  uint32_t nb[32];   // border units of the column object (border tiles)
  uint32_t off[32];
};

__device__ void run_tile(const PipeDev &p, uint32_t g, bool own, uint32_t rowtile, uint32_t coltile, uint32_t n,
                         uint32_t t, Counters &ct, HitRec *q, uint32_t &qn, HitWindow &w, ColTile &col) {
  const uint32_t lane = lane_id();
  const uint32_t base = p.grid_start[g];
  const uint32_t lt_mask = (1u << lane) - 1u;
  // column points
  uint32_t j = coltile * 32 + lane;
  bool vc = j < n;
  float4 cp = vc ? p.pts[base + j] : make_float4(0.f, 0.f, 0.f, 0.f);
  // row points
  float4 rp;
  uint32_t pid1 = 0;
  unsigned long long rank = 0;
  uint32_t i = rowtile * 32 + lane;
  bool vr;
  if (own) {
    vr = i < n;
    rp = vr ? p.pts[base + i] : make_float4(0.f, 0.f, 0.f, 0.f);
    pid1 = __float_as_uint(rp.w);
    rank = pid1;  // own-leaf unit of pid1 is grid_check[pid1] (tracing/filter.cpp:107-109)
  } else {
    uint32_t ub = p.bu_start[g], ue = p.bu_start[g + 1];
    uint32_t r = ub + i;
    vr = r < ue;
    rp = make_float4(0.f, 0.f, 0.f, 0.f);
    if (vr) {
      uint32_t pos = p.bu_sorted_pos[r];
      pid1 = p.bu_pid[pos];
      rank = (unsigned long long)p.N + pos;  // border units follow the N own units
      const Node *o = &p.sd.nodes[p.sd.gid_node[g]];
      double2 qq = p.xy[pid1];
      rp = make_float4(__double2float_rn(RN_SUB(qq.x, o->lo_x)), __double2float_rn(RN_SUB(qq.y, o->lo_y)),
                       metres_per_deg_lon_f(qq.y), 0.f);
    }
  }
  // A pair of a border row (pid1 outside leaf g) and member cpid occurs twice
  // in this step iff cpid also has a border unit targeting pid1's leaf.
  uint32_t row_leaf = (!own && vr) ? p.leaf_gid[pid1] : 0u;
  uint32_t col_nb = 0, col_off = 0;
  if (!own && vc) {
    uint32_t cpid0 = __float_as_uint(cp.w);
    col_nb = p.bcount[cpid0];
    col_off = col_nb ? p.boff[cpid0] : 0u;
  }
  // tile error margin
  float mx = warp_max(fmaxf(fabsf(rp.x), fabsf(cp.x)));
  float my = warp_max(fmaxf(fabsf(rp.y), fabsf(cp.y)));
  const float u = 5.9604645e-08f;
  const float r = (float)p.reach;
  float E = 2.1f * u * (2.0f * mx * STC_SMAX_F + 2.0f * my * STC_SLAT_F);
  float delta = 4.0f * E + 64.0f * u * r + 1e-6f * r;
  float lo = fmaxf(r - delta, 0.0f);
  float lo2 = lo * lo;
  float hi2 = (r + delta) * (r + delta);
  uint32_t kmax = n - coltile * 32;
  if (kmax > 32) kmax = 32;
  // stage the columns (the previous tile's reads are over)
  __syncwarp();
  col.xy[lane] = make_float2(cp.x, cp.y);
  col.pid[lane] = __float_as_uint(cp.w);
  col.nb[lane] = col_nb;
  col.off[lane] = col_off;
  __syncwarp();
  // this lane tests columns k in [kstart, kmax): an own-leaf unit pairs pid1
  // only with later members (tracing/refinement.cpp:30)
  int kstart = !vr ? 64 : (own ? (int)i - (int)(coltile * 32) + 1 : 0);
  if (kstart < 0) kstart = 0;
  if (kstart < (int)kmax) ct.tests += kmax - (uint32_t)kstart;
  // the column loop only marks hits (one bit per column); records are made
  // afterwards, one per lane per round, so that the loop carries no warp vote
  // or branch for them
  uint32_t hitmask = 0;
#pragma unroll 1
  for (uint32_t k = 0; k < kmax; k++) {
    const float2 c = col.xy[k];
    float dx = (rp.x - c.x) * rp.z;
    float dy = (rp.y - c.y) * STC_SLAT_F;
    float d2 = dx * dx + dy * dy;
    const bool valid = (int)k >= kstart;
    bool hit = valid && d2 <= lo2;
    if (valid && !hit && d2 < hi2) {
      ct.exact++;
      hit = exact_within(p, pid1, col.pid[k], ct.amb);
    }
    hitmask |= (uint32_t)hit << k;
  }
  ct.hits += __popc(hitmask);
  while (__any_sync(0xffffffffu, hitmask != 0)) {
    const bool has = hitmask != 0;
    const uint32_t k = has ? (uint32_t)(__ffs(hitmask) - 1) : 0u;
    hitmask &= hitmask - 1u;
    const uint32_t hm = __ballot_sync(0xffffffffu, has);
    if (has) {
      const uint32_t cpid = col.pid[k];
      HitRec h;
      h.a = pid1 < cpid ? pid1 : cpid;
      h.b = pid1 < cpid ? cpid : pid1;
      h.order = (rank << STC_ORDER_SHIFT) | (coltile * 32 + k);
      if (!own) {
        const uint32_t cnb = col.nb[k], coff = col.off[k];
        for (uint32_t u2 = 0; u2 < cnb; u2++)
          if (p.bu_gid[coff + u2] == row_leaf) h.order |= DUP_BIT;
      }
      q[qn + __popc(hm & lt_mask)] = h;
    }
    qn += __popc(hm);
    if (qn >= 32) {
      flush_queue(p, q, 32, t, w);
      uint32_t rest = qn - 32;
      HitRec mv;
      if (lane < rest) mv = q[32 + lane];
      __syncwarp();
      if (lane < rest) q[lane] = mv;
      __syncwarp();
      qn = rest;
    }
  }
}

// Slice `part` of `parts` runs job chunks [C * part / parts, C * (part + 1) / parts)
// of the C = ceil(jobs / p.job_chunk) chunks.
__global__ void __launch_bounds__(REFINE_THREADS, 4) k_refine_a(PipeDev p, uint32_t part, uint32_t parts) {
  const uint32_t t = p.st->step_t;
  __shared__ HitRec queues[REFINE_THREADS / 32][QCAP];
  __shared__ ColTile cols[REFINE_THREADS / 32];
  HitRec *q = queues[threadIdx.x >> 5];
  ColTile &col = cols[threadIdx.x >> 5];
  uint32_t qn = 0;  // warp-uniform queue length
  HitWindow w = {0, 0};
  const unsigned long long warp = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
  const unsigned long long J = p.st->jobs_total;
  const unsigned long long jc = p.job_chunk;
  const unsigned long long nchunks = (J + jc - 1) / jc;
  const unsigned long long c0 = nchunks * part / parts, c1 = nchunks * (part + 1) / parts;
  Counters ct = {0, 0, 0, 0};
  for (unsigned long long chunk = c0 + warp; chunk < c1; chunk += nwarps) {
    // one lane reads the flag so that the whole warp leaves together
    if (__shfl_sync(0xffffffffu, (int)stc_failed(p.st), 0)) break;
    unsigned long long j0 = chunk * jc;
    unsigned long long j1 = j0 + jc < J ? j0 + jc : J;
    // largest g with job_start[g] <= j0
    uint32_t lo = 0, hi = p.G;
    while (hi - lo > 1) {
      uint32_t mid = (lo + hi) >> 1;
      if (p.job_start[mid] <= j0) lo = mid; else hi = mid;
    }
    uint32_t g = lo;
    for (unsigned long long job = j0; job < j1; job++) {
      while (p.job_start[g + 1] <= job) g++;
      uint32_t local = (uint32_t)(job - p.job_start[g]);
      uint32_t cnt = p.grid_count[g];
      uint32_t n = cnt < p.leaf_cap ? cnt : p.leaf_cap;
      uint32_t R = (n + 31) / 32;
      uint32_t own = R * (R + 1) / 2;
      if (local < own) {
        // row-major upper triangle: row rc has R - rc tiles (fp32 estimate, exact fix-up)
        float b2 = 2.0f * (float)R + 1.0f;
        uint32_t rc = (uint32_t)fmaxf((b2 - sqrtf(fmaxf(b2 * b2 - 8.0f * (float)local, 0.0f))) * 0.5f, 0.0f);
        if (rc > R - 1) rc = R - 1;
        while (rc > 0 && rc * R - rc * (rc - 1) / 2 > local) rc--;
        while ((rc + 1) * R - (rc + 1) * rc / 2 <= local) rc++;
        uint32_t cc = rc + (local - (rc * R - rc * (rc - 1) / 2));
        run_tile(p, g, true, rc, cc, n, t, ct, q, qn, w, col);
      } else {
        uint32_t b = local - own;
        run_tile(p, g, false, b / R, b % R, n, t, ct, q, qn, w, col);
      }
    }
  }
  if (qn) flush_queue(p, q, qn, t, w);
  for (unsigned long long i = w.next + lane_id(); i < w.end; i += 32)
    if (i < p.hit_cap) p.hits[i].a = STC_NONE;
  // reduce counters per warp (64-bit sums)
  unsigned long long tests = ct.tests, exact = ct.exact, hits = ct.hits, amb = ct.amb;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    tests += __shfl_xor_sync(0xffffffffu, tests, o);
    exact += __shfl_xor_sync(0xffffffffu, exact, o);
    hits += __shfl_xor_sync(0xffffffffu, hits, o);
    amb += __shfl_xor_sync(0xffffffffu, amb, o);
  }
  if (lane_id() == 0) {
    if (tests) atomicAdd(&p.st->tests, tests);
    if (exact) atomicAdd(&p.st->exact_tests, exact);
    if (hits) atomicAdd(&p.st->hits, hits);
    if (amb) atomicAdd(&p.st->ambiguous, amb);
  }
}

// hit_bounds[part + 1] = the hit buffer's end after part `part` (its hits
// are [hit_bounds[part], hit_bounds[part + 1]): parts run in stream order)
__global__ void k_hit_mark(PipeDev p, uint32_t part) {
  const unsigned long long n = p.st->hit_count;
  p.hit_bounds[part + 1] = n < p.hit_cap ? n : p.hit_cap;
  if (part == 0) p.hit_bounds[0] = 0;
}

void step_pairs_part(PipeDev &p, uint32_t part, uint32_t parts, cudaStream_t s) {
  STC_KL k_refine_a<<<num_sms() * p.refine_bps, REFINE_THREADS, 0, s>>>(p, part, parts);
  STC_KL k_hit_mark<<<1, 1, 0, s>>>(p, part);
}

void step_hits_part(PipeDev &p, uint32_t part, uint32_t parts, cudaStream_t s) {
  STC_KL k_hits<<<num_sms() * p.hits_bps, 256, 0, s>>>(p, part, parts);
}

}  // namespace stc
