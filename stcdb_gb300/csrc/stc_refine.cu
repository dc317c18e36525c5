// Step kernel (b): proximity refinement fused with the first pass of the
// meeting-table insert.
//
// Work: every leaf's n kept members (the first leaf_cap in pid order,
// tracing/filter.cpp:100-104) are ordered by horizontal strips at least
// reach tall and, within small strips, by longitude (stc_partition.cu,
// k_strip_order). The reference tests every own-leaf pair (pid < q,
// tracing/refinement.cpp:30) and every (border unit, member) pair of the
// leaf (tracing/filter.cpp:248-259); a pair more than a strip apart, or
// farther apart in longitude than the leaf's window wx, is farther than
// reach, so only the pairs in a member's candidate windows -- the members
// after it in its strip up to its window's end and its window in the next
// strip, or for a border unit its window in the three strips beside its
// point -- can hit, and only those are tested. A job is 32 rows (members or
// border units) of one leaf, one per lane, each over one chunk of
// refine_chunk positions of its own contiguous segments (a dense leaf's
// n^2 / 2 pair tests spread over many jobs). Each hit keeps the reference's priority: the finding unit's
// rank and the member's index in pid order.
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
      // the box of both objects' float positions this step comes with the
      // record; the MBR only grows during a step, so a stale read of it can
      // only cause an extra atomic
      if (h.lo_x < mbr.x) atomic_min_f(&s->lo_x, h.lo_x);
      if (h.lo_y < mbr.y) atomic_min_f(&s->lo_y, h.lo_y);
      if (h.hi_x > mbr.z) atomic_max_f(&s->hi_x, h.hi_x);
      if (h.hi_y > mbr.w) atomic_max_f(&s->hi_y, h.hi_y);
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

// Direct emission: the round's records (one per lane with has set; hm =
// the ballot of has) go straight to the hit buffer at consecutive positions
// of the warp's window, a new window of HIT_CHUNK reserved when the round
// does not fit; records past the buffer are processed here.
__device__ __forceinline__ void emit_round(const PipeDev &p, const HitRec &h, bool has, uint32_t hm, uint32_t t,
                                           HitWindow &w) {
  const uint32_t lane = lane_id(), cnt = __popc(hm);
  if (w.end - w.next < cnt) {
    for (unsigned long long i = w.next + lane; i < w.end; i += 32)
      if (i < p.hit_cap) p.hits[i].a = STC_NONE;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&p.st->hit_count, (unsigned long long)HIT_CHUNK);
    base = __shfl_sync(0xffffffffu, base, 0);
    w.next = base;
    w.end = base + HIT_CHUNK;
  }
  if (has) {
    const unsigned long long pos = w.next + __popc(hm & ((1u << lane) - 1u));
    if (pos < p.hit_cap) p.hits[pos] = h;
    else process_hit(p, h, t);
  }
  w.next += cnt;
}

__device__ __forceinline__ HitRec load_hit(const HitRec *r) {
  // streamed once: evict-first loads keep L2 for the table and positions
  const ulonglong2 v = __ldcs((const ulonglong2 *)r);
  const float4 m = __ldcs((const float4 *)&r->lo_x);
  HitRec h;
  h.a = (uint32_t)v.x;
  h.b = (uint32_t)(v.x >> 32);
  h.order = v.y;
  h.lo_x = m.x;
  h.lo_y = m.y;
  h.hi_x = m.z;
  h.hi_y = m.w;
  return h;
}

// One thread per hit, two hits in flight per thread: both records and both
// home slots are requested before either is used.
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

// Lower bound of strip value v among the strip ids ((sorig >> 16) & 63,
// ascending) of a leaf's n members in strip order.
__device__ __forceinline__ uint32_t strip_lower_bound(const uint32_t *sorig, uint32_t n, uint32_t v) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (((__ldg(&sorig[mid]) >> 16) & 63u) < v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// First index in [lo, hi) of a longitude-ordered strip whose offset is
// greater than x (upper) or not below x (!upper).
__device__ __forceinline__ uint32_t strip_x_bound(const float4 *pts, uint32_t lo, uint32_t hi, float x, bool upper) {
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    const float v = __ldg(&pts[mid]).x;
    if (upper ? v <= x : v < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// One job: 32 rows of leaf g, each against its candidate ranges of members
// in (strip, longitude) order (stc_partition.cu, k_strip_order). Rows are
// the leaf's own members (own = true; row i tests the members after it in
// its strip up to its longitude window's end, and its window in the next
// strip, so every pair of members within reach is tested once) or 32 border
// units targeting the leaf (the members in the unit's longitude window in
// the three strips beside its point). A lane's candidates come in up to
// three contiguous segments, each read 32 at a time; hits are marked in a
// bitmask and turned into records after each group.
// DIRECT: records go straight to the hit buffer (emit_round) instead of
// through the warp's shared-memory queue; it pays where rows have many hits
// (dense leaves) and costs registers elsewhere.
template <bool DIRECT>
__device__ void run_rows(const PipeDev &p, uint32_t g, bool own, uint32_t rowblock, uint32_t chunk, uint32_t n,
                         uint32_t t, Counters &ct, HitRec *q, uint32_t &qn, HitWindow &w) {
  const uint32_t lane = lane_id();
  const uint32_t lt_mask = (1u << lane) - 1u;
  const uint32_t base = p.grid_start[g];
  const Node *o = &p.sd.nodes[p.sd.gid_node[g]];
  float4 rp = make_float4(0.f, 0.f, 0.f, 0.f);
  float2 fr = make_float2(0.f, 0.f);  // the row object's float position (fxy)
  uint32_t pid1 = 0, orig1 = 0, row_leaf = 0;
  uint32_t sa[3] = {0, 0, 0}, sl[3] = {0, 0, 0};  // candidate segments: start, length
  unsigned long long rank = 0;
  bool vr;
  if (own) {
    const uint32_t i = rowblock * 32 + lane;
    vr = i < n;
    if (vr) {
      rp = __ldg(&p.spts[base + i]);
      fr = __ldg(&p.sfxy[base + i]);
      pid1 = __float_as_uint(rp.w);
      orig1 = __ldg(&p.sorig[base + i]) & 0xFFFFu;
      const uint2 c = __ldg(&p.scand[base + i]);
      const uint32_t e1 = c.x & 0xFFFFu, a2 = c.x >> 16;
      sa[0] = i + 1;
      sl[0] = e1 > i + 1 ? e1 - (i + 1) : 0u;
      sa[1] = a2;
      sl[1] = c.y > a2 ? c.y - a2 : 0u;
    }
  } else {
    const uint32_t ub = p.bu_start[g], ue = p.bu_start[g + 1];
    const uint32_t r = ub + rowblock * 32 + lane;
    vr = r < ue;
    if (vr) {
      const uint32_t pos = p.bu_sorted_pos[r];
      pid1 = p.bu_pid[pos];
      rank = (unsigned long long)p.N + pos;  // border units follow the N own units
      const double2 qq = p.xy[pid1];
      fr = make_float2(__double2float_rn(qq.x), __double2float_rn(qq.y));
      rp = make_float4(__double2float_rn(RN_SUB(qq.x, o->lo_x)), __double2float_rn(RN_SUB(qq.y, o->lo_y)),
                       metres_per_deg_lon_f(qq.y), 0.f);
      // A pair of a border row (pid1 outside leaf g) and a member occurs
      // twice in this step iff the member also has a border unit targeting
      // pid1's leaf.
      row_leaf = p.leaf_gid[pid1];
      // candidates: the members in the point's longitude window of the
      // strips beside its own (all of a strip too large to be ordered)
      const float4 ls = __ldg(&p.lstrip[g]);
      const int H = (int)ls.y;
      const int c = (int)fminf(fmaxf(floorf(rp.y * ls.x), -4.0f), (float)H + 4.0f);
      const uint32_t *so = p.sorig + base;
      const float4 *sp = p.spts + base;
      int k = 0;
      for (int sidx = c - 1; sidx <= c + 1; sidx++, k++) {
        if (sidx < 0 || sidx >= H) continue;
        const uint32_t st = strip_lower_bound(so, n, (uint32_t)sidx);
        const uint32_t en = strip_lower_bound(so, n, (uint32_t)sidx + 1);
        if (st >= en) continue;
        uint32_t a = st, b = en;
        if (__ldg(&so[st]) & STRIP_XSORTED) {
          a = strip_x_bound(sp, st, en, rp.x - ls.z, false);
          b = strip_x_bound(sp, a, en, rp.x + ls.z, true);
        }
        sa[k] = a;
        sl[k] = b - a;
      }
    }
  }
  // this job's chunk: positions [chunk * refine_chunk, (chunk + 1) *
  // refine_chunk) of the lane's segments taken one after the other
  {
    uint32_t skip = chunk * p.refine_chunk, take = p.refine_chunk;
#pragma unroll
    for (int seg = 0; seg < 3; seg++) {
      const uint32_t d = min(skip, sl[seg]);
      sa[seg] += d;
      skip -= d;
      const uint32_t tk = min(take, sl[seg] - d);
      sl[seg] = tk;
      take -= tk;
    }
  }
  // error margin: offsets of the members are within the leaf's extent; a
  // border row's own offsets may exceed it
  const float wxl = (float)RN_SUB(o->hi_x, o->lo_x) * 1.000001f, wyl = (float)RN_SUB(o->hi_y, o->lo_y) * 1.000001f;
  const float mx = fmaxf(wxl, warp_max(fabsf(rp.x))), my = fmaxf(wyl, warp_max(fabsf(rp.y)));
  const float u = 5.9604645e-08f;
  const float r = (float)p.reach;
  const float E = 2.1f * u * (2.0f * mx * STC_SMAX_F + 2.0f * my * STC_SLAT_F);
  const float delta = 4.0f * E + 64.0f * u * r + 1e-6f * r;
  const float lo = fmaxf(r - delta, 0.0f);
  const float lo2 = lo * lo;
  const float hi2 = (r + delta) * (r + delta);
#pragma unroll 1
  for (int seg = 0; seg < 3; seg++) {
    const uint32_t a = sa[seg], len = sl[seg];
    ct.tests += len;
    const uint32_t maxlen = __reduce_max_sync(0xffffffffu, len);
    const float4 *cand = p.spts + base + a;
    for (uint32_t k0 = 0; k0 < maxlen; k0 += 32) {
      const uint32_t kn = maxlen - k0 < 32u ? maxlen - k0 : 32u;
      // the column loop only marks hits (one bit per candidate); records are
      // made afterwards, one per lane per round, so that the loop carries no
      // warp vote or branch for them
      uint32_t hitmask = 0;
#pragma unroll 4
      for (uint32_t kk = 0; kk < kn; kk++) {
        const bool valid = k0 + kk < len;
        const float4 c = valid ? __ldg(&cand[k0 + kk]) : make_float4(0.f, 0.f, 0.f, 0.f);
        const uint32_t pid2 = __float_as_uint(c.w);
        // the reference measures from the unit's point: an own pair from its
        // lower pid (tracing/refinement.cpp:30), a border pair from the unit
        const bool swap = own && pid2 < pid1;
        const float dx = (rp.x - c.x) * (swap ? c.z : rp.z);
        const float dy = (rp.y - c.y) * STC_SLAT_F;
        const float d2 = dx * dx + dy * dy;
        bool hit = valid && d2 <= lo2;
        if (valid && !hit && d2 < hi2) {
          ct.exact++;
          hit = swap ? exact_within(p, pid2, pid1, ct.amb) : exact_within(p, pid1, pid2, ct.amb);
        }
        hitmask |= (uint32_t)hit << kk;
      }
      ct.hits += __popc(hitmask);
      while (__any_sync(0xffffffffu, hitmask != 0)) {
        const bool has = hitmask != 0;
        const uint32_t kk = has ? (uint32_t)(__ffs(hitmask) - 1) : 0u;
        hitmask &= hitmask - 1u;
        const uint32_t hm = __ballot_sync(0xffffffffu, has);
        HitRec h;
        if (has) {
          const uint32_t j = a + k0 + kk;
          const uint32_t cpid = __float_as_uint(__ldg(&p.spts[base + j]).w);
          const uint32_t corig = __ldg(&p.sorig[base + j]) & 0xFFFFu;
          const float2 fc = __ldg(&p.sfxy[base + j]);
          const float2 fa = pid1 < cpid ? fr : fc, fb = pid1 < cpid ? fc : fr;
          h.a = pid1 < cpid ? pid1 : cpid;
          h.b = pid1 < cpid ? cpid : pid1;
          h.lo_x = fminf(fa.x, fb.x);
          h.lo_y = fminf(fa.y, fb.y);
          h.hi_x = fmaxf(fa.x, fb.x);
          h.hi_y = fmaxf(fa.y, fb.y);
          if (own) {
            // the pair is found by the lower pid's own unit (rank = its pid)
            // at the higher pid's place in the pid-ordered member list
            h.order = ((unsigned long long)h.a << STC_ORDER_SHIFT) | (pid1 < cpid ? corig : orig1);
          } else {
            h.order = (rank << STC_ORDER_SHIFT) | corig;
            const uint32_t cnb = p.bcount[cpid];
            const uint32_t coff = cnb ? p.boff[cpid] : 0u;
            for (uint32_t u2 = 0; u2 < cnb; u2++)
              if (p.bu_gid[coff + u2] == row_leaf) h.order |= DUP_BIT;
          }
          if (!DIRECT) q[qn + __popc(hm & lt_mask)] = h;
        }
        if (DIRECT) {
          emit_round(p, h, has, hm, t, w);
        } else {
          qn += __popc(hm);
          if (qn >= 32) {
            flush_queue(p, q, 32, t, w);
            const uint32_t rest = qn - 32;
            HitRec mv;
            if (lane < rest) mv = q[32 + lane];
            __syncwarp();
            if (lane < rest) q[lane] = mv;
            __syncwarp();
            qn = rest;
          }
        }
      }
    }
  }
}

// Slice `part` of `parts` runs job chunks [C * part / parts, C * (part + 1) / parts)
// of the C = ceil(jobs / p.job_chunk) chunks.
template <bool DIRECT>
__global__ void __launch_bounds__(REFINE_THREADS, 4) k_refine_a(PipeDev p, uint32_t part, uint32_t parts) {
  const uint32_t t = p.st->step_t;
  __shared__ HitRec queues[DIRECT ? 1 : REFINE_THREADS / 32][QCAP];
  HitRec *q = queues[DIRECT ? 0 : threadIdx.x >> 5];
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
      const uint32_t local = (uint32_t)(job - p.job_start[g]);
      const uint32_t cnt = p.grid_count[g];
      const uint32_t n = cnt < p.leaf_cap ? cnt : p.leaf_cap;
      const uint32_t R = (n + 31) / 32, cc = p.cchunks[g], own_jobs = R * cc;
      if (local < own_jobs) {
        run_rows<DIRECT>(p, g, true, local / cc, local % cc, n, t, ct, q, qn, w);
      } else {
        const uint32_t ccb = (n + p.refine_chunk - 1) / p.refine_chunk, b = local - own_jobs;
        run_rows<DIRECT>(p, g, false, b / ccb, b % ccb, n, t, ct, q, qn, w);
      }
    }
  }
  if (!DIRECT && qn) flush_queue(p, q, qn, t, w);
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
  if (p.direct_hits)
    STC_KL k_refine_a<true><<<num_sms() * p.refine_bps, REFINE_THREADS, 0, s>>>(p, part, parts);
  else
    STC_KL k_refine_a<false><<<num_sms() * p.refine_bps, REFINE_THREADS, 0, s>>>(p, part, parts);
  STC_KL k_hit_mark<<<1, 1, 0, s>>>(p, part);
}

void step_hits_part(PipeDev &p, uint32_t part, uint32_t parts, cudaStream_t s) {
  STC_KL k_hits<<<num_sms() * p.hits_bps, 256, 0, s>>>(p, part, parts);
}

}  // namespace stc
