// Step kernels (c): ordered insertion of new meetings and the expire/emit
// sweep of the meeting table.
//
// The reference inserts hits one by one in its processing order with linear
// probing from key % B and clears expired slots without tombstones
// (tracing/refinement.cpp:37-55, tracing/meeting.cpp:47-67). Which slot a
// new key lands in -- and therefore whether a later probe for a live meeting
// crosses a cleared slot and restarts it -- depends on that order. The
// sequential result is reproduced exactly:
//
//   Every candidate key k (distinct per step) walks from k % B over the
//   table as it stood before the step: slots holding other keys are passed,
//   a slot holding k itself ends the walk (the meeting is extended there),
//   and each empty slot is contended. Contention is resolved by priority =
//   the key's first position in the reference's processing order: a claim
//   word (key | CLAIM_BIT, priority) is installed with a 128-bit CAS, a
//   lower priority evicts a higher one, and the evicted key continues its
//   walk from the next slot. Slots prefer lower priorities and keys prefer
//   earlier slots, so this deferred acceptance converges to the unique stable
//   assignment, which is exactly what inserting the keys one by one in
//   priority order produces.
//
// The ordered walk itself lives in stc_insert.cuh; the refinement runs it for
// keys found once per step, k_insert_ordered for keys that may occur twice.
// The sweep turns claims into new meetings (start = end = t, MBR of both
// objects' current positions -- a new meeting has been seen in this step
// only), keeps active meetings, emits finished ones whose duration reaches
// min_meet_time (tracing/meeting.cpp:59, plus the map-box filter of
// cuda/geometry.cu:667) and clears the rest.
#include "stc_insert.cuh"

namespace stc {

__global__ void k_step_begin(DevState *st) {
  st->error = 0;
  st->error_info = 0;
  st->border_units = 0;
  st->border_points = 0;
  st->fast_claims = 0;
  st->hit_count = 0;
  st->jobs_total = 0;
  st->job_next = 0;
  st->cand_count = 0;
  st->tests = st->exact_tests = st->hits = st->ambiguous = 0;
  st->taken = 0;
  st->step_emitted = 0;
  st->da_iters = 0;
  st->splits = st->merges = st->events = 0;
  st->overflow_objects = 0;
}

// The step's time goes to the device from a page-locked word that the host
// sets before the step is issued (also when the step is replayed from a
// captured graph); the step's kernels read it from DevState::step_t.
void step_begin(PipeDev &p, const uint32_t *t_pinned, cudaStream_t s) {
  cudaMemcpyAsync(&p.st->step_t, t_pinned, sizeof(uint32_t), cudaMemcpyHostToDevice, s);
  STC_KL k_step_begin<<<1, 1, 0, s>>>(p.st);
}

__global__ void k_init_slots(Slot *slots, unsigned long long B) {
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < B;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    Slot s;
    s.key = STC_EMPTY_KEY;
    s.start = 0xFFFFFFFFu;
    s.end = 0xFFFFFFFFu;
    s.lo_x = STC_INIT_LO; s.lo_y = STC_INIT_LO; s.hi_x = STC_INIT_HI; s.hi_y = STC_INIT_HI;
    slots[i] = s;
  }
}

__global__ void k_init_cands(Cand *c, unsigned long long C) {
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < C;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    Cand x;
    x.key = STC_EMPTY_KEY;
    x.order = ~0ULL;
    x.lo_x = STC_INIT_LO; x.lo_y = STC_INIT_LO; x.hi_x = STC_INIT_HI; x.hi_y = STC_INIT_HI;
    c[i] = x;
  }
}

void init_tables(PipeDev &p, cudaStream_t s) {
  STC_KL k_init_slots<<<num_sms() * 8, 256, 0, s>>>(p.slots, p.B);
  STC_KL k_init_cands<<<num_sms() * 8, 256, 0, s>>>(p.cset, p.C);
}

// Candidates that may occur twice in a step: walk with their minimum
// priority once all instances are merged.
__global__ void k_insert_ordered(PipeDev p) {
  const uint32_t t = p.st->step_t;
  const unsigned long long nc = p.st->cand_count < p.cand_cap ? p.st->cand_count : p.cand_cap;
  for (unsigned long long c = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc;
       c += (unsigned long long)gridDim.x * blockDim.x) {
    if (stc_failed(p.st)) return;
    Cand *cp = &p.cset[p.cand_list[c]];
    unsigned long long key = cp->key, prio = cp->order;
    // last reader this step: reset the entry for the next one
    Cand x;
    x.key = STC_EMPTY_KEY;
    x.order = ~0ULL;
    x.lo_x = STC_INIT_LO; x.lo_y = STC_INIT_LO; x.hi_x = STC_INIT_HI; x.hi_y = STC_INIT_HI;
    *cp = x;
    if (!ordered_walk(p, key, prio, fast_mod(key, p.B, p.B_magic), t)) stc_set_error(p.st, ERR_DA, (uint32_t)c);
  }
}

void step_insert(PipeDev &p, cudaStream_t s) { STC_KL k_insert_ordered<<<num_sms() * 4, 256, 0, s>>>(p); }

// Sweep (tracing/meeting.cpp:32-76, cuda/geometry.cu:595-736).

// Loads slot i streaming: the table passes through once, so evict-first
// loads and stores leave L2 to the per-object positions read for new
// meetings.
__device__ __forceinline__ Slot load_slot_stream(const Slot *slots, unsigned long long i) {
  ulonglong2 a = __ldcs((const ulonglong2 *)&slots[i]);
  float4 b = __ldcs((const float4 *)&slots[i].lo_x);
  Slot s;
  s.key = a.x;
  s.start = (uint32_t)a.y;
  s.end = (uint32_t)(a.y >> 32);
  s.lo_x = b.x; s.lo_y = b.y; s.hi_x = b.z; s.hi_y = b.w;
  return s;
}

// One slot: finalise a meeting claimed this step, keep an extended one, or
// clear an ended one; returns whether the ended meeting is emitted.
// A claimed slot's pair: its objects' float positions this step (both
// requested before the slot is processed; a no-op for other slots).
struct ClaimPos {
  float2 fa, fb;
};
__device__ __forceinline__ ClaimPos claim_positions(const PipeDev &p, const Slot &s) {
  ClaimPos c;
  c.fa = c.fb = make_float2(0.f, 0.f);
  if (s.key != STC_EMPTY_KEY && (s.key & STC_CLAIM_BIT)) {
    uint32_t a, b;
    cantor_decode(s.key & ~STC_CLAIM_BIT, &a, &b);
    c.fa = __ldg(&p.fxy[a]);
    c.fb = __ldg(&p.fxy[b]);
  }
  return c;
}

__device__ __forceinline__ bool sweep_slot(const PipeDev &p, uint32_t t, unsigned long long i, const Slot &s,
                                           const ClaimPos &cp, unsigned long long &active,
                                           unsigned long long &fresh) {
  if (s.key == STC_EMPTY_KEY) return false;
  if (s.key & STC_CLAIM_BIT) {
    // new meeting of this step (cuda/geometry.cu:480-489): start = end = t,
    // MBR = init, then both objects' positions
    Slot nm;
    nm.key = s.key & ~STC_CLAIM_BIT;
    const float2 fa = cp.fa, fb = cp.fb;
    nm.start = t;
    nm.end = t;
    nm.lo_x = fminf(STC_INIT_LO, fminf(fa.x, fb.x));
    nm.lo_y = fminf(STC_INIT_LO, fminf(fa.y, fb.y));
    nm.hi_x = fmaxf(STC_INIT_HI, fmaxf(fa.x, fb.x));
    nm.hi_y = fmaxf(STC_INIT_HI, fmaxf(fa.y, fb.y));
    p.slots[i] = nm;
    active++;
    fresh++;
    return false;
  }
  if (s.end == t) {
    active++;
    return false;
  }
  bool emit = false;
  if (t - s.start >= p.min_meet_time + 1) {
    emit = !p.mbr_filter || (s.lo_x >= p.fmap_lo_x && s.hi_x <= p.fmap_hi_x && s.lo_y >= p.fmap_lo_y &&
                             s.hi_y <= p.fmap_hi_y);
  }
  Slot e;
  e.key = STC_EMPTY_KEY;
  e.start = 0xFFFFFFFFu;
  e.end = 0xFFFFFFFFu;
  e.lo_x = STC_INIT_LO; e.lo_y = STC_INIT_LO; e.hi_x = STC_INIT_HI; e.hi_y = STC_INIT_HI;
  p.slots[i] = e;
  return emit;
}

static constexpr uint32_t SWEEP_THREADS = 256;
static constexpr uint32_t SWEEP_BLOCKS_PER_SM = 5;
static constexpr uint32_t SWEEP_WARPS = SWEEP_THREADS / 32;
static constexpr uint32_t SWEEP_UNROLL = 2;                // slots per lane per pass
static constexpr uint32_t WARP_TILE = 32 * SWEEP_UNROLL;   // slots per warp pass
static constexpr uint32_t WARP_STAGE = 96;                 // staged meetings per warp

// Emitted meetings are staged per warp in shared memory and moved to the
// emit buffer with one reservation per few dozen meetings: one global
// counter bumped by every emitting warp serialises in L2.
__device__ __forceinline__ void flush_emits(const PipeDev &p, const stc_meeting *stage, uint32_t n) {
  const uint32_t lane = lane_id();
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(&p.st->emit_count, (unsigned long long)n);
  base = __shfl_sync(0xffffffffu, base, 0);
  for (uint32_t k = lane; k < n; k += 32) {
    unsigned long long pos = base + k;
    if (pos < p.E) {
      const uint4 *src = (const uint4 *)&stage[k];
      uint4 *dst = (uint4 *)&p.emit[pos];
      dst[0] = src[0];
      dst[1] = src[1];
    } else {
      stc_set_error(p.st, ERR_EMIT, (uint32_t)min(pos - p.E, 0xFFFFFFFFull));
    }
  }
  __syncwarp();
}

// Slice `part` of `parts` sweeps slots [B * part / parts, B * (part + 1) / parts).
__global__ void __launch_bounds__(SWEEP_THREADS, SWEEP_BLOCKS_PER_SM) k_sweep(PipeDev p, uint32_t part, uint32_t parts) {
  const uint32_t t = p.st->step_t;
  __shared__ __align__(16) stc_meeting stage_all[SWEEP_WARPS][WARP_STAGE];
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
  stc_meeting *stage = stage_all[warp];
  uint32_t n = 0;  // warp-uniform
  unsigned long long active = 0, fresh = 0, emitted = 0;
  const unsigned long long B0 = p.B * part / parts, B = p.B * (part + 1) / parts;
  const unsigned long long gw = (unsigned long long)blockIdx.x * SWEEP_WARPS + warp;
  const unsigned long long nw = (unsigned long long)gridDim.x * SWEEP_WARPS;
  for (unsigned long long bb = B0 + gw * WARP_TILE; bb < B; bb += nw * WARP_TILE) {
    Slot sl[SWEEP_UNROLL];
    unsigned long long idx[SWEEP_UNROLL];
#pragma unroll
    for (uint32_t u = 0; u < SWEEP_UNROLL; u++) {
      idx[u] = bb + u * 32 + lane;
      if (idx[u] < B) sl[u] = load_slot_stream(p.slots, idx[u]);
      else sl[u].key = STC_EMPTY_KEY;
    }
    // the positions of every claimed slot of the pass are requested before
    // any slot is processed
    ClaimPos cp[SWEEP_UNROLL];
#pragma unroll
    for (uint32_t u = 0; u < SWEEP_UNROLL; u++) cp[u] = claim_positions(p, sl[u]);
#pragma unroll
    for (uint32_t u = 0; u < SWEEP_UNROLL; u++) {
      bool emit = idx[u] < B && sweep_slot(p, t, idx[u], sl[u], cp[u], active, fresh);
      uint32_t ball = __ballot_sync(0xffffffffu, emit);
      if (emit) {
        stc_meeting m;
        cantor_decode(sl[u].key, &m.pid_lo, &m.pid_hi);
        m.start = sl[u].start;
        m.end = sl[u].end;
        m.mbr[0] = sl[u].lo_x; m.mbr[1] = sl[u].lo_y; m.mbr[2] = sl[u].hi_x; m.mbr[3] = sl[u].hi_y;
        stage[n + __popc(ball & ((1u << lane) - 1u))] = m;
      }
      n += __popc(ball);
    }
    __syncwarp();
    // room for the next pass (at most WARP_TILE more)
    if (n > WARP_STAGE - WARP_TILE) {
      flush_emits(p, stage, n);
      emitted += n;
      n = 0;
    }
  }
  __syncwarp();
  if (n) {
    flush_emits(p, stage, n);
    emitted += n;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    active += __shfl_xor_sync(0xffffffffu, active, o);
    fresh += __shfl_xor_sync(0xffffffffu, fresh, o);
  }
  if (lane == 0 && active) atomicAdd(&p.st->taken, active);
  if (lane == 0 && fresh) atomicAdd(&p.st->fast_claims, fresh);
  if (lane == 0 && emitted) atomicAdd(&p.st->step_emitted, emitted);
}

// The sweep's grid is SWEEP_WAVES times what the SMs hold at once, so that
// its blocks end and start again every few hundred microseconds: a query
// batch on a stream of higher priority gets SMs when the running wave ends,
// not after the whole 2.8 ms sweep (query p99 under ingest 3.65 -> 1.9 ms at
// 10M objects; the sweep's own time did not change).
static constexpr uint32_t SWEEP_WAVES = 8;

void step_sweep(PipeDev &p, cudaStream_t s) {
  for (uint32_t part = 0; part < p.slices; part++)
    STC_KL k_sweep<<<num_sms() * SWEEP_BLOCKS_PER_SM * SWEEP_WAVES, SWEEP_THREADS, 0, s>>>(p, part, p.slices);
}

}  // namespace stc
