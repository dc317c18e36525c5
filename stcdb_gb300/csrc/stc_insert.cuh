// Ordered insertion of new meetings into the meeting table (shared by the
// refinement kernel and the candidate pass of stc_meetings.cu).
//
// The reference inserts hits one by one in its processing order with linear
// probing from key % B and clears expired slots without tombstones
// (tracing/refinement.cpp:37-55, tracing/meeting.cpp:47-67). Which slot a new
// key takes -- and so whether a later probe for a live meeting crosses a
// cleared slot and restarts it -- depends on that order. It is reproduced
// exactly:
//
//   S0 is the table as it stood after the previous sweep; its keys do not
//   change during a step. A key found in its probe chain before the first
//   S0-empty slot is extended in place. Every other key walks on from that
//   slot: slots holding other S0 keys are passed, its own S0 entry ends the
//   walk (the meeting is extended there), and each S0-empty slot is contended
//   by priority = the key's first position in the reference's sequential
//   order. A claim word (key | CLAIM_BIT, priority) is installed with a
//   128-bit CAS; a lower priority evicts a higher one and the evicting thread
//   carries the evicted key on from the next slot. Slots prefer lower
//   priorities and keys prefer earlier slots, so this deferred acceptance
//   converges, independent of timing, to the unique stable assignment -- the
//   one produced by inserting the keys one by one in priority order.
//
// A pair can be produced twice in one step only by two border units that
// target each other's leaves; such keys first merge their instances (minimum
// priority) in the candidate set and walk after the refinement. All other
// keys walk as soon as they are found.
#pragma once
#include "stc_pipeline.cuh"

namespace stc {

// (key, claim) pair of a slot in one 16-byte load at L2 (claims change during
// the walk phase; a torn or stale value only makes a CAS fail and retry).
__device__ __forceinline__ U128 load_slot_pair(const Slot *s) {
  ulonglong2 v = __ldcg((const ulonglong2 *)s);
  U128 r;
  r.lo = v.x;
  r.hi = v.y;
  return r;
}

// Extends an existing meeting found by an ordered walk: end = t and the MBR
// grows by both objects' current float positions (cuda/geometry.cu:474-478).
__device__ __forceinline__ void extend_found(const PipeDev &p, Slot *s, unsigned long long key, uint32_t t) {
  uint32_t a, b;
  cantor_decode(key, &a, &b);
  float2 fa = p.fxy[a], fb = p.fxy[b];
  s->end = t;
  float lx = fminf(fa.x, fb.x), ly = fminf(fa.y, fb.y), hx = fmaxf(fa.x, fb.x), hy = fmaxf(fa.y, fb.y);
  if (lx < s->lo_x) atomic_min_f(&s->lo_x, lx);
  if (ly < s->lo_y) atomic_min_f(&s->lo_y, ly);
  if (hx > s->hi_x) atomic_max_f(&s->hi_x, hx);
  if (hy > s->hi_y) atomic_max_f(&s->hi_y, hy);
}

// Ordered walk of `key` with priority `prio` starting at `slot` (every slot
// before it in the key's chain holds another S0 key). `first`, when given,
// is a recent read of that slot's (key, claim) pair and saves one round trip
// (a stale value only makes the first CAS fail and retry). Returns false if
// the walk exceeded its bound.
__device__ inline bool ordered_walk(const PipeDev &p, unsigned long long key, unsigned long long prio,
                                    unsigned long long slot, uint32_t t, const U128 *first = nullptr) {
  const unsigned long long limit = STC_PROBE_LIMIT * 4;
  for (unsigned long long steps = 0; steps < limit; steps++) {
    Slot *s = &p.slots[slot];
    U128 cur = (steps == 0 && first) ? *first : load_slot_pair(s);
    if (cur.lo == key) {  // its own live entry
      extend_found(p, s, key, t);
      return true;
    }
    if (cur.lo != STC_EMPTY_KEY && !(cur.lo & STC_CLAIM_BIT)) {
      slot = slot + 1 == p.B ? 0 : slot + 1;
      continue;
    }
    bool advance = false;
    while (!advance) {
      if (cur.lo == STC_EMPTY_KEY) {
        U128 want = {key | STC_CLAIM_BIT, prio};
        U128 old = atomicCAS((U128 *)s, cur, want);
        if (old.lo == cur.lo && old.hi == cur.hi) return true;  // settled: a new meeting
        cur = old;
        continue;
      }
      unsigned long long other = cur.hi;  // claimed by another key
      if (prio < other) {
        U128 want = {key | STC_CLAIM_BIT, prio};
        U128 old = atomicCAS((U128 *)s, cur, want);
        if (old.lo == cur.lo && old.hi == cur.hi) {
          key = cur.lo & ~STC_CLAIM_BIT;  // carry the evicted key onward
          prio = other;
          advance = true;
        } else {
          cur = old;
        }
      } else {
        advance = true;  // lost this slot
      }
    }
    slot = slot + 1 == p.B ? 0 : slot + 1;
  }
  return false;
}

}  // namespace stc
