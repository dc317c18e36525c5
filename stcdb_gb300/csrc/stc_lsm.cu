// Memtable append and flush (layout and sequence in stc_lsm.cuh).
//
// Floating-point steps use explicit round-to-nearest intrinsics so that no
// multiply-add is contracted; conversions to integers use the round-toward-
// zero conversions the reference's casts compile to (NaN and negative values
// become 0, large values saturate).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "stc_lsm_kernels.cuh"

namespace stc {

namespace lsmk {

// ---- memtable --------------------------------------------------------------

__global__ void k_lsm_init_obox(uint4 *obox, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) obox[i] = make_uint4(OBOX_INIT, OBOX_INIT, 0u, 0u);
}

__global__ void k_lsm_reset_state(DevState *st) {
  st->kv_count = 0;
  st->lsm_sid_count = 0;
  st->lsm_over_count = 0;
}

// The emission branch of cuda_identify_meetings (cuda/geometry.cu:701-737):
// both directed keys of every meeting the step emitted, the per-object key
// count and box, and sid 1 for both objects of a meeting longer than
// max_meet_time.
__global__ void k_lsm_append(const stc_meeting *emit, unsigned long long E, LsmDev L) {
  DevState *st = L.st;
  if (stc_failed(st)) return;
  unsigned long long total = st->emit_count, n = st->step_emitted;
  if (total > E || n > total) return;  // the sweep has already reported the overflow
  unsigned long long begin = total - n;
  unsigned lane = threadIdx.x & 31u;
  for (unsigned long long i0 = begin + (unsigned long long)blockIdx.x * blockDim.x; i0 < total;
       i0 += (unsigned long long)gridDim.x * blockDim.x) {
    unsigned long long i = i0 + threadIdx.x;
    bool act = i < total;
    stc_meeting m;
    if (act) m = emit[i];
    uint32_t dur = act ? m.end - m.start : 0u;
    if (act && dur > L.max_meet) {
      atomicAdd(&st->lsm_over_count, 1u);
      L.sid[m.pid_lo] = 1;
      L.sid[m.pid_hi] = 1;
    }
    uint32_t ball = __ballot_sync(0xffffffffu, act);
    unsigned long long base = 0;
    if (lane == 0 && ball) base = atomicAdd(&st->kv_count, 2ull * __popc(ball));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (!act) continue;
    unsigned long long idx = base + 2ull * __popc(ball & ((1u << lane) - 1u));
    if (idx + 2 > L.cap) {
      stc_set_error(st, ERR_MEMTABLE, (uint32_t)min(idx - L.cap + 2, 0xFFFFFFFFull));
      continue;
    }
    uint32_t end_rel = m.end - L.end_time_min;
    float4 b = make_float4(m.mbr[0], m.mbr[1], m.mbr[2], m.mbr[3]);
    L.rec[idx] = make_uint4(m.pid_lo, m.pid_hi, dur, end_rel);
    L.rec[idx + 1] = make_uint4(m.pid_hi, m.pid_lo, dur, end_rel);
    L.box[idx] = b;
    L.box[idx + 1] = b;
    uint32_t lo0 = f2u_ref(b.x), lo1 = f2u_ref(b.y), hi0 = f2u_ref(b.z), hi1 = f2u_ref(b.w);
#pragma unroll
    for (int k = 0; k < 2; k++) {
      uint32_t pid = k ? m.pid_hi : m.pid_lo;
      atomicAdd(&L.cnt[pid], 1u);  // objects with keys are counted at the flush
      atomicMin(&L.obox[pid].x, lo0);
      atomicMax(&L.obox[pid].z, hi0);
      atomicMin(&L.obox[pid].y, lo1);
      atomicMax(&L.obox[pid].w, hi1);
    }
  }
}

// ---- flush -----------------------------------------------------------------

__global__ void k_lsm_flush_begin(DevState *st) {
  st->lsm_over_keys = 0;
  st->lsm_max_dur = 0;
  st->lsm_max_end = 0;
  st->lsm_os_min = 1u << 30;  // get_o_limit's initial values (cuda/geometry.cu:966)
  st->lsm_os_max = 0;
}

__global__ void k_lsm_set_counts(unsigned long long *n_dev, unsigned long long a, unsigned long long b,
                                 unsigned long long c) {
  n_dev[0] = a;
  n_dev[1] = b;
  n_dev[2] = c;
}

// set_oid (cuda/geometry.cu:740-767): objects whose key box is larger than
// the area restriction get sid 1; the others a midpoint (x from the low and
// high x, y from the high y taken twice, as the reference does).
__global__ void k_lsm_set_oid(LsmDev L) {
  uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
  // objects with at least one key (the reference counts them as their first
  // key arrives; counted here once instead of at every append)
  const unsigned has = __ballot_sync(0xffffffffu, id < L.N && L.cnt[id] >= 1u);
  if ((threadIdx.x & 31u) == 0 && has) atomicAdd(&L.st->lsm_sid_count, (uint32_t)__popc(has));
  if (id >= L.N) return;
  uint32_t mx = 0, my = 0;
  if (L.cnt[id] >= 1u) {
    uint4 ob = L.obox[id];
    float low0 = u2f_ref(ob.x), high0 = u2f_ref(ob.z), low1 = u2f_ref(ob.y), high1 = u2f_ref(ob.w);
    float area = __fmul_rn(__fsub_rn(high1, low1), __fsub_rn(high0, low0));
    if ((double)area > L.area) {
      atomicAdd(&L.st->lsm_over_count, 1u);
      L.sid[id] = 1;
    } else {
      mx = ob.x / 2 + ob.z / 2;
      my = ob.w / 2 + ob.w / 2;
    }
  }
  L.mid_lo[id] = my;
  L.mid_hi[id] = mx;
  L.sk[0][id] = id;
}

// The partition predicate of cuda/geometry.cu:1779-1796 (sid 1 -> oversize)
// and the largest duration / end offset (the sort's key widths).
__global__ void k_lsm_flags(LsmDev L, unsigned long long K) {
  uint32_t md = 0, me = 0;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < K;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    uint4 r = L.rec[i];
    bool o = L.sid[r.x] == 1;
    L.over[i] = o;
    if (o) agg_inc(&L.st->lsm_over_keys);
    md = max(md, r.z);
    me = max(me, r.w);
  }
  md = warp_max_u32(md);
  me = warp_max_u32(me);
  if ((threadIdx.x & 31u) == 0) {
    atomicMax(&L.st->lsm_max_dur, md);
    atomicMax(&L.st->lsm_max_end, me);
  }
}

__global__ void k_gather_u32(const uint32_t *src, const uint32_t *idx, uint32_t *dst, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[idx[i]];
}

// Slab sort keys: y of the object at position z + j, value j.
__global__ void k_slab_keys(const uint32_t *mid_lo, const uint32_t *oids, uint32_t z, uint32_t R, uint32_t *keys,
                            uint32_t *vals) {
  uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= R) return;
  keys[j] = mid_lo[oids[z + j]];
  vals[j] = j;
}

// Slab of an original position j: x slabs of xcap objects, the last one
// takes the rest (cuda/geometry.cu:1875-1889).
__global__ void k_slab_of(const uint32_t *jv, uint32_t R, uint32_t xcap, uint32_t split, uint32_t *keys) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= R) return;
  keys[i] = min(jv[i] / xcap, split - 1);
}

// make_sid (cuda/geometry.cu:780-796) and get_CTF_capacity (:808-818).
__global__ void k_make_sid(LsmDev L, const uint32_t *oids, const uint32_t *jv, uint32_t z, uint32_t R,
                           uint32_t xcap, uint32_t ycap) {
  extern __shared__ uint32_t s_cap[];
  for (uint32_t c = threadIdx.x; c < L.F; c += blockDim.x) s_cap[c] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x) {
    uint32_t oid = oids[z + jv[i]];
    uint32_t x_index = i / xcap;
    uint32_t y_index = (i - x_index * xcap) / ycap;
    uint16_t sid = (uint16_t)(x_index * L.split + y_index + 2);
    L.sid[oid] = sid;
    uint32_t c = (uint32_t)sid - 2u;
    if (c < L.F) atomicAdd(&s_cap[c], L.cnt[oid]);
  }
  __syncthreads();
  for (uint32_t c = threadIdx.x; c < L.F; c += blockDim.x)
    if (s_cap[c]) atomicAdd(&L.ctf_cap[c], s_cap[c]);
}

// One 32-bit word of the key sort. The order is (over, sid, pid, target,
// duration, end): the CTF keys by their 128-bit key sid:12 | pid:26 |
// target:26 | duration:32 | end:32 (cuda/geometry.cu:724-726, 799-806),
// then the oversize keys by theirs (sid 0). W_LOW and W_HIGH split the order
// in two words: the low target bits, duration and end; then the over flag,
// the object's rank in (sid, pid) order (its pid for an oversize key, whose
// sid counts as 0) and the high target bits.
__device__ __forceinline__ uint32_t low_word(const uint4 &r, const WordSpec &ws) {
  return r.w | (r.z << ws.a) | (r.y << ws.b);  // a = end bits, b = end + duration bits < 32
}
__device__ __forceinline__ uint32_t high_word(const uint4 &r, bool over, const uint32_t *rank, const WordSpec &ws) {
  // a = high target bits, b = low target bits, c = pid bits
  const uint32_t major = over ? r.x : rank[r.x];
  return (over ? 1u << (ws.c + ws.a) : 0u) | (major << ws.a) | (ws.a ? r.y >> ws.b : 0u);
}

__global__ void k_lsm_word(LsmDev L, unsigned long long K, const uint32_t *perm, uint32_t *keys, uint32_t *vals,
                           WordSpec ws) {
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < K;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    uint32_t src = perm ? perm[i] : (uint32_t)i;
    if (!perm) vals[i] = (uint32_t)i;
    uint4 r = L.rec[src];
    uint32_t w;
    switch (ws.kind) {
      case W_END_DUR: w = r.w | (r.z << ws.a); break;
      case W_END: w = r.w; break;
      case W_DUR: w = r.z; break;
      case W_TARGET: w = r.y; break;
      case W_SID_PID: w = r.x | ((L.over[src] ? 0u : (uint32_t)L.sid[r.x]) << ws.a); break;
      case W_PID: w = r.x; break;
      case W_SID: w = L.over[src] ? 0u : (uint32_t)L.sid[r.x]; break;
      default: w = L.over[src]; break;  // W_OVER (W_LOW / W_HIGH go through k_lsm_low_high)
    }
    keys[i] = w;
  }
}

// First pass of the two-word order, in memtable order: the low word as the
// sort key (value = the key's index) and the high word into `hi`, so that
// the second pass gathers one word a key instead of its record, over flag
// and object rank.
__global__ void k_lsm_low_high(LsmDev L, unsigned long long K, uint32_t *keys, uint32_t *vals, uint32_t *hi,
                               WordSpec lo, WordSpec hs, const uint32_t *rank) {
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < K;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const uint4 r = L.rec[i];
    vals[i] = (uint32_t)i;
    keys[i] = low_word(r, lo);
    hi[i] = high_word(r, L.over[i] != 0, rank, hs);
  }
}

// Objects by sid (stable): keys sid, values pid.
__global__ void k_sid_keys(const uint16_t *sid, uint32_t N, uint32_t *keys, uint32_t *vals) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) {
    keys[i] = sid[i];
    vals[i] = i;
  }
}

__global__ void k_rank_of(const uint32_t *order, uint32_t N, uint32_t *rank) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) rank[order[i]] = i;
}

__global__ void k_lsm_gather(LsmDev L, unsigned long long K, const uint32_t *perm) {
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < K;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    uint32_t src = perm[i];
    L.brec[i] = L.rec[src];
    L.bbox[i] = L.box[src];
  }
}

__global__ void k_lsm_limits_init(LsmDev L) {
  uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L.F) return;
  L.lim_box[c] = make_float4(100000.0f, 100000.0f, -100000.0f, -100000.0f);
  L.lim_time[c] = make_uint2(1u << 30, 0u);
}

// cuda_get_limit (cuda/geometry.cu:820-891): per CTF the box of its key
// boxes and the range of its start times, over its key range of the sorted
// keys (the range can reach into the oversize keys, as in the reference).
// LIM_PARTS blocks share a CTF; min and max are exact, so combining their
// results with atomics gives the reference's values in any order.
__global__ void k_lsm_limits(LsmDev L, unsigned long long K) {
  uint32_t c = blockIdx.x;
  unsigned long long a0 = min(L.ctf_first[c], K), b0 = min(L.ctf_first[c + 1], K);
  unsigned long long a = a0 + (b0 - a0) * blockIdx.y / LIM_PARTS;
  unsigned long long b = a0 + (b0 - a0) * (blockIdx.y + 1) / LIM_PARTS;
  if (a >= b) return;
  float lo0 = 100000.0f, lo1 = 100000.0f, hi0 = -100000.0f, hi1 = -100000.0f;
  uint32_t smin = 1u << 30, smax = 0;
  for (unsigned long long k = a + threadIdx.x; k < b; k += blockDim.x) {
    float4 bx = L.bbox[k];
    uint4 r = L.brec[k];
    lo0 = fminf(lo0, bx.x);
    lo1 = fminf(lo1, bx.y);
    hi0 = fmaxf(hi0, bx.z);
    hi1 = fmaxf(hi1, bx.w);
    uint32_t start = r.w + L.end_time_min - r.z;
    smin = min(smin, start);
    smax = max(smax, start);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo0 = fminf(lo0, __shfl_xor_sync(0xffffffffu, lo0, o));
    lo1 = fminf(lo1, __shfl_xor_sync(0xffffffffu, lo1, o));
    hi0 = fmaxf(hi0, __shfl_xor_sync(0xffffffffu, hi0, o));
    hi1 = fmaxf(hi1, __shfl_xor_sync(0xffffffffu, hi1, o));
    smin = min(smin, __shfl_xor_sync(0xffffffffu, smin, o));
    smax = max(smax, __shfl_xor_sync(0xffffffffu, smax, o));
  }
  __shared__ float4 s_box[32];
  __shared__ uint2 s_t[32];
  uint32_t w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if ((threadIdx.x & 31u) == 0) {
    s_box[w] = make_float4(lo0, lo1, hi0, hi1);
    s_t[w] = make_uint2(smin, smax);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float4 r = s_box[0];
    uint2 t = s_t[0];
    for (uint32_t i = 1; i < nw; i++) {
      r.x = fminf(r.x, s_box[i].x);
      r.y = fminf(r.y, s_box[i].y);
      r.z = fmaxf(r.z, s_box[i].z);
      r.w = fmaxf(r.w, s_box[i].w);
      t.x = min(t.x, s_t[i].x);
      t.y = max(t.y, s_t[i].y);
    }
    atomic_min_f(&L.lim_box[c].x, r.x);
    atomic_min_f(&L.lim_box[c].y, r.y);
    atomic_max_f(&L.lim_box[c].z, r.z);
    atomic_max_f(&L.lim_box[c].w, r.w);
    atomicMin(&L.lim_time[c].x, t.x);
    atomicMax(&L.lim_time[c].y, t.y);
  }
}

// get_o_limit and cuda_write_o_bitmap (cuda/geometry.cu:904-955): start
// times of the oversize keys and the edge x edge map bitmap of their boxes
// (in double, relative to the map box; edge is the reference's
// DEFAULT_bitmap_edge, util/util.h:47). Cells past the bitmap are skipped.
__global__ void k_lsm_oversize(LsmDev L, unsigned long long a, unsigned long long b) {
  uint32_t smin = 1u << 30, smax = 0;
  for (unsigned long long k = a + (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; k < b;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    uint4 r = L.brec[k];
    float4 bx = L.bbox[k];
    uint32_t start = r.w + L.end_time_min - r.z;
    smin = min(smin, start);
    smax = max(smax, start);
    double wx = __dsub_rn(L.map[2], L.map[0]), wy = __dsub_rn(L.map[3], L.map[1]);
    const double E = (double)L.edge;
    const uint32_t bits = L.edge * L.edge;
    uint32_t low0 = d2u_cell(__dmul_rn(__ddiv_rn(__dsub_rn((double)bx.x, L.map[0]), wx), E));
    uint32_t low1 = d2u_cell(__dmul_rn(__ddiv_rn(__dsub_rn((double)bx.y, L.map[1]), wy), E));
    uint32_t high0 = d2u_cell(__dmul_rn(__ddiv_rn(__dsub_rn((double)bx.z, L.map[0]), wx), E));
    uint32_t high1 = d2u_cell(__dmul_rn(__ddiv_rn(__dsub_rn((double)bx.w, L.map[1]), wy), E));
    // (i, j) past either bound gives a bit past the bitmap
    high0 = min(high0, bits - 1u);
    high1 = min(high1, L.edge - 1u);
    for (uint32_t i = low0; i <= high0; i++)
      for (uint32_t j = low1; j <= high1; j++) {
        uint32_t bit = i + j * L.edge;
        if (bit < bits) atomicOr(&L.obitmap[bit >> 5], 1u << (bit & 31u));
      }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    smin = min(smin, __shfl_xor_sync(0xffffffffu, smin, o));
    smax = max(smax, __shfl_xor_sync(0xffffffffu, smax, o));
  }
  if ((threadIdx.x & 31u) == 0) {
    atomicMin(&L.st->lsm_os_min, smin);
    atomicMax(&L.st->lsm_os_max, smax);
  }
}

// cuda_write_bitmap (cuda/geometry.cu:957-987) and write_key_and_mbr
// (:1062-1098) per key of the CTF ranges. The pid field keeps the sid above
// it for CTF keys (extract_fields does not mask it, cuda/cuda_util.cuh:164-169);
// oversize keys reached by a range carry none. In compaction mode the cells
// are clamped to the grid and the pid field is the object id alone.
//
// Each block takes one contiguous run of keys, which the CTF ranges split
// into one or a few pieces. Per group of 256 keys, those of the CTF the group
// starts in (the block's current CTF) set their bitmap bits in a shared copy
// of that CTF's bitmap, merged into the global one when the block moves to
// the next CTF, and their packed bytes are staged in shared memory and written
// out as whole 32-bit words; the group's other keys (past a CTF boundary) go
// to global memory directly.

// Bits i + j * x_grid for i in [l0, h0], j in [l1, h1], below 65536: per
// row one contiguous run, set a word at a time. In global memory a word is
// only updated when a bit of the run is still clear.
template <bool SHARED>
__device__ __forceinline__ void set_bitmap_runs(uint32_t *bm, uint32_t l0, uint32_t h0, uint32_t l1, uint32_t h1,
                                                uint32_t x_grid) {
  if (x_grid == 0) h1 = min(h1, l1);  // every row is the same run
  if (l0 > h0) return;
  for (uint32_t j = l1; j <= h1; j++) {
    const unsigned long long a = (unsigned long long)l0 + (unsigned long long)j * x_grid;
    if (a > 65535ull) break;  // later rows start no lower
    const uint32_t lo = (uint32_t)a;
    const uint32_t hi = (uint32_t)min((unsigned long long)h0 + (unsigned long long)j * x_grid, 65535ull);
    for (uint32_t w = lo >> 5; w <= (hi >> 5); w++) {
      const uint32_t b0 = max(lo, w << 5) & 31u, b1 = min(hi, (w << 5) + 31u) & 31u;
      const uint32_t mask = (0xFFFFFFFFu >> (31u - b1)) & (0xFFFFFFFFu << b0);
      if (SHARED) atomicOr(&bm[w], mask);
      else if ((__ldcg(&bm[w]) & mask) != mask) atomicOr(&bm[w], mask);
    }
  }
}

__device__ __forceinline__ uint32_t ctf_of(const unsigned long long *first, uint32_t F, unsigned long long kid,
                                           uint32_t from) {
  // largest c >= from with first[c] <= kid (empty CTFs share their start)
  uint32_t lo = from, hi = F - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi + 1) >> 1;
    if (first[mid] <= kid) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

constexpr uint32_t ENC_STAGE_WORDS = ENC_GROUP * 16 / 4 + 2;

__global__ void __launch_bounds__(ENC_GROUP) k_encode_keys(EncodeArgs L) {
  __shared__ unsigned long long s_first[MAX_CTF + 1];
  __shared__ uint32_t s_bm[STC_BITMAP_BYTES / 4];
  __shared__ uint32_t s_stage[ENC_STAGE_WORDS];
  __shared__ uint32_t s_c0;
  const unsigned long long total = L.total, slim = L.slim;
  for (uint32_t c = threadIdx.x; c <= L.F; c += blockDim.x) s_first[c] = L.ctf_first[c];
  for (uint32_t w = threadIdx.x; w < STC_BITMAP_BYTES / 4; w += blockDim.x) s_bm[w] = 0;
  const unsigned long long per = (total + gridDim.x - 1) / gridDim.x;
  const unsigned long long k0 = min(total, per * blockIdx.x), k1 = min(total, k0 + per);
  uint32_t cur = 0xFFFFFFFFu;  // CTF whose bits s_bm holds
  uint8_t *const stage = (uint8_t *)s_stage;
  for (unsigned long long base = k0; base < k1; base += ENC_GROUP) {
    __syncthreads();  // s_first and s_bm ready; the previous group's staging copied out
    if (threadIdx.x == 0) s_c0 = ctf_of(s_first, L.F, base, 0);
    __syncthreads();
    const uint32_t c0 = s_c0;
    if (c0 != cur) {
      if (cur != 0xFFFFFFFFu) {
        uint32_t *gbm = L.bitmaps + (size_t)cur * (STC_BITMAP_BYTES / 4);
        for (uint32_t w = threadIdx.x; w < STC_BITMAP_BYTES / 4; w += blockDim.x) {
          const uint32_t v = s_bm[w];
          if (v && (__ldcg(&gbm[w]) & v) != v) atomicOr(&gbm[w], v);
          s_bm[w] = 0;
        }
      }
      cur = c0;
      __syncthreads();
    }
    // the group's keys of CTF c0 are [base, g1)
    const unsigned long long g1 = min(min(base + ENC_GROUP, k1), s_first[c0 + 1] > base ? s_first[c0 + 1] : k1);
    const stc_ctf &t0 = L.ctfs[c0];
    const uint32_t kb0 = t0.key_bit / 8u;
    const unsigned long long g_start = t0.key_offset + (base - s_first[c0]) * kb0;  // byte of the group's first key
    const uint32_t lead = (uint32_t)(g_start & 3ull);
    const unsigned long long kid = base + threadIdx.x;
    if (kid < k1) {
      const uint32_t c = kid < g1 ? c0 : ctf_of(s_first, L.F, kid, c0);
      const stc_ctf &t = L.ctfs[c];
      float4 b = L.bbox[kid];
      uint4 r = L.brec[kid];
      float wx = __fsub_rn(t.mbr[2], t.mbr[0]), wy = __fsub_rn(t.mbr[3], t.mbr[1]);
      float gx = (float)t.x_grid, gy = (float)t.y_grid;
      uint32_t l0 = __float2uint_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.x, t.mbr[0]), wx), gx));
      uint32_t l1 = __float2uint_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.y, t.mbr[1]), wy), gy));
      uint32_t h0 = __float2uint_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.z, t.mbr[0]), wx), gx));
      uint32_t h1 = __float2uint_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.w, t.mbr[1]), wy), gy));
      if (L.compact) {
        // cells clamped to the grid (the merged block's rule)
        h0 = min(h0, (uint32_t)t.x_grid - 1u);
        h1 = min(h1, (uint32_t)t.y_grid - 1u);
      } else {
        // a box inside the CTF box gives cells <= the grid size; cells past
        // the 8 KB slot are skipped, so the loops stop where every bit would be
        h0 = min(h0, 65535u);
        h1 = min(h1, 65535u / max(1u, (uint32_t)t.x_grid));
      }
      if (c == c0) set_bitmap_runs<true>(s_bm, l0, h0, l1, h1, t.x_grid);
      else set_bitmap_runs<false>(L.bitmaps + (size_t)c * (STC_BITMAP_BYTES / 4), l0, h0, l1, h1, t.x_grid);
      unsigned long long pid_field =
          L.compact || kid >= slim ? r.x : (((unsigned long long)L.sid[r.x] << 26) | r.x);
      unsigned long long vm = serialize_mbr_dev(b, t);
      uint32_t s_end = t.mbr_bit, s_dur = t.end_bit + t.mbr_bit, s_tgt = t.duration_bit + t.end_bit + t.mbr_bit;
      uint32_t s_pid = t.id_bit + s_tgt;
      unsigned __int128 k = ((unsigned __int128)pid_field << s_pid) + ((unsigned __int128)r.y << s_tgt) +
                            ((unsigned __int128)r.z << s_dur) + ((unsigned __int128)r.w << s_end) +
                            (unsigned __int128)vm;
      const unsigned long long lo = (unsigned long long)k, hi = (unsigned long long)(k >> 64);
      const uint32_t kb = t.key_bit / 8u;
      if (c == c0) {
        uint8_t *dst = stage + lead + threadIdx.x * kb0;
#pragma unroll
        for (uint32_t i = 0; i < 16; i++)
          if (i < kb) dst[i] = (uint8_t)(i < 8 ? lo >> (8 * i) : hi >> (8 * (i - 8)));
      } else {
        uint8_t *dst = L.kbytes + t.key_offset + (kid - s_first[c]) * kb;
#pragma unroll
        for (uint32_t i = 0; i < 16; i++)
          if (i < kb) dst[i] = (uint8_t)(i < 8 ? lo >> (8 * i) : hi >> (8 * (i - 8)));
      }
    }
    __syncthreads();
    // the staged bytes [lead, lead + len) go to [g_start, g_start + len):
    // whole words where all four bytes are the group's, bytes at the ends
    const uint32_t len = (uint32_t)(g1 - base) * kb0, end = lead + len;
    uint32_t *gw = (uint32_t *)(L.kbytes + (g_start - lead));
    for (uint32_t w = threadIdx.x; w < (end + 3) / 4; w += blockDim.x) {
      const uint32_t b0 = 4 * w, b1 = b0 + 4;
      if (b0 >= lead && b1 <= end) {
        gw[w] = s_stage[w];
      } else {
        for (uint32_t x = max(b0, lead); x < min(b1, end); x++) L.kbytes[g_start - lead + x] = stage[x];
      }
    }
  }
  __syncthreads();
  if (cur != 0xFFFFFFFFu) {
    uint32_t *gbm = L.bitmaps + (size_t)cur * (STC_BITMAP_BYTES / 4);
    for (uint32_t w = threadIdx.x; w < STC_BITMAP_BYTES / 4; w += blockDim.x) {
      const uint32_t v = s_bm[w];
      if (v && (__ldcg(&gbm[w]) & v) != v) atomicOr(&gbm[w], v);
    }
  }
}

}  // namespace lsmk

using namespace lsmk;

static stc_status cuda_err(cudaError_t e, const char *where, std::string &err) {
  err = std::string(where) + ": " + cudaGetErrorString(e);
  return STC_ERR_CUDA;
}

// ---- host ------------------------------------------------------------------

static uint32_t min_bits_to_store(uint32_t v) {  // util/util.h:528-533
  if (v == 0) return 1;
  return (uint32_t)std::log2((double)v) + 1;
}
static uint32_t sat_u32(double x) {
  if (!(x > 0.0)) return 0;
  return x >= 4294967296.0 ? 0xFFFFFFFFu : (uint32_t)x;
}
static int32_t sat_i32(double x) {
  if (x != x) return 0;
  if (x <= -2147483648.0) return INT32_MIN;
  return x >= 2147483647.0 ? INT32_MAX : (int32_t)x;
}

bool ctf_bits(const float mbr[4], const double map[4], uint32_t num_objects, uint32_t max_meet_time,
              stc_ctf *c) {
  c->id_bit = (uint16_t)min_bits_to_store(num_objects);
  c->duration_bit = (uint16_t)min_bits_to_store(max_meet_time - 1);
  c->end_bit = c->duration_bit;
  // box corner at about 1/3000 (x) and 1/4200 (y) of the map
  double gx = (map[2] - map[0]) / 3000, gy = (map[3] - map[1]) / 4200;
  float wx = mbr[2] - mbr[0], wy = mbr[3] - mbr[1];
  uint32_t nx = sat_u32((double)wx / gx), ny = sat_u32((double)wy / gy);
  c->low_x_bit = (uint16_t)min_bits_to_store(std::max<uint32_t>(nx, 1) - 1);
  c->low_y_bit = (uint16_t)min_bits_to_store(std::max<uint32_t>(ny, 1) - 1);
  c->edge_bit = std::max(c->low_x_bit, c->low_y_bit);
  c->mbr_bit = (uint16_t)(c->low_x_bit + c->low_y_bit + 2 * c->edge_bit);
  uint32_t bits = 2u * c->id_bit + c->duration_bit + c->end_bit + c->mbr_bit;
  c->key_bit = (uint16_t)((bits + 7) / 8 * 8);
  // bitmap cells of about 100 m: 300 x 420 over the map, at least 32 a side,
  // both sides cut to 255 once either reaches 256
  int32_t ow = sat_i32((double)wx / (map[2] - map[0]) * 300);
  int32_t oh = sat_i32((double)wy / (map[3] - map[1]) * 420);
  int32_t xg = std::max(ow + 1, 32), yg = std::max(oh + 1, 32);
  if (xg >= 256 || yg >= 256) {
    xg = std::min(ow + 1, 255);
    yg = std::min(oh + 1, 255);
  }
  c->x_grid = (uint16_t)xg;
  c->y_grid = (uint16_t)yg;
  c->bitmap_bytes = ((uint32_t)c->x_grid * c->y_grid + 7) / 8;
  return c->mbr_bit <= 64 && bits <= 128;
}

size_t lsm_sort_words(const LsmDev &L) { return std::max<size_t>((size_t)L.cap, (size_t)L.N); }

static void reset_memtable(LsmDev &L, cudaStream_t s) {
  cudaMemsetAsync(L.cnt, 0, (size_t)L.N * sizeof(uint32_t), s);
  cudaMemsetAsync(L.sid, 0, (size_t)L.N * sizeof(uint16_t), s);
  STC_KL k_lsm_init_obox<<<nblk(L.N), 256, 0, s>>>(L.obox, L.N);
  STC_KL k_lsm_reset_state<<<1, 1, 0, s>>>(L.st);
}

void lsm_init(LsmDev &L, cudaStream_t s) {
  reset_memtable(L, s);
  cudaMemsetAsync(L.bsid, 0, (size_t)L.N * sizeof(uint16_t), s);
}

void lsm_append(const PipeDev &p, const LsmDev &L, cudaStream_t s) {
  STC_KL k_lsm_append<<<lsm_grid(), 256, 0, s>>>(p.emit, p.E, L);
}

void lsmk::sort_keys(const LsmDev &L, unsigned long long K, uint32_t N, uint32_t max_end, uint32_t max_dur,
                     uint32_t sid_bits, cudaStream_t s) {
  if (!K) return;
  uint32_t *const *sk = L.sk;
  WordSpec words[8];
  int nw = 0;
  const uint32_t eb = bits_for(max_end), db = bits_for(max_dur), ib = bits_for(N > 1 ? N - 1 : 1);
  const uint32_t low_t = eb + db < 32 ? 32 - eb - db : 0, th = ib > low_t ? ib - low_t : 0;
  const uint32_t *rank = nullptr;
  if (eb + db < 32 && 1 + ib + th <= 32) {
    // two words; the rank of each object in (sid, pid) order in sk[6]
    STC_KL k_sid_keys<<<nblk(N), 256, 0, s>>>(L.sid, N, sk[0], sk[1]);
    sort_words(L, sk[0], sk[1], sk[2], sk[3], sk[4], sk[5], 0, N, sid_bits, s);
    STC_KL k_rank_of<<<nblk(N), 256, 0, s>>>(sk[3], N, sk[6]);
    rank = sk[6];
    words[nw++] = {W_LOW, eb, eb + db, 0u, std::min(32u, eb + db + ib)};
    words[nw++] = {W_HIGH, th, low_t, ib, 1 + ib + th};
  } else {
    const uint32_t sb = sid_bits;
    if (eb + db <= 32) words[nw++] = {W_END_DUR, eb, 0u, 0u, eb + db};
    else { words[nw++] = {W_END, 0u, 0u, 0u, eb}; words[nw++] = {W_DUR, 0u, 0u, 0u, db}; }
    words[nw++] = {W_TARGET, 0u, 0u, 0u, ib};
    if (ib + sb <= 32) words[nw++] = {W_SID_PID, ib, 0u, 0u, ib + sb};
    else { words[nw++] = {W_PID, 0u, 0u, 0u, ib}; words[nw++] = {W_SID, 0u, 0u, 0u, sb}; }
    words[nw++] = {W_OVER, 0u, 0u, 0u, 1u};
  }
  const uint32_t *perm = nullptr;
  if (rank) {
    // the sorted records' buffer is free until the final gather: it holds
    // the high words meanwhile
    uint32_t *hi = reinterpret_cast<uint32_t *>(L.brec);
    STC_KL k_lsm_low_high<<<lsm_grid(), 256, 0, s>>>(L, K, sk[0], sk[1], hi, words[0], words[1], rank);
    sort_words(L, sk[0], sk[1], sk[2], sk[3], sk[4], sk[5], 2, K, words[0].bits, s);
    STC_KL k_gather_u32<<<nblk(K), 256, 0, s>>>(hi, sk[3], sk[0], (uint32_t)K);
    sort_words(L, sk[0], sk[3], sk[2], sk[1], sk[4], sk[5], 2, K, words[1].bits, s);
    perm = sk[1];
  } else {
    uint32_t *vbuf[2] = {sk[1], sk[3]};
    for (int w = 0; w < nw; w++) {
      uint32_t *vin = vbuf[w & 1], *vout = vbuf[(w + 1) & 1];
      STC_KL k_lsm_word<<<lsm_grid(), 256, 0, s>>>(L, K, perm, sk[0], perm ? nullptr : vin, words[w]);
      sort_words(L, sk[0], perm ? perm : vin, sk[2], vout, sk[4], sk[5], 2, K, words[w].bits, s);
      perm = vout;
    }
  }
  STC_KL k_lsm_gather<<<lsm_grid(), 256, 0, s>>>(L, K, perm);
}

// Stable sort of n (key, value) words; returns the buffers holding the result.
void lsmk::sort_words(const LsmDev &L, const uint32_t *k, const uint32_t *v, uint32_t *ko, uint32_t *vo,
                      uint32_t *kt, uint32_t *vt, int count_slot, size_t n, uint32_t bits, cudaStream_t s) {
  radix_sort_u32(k, v, ko, vo, kt, vt, L.n_dev + count_slot, n, (int)bits, L.hist, L.scan, s);
}

stc_status lsm_flush(LsmDev &L, LsmHost &H, uint32_t t, cudaStream_t s, DevState *st_host, std::string &err,
                     const cudaEvent_t *marks) {
  auto mark = [&](int i) {
    if (marks) cudaEventRecord(marks[i], s);
  };
  cudaError_t e;
  auto read_state = [&]() -> cudaError_t {
    cudaError_t r = cudaMemcpyAsync(st_host, L.st, sizeof(DevState), cudaMemcpyDeviceToHost, s);
    if (r == cudaSuccess) r = cudaStreamSynchronize(s);
    if (r == cudaSuccess) r = cudaGetLastError();
    return r;
  };
  if ((e = read_state()) != cudaSuccess) return cuda_err(e, "flush", err);
  const unsigned long long K = st_host->kv_count;
  const uint32_t N = L.N, F = L.F, S = L.split;
  uint32_t **sk = L.sk;
  STC_KL k_lsm_flush_begin<<<1, 1, 0, s>>>(L.st);
  cudaMemsetAsync(L.ctf_cap, 0, (size_t)F * sizeof(uint32_t), s);
  cudaMemsetAsync(L.bitmaps, 0, (size_t)F * STC_BITMAP_BYTES, s);
  cudaMemsetAsync(L.obitmap, 0, STC_MAP_BITMAP_BYTES(L.edge), s);
  // 1. object boxes -> oversize objects and STR midpoints; key partition flags
  STC_KL k_lsm_set_oid<<<nblk(N), 256, 0, s>>>(L);
  STC_KL k_lsm_flags<<<lsm_grid(), 256, 0, s>>>(L, K);
  // 2. order objects by midpoint (x, then y): stable sort by y, then by x
  STC_KL k_lsm_set_counts<<<1, 1, 0, s>>>(L.n_dev, N, 0, K);
  sort_words(L, L.mid_lo, sk[0], sk[1], sk[2], sk[3], sk[4], 0, N, 32, s);
  STC_KL k_gather_u32<<<nblk(N), 256, 0, s>>>(L.mid_hi, sk[2], sk[5], N);
  sort_words(L, sk[5], sk[2], sk[1], sk[6], sk[3], sk[4], 0, N, 32, s);  // sk[6]: objects in STR order
  if ((e = read_state()) != cudaSuccess) return cuda_err(e, "flush", err);
  const uint32_t sid_count = st_host->lsm_sid_count, over_count = st_host->lsm_over_count;
  const unsigned long long over_keys = st_host->lsm_over_keys;
  const uint32_t max_dur = st_host->lsm_max_dur, max_end = st_host->lsm_max_end;
  // 3. y slabs and sids (cuda/geometry.cu:1871-1898): positions < z hold the
  // objects without keys and the oversize ones
  const uint32_t z = (N - sid_count) + over_count;
  const uint32_t xcap = (sid_count - over_count) / S + 1, ycap = xcap / S + 1;
  const uint32_t R = z < N ? N - z : 0;
  if (R) {
    STC_KL k_lsm_set_counts<<<1, 1, 0, s>>>(L.n_dev, N, R, K);
    STC_KL k_slab_keys<<<nblk(R), 256, 0, s>>>(L.mid_lo, sk[6], z, R, sk[0], sk[2]);
    sort_words(L, sk[0], sk[2], sk[1], sk[5], sk[3], sk[4], 1, R, 32, s);
    STC_KL k_slab_of<<<nblk(R), 256, 0, s>>>(sk[5], R, xcap, S, sk[0]);
    sort_words(L, sk[0], sk[5], sk[1], sk[2], sk[3], sk[4], 1, R, bits_for(S - 1), s);
    STC_KL k_make_sid<<<num_sms(), 512, F * sizeof(uint32_t), s>>>(L, sk[6], sk[2], z, R, xcap, ycap);
  }
  mark(0);
  // 4. sort the keys: (over, sid, pid, target, duration, end)
  sort_keys(L, K, N, max_end, max_dur, bits_for(S * S + 1), s);
  mark(1);
  // 5. CTF key ranges
  std::vector<uint32_t> cap(F);
  e = cudaMemcpyAsync(cap.data(), L.ctf_cap, (size_t)F * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_err(e, "flush", err);
  std::vector<unsigned long long> first(F + 1, 0);
  for (uint32_t c = 0; c < F; c++) first[c + 1] = first[c] + cap[c];
  const unsigned long long slim = K - over_keys;
  const unsigned long long total = std::min<unsigned long long>(first[F], K);
  cudaMemcpyAsync(L.ctf_first, first.data(), (F + 1) * sizeof(unsigned long long), cudaMemcpyHostToDevice, s);
  STC_KL k_lsm_limits_init<<<nblk(F), 256, 0, s>>>(L);
  STC_KL k_lsm_limits<<<dim3(F, LIM_PARTS), 256, 0, s>>>(L, K);
  if (K > slim) STC_KL k_lsm_oversize<<<lsm_grid(), 256, 0, s>>>(L, slim, K);
  std::vector<float4> lb(F);
  std::vector<uint2> lt(F);
  e = cudaMemcpyAsync(lb.data(), L.lim_box, F * sizeof(float4), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(lt.data(), L.lim_time, F * sizeof(uint2), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = read_state();
  if (e != cudaSuccess) return cuda_err(e, "flush", err);
  // 6. per-CTF metadata on the host, as the reference (cuda/geometry.cu:1960-1963)
  H.ctfs.assign(F, stc_ctf{});
  unsigned long long off = 0;
  bool fits = true;
  for (uint32_t c = 0; c < F; c++) {
    stc_ctf &x = H.ctfs[c];
    x.mbr[0] = lb[c].x; x.mbr[1] = lb[c].y; x.mbr[2] = lb[c].z; x.mbr[3] = lb[c].w;
    x.kv_count = cap[c];
    x.start_time_min = lt[c].x;
    x.start_time_max = lt[c].y;
    x.end_time_min = L.end_time_min;
    x.end_time_max = t;
    fits &= ctf_bits(x.mbr, L.map, N, L.max_meet, &x);
    x.first_key = first[c];
    x.key_offset = off;
    off += (unsigned long long)cap[c] * (x.key_bit / 8u);
  }
  if (!fits) {
    err = "flush: a CTF key needs more than 64 box bits or 128 bits in all";
    return STC_ERR_CAPACITY;
  }
  if (off > L.cap * 16ull) {
    err = "flush: packed keys exceed the key buffer";
    return STC_ERR_CAPACITY;
  }
  cudaMemcpyAsync(L.ctfs, H.ctfs.data(), F * sizeof(stc_ctf), cudaMemcpyHostToDevice, s);
  mark(2);
  // 7. bitmaps and packed keys
  if (total)
    STC_KL k_encode_keys<<<lsm_grid(), ENC_GROUP, 0, s>>>(
        EncodeArgs{L.brec, L.bbox, L.ctfs, L.ctf_first, L.sid, L.bitmaps, L.kbytes, total, slim, L.F, false});
  mark(3);
  // 8. keep the sids of the block; empty the memtable
  cudaMemcpyAsync(L.bsid, L.sid, (size_t)N * sizeof(uint16_t), cudaMemcpyDeviceToDevice, s);
  stc_ctb_info in{};
  in.index = H.next_index;
  in.ctf_count = F;
  in.flush_time = t;
  in.end_time_min = L.end_time_min;
  in.kv_count = K;
  in.ctf_kv_count = slim;
  in.oversize_kv_count = over_keys;
  in.key_bytes = off;
  in.sid_count = sid_count;
  in.oversize_oid_count = st_host->lsm_over_count;
  in.o_start_time_min = st_host->lsm_os_min;
  in.o_start_time_max = st_host->lsm_os_max;
  in.o_end_time_min = L.end_time_min;
  in.o_end_time_max = t;
  in.bitmap_edge = L.edge;
  reset_memtable(L, s);  // after the encode on the same stream, which reads the sids
  if ((e = read_state()) != cudaSuccess) return cuda_err(e, "flush", err);
  H.info = in;
  H.has_block = true;
  H.flushes++;
  H.next_index++;
  L.end_time_min = t;  // straight_dump: the next block starts at the flush step (process.cpp:271)
  return STC_OK;
}

}  // namespace stc
