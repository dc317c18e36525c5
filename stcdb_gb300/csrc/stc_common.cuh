// Shared device-side definitions of the GB300 co-occurrence pipeline.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "stc.h"
#include "stc_refmath.h"

#define STC_CLAIM_BIT (1ULL << 63)
#define STC_INIT_LO 100000.0f
#define STC_INIT_HI -100000.0f
#define STC_NONE 0xFFFFFFFFu
#define STC_ORDER_SHIFT 24          // order = unit_rank << 24 | member index
#define STC_MAX_LEAF_CAP (1u << 16)    // leaf list capacity bound (tile counts fit in 32 bits)
#define STC_MAX_DEPTH 96            // descent / lookup depth bound
#define STC_PROBE_LIMIT (1ULL << 16)  // longest probe walk before the table counts as full

enum { NODE_INVALID = 0, NODE_BRANCH = 1, NODE_LEAF = 2 };  // index/QTree.h:43-47

// Device error codes (stored in DevState::error, first one wins).
enum {
  ERR_NONE = 0,
  ERR_DESCENT = 1,     // descent reached an invalid node or ran too deep
  ERR_UNITS = 2,       // border checking units exceed refine_size * N
  ERR_PROBE = 3,       // meeting table probe walk exceeded its bound (table full)
  ERR_CAND = 4,        // candidate set / list full
  ERR_DA = 5,          // ordered insertion exceeded its bound
  ERR_EMIT = 6,        // emit buffer full
  ERR_SCHEMA = 7,      // schema or grid stack exhausted
  ERR_LOOKUP = 8,      // border lookup stack overflow
  ERR_BUILD = 9,       // initial quadtree build exceeded capacity
  ERR_MEMTABLE = 10,   // memtable full
  ERR_COMPACT = 11,    // a key to compact lies outside its CTF or names an unknown object
};

// One meeting-table slot (32 B; the reference's meeting_unit of
// tracing/workbench.h:62-83 with the f_box of cuda/geometry.cu).
// While an ordered insertion runs, an empty slot's (start, end) word holds
// the priority of the key claiming it and the key carries STC_CLAIM_BIT.
struct __align__(32) Slot {
  unsigned long long key;
  uint32_t start, end;
  float lo_x, lo_y, hi_x, hi_y;
};

// Distinct keys of one step that were not found by a plain probe.
struct __align__(32) Cand {
  unsigned long long key;
  unsigned long long order;   // first occurrence in the reference's processing order
  float lo_x, lo_y, hi_x, hi_y;
};

// Quadtree node geometry (index/QTree.h:49-62 QTSchema, split in two arrays).
struct __align__(64) Node {
  double mid_x, mid_y, lo_x, lo_y, hi_x, hi_y;
  uint32_t child[4];
};

struct NodeMeta {
  int16_t type, level, overflow, underflow;
  uint32_t grid_id;
  uint32_t parent;
};

// One pair within reach found by the refinement, waiting to be applied to
// the meeting table: the pair (a < b; a = STC_NONE marks an unused record),
// its priority and its MBR contribution, the box of the two objects' float
// positions of the step (fxy; lo = fminf(a's, b's), hi = fmaxf(a's, b's)).
// The key cantor(a, b) is rebuilt when applied. Carrying the box saves the
// table update two dependent random reads of fxy per extended meeting.
struct __align__(32) HitRec {
  uint32_t a, b;
  unsigned long long order;  // bit 63: the pair may occur twice this step
  float lo_x, lo_y, hi_x, hi_y;
};

struct __align__(16) U128 {
  unsigned long long lo, hi;
};

// Small device-resident control block.
struct DevState {
  uint32_t schema_stack_index, grids_stack_index;
  uint32_t error, error_info;
  unsigned long long border_units;
  unsigned long long jobs_total;
  unsigned long long job_next;
  unsigned long long cand_count;
  unsigned long long emit_count;      // records in the emit buffer (pending drain)
  unsigned long long tests, exact_tests, hits, ambiguous;
  unsigned long long taken;
  unsigned long long step_emitted;
  unsigned long long da_iters;
  uint32_t splits, merges, events, overflow_objects;
  uint32_t build_nodes, build_leaves, build_active, build_level;
  uint32_t work_next;                 // generic persistent-kernel work counter
  uint32_t step_t;                    // time of the step in flight (set at its start)
  uint32_t pad[2];
  unsigned long long border_points;   // points whose lookup starts above their leaf
  unsigned long long fast_claims;     // new meetings started this step (claims finalised by the sweep)
  unsigned long long hit_count;       // hits appended to the hit buffer this step
  uint32_t schema_path;               // 1 parallel replay, 2 serial (cascade), 0 serial (other)
  uint32_t pad2;
  // memtable (stc_lsm.cu)
  unsigned long long kv_count;        // directed keys in the memtable
  unsigned long long lsm_over_keys;   // keys partitioned to the oversize buffer (flush)
  uint32_t lsm_sid_count;             // objects with at least one key
  uint32_t lsm_over_count;            // the reference's oversize_oid_count
  uint32_t lsm_max_dur, lsm_max_end;  // largest duration / end offset (flush sort widths)
  uint32_t lsm_os_min, lsm_os_max;    // oversize buffer start times (flush)
};

__device__ __forceinline__ void stc_set_error(DevState *st, uint32_t code, uint32_t info) {
  if (atomicCAS(&st->error, 0u, code) == 0u) st->error_info = info;
}

// Float min/max on the IEEE bit pattern (valid for any mix of signs, no NaN).
__device__ __forceinline__ void atomic_min_f(float *a, float v) {
  if (v >= 0.0f) atomicMin((int *)a, __float_as_int(v));
  else atomicMax((unsigned int *)a, __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float *a, float v) {
  if (v >= 0.0f) atomicMax((int *)a, __float_as_int(v));
  else atomicMin((unsigned int *)a, __float_as_uint(v));
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// x % d for a fixed divisor with m = ceil(2^64 / d) (computed on the host):
// the multiply-high quotient is exact or one too large; 64-bit division
// would run through the FP64 pipe.
__device__ __forceinline__ unsigned long long fast_mod(unsigned long long x, unsigned long long d,
                                                       unsigned long long m) {
  unsigned long long q = __umul64hi(x, m);
  unsigned long long r = x - q * d;
  return (long long)r < 0 ? r + d : r;
}

__device__ __forceinline__ bool stc_failed(const DevState *st) {
  return *(volatile const uint32_t *)&st->error != 0u;
}

// Warp-aggregated fetch-add of 1 on a global counter by the lanes that reach
// this call together.
__device__ __forceinline__ unsigned long long agg_inc(unsigned long long *ctr) {
  unsigned m = __activemask();
  unsigned lane = threadIdx.x & 31u;
  int leader = __ffs(m) - 1;
  unsigned long long base = 0;
  if ((int)lane == leader) base = atomicAdd(ctr, (unsigned long long)__popc(m));
  base = __shfl_sync(m, base, leader);
  return base + __popc(m & ((1u << lane) - 1u));
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z ^= z >> 33;
  z *= 0xff51afd7ed558ccdULL;
  z ^= z >> 33;
  z *= 0xc4ceb9fe1a85ec53ULL;
  z ^= z >> 33;
  return z;
}

// Exact integer inverse of the Cantor pairing (util/util.h:72-78 uses a
// double sqrt, which is exact only while 8z+1 < 2^53). 64-bit integer <->
// float conversions run on the FP64 pipe, so the first guess comes from the
// top 32 bits in fp32 (relative error ~2^-22, i.e. a few units for
// v < 2^62); exact integer steps correct it.
__device__ __forceinline__ void cantor_decode(unsigned long long z, uint32_t *a, uint32_t *b) {
  unsigned long long v = 8ULL * z + 1ULL;
  int sh = 64 - __clzll(v);
  sh = sh > 32 ? ((sh - 32 + 1) & ~1) : 0;  // even shift keeps sqrt(v >> sh) * 2^(sh/2)
  float fv = __uint2float_rn((uint32_t)(v >> sh));
  // scale in fp32 before rounding to an integer (r < 2^30 for v < 2^60)
  float rf = sqrtf(fv) * __int_as_float((127 + sh / 2) << 23);
  unsigned long long r = __float2uint_rn(rf);
  while (r * r > v) r--;
  while ((r + 1) * (r + 1) <= v) r++;
  unsigned long long w = (r - 1) / 2;
  unsigned long long t = (w * w + w) / 2;
  *b = (uint32_t)(z - t);
  *a = (uint32_t)(w - (z - t));
}

// metres per degree of longitude at latitude y (1/dpml), single precision;
// used only by the conservative pre-filter, never for a decision by itself.
__device__ __forceinline__ float metres_per_deg_lon_f(double y) {
  float absla = (float)fabs(y);
  float arg = (90.0f - absla) * (3.14159265f / 180.0f);
  return sinf(arg) * 111322.2222222f;
}

#define STC_SLAT_F 111322.2222222f   // metres per degree of latitude (1/dpm_lat)
#define STC_SMAX_F 111322.2222222f   // upper bound of metres per degree of longitude

// ---------------------------------------------------------------------------
namespace stc {

// Kernel launches issued by this thread (counted per step in stc_stats).
extern thread_local unsigned long long tl_launches;

// Streaming multiprocessors of the current device
// (cudaDevAttrMultiProcessorCount, looked up once per device): grid-stride
// launches are sized in multiples of it.
int num_sms();

}  // namespace stc

// Prefix for every kernel launch statement: `STC_KL k<<<g, b, 0, s>>>(...);`
#define STC_KL ::stc::tl_launches++,

// Primitives implemented in stc_sort.cu.
#define STC_SCAN_TILE 2048  // items per scan block
#define STC_RS_TILE 4096    // items per radix-sort block
namespace stc {

// Exclusive scan of n uint32 values (in place allowed). total (device ptr,
// optional) receives the sum as uint64. tmp must hold scan_tmp_words(n) words.
size_t scan_tmp_words(size_t n);
void exclusive_scan_u32(const uint32_t *in, uint32_t *out, size_t n, unsigned long long *total, uint32_t *tmp,
                        cudaStream_t s);

// Stable LSD radix sort of (key, value) uint32 pairs on the low `bits` key
// bits. n_dev (device) holds the item count, n_max bounds it. Result lands
// in (k_out, v_out); k_tmp/v_tmp are scratch of n_max words. hist must hold
// radix_hist_words(n_max) words.
size_t radix_hist_words(size_t n_max);
void radix_sort_u32(const uint32_t *k_in, const uint32_t *v_in, uint32_t *k_out, uint32_t *v_out,
                    uint32_t *k_tmp, uint32_t *v_tmp, const unsigned long long *n_dev, size_t n_max, int bits,
                    uint32_t *hist, uint32_t *scan_tmp, cudaStream_t s);

void iota_u32(uint32_t *out, size_t n, cudaStream_t s);

}  // namespace stc
