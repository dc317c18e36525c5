// Device helpers and kernels of the memtable flush (stc_lsm.cu) that the
// compaction of flushed blocks (stc_compact.cu) runs as well.
#pragma once
#include <algorithm>

#include "stc_lsm.cuh"

namespace stc {
namespace lsmk {

inline unsigned nblk(size_t n, unsigned t = 256) { return (unsigned)std::max<size_t>((n + t - 1) / t, 1); }

// Smallest b >= 1 with v < 2^b.
inline uint32_t bits_for(unsigned long long v) {
  uint32_t b = 1;
  while (b < 64 && (v >> b)) b++;
  return b;
}

inline unsigned lsm_grid() { return (unsigned)num_sms() * 8; }  // grid-stride kernels over keys
constexpr uint32_t OBOX_INIT = 100000000u;  // uint_box initial low (geometry/geometry.h:320-324)
constexpr uint32_t LIM_PARTS = 32;          // blocks per CTF in k_lsm_limits
constexpr uint32_t MAX_CTF = 3969;          // 63^2: sids 2..3970 fit the 12-bit sid field

// float_to_uint / uint_to_float (cuda/cuda_util.cuh:116-125)
__device__ __forceinline__ uint32_t f2u_ref(float xy) {
  return __float2uint_rz(__fmul_rn(__fadd_rn(xy, 180.0f), 100000.0f));
}
__device__ __forceinline__ float u2f_ref(uint32_t f) {
  return __fsub_rn(__fdiv_rn(__uint2float_rn(f), 100000.0f), 180.0f);
}

__device__ __forceinline__ uint32_t warp_max_u32(uint32_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ uint32_t d2u_cell(double v) { return __double2uint_rz(v); }

// serialize_mbr (cuda/geometry.cu:161-171)
__device__ __forceinline__ unsigned long long serialize_mbr_dev(float4 b, const stc_ctf &c) {
  float wx = __fsub_rn(c.mbr[2], c.mbr[0]), wy = __fsub_rn(c.mbr[3], c.mbr[1]);
  float le = fmaxf(wx, wy);
  float fx = __ull2float_rn((1ull << c.low_x_bit) - 1), fy = __ull2float_rn((1ull << c.low_y_bit) - 1);
  float fe = __ull2float_rn((1ull << c.edge_bit) - 1);
  unsigned long long low0 = __float2ull_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.x, c.mbr[0]), wx), fx));
  unsigned long long low1 = __float2ull_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.y, c.mbr[1]), wy), fy));
  unsigned long long x = __float2ull_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.z, b.x), le), fe));
  unsigned long long y = __float2ull_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.w, b.y), le), fe));
  return (low0 << (c.low_y_bit + 2 * c.edge_bit)) + (low1 << (2 * c.edge_bit)) + (x << c.edge_bit) + y;
}

// One 32-bit word of the key sort. The order is (over, sid, pid, target,
// duration, end): the CTF keys by their 128-bit key sid:12 | pid:26 |
// target:26 | duration:32 | end:32 (cuda/geometry.cu:724-726, 799-806),
// then the oversize keys by theirs (sid 0).
enum WordKind : int { W_END_DUR, W_END, W_DUR, W_TARGET, W_SID_PID, W_PID, W_SID, W_OVER, W_LOW, W_HIGH };

// One word of the key sort: its kind, the field shifts it needs and its
// significant bits.
struct WordSpec {
  int kind;
  uint32_t a, b, c, bits;
};

__global__ void k_lsm_set_counts(unsigned long long *n_dev, unsigned long long a, unsigned long long b,
                                 unsigned long long c);
__global__ void k_gather_u32(const uint32_t *src, const uint32_t *idx, uint32_t *dst, uint32_t n);
__global__ void k_slab_keys(const uint32_t *mid_lo, const uint32_t *oids, uint32_t z, uint32_t R, uint32_t *keys,
                            uint32_t *vals);
__global__ void k_slab_of(const uint32_t *jv, uint32_t R, uint32_t xcap, uint32_t split, uint32_t *keys);
__global__ void k_make_sid(LsmDev L, const uint32_t *oids, const uint32_t *jv, uint32_t z, uint32_t R,
                           uint32_t xcap, uint32_t ycap);
__global__ void k_lsm_word(LsmDev L, unsigned long long K, const uint32_t *perm, uint32_t *keys, uint32_t *vals,
                           WordSpec w);
__global__ void k_lsm_low_high(LsmDev L, unsigned long long K, uint32_t *keys, uint32_t *vals, uint32_t *hi,
                               WordSpec lo, WordSpec hs, const uint32_t *rank);
__global__ void k_lsm_gather(LsmDev L, unsigned long long K, const uint32_t *perm);

// Bitmaps and packed keys of the sorted keys [0, total) over CTF ranges
// ctf_first[0..F] (k_encode_keys, launched with ENC_GROUP threads a block).
struct EncodeArgs {
  const uint4 *brec;
  const float4 *bbox;
  const stc_ctf *ctfs;
  const unsigned long long *ctf_first;
  const uint16_t *sid;
  uint32_t *bitmaps;
  uint8_t *kbytes;
  unsigned long long total, slim;
  uint32_t F;
  bool compact;
};
constexpr uint32_t ENC_GROUP = 256;
__global__ void k_encode_keys(EncodeArgs a);
__global__ void k_lsm_limits(LsmDev L, unsigned long long K);
__global__ void k_lsm_oversize(LsmDev L, unsigned long long a, unsigned long long b);

// Stable sort of n (key, value) words with L's radix-sort scratch; the item
// count is read from L.n_dev[count_slot].
void sort_words(const LsmDev &L, const uint32_t *k, const uint32_t *v, uint32_t *ko, uint32_t *vo, uint32_t *kt,
                uint32_t *vt, int count_slot, size_t n, uint32_t bits, cudaStream_t s);

// The K records (L.rec, L.box) into (L.brec, L.bbox), stably ordered by
// (over, sid, pid, target, duration, end). L.sid holds each object's sid
// (below 2^sid_bits); L.n_dev[0] = N and L.n_dev[2] = K; L.sk[0..6] are
// scratch (sk[6] free on entry).
void sort_keys(const LsmDev &L, unsigned long long K, uint32_t N, uint32_t max_end, uint32_t max_dur,
               uint32_t sid_bits, cudaStream_t s);

}  // namespace lsmk
}  // namespace stc
