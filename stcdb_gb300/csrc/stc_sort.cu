// Device-wide exclusive scan and stable LSD radix sort (hand-written; no
// CUB/thrust). The reference sorts with thrust::sort_by_key
// (cuda/geometry.cu:1809-1907); here the partition step uses these kernels
// to group object ids by quadtree leaf in pid order.
#include <atomic>

#include "stc_common.cuh"

namespace stc {

thread_local unsigned long long tl_launches = 0;

int num_sms() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
  std::atomic<int> *slot = dev < 64 ? &cache[dev] : nullptr;
  int v = slot ? slot->load(std::memory_order_relaxed) : 0;
  if (v > 0) return v;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
    cudaGetLastError();
    v = 1;  // a device that cannot be asked gets minimal grids (its launches fail on their own)
  }
  if (slot) slot->store(v, std::memory_order_relaxed);
  return v;
}

static constexpr int SCAN_THREADS = 256;
static constexpr int SCAN_ITEMS = 8;
static constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
static_assert(SCAN_TILE == STC_SCAN_TILE, "scan tile");

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  uint32_t lane = threadIdx.x & 31u;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= (uint32_t)o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns exclusive prefix,
// *total receives the block sum. blockDim.x must be a multiple of 32, <= 1024.
__device__ uint32_t block_excl_scan(uint32_t v, uint32_t *total) {
  __shared__ uint32_t warp_sums[32];
  __shared__ uint32_t block_total;
  uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t incl = warp_incl_scan(v);
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  uint32_t nw = blockDim.x >> 5;
  if (warp == 0) {
    uint32_t s = lane < nw ? warp_sums[lane] : 0u;
    uint32_t si = warp_incl_scan(s);
    if (lane < nw) warp_sums[lane] = si - s;
    if (lane == 31) block_total = si;
  }
  __syncthreads();
  uint32_t res = incl - v + warp_sums[warp];
  uint32_t tot = block_total;
  __syncthreads();
  *total = tot;
  return res;
}

__global__ void k_scan_reduce(const uint32_t *in, size_t n, uint32_t *sums) {
  size_t base = (size_t)blockIdx.x * SCAN_TILE;
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    size_t idx = base + (size_t)i * SCAN_THREADS + threadIdx.x;
    if (idx < n) s += in[idx];
  }
  uint32_t tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_sums(uint32_t *sums, size_t nb, unsigned long long *total) {
  // one block of 1024 threads, each owns a contiguous chunk
  size_t per = (nb + blockDim.x - 1) / blockDim.x;
  size_t b0 = (size_t)threadIdx.x * per, b1 = b0 + per < nb ? b0 + per : nb;
  uint32_t s = 0;
  for (size_t i = b0; i < b1; i++) s += sums[i];
  uint32_t tot;
  uint32_t off = block_excl_scan(s, &tot);
  for (size_t i = b0; i < b1; i++) {
    uint32_t v = sums[i];
    sums[i] = off;
    off += v;
  }
  if (threadIdx.x == 0 && total) *total = tot;
}

__global__ void k_scan_down(const uint32_t *in, uint32_t *out, size_t n, const uint32_t *sums) {
  size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS];
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    size_t idx = base + i;
    v[i] = idx < n ? in[idx] : 0u;
    s += v[i];
  }
  uint32_t tot;
  uint32_t off = block_excl_scan(s, &tot) + sums[blockIdx.x];
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    size_t idx = base + i;
    if (idx < n) out[idx] = off;
    off += v[i];
  }
}

size_t scan_tmp_words(size_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE + 1; }

void exclusive_scan_u32(const uint32_t *in, uint32_t *out, size_t n, unsigned long long *total, uint32_t *tmp,
                        cudaStream_t s) {
  if (n == 0) {
    if (total) cudaMemsetAsync(total, 0, sizeof(unsigned long long), s);
    return;
  }
  size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  STC_KL k_scan_reduce<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, tmp);
  STC_KL k_scan_sums<<<1, 1024, 0, s>>>(tmp, nb, total);
  STC_KL k_scan_down<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, out, n, tmp);
}

// ---------------------------------------------------------------------------
// Radix sort: 8-bit digits, tiles of 256 threads x 16 items.

static constexpr int RS_THREADS = 256;
static constexpr int RS_ITEMS = 16;
static constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
static_assert(RS_TILE == STC_RS_TILE, "radix tile");
static constexpr int RS_WARPS = RS_THREADS / 32;
// the histogram, scan and scatter kernels give each of the 256 digits its
// own thread (per-digit shared arrays and histogram rows are indexed by it)
static_assert(RS_THREADS == 256, "one thread per 8-bit digit");

size_t radix_hist_words(size_t n_max) { return 256 * ((n_max + RS_TILE - 1) / RS_TILE) + 1; }

__global__ void k_rs_hist(const uint32_t *keys, const unsigned long long *n_dev, size_t n_max, int shift,
                          uint32_t dmask, uint32_t *hist, uint32_t nb) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  size_t n = (size_t)*n_dev;
  if (n > n_max) n = n_max;
  size_t base = (size_t)blockIdx.x * RS_TILE;
  if (base < n) {
    // all of the thread's items are requested before any is counted
    uint32_t kr[RS_ITEMS];
#pragma unroll
    for (int i = 0; i < RS_ITEMS; i++) {
      size_t idx = base + (size_t)i * RS_THREADS + threadIdx.x;
      kr[i] = idx < n ? keys[idx] : 0u;  // kept in L2 for the scatter that follows
    }
#pragma unroll
    for (int i = 0; i < RS_ITEMS; i++) {
      size_t idx = base + (size_t)i * RS_THREADS + threadIdx.x;
      if (idx < n) atomicAdd(&h[(kr[i] >> shift) & dmask], 1u);
    }
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * nb + blockIdx.x] = h[threadIdx.x];
}

// One tile of RS_TILE items, stable. Warp w takes the tile's items
// [w * 512, (w + 1) * 512) in order, 32 at a time, and ranks each among the
// warp's earlier items of its digit with a warp-private histogram; one scan
// over (digit, warp) then places every item in a shared-memory copy of the
// tile ordered by digit, which is written out one digit run after another,
// so that neighbouring threads write neighbouring addresses. hist holds the
// exclusive scan of the counts laid out [digit][tile].
static constexpr int RS_WARP_ITEMS = RS_TILE / RS_WARPS;  // 512
static_assert(RS_WARP_ITEMS == 32 * RS_ITEMS, "warp share");

// Ranks the thread's RS_ITEMS items among the warp's earlier items of their
// digit (pr) and counts the warp's items per digit (wh). FULL: every item of
// the tile is valid (all tiles but the last), so no lane needs masking.
template <bool FULL>
__device__ __forceinline__ void rank_items(const uint32_t *kr, uint32_t *pr, uint32_t *wh, uint32_t warp,
                                           uint32_t lane, uint32_t in_tile, int shift, uint32_t dmask) {
  const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
  for (int it = 0; it < RS_ITEMS; it++) {
    const uint32_t li = warp * RS_WARP_ITEMS + (uint32_t)it * 32u + lane;
    const bool valid = FULL || li < in_tile;
    const uint32_t digit = (kr[it] >> shift) & dmask;
    // lanes with the same digit: one vote per digit bit (valid lanes only)
    uint32_t peers = FULL ? 0xffffffffu : __ballot_sync(0xffffffffu, valid);
#pragma unroll
    for (int b = 0; b < 8; b++) {
      const bool bit = (digit >> b) & 1u;
      const uint32_t m = __ballot_sync(0xffffffffu, bit);
      peers &= bit ? m : ~m;
    }
    if (!FULL && !valid) peers = 1u << lane;
    const uint32_t rank = __popc(peers & lt_mask);
    const uint32_t leader = __ffs(peers) - 1u;
    uint32_t before = 0;
    if (valid && rank == 0) {
      before = wh[digit];
      wh[digit] = before + __popc(peers);
    }
    before = __shfl_sync(0xffffffffu, before, leader);
    pr[it] = before + rank;  // position among the warp's items of this digit
    __syncwarp();
  }
}

__global__ void __launch_bounds__(RS_THREADS, 3) k_rs_scatter(const uint32_t *k_in, const uint32_t *v_in,
                                                           uint32_t *k_out, uint32_t *v_out,
                                                           const unsigned long long *n_dev, size_t n_max, int shift,
                                                           uint32_t dmask, const uint32_t *hist, uint32_t nb) {
  __shared__ uint2 s_kv[RS_TILE];     // the tile in digit order
  __shared__ uint32_t base_off[256];  // output position of tile position i of digit d, less i
  // per warp and digit: counts, then the tile position of the warp's first item of the digit
  __shared__ uint32_t whist[RS_WARPS][256];
  __shared__ uint32_t scan_tmp[RS_WARPS];
  size_t n = (size_t)*n_dev;
  if (n > n_max) n = n_max;
  size_t tile = (size_t)blockIdx.x * RS_TILE;
  if (tile >= n) return;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t in_tile = (uint32_t)min((size_t)RS_TILE, n - tile);
  const bool full = in_tile == RS_TILE;
  base_off[threadIdx.x] = hist[(size_t)threadIdx.x * nb + blockIdx.x];
  for (int w = 0; w < RS_WARPS; w++) whist[w][threadIdx.x] = 0;
  // all of the thread's items are requested before the ranking starts
  uint32_t kr[RS_ITEMS], vr[RS_ITEMS], pr[RS_ITEMS];
#pragma unroll
  for (int it = 0; it < RS_ITEMS; it++) {
    const uint32_t li = warp * RS_WARP_ITEMS + (uint32_t)it * 32u + lane;
    kr[it] = li < in_tile ? __ldcs(&k_in[tile + li]) : 0u;
    vr[it] = li < in_tile ? __ldcs(&v_in[tile + li]) : 0u;
  }
  __syncthreads();
  if (full) rank_items<true>(kr, pr, whist[warp], warp, lane, in_tile, shift, dmask);
  else rank_items<false>(kr, pr, whist[warp], warp, lane, in_tile, shift, dmask);
  __syncthreads();
  {
    // per digit: the tile's exclusive offset (block scan over digits), then
    // each warp's first tile position of the digit
    const uint32_t d = threadIdx.x;
    uint32_t c[RS_WARPS], cnt = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) {
      c[w] = whist[w][d];
      cnt += c[w];
    }
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += v;
    }
    if (lane == 31) scan_tmp[warp] = incl;
    __syncthreads();
    uint32_t before = 0;
    for (uint32_t w = 0; w < warp; w++) before += scan_tmp[w];
    uint32_t start = before + incl - cnt;
    base_off[d] -= start;
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) {
      whist[w][d] = start;
      start += c[w];
    }
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < RS_ITEMS; it++) {
    const uint32_t li = warp * RS_WARP_ITEMS + (uint32_t)it * 32u + lane;
    if (full || li < in_tile) {
      const uint32_t digit = (kr[it] >> shift) & dmask;
      s_kv[whist[warp][digit] + pr[it]] = make_uint2(kr[it], vr[it]);
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < in_tile; i += RS_THREADS) {
    const uint2 kv = s_kv[i];
    const uint32_t pos = base_off[(kv.x >> shift) & dmask] + i;
    k_out[pos] = kv.x;
    v_out[pos] = kv.y;
  }
}

void radix_sort_u32(const uint32_t *k_in, const uint32_t *v_in, uint32_t *k_out, uint32_t *v_out,
                    uint32_t *k_tmp, uint32_t *v_tmp, const unsigned long long *n_dev, size_t n_max, int bits,
                    uint32_t *hist, uint32_t *scan_tmp, cudaStream_t s) {
  uint32_t nb = (uint32_t)((n_max + RS_TILE - 1) / RS_TILE);
  if (nb == 0) return;
  int passes = (bits + 7) / 8;
  if (passes < 1) passes = 1;
  // ping-pong so that the last pass writes (k_out, v_out)
  const uint32_t *ki = k_in, *vi = v_in;
  for (int p = 0; p < passes; p++) {
    bool to_out = ((passes - 1 - p) % 2) == 0;
    uint32_t *ko = to_out ? k_out : k_tmp;
    uint32_t *vo = to_out ? v_out : v_tmp;
    // the last digit covers only the key bits that remain
    int left = bits - 8 * p;
    uint32_t dmask = left >= 8 ? 255u : (1u << left) - 1u;
    STC_KL k_rs_hist<<<nb, RS_THREADS, 0, s>>>(ki, n_dev, n_max, 8 * p, dmask, hist, nb);
    exclusive_scan_u32(hist, hist, (size_t)256 * nb, nullptr, scan_tmp, s);
    STC_KL k_rs_scatter<<<nb, RS_THREADS, 0, s>>>(ki, vi, ko, vo, n_dev, n_max, 8 * p, dmask, hist, nb);
    ki = ko;
    vi = vo;
  }
}

__global__ void k_iota(uint32_t *out, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (uint32_t)i;
}

void iota_u32(uint32_t *out, size_t n, cudaStream_t s) {
  if (n == 0) return;
  STC_KL k_iota<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, n);
}

}  // namespace stc
