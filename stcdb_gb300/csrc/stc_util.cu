// Context-free C ABI utilities (include/stc.h).
#include <mutex>
#include <string>

#include "stc_common.cuh"

namespace stc {
void set_thread_error(const std::string &msg);
}

using namespace stc;

namespace {

__global__ void k_set_count(unsigned long long *dst, unsigned long long v) { *dst = v; }

thread_local float t_last_sort_ms = 0.0f;

// Device time of the sort kernels (events around them on stream 0).
struct SortTimer {
  cudaEvent_t a = nullptr, b = nullptr;
  SortTimer() {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  ~SortTimer() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
  void start() { cudaEventRecord(a, 0); }
  void stop() { cudaEventRecord(b, 0); }
  void read() {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, a, b) == cudaSuccess) t_last_sort_ms = ms;
    cudaGetLastError();
  }
};

stc_status sort_args_ok(const uint32_t *keys, const uint32_t *values, uint32_t *keys_out, uint32_t *values_out,
                        size_t n, uint32_t key_bits, const char *who) {
  if (key_bits < 1 || key_bits > 32 || n > (size_t)1 << 31 ||
      (n && (!keys || !values || !keys_out || !values_out)) || (n && (keys == keys_out || values == values_out))) {
    set_thread_error(std::string(who) + ": invalid arguments");
    return STC_ERR_INVALID_ARG;
  }
  return STC_OK;
}

}  // namespace

extern "C" stc_status stc_sort_pairs_u32(const uint32_t *keys, const uint32_t *values, uint32_t *keys_out,
                                         uint32_t *values_out, size_t n, uint32_t key_bits, uint32_t device) {
  stc_status st = sort_args_ok(keys, values, keys_out, values_out, n, key_bits, "stc_sort_pairs_u32");
  if (st != STC_OK || n == 0) return st;
  cudaError_t e = cudaSetDevice((int)device);
  uint32_t *ktmp = nullptr, *vtmp = nullptr, *hist = nullptr, *scan = nullptr;
  unsigned long long *n_dev = nullptr;
  size_t hw = radix_hist_words(n);
  if (e == cudaSuccess) e = cudaMalloc(&ktmp, n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&vtmp, n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&hist, hw * 4);
  if (e == cudaSuccess) e = cudaMalloc(&scan, scan_tmp_words(hw) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&n_dev, sizeof(unsigned long long));
  if (e == cudaSuccess) {
    SortTimer tm;
    STC_KL k_set_count<<<1, 1, 0, 0>>>(n_dev, (unsigned long long)n);
    tm.start();
    radix_sort_u32(keys, values, keys_out, values_out, ktmp, vtmp, n_dev, n, (int)key_bits, hist, scan, 0);
    tm.stop();
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e == cudaSuccess) tm.read();
  }
  cudaFree(ktmp);
  cudaFree(vtmp);
  cudaFree(hist);
  cudaFree(scan);
  cudaFree(n_dev);
  if (e != cudaSuccess) {
    set_thread_error(std::string("stc_sort_pairs_u32: ") + cudaGetErrorString(e));
    return STC_ERR_CUDA;
  }
  return STC_OK;
}

// ---------------------------------------------------------------------------
// stc_sort_pairs_u32_noalloc: the same sort with its scratch in a fixed
// device array that belongs to the library, for callers that must not have
// device memory allocated on their behalf (see include/stc.h).

namespace {

constexpr size_t NA_MAX = STC_SORT_NOALLOC_MAX_PAIRS;
constexpr size_t NA_HIST = 256 * ((NA_MAX + STC_RS_TILE - 1) / STC_RS_TILE) + 1;  // radix histograms
constexpr size_t NA_SCAN = (NA_HIST + STC_SCAN_TILE - 1) / STC_SCAN_TILE + 1;       // scan block sums
constexpr size_t NA_COUNT_AT = (2 * NA_MAX + NA_HIST + NA_SCAN + 1) & ~(size_t)1;  // 8-byte aligned word
constexpr size_t NA_WORDS = NA_COUNT_AT + 2;

// Every process that loads the library holds this array on every device it
// touches, until exit (about 8.7 MB).
__device__ __align__(256) uint32_t g_sort_scratch[NA_WORDS];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mutex;
uint32_t *g_na_addr[NA_MAX_DEVICES] = {};

// Device address of g_sort_scratch on `device` (which must be current). The
// symbol's name in host code is only a host-side handle, so the address is
// looked up once per device and cached.
stc_status sort_scratch(int device, uint32_t **out) {
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_addr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess || !p) {
      set_thread_error(std::string("stc_sort_pairs_u32_noalloc: cudaGetSymbolAddress failed: ") +
                       cudaGetErrorString(e));
      return STC_ERR_CUDA;
    }
    g_na_addr[device] = (uint32_t *)p;
  }
  *out = g_na_addr[device];
  return STC_OK;
}

}  // namespace

extern "C" stc_status stc_sort_pairs_u32_noalloc(const uint32_t *keys, const uint32_t *values, uint32_t *keys_out,
                                                 uint32_t *values_out, size_t n, uint32_t key_bits,
                                                 uint32_t device) {
  stc_status st = sort_args_ok(keys, values, keys_out, values_out, n, key_bits, "stc_sort_pairs_u32_noalloc");
  if (st != STC_OK) return st;
  if (n > NA_MAX) {
    set_thread_error("stc_sort_pairs_u32_noalloc: n = " + std::to_string(n) + " exceeds the " +
                     std::to_string(NA_MAX) + " pairs its fixed scratch holds");
    return STC_ERR_CAPACITY;
  }
  if (device >= (uint32_t)NA_MAX_DEVICES) {
    set_thread_error("stc_sort_pairs_u32_noalloc: device ordinal out of range");
    return STC_ERR_INVALID_ARG;
  }
  if (n == 0) return STC_OK;
  cudaError_t e = cudaSetDevice((int)device);
  if (e != cudaSuccess) {
    set_thread_error(std::string("stc_sort_pairs_u32_noalloc: ") + cudaGetErrorString(e));
    return STC_ERR_CUDA;
  }
  uint32_t *scratch = nullptr;
  st = sort_scratch((int)device, &scratch);
  if (st != STC_OK) return st;
  uint32_t *ktmp = scratch, *vtmp = scratch + NA_MAX, *hist = vtmp + NA_MAX, *scan = hist + NA_HIST;
  unsigned long long *n_dev = (unsigned long long *)(scratch + NA_COUNT_AT);
  // the count and every histogram word the call reads are written by the
  // call itself, so nothing left by an earlier call is used
  STC_KL k_set_count<<<1, 1, 0, 0>>>(n_dev, (unsigned long long)n);
  radix_sort_u32(keys, values, keys_out, values_out, ktmp, vtmp, n_dev, n, (int)key_bits, hist, scan, 0);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  if (e != cudaSuccess) {
    set_thread_error(std::string("stc_sort_pairs_u32_noalloc: ") + cudaGetErrorString(e));
    return STC_ERR_CUDA;
  }
  return STC_OK;
}

extern "C" float stc_last_sort_ms(void) { return t_last_sort_ms; }

namespace {

// Slot s of the probe table holds key mix64(s).
__global__ void k_ra_init(Slot *slots, unsigned long long n) {
  for (unsigned long long s = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; s < n;
       s += (unsigned long long)gridDim.x * blockDim.x) {
    Slot v = {};
    v.key = mix64(s);
    slots[s] = v;
  }
}

// Access i reads the first 16 bytes of slot mix64(i + salt) & mask at L2 and
// stores its end word: the access pattern of the meeting-table update, where
// a hit reads its home slot and writes it (an extension its end time, a new
// meeting its claim).
__global__ void k_ra_access(Slot *slots, unsigned long long mask, unsigned long long n,
                            unsigned long long salt, uint32_t t, unsigned long long *sink) {
  unsigned long long acc = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long s = mix64(i + salt) & mask;
    const ulonglong2 v = __ldcg((const ulonglong2 *)&slots[s]);
    acc += v.x;
    slots[s].end = t + (uint32_t)v.y;
  }
  if (acc == 0x5A5A5A5A5A5A5A5Aull) *sink = acc;  // keeps the loads
}

}  // namespace

extern "C" stc_status stc_measure_random_access(uint32_t table_log2, unsigned long long accesses,
                                                uint32_t device, float *ms) {
  if (table_log2 < 10 || table_log2 > 32 || accesses == 0 || accesses > (1ull << 34) || !ms) {
    set_thread_error("stc_measure_random_access: invalid arguments");
    return STC_ERR_INVALID_ARG;
  }
  *ms = 0.0f;
  const unsigned long long n = 1ull << table_log2;
  cudaError_t e = cudaSetDevice((int)device);
  Slot *slots = nullptr;
  unsigned long long *sink = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&slots, n * sizeof(Slot));
  if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  float best = 0.0f;
  if (e == cudaSuccess) {
    const int grid = num_sms() * 16;
    STC_KL k_ra_init<<<grid, 256>>>(slots, n);
    for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {  // one warm-up, three timed
      cudaEventRecord(a, 0);
      STC_KL k_ra_access<<<grid, 256>>>(slots, n - 1, accesses, 0x9E3779B97F4A7C15ull * (rep + 1), rep, sink);
      cudaEventRecord(b, 0);
      e = cudaEventSynchronize(b);
      float t = 0.0f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
      if (e == cudaSuccess && rep > 0 && (best == 0.0f || t < best)) best = t;
    }
    if (e == cudaSuccess) e = cudaGetLastError();
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  cudaFree(slots);
  cudaFree(sink);
  if (e != cudaSuccess) {
    set_thread_error(std::string("stc_measure_random_access: ") + cudaGetErrorString(e));
    return STC_ERR_CUDA;
  }
  *ms = best;
  return STC_OK;
}
