// Context-free C ABI utilities (include/stc.h).
#include <string>

#include "stc_common.cuh"

namespace stc {
void set_thread_error(const std::string &msg);
}

using namespace stc;

namespace {

__global__ void k_set_count(unsigned long long *dst, unsigned long long v) { *dst = v; }

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
    STC_KL k_set_count<<<1, 1, 0, 0>>>(n_dev, (unsigned long long)n);
    radix_sort_u32(keys, values, keys_out, values_out, ktmp, vtmp, n_dev, n, (int)key_bits, hist, scan, 0);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
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
