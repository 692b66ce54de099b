// te_common.cu -- error reporting and launch-shape helpers of libtegpu.
#include <cstdarg>
#include <cstdio>

#include <map>
#include <mutex>
#include <tuple>

#include "te_internal.cuh"

static thread_local char g_last_error[512] = "";

void te_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

int te_cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return TE_OK;
  te_set_error("CUDA error in %s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? TE_ERR_OUT_OF_MEMORY : TE_ERR_CUDA;
}

int te_num_sms() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

// Grid for a grid-stride kernel: enough blocks to cover the items, at most
// blocks_per_sm resident blocks on every SM.
int te_grid_for(int64_t n_items, int threads, int blocks_per_sm) {
  int64_t need = (n_items + threads - 1) / threads;
  int64_t cap = (int64_t)te_num_sms() * blocks_per_sm;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}

int te_kernel_blocks_per_sm(const void* kernel, int threads, size_t dyn_smem) {
  static std::mutex mu;
  static std::map<std::tuple<const void*, int, size_t>, int> cache;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_tuple(kernel, threads, dyn_smem);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, threads, dyn_smem) != cudaSuccess || blocks < 1) {
    cudaGetLastError();
    blocks = 1;
  }
  cache[key] = blocks;
  return blocks;
}

int te_grid_fit(const void* kernel, int64_t n_items, int threads, size_t dyn_smem) {
  const int64_t cap = (int64_t)te_num_sms() * te_kernel_blocks_per_sm(kernel, threads, dyn_smem);
  const int64_t need = (n_items + threads - 1) / threads;
  // more items than one wave of threads: exactly one wave, so that every SM
  // holds the same number of blocks (threads differ by at most one item)
  return (int)(need <= cap ? std::max<int64_t>(need, 1) : cap);
}

bool te_grid_saturated(const void* kernel, int64_t n_items, int threads, size_t dyn_smem) {
  const int64_t cap = (int64_t)te_num_sms() * te_kernel_blocks_per_sm(kernel, threads, dyn_smem);
  return (n_items + threads - 1) / threads > cap;
}

extern "C" const char* te_last_error(void) { return g_last_error; }
extern "C" int te_abi_version(void) { return TEGPU_ABI_VERSION; }
extern "C" int te_set_device(int device) { return te_cuda_check(cudaSetDevice(device), "cudaSetDevice"); }
