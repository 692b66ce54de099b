// te_common.cu -- error reporting and launch-shape helpers of libtegpu.
#include <cstdarg>
#include <cstdio>

#include <map>
#include <mutex>
#include <thread>
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

// Sum of squares of a host array (the normalisation check of a start vector,
// krylovTimeEvolver.cpp:45-48): 8 independent partial sums per part, and 8
// parts on their own threads from 2^21 values on, combined in a fixed order,
// so the result depends on len only.  A single running sum was a chain of
// dependent adds: about 2 ms for the 2.7 M values of a dim-1.35 M vector.
double te_host_sumsq(const double* x, int64_t len) {
  auto part = [x](int64_t a, int64_t b) {
    double s[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    int64_t i = a;
    for (; i + 8 <= b; i += 8)
      for (int k = 0; k < 8; ++k) s[k] += x[i + k] * x[i + k];
    for (; i < b; ++i) s[0] += x[i] * x[i];
    return ((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]));
  };
  constexpr int kParts = 8;
  if (len < ((int64_t)1 << 21)) return part(0, len);
  double res[kParts];
  std::vector<std::thread> pool;
  for (int t = 1; t < kParts; ++t)
    pool.emplace_back([&, t]() { res[t] = part(len * t / kParts, len * (t + 1) / kParts); });
  res[0] = part(0, len / kParts);
  for (auto& th : pool) th.join();
  double tot = 0.0;
  for (int t = 0; t < kParts; ++t) tot += res[t];
  return tot;
}

extern "C" const char* te_last_error(void) { return g_last_error; }
extern "C" int te_abi_version(void) { return TEGPU_ABI_VERSION; }
extern "C" int te_set_device(int device) { return te_cuda_check(cudaSetDevice(device), "cudaSetDevice"); }
