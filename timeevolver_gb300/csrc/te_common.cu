// te_common.cu -- error reporting, launch-shape helpers and the buffer cache
// of libtegpu.
#include <cstdarg>
#include <cstdio>

#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <unordered_map>

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

// ----------------------------------------------------------- buffer cache
// Device buffers of at least 1 MiB and small pinned host buffers are kept
// after te_free / te_free_host and handed out again to a request of exactly
// the same size on the same device: repeated evolutions of one dimension
// (the matrices, the Krylov basis, the fixed-point copies) then skip the
// driver's allocation and release, about 3 ms per L=12 evolution.  A block
// goes into the cache only after the device is idle (a cudaFree would have
// waited for it too).  The cached bytes are capped (te_set_buffer_cache_limit,
// default 8 GiB of device memory; 64 MiB of pinned host memory), and a failed
// allocation releases the cache and tries again.
namespace {

constexpr size_t kCacheMinBytes = (size_t)1 << 20;
constexpr size_t kHostCacheMaxBlock = (size_t)1 << 20;  // pinned blocks up to this size are cached

struct BufferCache {
  std::mutex mu;
  // key (device, bytes); host blocks use device -1
  std::multimap<std::pair<int, size_t>, void*> free_blocks;
  std::unordered_map<void*, std::pair<int, size_t>> live;
  size_t cached_dev = 0, cached_host = 0;
  size_t limit_dev = (size_t)8 << 30, limit_host = (size_t)64 << 20;
};

BufferCache& cache() {
  static BufferCache* c = new BufferCache();  // never destroyed: usable from other static destructors
  return *c;
}

// Release every cached block of `device` (-2: all devices and host).  The
// caller holds the lock.
void release_locked(BufferCache& c, int device) {
  int cur = 0;
  cudaGetDevice(&cur);
  for (auto it = c.free_blocks.begin(); it != c.free_blocks.end();) {
    const int d = it->first.first;
    if (device == -2 || d == device) {
      if (d == -1) {
        cudaFreeHost(it->second);
        c.cached_host -= it->first.second;
      } else {
        if (d != cur) cudaSetDevice(d);
        cudaFree(it->second);
        if (d != cur) cudaSetDevice(cur);
        c.cached_dev -= it->first.second;
      }
      it = c.free_blocks.erase(it);
    } else {
      ++it;
    }
  }
}

}  // namespace

cudaError_t te_malloc_bytes(void** p, size_t bytes) {
  if (bytes < kCacheMinBytes) return cudaMalloc(p, bytes);
  int dev = 0;
  cudaGetDevice(&dev);
  BufferCache& c = cache();
  std::lock_guard<std::mutex> lock(c.mu);
  auto it = c.free_blocks.find({dev, bytes});
  if (it != c.free_blocks.end()) {
    *p = it->second;
    c.free_blocks.erase(it);
    c.cached_dev -= bytes;
    c.live[*p] = {dev, bytes};
    return cudaSuccess;
  }
  cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaErrorMemoryAllocation && c.cached_dev > 0) {
    cudaGetLastError();
    release_locked(c, dev);
    e = cudaMalloc(p, bytes);
  }
  if (e == cudaSuccess) c.live[*p] = {dev, bytes};
  return e;
}

cudaError_t te_free(void* p) {
  if (!p) return cudaSuccess;
  BufferCache& c = cache();
  std::lock_guard<std::mutex> lock(c.mu);
  auto it = c.live.find(p);
  if (it == c.live.end()) return cudaFree(p);  // small or not from te_malloc
  const int dev = it->second.first;
  const size_t bytes = it->second.second;
  c.live.erase(it);
  int cur = 0;
  cudaGetDevice(&cur);
  if (dev != cur || c.cached_dev + bytes > c.limit_dev) return cudaFree(p);
  const cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cudaFree(p);
  c.free_blocks.insert({{dev, bytes}, p});
  c.cached_dev += bytes;
  return cudaSuccess;
}

cudaError_t te_malloc_host_bytes(void** p, size_t bytes) {
  if (bytes > kHostCacheMaxBlock) return cudaMallocHost(p, bytes);
  BufferCache& c = cache();
  std::lock_guard<std::mutex> lock(c.mu);
  auto it = c.free_blocks.find({-1, bytes});
  if (it != c.free_blocks.end()) {
    *p = it->second;
    c.free_blocks.erase(it);
    c.cached_host -= bytes;
    c.live[*p] = {-1, bytes};
    return cudaSuccess;
  }
  const cudaError_t e = cudaMallocHost(p, bytes);
  if (e == cudaSuccess) c.live[*p] = {-1, bytes};
  return e;
}

cudaError_t te_free_host(void* p) {
  if (!p) return cudaSuccess;
  BufferCache& c = cache();
  std::lock_guard<std::mutex> lock(c.mu);
  auto it = c.live.find(p);
  if (it == c.live.end()) return cudaFreeHost(p);
  const size_t bytes = it->second.second;
  c.live.erase(it);
  if (c.cached_host + bytes > c.limit_host) return cudaFreeHost(p);
  const cudaError_t e = cudaDeviceSynchronize();  // no copy into the block is still in flight
  if (e != cudaSuccess) return cudaFreeHost(p);
  c.free_blocks.insert({{-1, bytes}, p});
  c.cached_host += bytes;
  return cudaSuccess;
}

extern "C" int te_release_buffers(void) {
  BufferCache& c = cache();
  std::lock_guard<std::mutex> lock(c.mu);
  release_locked(c, -2);
  return te_cuda_check(cudaGetLastError(), "te_release_buffers");
}

extern "C" int te_set_buffer_cache_limit(int64_t device_bytes) {
  if (device_bytes < 0) {
    te_set_error("te_set_buffer_cache_limit: negative limit");
    return TE_ERR_INVALID_ARG;
  }
  BufferCache& c = cache();
  std::lock_guard<std::mutex> lock(c.mu);
  c.limit_dev = (size_t)device_bytes;
  if (c.cached_dev > c.limit_dev) {
    for (auto it = c.free_blocks.begin(); it != c.free_blocks.end();) {  // devices only
      if (it->first.first >= 0) {
        int cur = 0;
        cudaGetDevice(&cur);
        if (it->first.first != cur) cudaSetDevice(it->first.first);
        cudaFree(it->second);
        if (it->first.first != cur) cudaSetDevice(cur);
        c.cached_dev -= it->first.second;
        it = c.free_blocks.erase(it);
      } else {
        ++it;
      }
    }
  }
  return TE_OK;
}

extern "C" int64_t te_buffer_cache_bytes(void) {
  BufferCache& c = cache();
  std::lock_guard<std::mutex> lock(c.mu);
  return (int64_t)c.cached_dev;
}

extern "C" const char* te_last_error(void) { return g_last_error; }
extern "C" int te_abi_version(void) { return TEGPU_ABI_VERSION; }
extern "C" int te_set_device(int device) { return te_cuda_check(cudaSetDevice(device), "cudaSetDevice"); }
