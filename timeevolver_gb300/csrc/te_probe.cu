// te_probe.cu -- FP64 FMA throughput and issue probes, and the gather probe
// (include/te_diag.h).
#include <cuda.h>
#include <cudaTypedefs.h>

#include "../../include/te_diag.h"
#include "te_internal.cuh"

__global__ void fp64_fma_probe(double* out, int iters, double a, double b) {
  double c0 = threadIdx.x, c1 = c0 + 1, c2 = c0 + 2, c3 = c0 + 3, c4 = c0 + 4, c5 = c0 + 5, c6 = c0 + 6,
         c7 = c0 + 7;
  for (int i = 0; i < iters; ++i) {
    c0 = fma(c0, a, b);
    c1 = fma(c1, a, b);
    c2 = fma(c2, a, b);
    c3 = fma(c3, a, b);
    c4 = fma(c4, a, b);
    c5 = fma(c5, a, b);
    c6 = fma(c6, a, b);
    c7 = fma(c7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = c0 + c1 + c2 + c3 + c4 + c5 + c6 + c7;
}

extern "C" int te_probe_fp64_tflops(double* tflops) {
  if (!tflops) return TE_ERR_INVALID_ARG;
  const int blocks = te_num_sms() * 4, threads = 256, iters = 1024;
  double* out = nullptr;
  TE_CUDA(te_malloc(&out, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fp64_fma_probe<<<blocks, threads>>>(out, 16, 1.0000001, 1e-9);  // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    fp64_fma_probe<<<blocks, threads>>>(out, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  int rc = te_cuda_check(cudaGetLastError(), "fp64 probe");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  te_free(out);
  if (rc != TE_OK) return rc;
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return TE_OK;
}

// One dependent FMA chain per thread (the latency a warp sees).
__global__ void fp64_chain_probe(double* out, int iters, double a, double b) {
  double c0 = threadIdx.x;
  for (int i = 0; i < iters; ++i) c0 = fma(c0, a, b);
  out[blockIdx.x * blockDim.x + threadIdx.x] = c0;
}

extern "C" int te_probe_fp64_issue(int warps, int blocks, double* cycles_indep, double* cycles_chain) {
  if (!cycles_indep || !cycles_chain || warps < 1 || warps > 32 || blocks < 1 || blocks > 65535)
    return TE_ERR_INVALID_ARG;
  const int threads = 32 * warps, iters = 20000;
  int dev = 0, khz = 0;
  cudaGetDevice(&dev);
  TE_CUDA(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev));
  double* out = nullptr;
  TE_CUDA(te_malloc(&out, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float ms[2] = {0.f, 0.f};
  for (int kind = 0; kind < 2; ++kind) {
    for (int rep = 0; rep < 2; ++rep) {  // the first launch warms up
      cudaEventRecord(e0);
      if (kind == 0)
        fp64_fma_probe<<<blocks, threads>>>(out, iters, 0.999999, 1.0);
      else
        fp64_chain_probe<<<blocks, threads>>>(out, iters, 0.999999, 1.0);
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      cudaEventElapsedTime(&ms[kind], e0, e1);
    }
  }
  int rc = te_cuda_check(cudaGetLastError(), "fp64 issue probe");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  te_free(out);
  if (rc != TE_OK) return rc;
  const double cycles_per_ms = (double)khz;  // clock rate in kHz = cycles per ms
  *cycles_indep = ms[0] * cycles_per_ms / (8.0 * iters * warps);
  *cycles_chain = ms[1] * cycles_per_ms / iters;
  return TE_OK;
}

// ---------------------------------------------------------------------------
// Gather probe: one 16-byte row of a table per index, the access of the SpMV
// passes' X gathers.  Each warp walks its own run of "slot rows" of 32
// indices.  Mode 0 gathers with ordinary loads (depth rows in flight per
// lane); mode 1 with TMA tile::gather4 copies (one thread copies 4 rows into
// shared memory, completion on an mbarrier; depth stages of 32 rows per warp).
// Both fold the rows into the same per-lane checksum.

namespace {

__device__ __forceinline__ uint32_t probe_smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool probe_mb_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
               : "=r"(ok)
               : "r"(bar), "r"(parity)
               : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool probe_mb_wait(uint32_t bar, uint32_t parity, int limit) {
  for (int i = 0; i < limit; ++i)
    if (probe_mb_try(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void probe_fold(int4& a, const int4 v) {
  a.x ^= v.x;
  a.y += v.y;
  a.z ^= v.z;
  a.w += v.w;
}

template <int U>
__global__ void __launch_bounds__(256) gather_lsu_probe(const int4* __restrict__ X, const int32_t* __restrict__ idx,
                                                        int rows, int4* out) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int32_t* my = idx + gw * (int64_t)rows * 32;
  int4 acc = make_int4(0, 0, 0, 0);
#pragma unroll(U)
  for (int r = 0; r < rows; ++r) probe_fold(acc, __ldg(X + __ldcs(my + (int64_t)r * 32 + lane)));
  out[gw * 32 + lane] = acc;
}

// Shared memory: 8 warps x S mbarriers in the first 1 KB, then from the next
// 1 KB boundary 8 warps x S stages x 1 KB; group g of a stage (rows 4g..4g+3,
// 64 bytes) starts at 128 g.
template <int S>
__global__ void __launch_bounds__(256) gather_tma_probe(const __grid_constant__ CUtensorMap tm,
                                                        const int32_t* __restrict__ idx, int rows, int4* out,
                                                        unsigned int* err, int limit) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const uint32_t base_s = probe_smem_addr(smem);
  const uint32_t data_s = (base_s + 1024u + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t bar0 = base_s + 8u * (uint32_t)(warp * S);
  const uint32_t wd_s = data_s + (uint32_t)(warp * S) * 1024u;
  const unsigned char* wd = smem + (wd_s - base_s);
  if (lane == 0)
    for (int s = 0; s < S; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8u * s) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  __syncwarp();
  const int64_t gw = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  const int32_t* my = idx + gw * (int64_t)rows * 32;
  auto issue = [&](int r) {
    const int s = r % S;
    const int c0 = __ldcs(my + (int64_t)r * 32 + lane);
    const int c1 = __shfl_down_sync(0xffffffffu, c0, 1), c2 = __shfl_down_sync(0xffffffffu, c0, 2),
              c3 = __shfl_down_sync(0xffffffffu, c0, 3);
    const uint32_t bar = bar0 + 8u * s;
    if (lane == 0)
      asm volatile("{ .reg .b64 st; mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], 512; }" ::"r"(bar) : "memory");
    __syncwarp();
    if ((lane & 3) == 0)
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes "
          "[%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(wd_s + (uint32_t)s * 1024u + (uint32_t)(lane >> 2) * 128u),
          "l"((uint64_t)&tm), "r"(0), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
          : "memory");
  };
  for (int r = 0; r < rows && r < S; ++r) issue(r);
  int4 acc = make_int4(0, 0, 0, 0);
  int r = 0;
  bool ok = true;
  for (; r < rows; ++r) {
    const int s = r % S;
    if (!probe_mb_wait(bar0 + 8u * s, (uint32_t)((r / S) & 1), limit)) {
      ok = false;
      break;
    }
    probe_fold(acc, *reinterpret_cast<const int4*>(wd + s * 1024 + (lane >> 2) * 128 + (lane & 3) * 16));
    __syncwarp();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // reads before the next copy into the stage
    if (r + S < rows) issue(r + S);
  }
  if (!ok) {
    if (lane == 0) atomicOr(err, 1u);
    for (int q = r; q < rows && q < r + S; ++q) probe_mb_wait(bar0 + 8u * (q % S), (uint32_t)((q / S) & 1), limit);
  }
  out[gw * 32 + lane] = acc;
}

__global__ void gather_random_indices(int32_t* idx, int64_t count, int64_t n_rows, uint64_t seed) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t z = seed + 0x9e3779b97f4a7c15ull * (uint64_t)(i + 1);  // splitmix64
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    idx[i] = (int32_t)(z % (uint64_t)n_rows);
  }
}

__global__ void gather_fill_table(int4* X, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    X[i] = make_int4((int)i, (int)(3 * i), (int)(i ^ 0x5a5a), 1);
}

__global__ void gather_checksum(const int4* out, int64_t count, unsigned long long* sum) {
  unsigned long long s = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const int4 v = out[i];
    s += (unsigned long long)(unsigned)v.x * 3ull + (unsigned long long)(unsigned)v.y * 5ull +
         (unsigned long long)(unsigned)v.z * 7ull + (unsigned long long)(unsigned)v.w * 11ull;
  }
  atomicAdd(sum, s);
}

}  // namespace

extern "C" int te_probe_gather(te_matrix M, int64_t n_rows, int64_t n_gathers, int mode, int depth,
                               int blocks_per_sm, double* rows_per_s, unsigned long long* checksum) {
  const bool mode_ok = (mode == 0 && (depth == 1 || depth == 2 || depth == 4)) ||
                       (mode == 1 && (depth == 4 || depth == 8 || depth == 16));
  if (!rows_per_s || !checksum || !mode_ok || blocks_per_sm < 1 || blocks_per_sm > 8 ||
      (!M && (n_rows < 1 || n_rows > INT32_MAX || n_gathers < 32))) {
    te_set_error("te_probe_gather: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  if (M && (M->sell.slots < 32 || !M->sell.col)) {
    te_set_error("te_probe_gather: the matrix has no SELL slots");
    return TE_ERR_INVALID_ARG;
  }
  const int64_t table = M ? M->sell.n : n_rows;
  const int64_t count = M ? M->sell.slots : n_gathers / 32 * 32;
  const int sms = te_num_sms(), threads = 256;
  const int blocks = sms * blocks_per_sm;
  const int64_t warps = (int64_t)blocks * (threads / 32);
  const int64_t rows64 = count / 32 / warps;
  if (rows64 < 1 || rows64 > INT32_MAX) {
    te_set_error("te_probe_gather: %lld gathers are too few or too many for %d blocks", (long long)count, blocks);
    return TE_ERR_UNSUPPORTED;
  }
  const int rows = (int)rows64;
  const void* kern = nullptr;
  size_t smem = 0;
  if (mode == 0) {
    kern = depth == 1 ? (const void*)gather_lsu_probe<1> : depth == 2 ? (const void*)gather_lsu_probe<2>
                                                                      : (const void*)gather_lsu_probe<4>;
  } else {
    kern = depth == 4 ? (const void*)gather_tma_probe<4> : depth == 8 ? (const void*)gather_tma_probe<8>
                                                                      : (const void*)gather_tma_probe<16>;
    smem = 2048 + (size_t)(threads / 32) * depth * 1024;
    TE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  int occ = 0;
  TE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, smem));
  if (occ < blocks_per_sm) {
    te_set_error("te_probe_gather: %d blocks per SM do not fit (%d)", blocks_per_sm, occ);
    return TE_ERR_UNSUPPORTED;
  }
  int4 *X = nullptr, *out = nullptr;
  int32_t* own_idx = nullptr;
  unsigned int* err = nullptr;
  unsigned long long* sum = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto done = [&](int rc) {
    te_free(X);
    te_free(out);
    te_free(own_idx);
    te_free(err);
    te_free(sum);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return rc;
  };
  if (te_cuda_check(te_malloc(&X, sizeof(int4) * table), "gather probe") != TE_OK ||
      te_cuda_check(te_malloc(&out, sizeof(int4) * warps * 32), "gather probe") != TE_OK ||
      te_cuda_check(te_malloc(&err, sizeof(unsigned int)), "gather probe") != TE_OK ||
      te_cuda_check(te_malloc(&sum, sizeof(unsigned long long)), "gather probe") != TE_OK ||
      te_cuda_check(cudaMemset(err, 0, sizeof(unsigned int)), "gather probe") != TE_OK ||
      te_cuda_check(cudaMemset(sum, 0, sizeof(unsigned long long)), "gather probe") != TE_OK)
    return done(TE_ERR_CUDA);
  gather_fill_table<<<te_grid_for(table, 256, 4), 256>>>(X, table);
  const int32_t* idx = M ? M->sell.col : nullptr;
  if (!M) {
    if (te_cuda_check(te_malloc(&own_idx, sizeof(int32_t) * count), "gather probe") != TE_OK) return done(TE_ERR_CUDA);
    gather_random_indices<<<te_grid_for(count, 256, 4), 256>>>(own_idx, count, table, 0x5eedull);
    idx = own_idx;
  }
  CUtensorMap tm;
  if (mode == 1) {
    PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", (void**)&encode, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !encode) {
      te_set_error("te_probe_gather: cuTensorMapEncodeTiled is not available");
      return done(TE_ERR_UNSUPPORTED);
    }
    // the table as int32 [table][4]: box of one row of 16 bytes
    const cuuint64_t gdim[2] = {4, (cuuint64_t)table};
    const cuuint64_t gstride[1] = {16};
    const cuuint32_t box[2] = {4, 1};
    const cuuint32_t estride[2] = {1, 1};
    if (encode(&tm, CU_TENSOR_MAP_DATA_TYPE_INT32, 2, X, gdim, gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
      te_set_error("te_probe_gather: tensor map encoding failed");
      return done(TE_ERR_UNSUPPORTED);
    }
  }
  if (te_cuda_check(cudaEventCreate(&e0), "gather probe") != TE_OK ||
      te_cuda_check(cudaEventCreate(&e1), "gather probe") != TE_OK)
    return done(TE_ERR_CUDA);
  const int limit = 1 << 22;
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {  // the first launch warms up
    cudaEventRecord(e0);
    if (mode == 0) {
      if (depth == 1) gather_lsu_probe<1><<<blocks, threads>>>(X, idx, rows, out);
      else if (depth == 2) gather_lsu_probe<2><<<blocks, threads>>>(X, idx, rows, out);
      else gather_lsu_probe<4><<<blocks, threads>>>(X, idx, rows, out);
    } else {
      if (depth == 4) gather_tma_probe<4><<<blocks, threads, smem>>>(tm, idx, rows, out, err, limit);
      else if (depth == 8) gather_tma_probe<8><<<blocks, threads, smem>>>(tm, idx, rows, out, err, limit);
      else gather_tma_probe<16><<<blocks, threads, smem>>>(tm, idx, rows, out, err, limit);
    }
    cudaEventRecord(e1);
    if (te_cuda_check(cudaEventSynchronize(e1), "gather probe") != TE_OK) return done(TE_ERR_CUDA);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  gather_checksum<<<te_grid_for(warps * 32, 256, 4), 256>>>(out, warps * 32, sum);
  unsigned int herr = 0;
  unsigned long long hsum = 0;
  if (te_cuda_check(cudaMemcpy(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost), "gather probe") != TE_OK ||
      te_cuda_check(cudaMemcpy(&hsum, sum, sizeof(hsum), cudaMemcpyDeviceToHost), "gather probe") != TE_OK)
    return done(TE_ERR_CUDA);
  if (herr) {
    te_set_error("te_probe_gather: an mbarrier wait gave up");
    return done(TE_ERR_DEVICE_TIMEOUT);
  }
  *rows_per_s = (double)warps * rows * 32 / (best * 1e-3);
  *checksum = hsum;
  return done(TE_OK);
}
