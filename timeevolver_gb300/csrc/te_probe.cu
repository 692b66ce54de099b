// te_probe.cu -- FP64 FMA throughput and issue probes (include/te_diag.h).
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
  TE_CUDA(cudaMalloc(&out, sizeof(double) * blocks * threads));
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
  cudaFree(out);
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
  TE_CUDA(cudaMalloc(&out, sizeof(double) * blocks * threads));
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
  cudaFree(out);
  if (rc != TE_OK) return rc;
  const double cycles_per_ms = (double)khz;  // clock rate in kHz = cycles per ms
  *cycles_indep = ms[0] * cycles_per_ms / (8.0 * iters * warps);
  *cycles_chain = ms[1] * cycles_per_ms / iters;
  return TE_OK;
}
