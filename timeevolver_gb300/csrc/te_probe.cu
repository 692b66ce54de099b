// te_probe.cu -- FP64 FMA throughput probe (include/te_diag.h).
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
