// te_reduce.cuh -- deterministic block and grid reductions.
//
// Grid reductions use the "last block finishes" pattern: every block writes
// its partial sums to partials[value * gridDim.x + block], fences, and bumps a
// counter; the block that brings the counter to gridDim.x sums all partials in
// a fixed order (thread t takes blocks t, t+blockDim, ... sequentially, then a
// fixed tree), so the result does not depend on which block finished last.
#pragma once
#include "te_internal.cuh"

__device__ __forceinline__ double te_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Block sum of NV values per thread; result valid in thread 0.  scratch must
// hold NV * 32 doubles.
template <int NV>
__device__ __forceinline__ void te_block_sum(double (&v)[NV], double* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = te_warp_sum(v[k]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) scratch[k * 32 + warp] = v[k];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = lane < nw ? scratch[k * 32 + lane] : 0.0;
      v[k] = te_warp_sum(x);
    }
  }
  __syncthreads();
}

// Block sum through shared memory first: every thread stores its NV values
// (wide: NV * blockDim.x doubles), then warp 0 adds blockDim.x / 32 values per
// lane and finishes with one shuffle tree.  The FP64 pipe sees
// blockDim.x / 32 + 5 warp-wide additions per value instead of 5 per warp and
// 5 more, which matters for passes bound by FP64 issue.  Result in thread 0.
template <int NV>
__device__ __forceinline__ void te_block_sum_wide(double (&v)[NV], double* wide) {
  const int t = threadIdx.x, B = blockDim.x;
#pragma unroll
  for (int k = 0; k < NV; ++k) wide[k * B + t] = v[k];
  __syncthreads();
  if (t < 32) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = wide[k * B + t];
      for (int i = t + 32; i < B; i += 32) s += wide[k * B + i];
      v[k] = te_warp_sum(s);
    }
  }
  __syncthreads();
}

// Publish NV per-block partials and return true in the block that must do
// the final reduction.  Call from all threads; thread 0 holds the values.
template <int NV>
__device__ __forceinline__ bool te_publish_partials(const double (&v)[NV], double* partials, unsigned int* counter) {
  __shared__ bool is_last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[k * gridDim.x + blockIdx.x] = v[k];
    __threadfence();
    unsigned int prev = atomicAdd(counter, 1u);
    is_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (is_last) __threadfence();
  return is_last;
}

// In the last block: sum the partials of NV values over all blocks in a fixed
// order.  Result valid in thread 0; resets the counter.  extra(out) may add
// further per-thread terms (in an order fixed by the thread index) before the
// block tree.
template <int NV, typename Extra>
__device__ __forceinline__ void te_final_sum(double (&out)[NV], const double* partials, unsigned int* counter,
                                             double* scratch, Extra extra) {
#pragma unroll
  for (int k = 0; k < NV; ++k) out[k] = 0.0;
  // blocks ascending per thread for every value (the loads of consecutive
  // iterations are independent, so the unrolled loop keeps several in flight)
#pragma unroll 4
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] += __ldcg(partials + k * gridDim.x + b);
  }
  extra(out);
  te_block_sum<NV>(out, scratch);
  if (threadIdx.x == 0) *counter = 0u;
}

template <int NV>
__device__ __forceinline__ void te_final_sum(double (&out)[NV], const double* partials, unsigned int* counter,
                                             double* scratch) {
  te_final_sum<NV>(out, partials, counter, scratch, [](double (&)[NV]) {});
}

// Grid barrier with a bounded wait.  Arrival after a fence; the block that
// brings the count to `arrivals` resets it and bumps the generation.  A wait
// that gives up after spin_limit polls sets fatal = TE_ERR_DEVICE_TIMEOUT and
// returns false (the kernel then exits).
__device__ __forceinline__ bool te_grid_barrier(unsigned int* count, unsigned int* gen, int* fatal,
                                                unsigned int spin_limit, unsigned int arrivals) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned int* vgen = gen;
    const unsigned int g0 = *vgen;
    __threadfence();
    if (atomicAdd(count, 1u) == arrivals - 1) {
      atomicExch(count, 0u);
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      unsigned int spins = 0;
      while (*vgen == g0) {
        __nanosleep(32);
        if (++spins > spin_limit) {
          ok = 0;
          atomicExch(fatal, TE_ERR_DEVICE_TIMEOUT);
          break;
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}
