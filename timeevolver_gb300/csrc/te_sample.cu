// te_sample.cu -- states and observables from the Krylov basis.
//
// Replaces, in krylovTimeEvolver::timeEvolve (core/krylovTimeEvolver.cpp):
//   currentVec = V w                 (:382, cblas_zgemv n x m)
//   sampledState = V y(t_sampling)   (:409-421)
//   sample() -> observable->expectation (:120-126, krylovObservables.cpp:173-236)
//   the final norm check            (:446-452, cblas_dznrm2)
// One pass over the m basis columns produces every output of a batch (the
// next start vector and the batch's samples), so V is read once per batch;
// diagonal and vector observables are reduced in one further pass over the
// batch.  All reductions finish in the last block to complete, in a fixed
// order.
#include "te_internal.cuh"
#include "te_reduce.cuh"
#include "te_rowdot.cuh"

#define TE_COMBINE_GROUP 4

// psi_o = sum_j u_j Y[slot_o][j] for the outputs of this batch.
__global__ void __launch_bounds__(TE_THREADS) combine_kernel(TeCombineArgs a, TeDevState* ds, double2* last_out) {
  __shared__ double2 ys[TE_COMBINE_GROUP][TE_MMAX];
  __shared__ int slot_s[TE_COMBINE_GROUP];
  if (ds->fatal != 0) return;
  const int want_w = ds->want_w;
  const int S = ds->samples_in_batch;
  const int nout = want_w + S;
  const int m = min(a.m, ds->m_eff);  // a lucky breakdown shrinks the basis of this step
  for (int g0 = 0; g0 < nout; g0 += TE_COMBINE_GROUP) {
    const int G = min(TE_COMBINE_GROUP, nout - g0);
    __syncthreads();
    if (threadIdx.x < TE_COMBINE_GROUP) {
      int o = g0 + threadIdx.x;
      slot_s[threadIdx.x] = want_w ? o : o + 1;  // slot 0 = w, slots 1.. = samples
    }
    __syncthreads();
    for (int i = threadIdx.x; i < G * TE_MMAX; i += blockDim.x) {
      int o = i / TE_MMAX, j = i % TE_MMAX;
      ys[o][j] = j < m ? ds->Y[slot_s[o] * TE_MMAX + j] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.n; r += (int64_t)gridDim.x * blockDim.x) {
      double2 acc[TE_COMBINE_GROUP];
#pragma unroll
      for (int o = 0; o < TE_COMBINE_GROUP; ++o) acc[o] = make_double2(0.0, 0.0);
      for (int j = 0; j < m; ++j) {
        const double2 u = a.cols[j][r];
#pragma unroll
        for (int o = 0; o < TE_COMBINE_GROUP; ++o) {
          if (o < G) {
            const double2 y = ys[o][j];
            acc[o].x = fma(u.x, y.x, fma(-u.y, y.y, acc[o].x));
            acc[o].y = fma(u.x, y.y, fma(u.y, y.x, acc[o].y));
          }
        }
      }
#pragma unroll
      for (int o = 0; o < TE_COMBINE_GROUP; ++o) {
        if (o < G) {
          const int slot = slot_s[o];
          if (slot == 0) {
            a.w_out[r] = acc[o];
          } else {
            a.sample_out[(int64_t)(slot - 1) * a.n + r] = acc[o];
            if (slot == S) last_out[r] = acc[o];
          }
        }
      }
    }
  }
}

void te_launch_combine(const TeCombineArgs& a, TeDevState* ds, double2* last_out, cudaStream_t st) {
  combine_kernel<<<te_grid_for(a.n, TE_THREADS, 8), TE_THREADS, 0, st>>>(a, ds, last_out);
}

// Diagonal observables: Re sum_i O_ii |psi_i|^2 (= Re zdotc(psi, O psi) for a
// diagonal O); vector observables: |sum_i conj(psi_i) o_i|^2.  Up to
// TE_FUSED_DIAG + TE_FUSED_VEC observables per launch.
__global__ void __launch_bounds__(TE_THREADS) fused_obs_kernel(int64_t n, const double2* __restrict__ psi_base,
                                                               TeFusedObs f, TeDevState* ds, double* partials,
                                                               double* results, int n_samples_total) {
  __shared__ double scratch[TE_FUSED_VALS * 32];
  __shared__ bool is_last;
  if (ds->fatal != 0) return;
  const int S = ds->samples_in_batch;
  const int base = ds->sample_base;
  const int nd = f.n_diag, nv = f.n_vec;
  for (int s = 0; s < S; ++s) {
    const double2* __restrict__ psi = psi_base + (int64_t)s * n;
    double acc[TE_FUSED_VALS];
#pragma unroll
    for (int v = 0; v < TE_FUSED_VALS; ++v) acc[v] = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
      const double2 p = psi[r];
      const double p2 = fma(p.x, p.x, p.y * p.y);
#pragma unroll
      for (int v = 0; v < TE_FUSED_DIAG; ++v) {
        if (v < nd) acc[v] = fma(__ldg(f.diag[v] + r), p2, acc[v]);
      }
#pragma unroll
      for (int v = 0; v < TE_FUSED_VEC; ++v) {
        if (v < nv) {
          const double2 o = __ldg(f.vec[v] + r);
          // conj(psi) * o
          acc[TE_FUSED_DIAG + 2 * v] = fma(p.x, o.x, fma(p.y, o.y, acc[TE_FUSED_DIAG + 2 * v]));
          acc[TE_FUSED_DIAG + 2 * v + 1] = fma(p.x, o.y, fma(-p.y, o.x, acc[TE_FUSED_DIAG + 2 * v + 1]));
        }
      }
    }
    te_block_sum<TE_FUSED_VALS>(acc, scratch);
    if (threadIdx.x == 0)
      for (int v = 0; v < TE_FUSED_VALS; ++v)
        partials[((int64_t)s * TE_FUSED_VALS + v) * gridDim.x + blockIdx.x] = acc[v];
  }
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned int prev = atomicAdd(&ds->counter[2], 1u);
    is_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  for (int s = 0; s < S; ++s) {
    double tot[TE_FUSED_VALS];
#pragma unroll
    for (int v = 0; v < TE_FUSED_VALS; ++v) {
      double sum = 0.0;
      for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
        sum += __ldcg(partials + ((int64_t)s * TE_FUSED_VALS + v) * gridDim.x + b);
      tot[v] = sum;
    }
    te_block_sum<TE_FUSED_VALS>(tot, scratch);
    if (threadIdx.x == 0) {
      for (int v = 0; v < nd; ++v) results[(int64_t)f.row_diag[v] * n_samples_total + base + s] = tot[v];
      for (int v = 0; v < nv; ++v) {
        const double re = tot[TE_FUSED_DIAG + 2 * v], im = tot[TE_FUSED_DIAG + 2 * v + 1];
        results[(int64_t)f.row_vec[v] * n_samples_total + base + s] = re * re + im * im;
      }
    }
  }
  if (threadIdx.x == 0) ds->counter[2] = 0u;
}

void te_launch_fused_obs(int64_t n, const double2* psi, const TeFusedObs& f, TeDevState* ds, double* partials,
                         double* results, int n_samples_total, cudaStream_t st) {
  fused_obs_kernel<<<te_grid_for(n, TE_THREADS, 4), TE_THREADS, 0, st>>>(n, psi, f, ds, partials, results,
                                                                         n_samples_total);
}

// General sparse observable: Re sum_i conj(psi_i) (O psi)_i on the original
// ordering (krylovObservables.cpp:187-189).  Result goes to results_row[base + s].
template <bool REAL>
__global__ void __launch_bounds__(TE_THREADS) general_obs_kernel(int64_t n, const int32_t* __restrict__ row_ptr,
                                                                 const int32_t* __restrict__ col,
                                                                 const double* __restrict__ val,
                                                                 const double2* __restrict__ psi, TeDevState* ds,
                                                                 int sample_in_batch, double* partials,
                                                                 double* results_row) {
  __shared__ double scratch[32];
  if (ds->fatal != 0) return;
  double acc[1] = {0.0};
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const double2 y = te_row_dot<REAL>(row_ptr, col, val, psi, (int32_t)r);
    const double2 p = psi[r];
    acc[0] = fma(p.x, y.x, fma(p.y, y.y, acc[0]));
  }
  te_block_sum<1>(acc, scratch);
  if (te_publish_partials<1>(acc, partials, &ds->counter[3])) {
    double tot[1];
    te_final_sum<1>(tot, partials, &ds->counter[3], scratch);
    if (threadIdx.x == 0) results_row[ds->sample_base + sample_in_batch] = tot[0];
  }
}

void te_launch_general_obs(const te_matrix_s& O, const double2* psi_orig, TeDevState* ds, int sample_in_batch,
                           double* partials, double* results_row, cudaStream_t st) {
  const int grid = te_grid_for(O.n_rows, TE_THREADS, 8);
  if (O.is_real)
    general_obs_kernel<true><<<grid, TE_THREADS, 0, st>>>(O.n_rows, O.row_ptr, O.col, O.val, psi_orig, ds,
                                                          sample_in_batch, partials, results_row);
  else
    general_obs_kernel<false><<<grid, TE_THREADS, 0, st>>>(O.n_rows, O.row_ptr, O.col, O.val, psi_orig, ds,
                                                           sample_in_batch, partials, results_row);
}

// ||x||^2 into ds->norm2_final (cblas_dznrm2 of :446).
__global__ void __launch_bounds__(TE_THREADS) norm2_kernel(int64_t n, const double2* __restrict__ x, TeDevState* ds,
                                                           double* partials) {
  __shared__ double scratch[32];
  double acc[1] = {0.0};
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const double2 p = x[r];
    acc[0] = fma(p.x, p.x, fma(p.y, p.y, acc[0]));
  }
  te_block_sum<1>(acc, scratch);
  if (te_publish_partials<1>(acc, partials, &ds->counter[3])) {
    double tot[1];
    te_final_sum<1>(tot, partials, &ds->counter[3], scratch);
    if (threadIdx.x == 0) ds->norm2_final = tot[0];
  }
}

void te_launch_norm2(int64_t n, const double2* x, double* partials, TeDevState* ds, cudaStream_t st) {
  norm2_kernel<<<te_grid_for(n, TE_THREADS, 8), TE_THREADS, 0, st>>>(n, x, ds, partials);
}
