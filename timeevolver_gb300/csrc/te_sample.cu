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
#include "te_fixed.cuh"
#include "te_internal.cuh"
#include "te_reduce.cuh"
#include "te_rowdot.cuh"

#define TE_COMBINE_GROUP 4

// Rows of G outputs: psi_o[r] = sum_j u_j[r] ys[o][j].  G is a compile-time
// count: on GB300 a predicated-off FP64 instruction still occupies the FP64
// pipe, so every output slot that exists in the code must be a real output.
template <int G>
__device__ __forceinline__ void combine_rows(const TeCombineArgs& a, const double2* const* cols, int m,
                                             const double2 (*ys)[TE_MMAX], const int* slot_s, int S,
                                             double2* last_out, double2* store, int64_t store_ld, int base) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.n; r += (int64_t)gridDim.x * blockDim.x) {
    double2 acc[G];
#pragma unroll
    for (int o = 0; o < G; ++o) acc[o] = make_double2(0.0, 0.0);
    for (int j = 0; j < m; ++j) {
      const double2 u = cols[j][r];
#pragma unroll
      for (int o = 0; o < G; ++o) {
        const double2 y = ys[o][j];
        acc[o].x = fma(u.x, y.x, fma(-u.y, y.y, acc[o].x));
        acc[o].y = fma(u.x, y.y, fma(u.y, y.x, acc[o].y));
      }
    }
#pragma unroll
    for (int o = 0; o < G; ++o) {
      const int slot = slot_s[o];
      if (slot == 0) {
        a.w_out[r] = acc[o];
      } else {
        a.sample_out[(int64_t)(slot - 1) * a.n + r] = acc[o];
        if (slot == S) last_out[r] = acc[o];
        if (store) store[(int64_t)(base + slot - 1) * store_ld + r] = acc[o];
      }
    }
  }
}

// Basis vectors of a row in flight per thread in the fixed-point combine: 8
// measured 10.4 ms per L=12 solve against 11.2 (4) and 13.4 (1).
constexpr int kCombineUnroll = 8;

// The same outputs from the fixed-point copies X_j = round(u_j 2^xs_j) of the
// basis (te_fixed.cuh), on the integer pipes: with c_oj = Y[slot_o][j] 2^-xs_j
// (so that c_oj X_j = Y[slot_o][j] u_j) quantised per output as
// C_oj = round(c_oj 2^sc_o), sc_o putting sum_j (|Re c_oj| + |Im c_oj|) below
// 2^61, psi_o = 2^(62 - sc_o) sum_j C_oj X_j with the limb products of
// te_fix_mac (complex: Re = Cr Xr - Ci Xi, Im = Cr Xi + Ci Xr).  Error per
// component below 4 m 1.25 2^-56 + (m + 1) 2^-61 of sum_j |Y_oj| max|u_j|.
template <int G>
__device__ __forceinline__ void combine_rows_fix(const TeCombineArgs& a, int m, const int4 (*C)[TE_MMAX],
                                                 const int* sc, const int* slot_s, int S, double2* last_out,
                                                 double2* store, int64_t store_ld, int base) {
  const int64_t n = a.n;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    int64_t sr[G], si[G];
#pragma unroll
    for (int o = 0; o < G; ++o) sr[o] = si[o] = 0;
#pragma unroll(kCombineUnroll)
    for (int j = 0; j < m; ++j) {
      const int4 x = __ldcs(a.fx + (int64_t)j * n + r);  // {re0, re1, im0, im1}
#pragma unroll
      for (int o = 0; o < G; ++o) {
        const int4 c = C[o][j];  // {re0, re1, im0, im1}
        sr[o] += te_fix_prod(c.x, c.y, x.x, x.y) - te_fix_prod(c.z, c.w, x.z, x.w);
        si[o] += te_fix_prod(c.x, c.y, x.z, x.w) + te_fix_prod(c.z, c.w, x.x, x.y);
      }
    }
#pragma unroll
    for (int o = 0; o < G; ++o) {
      const double2 v = make_double2(te_i64_to_double(sr[o], 62 - sc[o]), te_i64_to_double(si[o], 62 - sc[o]));
      const int slot = slot_s[o];
      if (slot == 0) {
        a.w_out[r] = v;
      } else {
        a.sample_out[(int64_t)(slot - 1) * n + r] = v;
        if (slot == S) last_out[r] = v;
        if (store) store[(int64_t)(base + slot - 1) * store_ld + r] = v;
      }
    }
  }
}

// psi_o = sum_j u_j Y[slot_o][j] for the outputs of this batch (the step's
// next start vector w, then its samples), one pass over V per group of up to
// four outputs.
__global__ void __launch_bounds__(TE_THREADS) combine_kernel(TeCombineArgs a, TeDevState* ds, double2* last_out) {
  __shared__ double2 ys[TE_COMBINE_GROUP][TE_MMAX];
  __shared__ int4 cfix[TE_COMBINE_GROUP][TE_MMAX];  // fixed-point coefficients (a.fx)
  __shared__ int sc_s[TE_COMBINE_GROUP];
  __shared__ int slot_s[TE_COMBINE_GROUP];
  __shared__ const double2* cols[TE_MMAX];
  if (ds->fatal != 0) return;
  const int want_w = ds->want_w;
  const int S = ds->samples_in_batch;
  const int nout = want_w + S;
  const int m = min(a.m, ds->m_eff);  // a lucky breakdown shrinks the basis of this step
  if (threadIdx.x < TE_MMAX) cols[threadIdx.x] = threadIdx.x < m ? a.cols[threadIdx.x] : nullptr;
  for (int g0 = 0; g0 < nout; g0 += TE_COMBINE_GROUP) {
    const int G = min(TE_COMBINE_GROUP, nout - g0);
    __syncthreads();
    if (threadIdx.x < TE_COMBINE_GROUP) {
      const int o = g0 + threadIdx.x;
      slot_s[threadIdx.x] = want_w ? o : o + 1;  // slot 0 = w, slots 1.. = samples
    }
    __syncthreads();
    for (int i = threadIdx.x; i < G * TE_MMAX; i += blockDim.x) {
      const int o = i / TE_MMAX, j = i % TE_MMAX;
      ys[o][j] = j < m ? ds->Y[slot_s[o] * TE_MMAX + j] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    double2* store = ds->state_store;
    const int64_t sld = ds->store_ld;
    const int base = ds->sample_base;
    if (a.fx) {
      // coefficients c_oj = Y_oj 2^-xs_j in fixed point, per output scale
      if (threadIdx.x < G) {
        double b = 0.0;
        for (int j = 0; j < m; ++j) {
          const int xs = ds->fx_xs[j];
          b += ldexp(fabs(ys[threadIdx.x][j].x), -xs) + ldexp(fabs(ys[threadIdx.x][j].y), -xs);
        }
        sc_s[threadIdx.x] = te_fix_scale(b * (1.0 + 1e-12));
      }
      __syncthreads();
      for (int i = threadIdx.x; i < G * TE_MMAX; i += blockDim.x) {
        const int o = i / TE_MMAX, j = i % TE_MMAX;
        int4 c = make_int4(0, 0, 0, 0);
        if (j < m) {
          const int xs = ds->fx_xs[j];
          const int2 cr = te_fix_split(te_fix_encode(ldexp(ys[o][j].x, -xs), sc_s[o]));
          const int2 ci = te_fix_split(te_fix_encode(ldexp(ys[o][j].y, -xs), sc_s[o]));
          c = make_int4(cr.x, cr.y, ci.x, ci.y);
        }
        cfix[o][j] = c;
      }
      __syncthreads();
      switch (G) {
        case 1: combine_rows_fix<1>(a, m, cfix, sc_s, slot_s, S, last_out, store, sld, base); break;
        case 2: combine_rows_fix<2>(a, m, cfix, sc_s, slot_s, S, last_out, store, sld, base); break;
        case 3: combine_rows_fix<3>(a, m, cfix, sc_s, slot_s, S, last_out, store, sld, base); break;
        default: combine_rows_fix<4>(a, m, cfix, sc_s, slot_s, S, last_out, store, sld, base); break;
      }
      continue;
    }
    switch (G) {
      case 1: combine_rows<1>(a, cols, m, ys, slot_s, S, last_out, store, sld, base); break;
      case 2: combine_rows<2>(a, cols, m, ys, slot_s, S, last_out, store, sld, base); break;
      case 3: combine_rows<3>(a, cols, m, ys, slot_s, S, last_out, store, sld, base); break;
      default: combine_rows<4>(a, cols, m, ys, slot_s, S, last_out, store, sld, base); break;
    }
  }
}

void te_launch_combine(const TeCombineArgs& a, TeDevState* ds, double2* last_out, cudaStream_t st) {
  combine_kernel<<<te_grid_fit((const void*)combine_kernel, a.n, TE_THREADS), TE_THREADS, 0, st>>>(a, ds, last_out);
}

// Diagonal observables: Re sum_i O_ii |psi_i|^2 (= Re zdotc(psi, O psi) for a
// diagonal O); vector observables: |sum_i conj(psi_i) o_i|^2.  ND diagonal and
// NV vector observables per launch, compile-time counts (no predicated FP64).
template <int ND, int NV>
__global__ void __launch_bounds__(TE_THREADS) fused_obs_kernel(int64_t n, const double2* __restrict__ psi_base,
                                                               TeFusedObs f, TeDevState* ds, double* partials,
                                                               double* results, int n_samples_total) {
  constexpr int V = ND + 2 * NV;
  __shared__ double scratch[V * 32];
  __shared__ bool is_last;
  if (ds->fatal != 0) return;
  const int S = ds->samples_in_batch;
  const int base = ds->sample_base;
  for (int s = 0; s < S; ++s) {
    const double2* __restrict__ psi = psi_base + (int64_t)s * n;
    double acc[V];
#pragma unroll
    for (int v = 0; v < V; ++v) acc[v] = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
      const double2 p = psi[r];
      if (ND > 0) {
        const double p2 = fma(p.x, p.x, p.y * p.y);
#pragma unroll
        for (int v = 0; v < ND; ++v) acc[v] = fma(__ldg(f.diag[v] + r), p2, acc[v]);
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const double2 o = __ldg(f.vec[v] + r);
        // conj(psi) * o
        acc[ND + 2 * v] = fma(p.x, o.x, fma(p.y, o.y, acc[ND + 2 * v]));
        acc[ND + 2 * v + 1] = fma(p.x, o.y, fma(-p.y, o.x, acc[ND + 2 * v + 1]));
      }
    }
    te_block_sum<V>(acc, scratch);
    if (threadIdx.x == 0)
#pragma unroll
      for (int v = 0; v < V; ++v) partials[((int64_t)s * V + v) * gridDim.x + blockIdx.x] = acc[v];
  }
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int prev = atomicAdd(&ds->counter[2], 1u);
    is_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  for (int s = 0; s < S; ++s) {
    double tot[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
      double sum = 0.0;
      for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
        sum += __ldcg(partials + ((int64_t)s * V + v) * gridDim.x + b);
      tot[v] = sum;
    }
    te_block_sum<V>(tot, scratch);
    if (threadIdx.x == 0) {
#pragma unroll
      for (int v = 0; v < ND; ++v) results[(int64_t)f.row_diag[v] * n_samples_total + base + s] = tot[v];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const double re = tot[ND + 2 * v], im = tot[ND + 2 * v + 1];
        results[(int64_t)f.row_vec[v] * n_samples_total + base + s] = re * re + im * im;
      }
    }
  }
  if (threadIdx.x == 0) ds->counter[2] = 0u;
}

template <int ND, int NV>
static void launch_fused(int64_t n, const double2* psi, const TeFusedObs& f, TeDevState* ds, double* partials,
                         double* results, int n_samples_total, cudaStream_t st) {
  fused_obs_kernel<ND, NV><<<te_grid_fit((const void*)fused_obs_kernel<ND, NV>, n, TE_THREADS), TE_THREADS, 0, st>>>(n, psi, f, ds, partials, results,
                                                                                 n_samples_total);
}

void te_launch_fused_obs(int64_t n, const double2* psi, const TeFusedObs& f, TeDevState* ds, double* partials,
                         double* results, int n_samples_total, cudaStream_t st) {
  typedef void (*L)(int64_t, const double2*, const TeFusedObs&, TeDevState*, double*, double*, int, cudaStream_t);
  static const L table[TE_FUSED_DIAG + 1][TE_FUSED_VEC + 1] = {
      {nullptr, launch_fused<0, 1>, launch_fused<0, 2>},
      {launch_fused<1, 0>, launch_fused<1, 1>, launch_fused<1, 2>},
      {launch_fused<2, 0>, launch_fused<2, 1>, launch_fused<2, 2>},
      {launch_fused<3, 0>, launch_fused<3, 1>, launch_fused<3, 2>},
      {launch_fused<4, 0>, launch_fused<4, 1>, launch_fused<4, 2>}};
  L fn = table[f.n_diag][f.n_vec];
  if (fn) fn(n, psi, f, ds, partials, results, n_samples_total, st);
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

// Dense observable: Re sum_i conj(psi_i) (O psi)_i for a column-major complex O
// on the original ordering (the zgemv + zdotc of krylovObservables.cpp:119-138).
// One thread per row (column-major: a warp reads 32 consecutive entries of a
// column); psi is staged through shared memory in tiles.
#define TE_DENSE_TILE 1024
__global__ void __launch_bounds__(TE_THREADS) dense_obs_kernel(int64_t n, const double2* __restrict__ O,
                                                               const double2* __restrict__ psi, TeDevState* ds,
                                                               int sample_in_batch, double* partials,
                                                               double* results_row) {
  __shared__ double2 tile[TE_DENSE_TILE];
  __shared__ double scratch[32];
  if (ds->fatal != 0) return;
  double acc[1] = {0.0};
  const int64_t rows_per_pass = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r0 = (int64_t)blockIdx.x * blockDim.x; r0 < n; r0 += rows_per_pass) {
    const int64_t r = r0 + threadIdx.x;
    double yr = 0.0, yi = 0.0;
    for (int64_t j0 = 0; j0 < n; j0 += TE_DENSE_TILE) {
      const int64_t jn = min((int64_t)TE_DENSE_TILE, n - j0);
      __syncthreads();
      for (int64_t k = threadIdx.x; k < jn; k += blockDim.x) tile[k] = psi[j0 + k];
      __syncthreads();
      if (r < n) {
        const double2* __restrict__ col = O + j0 * n + r;
        for (int64_t k = 0; k < jn; ++k) {
          const double2 a = col[k * n];
          const double2 x = tile[k];
          yr = fma(a.x, x.x, fma(-a.y, x.y, yr));
          yi = fma(a.x, x.y, fma(a.y, x.x, yi));
        }
      }
    }
    if (r < n) {
      const double2 p = psi[r];
      acc[0] = fma(p.x, yr, fma(p.y, yi, acc[0]));
    }
  }
  te_block_sum<1>(acc, scratch);
  if (te_publish_partials<1>(acc, partials, &ds->counter[3])) {
    double tot[1];
    te_final_sum<1>(tot, partials, &ds->counter[3], scratch);
    if (threadIdx.x == 0) results_row[ds->sample_base + sample_in_batch] = tot[0];
  }
}

void te_launch_dense_obs(int64_t n, const double2* O, const double2* psi_orig, TeDevState* ds, int sample_in_batch,
                         double* partials, double* results_row, cudaStream_t st) {
  const int grid = te_grid_fit((const void*)dense_obs_kernel, n, TE_THREADS);
  dense_obs_kernel<<<grid, TE_THREADS, 0, st>>>(n, O, psi_orig, ds, sample_in_batch, partials, results_row);
}

__global__ void stop_check_kernel(TeStopConds c, const double* __restrict__ results, int n_samples_total,
                                  TeDevState* ds) {
  if (threadIdx.x != 0 || ds->fatal != 0 || ds->stop_flag != 0) return;
  const int S = ds->samples_in_batch, base = ds->sample_base;
  for (int s = 0; s < S; ++s)
    for (int k = 0; k < c.count; ++k) {
      const double v = results[(int64_t)c.obs[k] * n_samples_total + base + s];
      if (c.direction[k] > 0 ? v >= c.threshold[k] : v <= c.threshold[k]) {
        ds->stop_flag = s + 1;
        return;
      }
    }
}

void te_launch_stop_check(const TeStopConds& c, const double* results, int n_samples_total, TeDevState* ds,
                          cudaStream_t st) {
  stop_check_kernel<<<1, 32, 0, st>>>(c, results, n_samples_total, ds);
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
  norm2_kernel<<<te_grid_fit((const void*)norm2_kernel, n, TE_THREADS), TE_THREADS, 0, st>>>(n, x, ds, partials);
}
