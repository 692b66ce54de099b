// te_lanczos.cu -- one Lanczos iteration of arnoldiAlgorithm
// (core/krylovTimeEvolver.cpp:523-571) as two grid passes.
//
// The basis is kept unnormalised: u_0 = currentVec, v_j = s_j u_j with
// s_j = 1/beta_j.  Iteration j:
//   pass 1 (apply):  w = A v_j + beta_j v_{j-1}       (A = -i expFactor H; the
//                    reference subtracts H[j-1,j] = -beta_j, :537-541)
//                    alpha_j = <v_j, w>                (:542-543)
//   pass 2 (update): u_{j+1} = w - alpha_j v_j         (:544-546)
//                    beta_{j+1} = ||u_{j+1}||          (:548)
//                    lucky breakdown if beta_{j+1} < tolRate (:551-555)
// The 1/beta scaling of :558-565 is deferred into s_{j+1}, so no pass rewrites
// a vector.  Each pass finishes its reduction in the last block to complete
// (fixed order), so the Krylov coefficients never leave the device.  Pass 1
// runs on the SELL-32 layout: a warp owns 32 equal-length rows.
#include "te_internal.cuh"
#include "te_reduce.cuh"
#include "te_sell.cuh"

__device__ __forceinline__ bool te_step_inactive(const TeDevState* ds) {
  return ds->fatal != 0 || ds->done != 0 || ds->breakdown != 0;
}

template <bool REAL, bool HAS_PREV>
__global__ void __launch_bounds__(TE_THREADS) lanczos_apply_kernel(
    int64_t n, int64_t n_chunks, const int64_t* __restrict__ chunk_off, const int32_t* __restrict__ col,
    const double* __restrict__ val, const double2* __restrict__ u_j, const double2* __restrict__ u_jm1,
    double2* __restrict__ w, TeDevState* ds, double* partials, int j) {
  __shared__ double scratch[2 * 32];
  if (te_step_inactive(ds)) return;
  const int lane = threadIdx.x & 31;
  const double sj = ds->s[j];
  const double g = ds->exp_factor * sj;  // A v_j = -i g H u_j
  const double cprev = HAS_PREV ? ds->beta[j] * ds->s[j - 1] : 0.0;
  double acc[2] = {0.0, 0.0};
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t c = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < n_chunks; c += warps) {
    double2 y = te_sell_row<REAL>(chunk_off, col, val, u_j, c, lane);
    const int64_t r = c * 32 + lane;
    if (r < n) {
      double2 wr;
      if (HAS_PREV) {
        double2 up = u_jm1[r];
        wr.x = fma(cprev, up.x, g * y.y);
        wr.y = fma(cprev, up.y, -g * y.x);
      } else {
        wr.x = g * y.y;
        wr.y = -g * y.x;
      }
      w[r] = wr;
      double2 uj = u_j[r];
      // conj(u_j) * w
      acc[0] = fma(uj.x, wr.x, fma(uj.y, wr.y, acc[0]));
      acc[1] = fma(uj.x, wr.y, fma(-uj.y, wr.x, acc[1]));
    }
  }
  te_block_sum<2>(acc, scratch);
  if (te_publish_partials<2>(acc, partials, &ds->counter[0])) {
    double tot[2];
    te_final_sum<2>(tot, partials, &ds->counter[0], scratch);
    if (threadIdx.x == 0) ds->alpha[j] = make_double2(sj * tot[0], sj * tot[1]);
  }
}

template <bool STORE>
__global__ void __launch_bounds__(TE_THREADS) lanczos_update_kernel(int64_t n, const double2* __restrict__ w,
                                                                    const double2* __restrict__ u_j,
                                                                    double2* __restrict__ u_jp1, TeDevState* ds,
                                                                    double* partials, int j) {
  __shared__ double scratch[32];
  if (te_step_inactive(ds)) return;
  const double sj = ds->s[j];
  const double2 a = ds->alpha[j];
  const double gr = a.x * sj, gi = a.y * sj;  // gamma = alpha_j s_j
  double acc[1] = {0.0};
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double2 wv = w[r];
    double2 u = u_j[r];
    double2 o;
    o.x = fma(-gr, u.x, fma(gi, u.y, wv.x));
    o.y = fma(-gr, u.y, fma(-gi, u.x, wv.y));
    if (STORE) u_jp1[r] = o;
    acc[0] = fma(o.x, o.x, fma(o.y, o.y, acc[0]));
  }
  te_block_sum<1>(acc, scratch);
  if (te_publish_partials<1>(acc, partials, &ds->counter[1])) {
    double tot[1];
    te_final_sum<1>(tot, partials, &ds->counter[1], scratch);
    if (threadIdx.x == 0) {
      const double beta = sqrt(tot[0]);
      const int m = ds->m_cur;
      if (beta < ds->tol_rate) {  // lucky breakdown (:551-555)
        ds->breakdown = 1;
        ds->m_eff = j + 1;
        ds->h = beta;
      } else if (j + 1 != m) {
        ds->beta[j + 1] = beta;
        ds->s[j + 1] = 1.0 / beta;
      } else {
        ds->h = beta;
        ds->m_eff = m;
      }
    }
  }
}

void te_launch_lanczos_apply(const TeSell& A, bool is_real, const double2* u_j, const double2* u_jm1, double2* w,
                             TeDevState* ds, double* partials, int j, cudaStream_t st) {
  const int grid = te_grid_for(A.n_chunks * 32, TE_THREADS, 8);
  if (is_real) {
    if (j > 0)
      lanczos_apply_kernel<true, true><<<grid, TE_THREADS, 0, st>>>(A.n, A.n_chunks, A.chunk_off, A.col, A.val, u_j,
                                                                    u_jm1, w, ds, partials, j);
    else
      lanczos_apply_kernel<true, false><<<grid, TE_THREADS, 0, st>>>(A.n, A.n_chunks, A.chunk_off, A.col, A.val, u_j,
                                                                     u_jm1, w, ds, partials, j);
  } else {
    if (j > 0)
      lanczos_apply_kernel<false, true><<<grid, TE_THREADS, 0, st>>>(A.n, A.n_chunks, A.chunk_off, A.col, A.val, u_j,
                                                                     u_jm1, w, ds, partials, j);
    else
      lanczos_apply_kernel<false, false><<<grid, TE_THREADS, 0, st>>>(A.n, A.n_chunks, A.chunk_off, A.col, A.val,
                                                                      u_j, u_jm1, w, ds, partials, j);
  }
}

void te_launch_lanczos_update(int64_t n, const double2* w, const double2* u_j, double2* u_jp1, TeDevState* ds,
                              double* partials, int j, cudaStream_t st) {
  const int grid = te_grid_for(n, TE_THREADS, 8);
  if (u_jp1)
    lanczos_update_kernel<true><<<grid, TE_THREADS, 0, st>>>(n, w, u_j, u_jp1, ds, partials, j);
  else
    lanczos_update_kernel<false><<<grid, TE_THREADS, 0, st>>>(n, w, u_j, u_jp1, ds, partials, j);
}
