// te_adjoint.cu -- gradients of a sampled expectation value with respect to
// the couplings of H = sum_k theta_k H_k.
//
// Loss L(theta) = <psi(T)|O|psi(T)>, psi(T) = exp(-i H T) v.  With the costate
// lambda(s) = exp(+i H (T - s)) O psi(T) (Duhamel's formula),
//   dL/dtheta_k = 2 Im int_0^T <lambda(s)| H_k |psi(s)> ds.
// Pipeline, all on the GPU through the evolver of te_evolver.cu:
//   1. forward evolution of v under H(theta) to T, sampling psi at the
//      Gauss-Legendre nodes of every checkpoint interval [c, c + dt] (and at 0,
//      T); the sampled states come from the Krylov basis of the step that
//      contains them, so no extra Lanczos work is done, and they are kept in
//      HBM (the memory-lean variant would keep one state per interval and
//      recompute the interval);
//   2. lambda(T) = O psi(T), normalised, evolved with exp(+i H tau) (expFactor
//      -1) to tau = T, sampled at tau = T - s for the same nodes s;
//   3. one fused bilinear pass over all terms and nodes:
//      S[q][k] = Im sum_i conj(lambda_i(s_q)) (H_k psi(s_q))_i, and
//      grad_k = 2 ||lambda(T)|| sum_q w_q S[q][k].
// No counterpart in the reference (which has no differentiation); the forward
// evolution is the reference's krylovTimeEvolver algorithm.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "te_internal.cuh"
#include "te_reduce.cuh"

namespace {

// Gauss-Legendre nodes / weights on [-1, 1] by Newton iteration on P_q.
void gauss_legendre(int q, std::vector<double>& x, std::vector<double>& w) {
  x.resize(q);
  w.resize(q);
  for (int i = 0; i < q; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (q + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= q; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      double pp = q * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / pp;
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= q; ++k) {
      double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    double pp = q * (z * p1 - p0) / (z * z - 1.0);
    x[i] = -z;  // ascending
    w[i] = 2.0 / ((1.0 - z * z) * pp * pp);
  }
}

__global__ void scale_kernel(int64_t n, const double2* __restrict__ in, double s, double2* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = in[i];
    out[i] = make_double2(s * v.x, s * v.y);
  }
}

// ||x||^2 with the last-block reduction (fixed order).
__global__ void __launch_bounds__(TE_THREADS) norm2_simple_kernel(int64_t n, const double2* __restrict__ x,
                                                                  double* partials, unsigned int* counter,
                                                                  double* out) {
  __shared__ double scratch[32];
  double acc[1] = {0.0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = x[i];
    acc[0] = fma(v.x, v.x, fma(v.y, v.y, acc[0]));
  }
  te_block_sum<1>(acc, scratch);
  if (te_publish_partials<1>(acc, partials, counter)) {
    double tot[1];
    te_final_sum<1>(tot, partials, counter, scratch);
    if (threadIdx.x == 0) *out = tot[0];
  }
}

struct TermGeom {
  int n_terms;
  int64_t n, n_pad;                // rows per term, padded to whole warps
  const int32_t* const* row_ptr;   // device array of K pointers (original order CSR)
  const int32_t* const* col;
  const double* const* val;
  const unsigned char* is_real;    // per term
  const int32_t* iperm;            // original index -> evolver row
};

// S[q][chunk] partials: for node q (forward index qf, backward index qb) and
// the 32-row chunk `chunk` of term k = chunk / (n_pad / 32):
//   Im sum_rows conj(lambda_i) (H_k psi)_i.
__global__ void __launch_bounds__(TE_THREADS) bilinear_kernel(TermGeom g, const double2* __restrict__ psi_store,
                                                              const double2* __restrict__ lam_store, int64_t ld,
                                                              const int* __restrict__ fwd_index,
                                                              const int* __restrict__ bwd_index, int n_nodes,
                                                              double* __restrict__ partials) {
  const int lane = threadIdx.x & 31;
  const int64_t chunks_per_term = g.n_pad / 32;
  const int64_t n_chunks = chunks_per_term * g.n_terms;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t c = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < n_chunks; c += warps) {
    const int k = (int)(c / chunks_per_term);
    const int64_t i = (c - (int64_t)k * chunks_per_term) * 32 + lane;
    const bool valid = i < g.n;
    const int32_t* __restrict__ rp = g.row_ptr[k];
    const int32_t* __restrict__ ci = g.col[k];
    const double* __restrict__ vv = g.val[k];
    const bool real = g.is_real[k] != 0;
    const int32_t b = valid ? rp[i] : 0, e = valid ? rp[i + 1] : 0;
    const int32_t ri = valid ? g.iperm[i] : 0;
    for (int q = 0; q < n_nodes; ++q) {
      const double2* __restrict__ psi = psi_store + (int64_t)fwd_index[q] * ld;
      const double2* __restrict__ lam = lam_store + (int64_t)bwd_index[q] * ld;
      double yr = 0.0, yi = 0.0;
      for (int32_t p = b; p < e; ++p) {
        const double2 x = psi[g.iperm[ci[p]]];
        if (real) {
          const double a = vv[p];
          yr = fma(a, x.x, yr);
          yi = fma(a, x.y, yi);
        } else {
          const double2 a = reinterpret_cast<const double2*>(vv)[p];
          yr = fma(a.x, x.x, fma(-a.y, x.y, yr));
          yi = fma(a.x, x.y, fma(a.y, x.x, yi));
        }
      }
      double im = 0.0;
      if (valid) {
        const double2 l = lam[ri];
        im = fma(l.x, yi, -l.y * yr);  // Im(conj(l) y)
      }
      im = te_warp_sum(im);
      if (lane == 0) partials[(int64_t)q * n_chunks + c] = im;
    }
  }
}

// grad[k] = scale * sum_q w_q sum_{chunks of term k} partials[q][chunk] (one block per term).
__global__ void __launch_bounds__(TE_THREADS) bilinear_reduce_kernel(int n_terms, int64_t chunks_per_term,
                                                                     const double* __restrict__ partials,
                                                                     const double* __restrict__ weights, int n_nodes,
                                                                     double scale, double* grad) {
  __shared__ double scratch[32];
  const int k = blockIdx.x;
  const int64_t n_chunks = chunks_per_term * n_terms;
  double acc[1] = {0.0};
  for (int q = 0; q < n_nodes; ++q) {
    double s = 0.0;
    for (int64_t c = threadIdx.x; c < chunks_per_term; c += blockDim.x)
      s += partials[(int64_t)q * n_chunks + (int64_t)k * chunks_per_term + c];
    acc[0] = fma(weights[q], s, acc[0]);
  }
  te_block_sum<1>(acc, scratch);
  if (threadIdx.x == 0) grad[k] = scale * acc[0];
}

}  // namespace

struct te_adjoint_s {
  int K = 0;
  std::vector<te_matrix> terms;
  te_matrix O = nullptr;
  int64_t n = 0;
  std::vector<double> v0;
  double T = 0, tol = 0, interval = 0;
  int m = 40, q = 0;
  std::vector<double> times, weights;  // forward sample times and their quadrature weights
  // host CSR copies of the terms (original order) for assembling H(theta)
  std::vector<std::vector<int32_t>> rp, ci;
  std::vector<std::vector<double>> vals;  // interleaved complex
  // device
  double2* store_psi = nullptr;
  double2* store_lam = nullptr;
  double2* lam0 = nullptr;
  double* partials = nullptr;
  double* red = nullptr;  // reduction partials for norms
  unsigned int* counter = nullptr;
  double* d_scalar = nullptr;
  double* d_weights = nullptr;
  int* d_fwd = nullptr;
  int* d_bwd = nullptr;
  double* d_grad = nullptr;
  const int32_t** d_rp = nullptr;
  const int32_t** d_ci = nullptr;
  const double** d_val = nullptr;
  unsigned char* d_real = nullptr;
  te_result fwd{}, bwd{};
  int64_t launches = 0;
};

namespace {

void free_adjoint(te_adjoint a) {
  if (!a) return;
  cudaFree(a->store_psi);
  cudaFree(a->store_lam);
  cudaFree(a->lam0);
  cudaFree(a->partials);
  cudaFree(a->red);
  cudaFree(a->counter);
  cudaFree(a->d_scalar);
  cudaFree(a->d_weights);
  cudaFree(a->d_fwd);
  cudaFree(a->d_bwd);
  cudaFree(a->d_grad);
  cudaFree(a->d_rp);
  cudaFree(a->d_ci);
  cudaFree(a->d_val);
  cudaFree(a->d_real);
  delete a;
}

// H(theta) = sum_k theta_k H_k as one matrix (rows keep the term order).
int assemble(te_adjoint a, const double* theta, te_matrix* out) {
  const int64_t n = a->n;
  std::vector<int64_t> rp(n + 1, 0);
  for (int k = 0; k < a->K; ++k)
    for (int64_t r = 0; r < n; ++r) rp[r + 1] += a->rp[k][r + 1] - a->rp[k][r];
  for (int64_t r = 0; r < n; ++r) rp[r + 1] += rp[r];
  const int64_t nnz = rp[n];
  std::vector<int32_t> ci(nnz);
  std::vector<double> vv(2 * nnz);
  std::vector<int64_t> fill(rp.begin(), rp.end() - 1);
  for (int64_t r = 0; r < n; ++r)
    for (int k = 0; k < a->K; ++k)
      for (int32_t p = a->rp[k][r]; p < a->rp[k][r + 1]; ++p) {
        const int64_t d = fill[r]++;
        ci[d] = a->ci[k][p];
        vv[2 * d] = theta[k] * a->vals[k][2 * p];
        vv[2 * d + 1] = theta[k] * a->vals[k][2 * p + 1];
      }
  return te_matrix_create_csr(n, n, nnz, rp.data(), ci.data(), vv.data(), 1, out);
}

int evolve_fixed(te_matrix H, const double* v_host, const double* v_dev, double T, double sampling, double exp_factor,
                 double tol, int m, const std::vector<double>* times, double2* store, int64_t ld, te_matrix O,
                 te_result* res, double* last_sample, double2* last_state_dev, int64_t* launches) {
  te_params p{};
  p.t = T;
  p.sampling_step = sampling;
  p.exp_factor = exp_factor;
  p.tol = tol;
  p.m = m;
  std::vector<double> zero;
  te_evolver ev = nullptr;
  int rc;
  if (v_host) {
    rc = te_evolver_create(H, v_host, &p, &ev);
  } else {
    // a normalised placeholder for creation, then the device start vector
    zero.assign(2 * H->n_rows, 0.0);
    zero[0] = 1.0;
    rc = te_evolver_create(H, zero.data(), &p, &ev);
    if (rc == TE_OK) rc = te_evolver_reset(ev, v_dev, 1);
  }
  if (rc != TE_OK) return rc;
  if (times) rc = te_evolver_set_schedule(ev, times->data(), (int64_t)times->size(), store, ld);
  if (rc == TE_OK && O) rc = te_evolver_add_sparse_observable(ev, O);
  if (rc == TE_OK) rc = te_evolver_run(ev, res);
  if (rc == TE_OK && O && last_sample) {
    const int64_t ns = times ? (int64_t)times->size() : (int64_t)std::floor(T / sampling) + 1;
    std::vector<double> s(ns);
    rc = te_evolver_samples(ev, 0, s.data(), ns);
    *last_sample = s[ns - 1];
  }
  if (rc == TE_OK && last_state_dev) {
    const double* st = nullptr;
    rc = te_evolver_state_device(ev, &st);
    if (rc == TE_OK)
      rc = te_cuda_check(cudaMemcpy(last_state_dev, st, sizeof(double2) * H->n_rows, cudaMemcpyDeviceToDevice),
                         "state copy");
  }
  if (launches) *launches += te_evolver_launch_count(ev);
  te_evolver_destroy(ev);
  return rc;
}

}  // namespace

extern "C" int te_adjoint_create(int n_terms, const te_matrix* terms, te_matrix O, const double* v_host, double T,
                                 double tol, int m, double checkpoint_interval, int nodes_per_interval,
                                 te_adjoint* out) {
  if (n_terms < 1 || !terms || !O || !v_host || !out || !(T > 0) || !(tol > 0) || m < 1 ||
      !(checkpoint_interval > 0) || nodes_per_interval < 1 || nodes_per_interval > 256) {
    te_set_error("te_adjoint_create: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  const int64_t n = terms[0]->n_rows;
  for (int k = 0; k < n_terms; ++k)
    if (!terms[k] || terms[k]->n_rows != n || terms[k]->n_cols != n) {
      te_set_error("te_adjoint_create: every term must be a square matrix of the same size");
      return TE_ERR_DIM;
    }
  if (O->n_rows != n || O->n_cols != n) {
    te_set_error("Incompatible dimensions");
    return TE_ERR_DIM;
  }
  te_adjoint a = new te_adjoint_s();
  auto fail = [&](int rc) {
    free_adjoint(a);
    return rc;
  };
  a->K = n_terms;
  a->terms.assign(terms, terms + n_terms);
  a->O = O;
  a->n = n;
  a->v0.assign(v_host, v_host + 2 * n);
  a->T = T;
  a->tol = tol;
  a->m = m;
  a->interval = checkpoint_interval;
  a->q = nodes_per_interval;
  // host copies of the terms
  a->rp.resize(n_terms);
  a->ci.resize(n_terms);
  a->vals.resize(n_terms);
  for (int k = 0; k < n_terms; ++k) {
    te_matrix H = terms[k];
    a->rp[k].resize(n + 1);
    a->ci[k].resize(H->nnz);
    a->vals[k].assign(2 * H->nnz, 0.0);
    int rc = te_cuda_check(cudaMemcpy(a->rp[k].data(), H->row_ptr, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost),
                           "term");
    if (rc == TE_OK && H->nnz)
      rc = te_cuda_check(cudaMemcpy(a->ci[k].data(), H->col, sizeof(int32_t) * H->nnz, cudaMemcpyDeviceToHost), "term");
    if (rc == TE_OK && H->nnz) {
      if (H->is_real) {
        std::vector<double> re(H->nnz);
        rc = te_cuda_check(cudaMemcpy(re.data(), H->val, sizeof(double) * H->nnz, cudaMemcpyDeviceToHost), "term");
        for (int64_t p = 0; p < H->nnz; ++p) a->vals[k][2 * p] = re[p];
      } else {
        rc = te_cuda_check(cudaMemcpy(a->vals[k].data(), H->val, sizeof(double) * 2 * H->nnz, cudaMemcpyDeviceToHost),
                           "term");
      }
    }
    if (rc != TE_OK) return fail(rc);
  }
  // sample times: 0, Gauss nodes of every interval, T
  std::vector<double> gx, gw;
  gauss_legendre(nodes_per_interval, gx, gw);
  a->times.push_back(0.0);
  a->weights.push_back(0.0);
  for (double c = 0.0; c < T * (1 - 1e-15); c += checkpoint_interval) {
    const double b = std::min(T, c + checkpoint_interval), h = 0.5 * (b - c), mid = 0.5 * (b + c);
    for (int i = 0; i < nodes_per_interval; ++i) {
      a->times.push_back(mid + h * gx[i]);
      a->weights.push_back(h * gw[i]);
    }
  }
  a->times.push_back(T);
  a->weights.push_back(0.0);
  const int64_t nt = (int64_t)a->times.size();
  // device buffers
  const int64_t n_pad = (n + 31) / 32 * 32;
  const int64_t n_chunks = n_pad / 32 * n_terms;
  int rc = TE_OK;
  if ((rc = te_cuda_check(cudaMalloc(&a->store_psi, sizeof(double2) * n * nt), "psi store")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(cudaMalloc(&a->store_lam, sizeof(double2) * n * nt), "lambda store")) != TE_OK)
    return fail(rc);
  if ((rc = te_cuda_check(cudaMalloc(&a->lam0, sizeof(double2) * n * 2), "lambda")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(cudaMalloc(&a->partials, sizeof(double) * n_chunks * nt), "partials")) != TE_OK)
    return fail(rc);
  if ((rc = te_cuda_check(cudaMalloc(&a->red, sizeof(double) * 4096), "red")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(cudaMalloc(&a->counter, sizeof(unsigned int)), "counter")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(cudaMemset(a->counter, 0, sizeof(unsigned int)), "counter")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(cudaMalloc(&a->d_scalar, sizeof(double)), "scalar")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(cudaMalloc(&a->d_weights, sizeof(double) * nt), "weights")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(cudaMalloc(&a->d_fwd, sizeof(int) * nt), "index")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(cudaMalloc(&a->d_bwd, sizeof(int) * nt), "index")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(cudaMalloc(&a->d_grad, sizeof(double) * n_terms), "grad")) != TE_OK) return fail(rc);
  std::vector<int> fi(nt), bi(nt);
  for (int64_t i = 0; i < nt; ++i) {
    fi[i] = (int)i;
    bi[i] = (int)(nt - 1 - i);
  }
  TE_CUDA(cudaMemcpy(a->d_weights, a->weights.data(), sizeof(double) * nt, cudaMemcpyHostToDevice));
  TE_CUDA(cudaMemcpy(a->d_fwd, fi.data(), sizeof(int) * nt, cudaMemcpyHostToDevice));
  TE_CUDA(cudaMemcpy(a->d_bwd, bi.data(), sizeof(int) * nt, cudaMemcpyHostToDevice));
  std::vector<const int32_t*> hrp(n_terms), hci(n_terms);
  std::vector<const double*> hval(n_terms);
  std::vector<unsigned char> hreal(n_terms);
  for (int k = 0; k < n_terms; ++k) {
    hrp[k] = terms[k]->row_ptr;
    hci[k] = terms[k]->col;
    hval[k] = terms[k]->val;
    hreal[k] = terms[k]->is_real ? 1 : 0;
  }
  if ((rc = te_cuda_check(cudaMalloc(&a->d_rp, sizeof(void*) * n_terms), "terms")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(cudaMalloc(&a->d_ci, sizeof(void*) * n_terms), "terms")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(cudaMalloc(&a->d_val, sizeof(void*) * n_terms), "terms")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(cudaMalloc(&a->d_real, n_terms), "terms")) != TE_OK) return fail(rc);
  TE_CUDA(cudaMemcpy(a->d_rp, hrp.data(), sizeof(void*) * n_terms, cudaMemcpyHostToDevice));
  TE_CUDA(cudaMemcpy(a->d_ci, hci.data(), sizeof(void*) * n_terms, cudaMemcpyHostToDevice));
  TE_CUDA(cudaMemcpy(a->d_val, hval.data(), sizeof(void*) * n_terms, cudaMemcpyHostToDevice));
  TE_CUDA(cudaMemcpy(a->d_real, hreal.data(), n_terms, cudaMemcpyHostToDevice));
  *out = a;
  return TE_OK;
}

extern "C" int te_adjoint_destroy(te_adjoint a) {
  free_adjoint(a);
  return TE_OK;
}

extern "C" int te_adjoint_forward(te_adjoint a, const double* theta, double* loss) {
  if (!a || !theta || !loss) {
    te_set_error("te_adjoint_forward: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  te_matrix H = nullptr;
  int rc = assemble(a, theta, &H);
  if (rc != TE_OK) return rc;
  a->launches = 0;
  rc = evolve_fixed(H, a->v0.data(), nullptr, a->T, a->T, 1.0, a->tol, a->m, nullptr, nullptr, 0, a->O, &a->fwd, loss,
                    nullptr, &a->launches);
  te_matrix_destroy(H);
  return rc;
}

extern "C" int te_adjoint_run(te_adjoint a, const double* theta, double* loss, double* grad) {
  if (!a || !theta || !loss || !grad) {
    te_set_error("te_adjoint_run: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  const int64_t n = a->n, nt = (int64_t)a->times.size();
  te_matrix H = nullptr;
  int rc = assemble(a, theta, &H);
  if (rc != TE_OK) return rc;
  a->launches = 0;
  double2* psiT = a->lam0 + n;  // scratch: psi(T) in the original order
  // 1. forward, sampling psi at every node
  rc = evolve_fixed(H, a->v0.data(), nullptr, a->T, a->T, 1.0, a->tol, a->m, &a->times, a->store_psi, n, a->O,
                    &a->fwd, loss, psiT, &a->launches);
  // 2. costate lambda(T) = O psi(T), normalised, evolved with exp(+i H tau)
  double lam_norm = 0.0;
  if (rc == TE_OK) rc = te_matrix_spmv(a->O, 1.0, 0.0, (const double*)psiT, (double*)a->lam0, nullptr);
  if (rc == TE_OK) {
    norm2_simple_kernel<<<te_grid_for(n, TE_THREADS, 4), TE_THREADS>>>(n, a->lam0, a->red, a->counter, a->d_scalar);
    double nrm2 = 0.0;
    rc = te_cuda_check(cudaMemcpy(&nrm2, a->d_scalar, sizeof(double), cudaMemcpyDeviceToHost), "norm");
    lam_norm = std::sqrt(nrm2);
    a->launches += 3;
  }
  if (rc == TE_OK && lam_norm > 0.0) {
    scale_kernel<<<te_grid_for(n, TE_THREADS, 4), TE_THREADS>>>(n, a->lam0, 1.0 / lam_norm, a->lam0);
    std::vector<double> tau(nt);
    for (int64_t i = 0; i < nt; ++i) tau[i] = a->T - a->times[nt - 1 - i];
    tau[0] = 0.0;
    for (int64_t i = 1; i < nt; ++i) tau[i] = std::max(tau[i], tau[i - 1]);
    rc = te_cuda_check(cudaDeviceSynchronize(), "scale");
    if (rc == TE_OK)
      rc = evolve_fixed(H, nullptr, (const double*)a->lam0, a->T, a->T, -1.0, a->tol, a->m, &tau, a->store_lam, n,
                        nullptr, &a->bwd, nullptr, nullptr, &a->launches);
  }
  // 3. fused bilinear pass over all terms and nodes, then the weighted sums
  if (rc == TE_OK) {
    TermGeom g;
    g.n_terms = a->K;
    g.n = n;
    g.n_pad = (n + 31) / 32 * 32;
    g.row_ptr = a->d_rp;
    g.col = a->d_ci;
    g.val = a->d_val;
    g.is_real = a->d_real;
    g.iperm = H->sell.iperm;
    const int64_t chunks = g.n_pad / 32 * a->K;
    if (lam_norm > 0.0) {
      bilinear_kernel<<<te_grid_for(chunks * 32, TE_THREADS, 8), TE_THREADS>>>(
          g, a->store_psi, a->store_lam, n, a->d_fwd, a->d_bwd, (int)nt, a->partials);
      bilinear_reduce_kernel<<<a->K, TE_THREADS>>>(a->K, g.n_pad / 32, a->partials, a->d_weights, (int)nt,
                                                   2.0 * lam_norm, a->d_grad);
      a->launches += 2;
      rc = te_cuda_check(cudaMemcpy(grad, a->d_grad, sizeof(double) * a->K, cudaMemcpyDeviceToHost), "grad");
    } else {
      for (int k = 0; k < a->K; ++k) grad[k] = 0.0;
    }
  }
  te_matrix_destroy(H);
  return rc == TE_OK ? te_cuda_check(cudaGetLastError(), "adjoint") : rc;
}

extern "C" int te_adjoint_stats(te_adjoint a, te_result* forward, te_result* backward, int64_t* launches,
                                int64_t* n_nodes) {
  if (!a) return TE_ERR_INVALID_ARG;
  if (forward) *forward = a->fwd;
  if (backward) *backward = a->bwd;
  if (launches) *launches = a->launches;
  if (n_nodes) *n_nodes = (int64_t)a->times.size();
  return TE_OK;
}
