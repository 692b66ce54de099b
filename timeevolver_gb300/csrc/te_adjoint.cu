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
//   3. one bilinear pass over the entries of H(theta)'s SELL layout (rows
//      and columns in the evolver's order, every slot tagged with its term):
//        G_p = sum_q w_q conj(lambda_i(s_q)) psi_j(s_q)   for entry p = (i, j),
//      then grad_k = 2 ||lambda(T)|| sum_{p in term k} Im(a_p G_p), a_p the
//      entry of H_k, summed per term in a fixed order.
// No counterpart in the reference (which has no differentiation); the forward
// evolution is the reference's krylovTimeEvolver algorithm.
#include <algorithm>
#include <chrono>
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

// values of H(theta) from the per-entry term index and the theta = 1 values
template <typename V>
__global__ void refresh_values_kernel(int64_t count, const int32_t* __restrict__ term, const V* __restrict__ base,
                                      const double* __restrict__ theta, V* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const int k = term[i];
    const double th = k >= 0 ? theta[k] : 0.0;
    out[i] = base[i] * th;
  }
}

__device__ __forceinline__ double2 operator*(const double2& a, double s) { return make_double2(a.x * s, a.y * s); }

// 1-norm of H(theta) (maximum absolute column sum, matrixDataTypes.cpp:67-79):
// one thread per column sums |theta_term| |a| over the column's entries in
// ascending entry order; the maximum goes through the bit patterns of the
// (non-negative) sums, so the result does not depend on the schedule.
__global__ void norm1_kernel(int64_t n, const int64_t* __restrict__ col_ptr, const int32_t* __restrict__ col_entry,
                             const int32_t* __restrict__ term, const double* __restrict__ absval,
                             const double* __restrict__ theta, unsigned long long* max_bits) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int64_t p = col_ptr[c]; p < col_ptr[c + 1]; ++p) {
      const int32_t e = col_entry[p];
      s = __dadd_rn(s, __dmul_rn(fabs(theta[term[e]]), absval[e]));
    }
    atomicMax(max_bits, (unsigned long long)__double_as_longlong(s));
  }
}

// Per-slot contributions Im(a_p G_p) of the bilinear form (see the file head).
// One warp per 32-row chunk; the slots are visited in groups of G so that a
// group's columns and sums stay in registers while the nodes stream past.
template <bool REAL, int G>
__global__ void __launch_bounds__(TE_THREADS) bilinear_kernel(
    int64_t n, int64_t n_chunks, const int64_t* __restrict__ chunk_off, const int32_t* __restrict__ scol,
    const double* __restrict__ base, const double2* __restrict__ psi_store, const double2* __restrict__ lam_store,
    int64_t ld, const int* __restrict__ fwd_index, const int* __restrict__ bwd_index,
    const double* __restrict__ weights, int n_nodes, double* __restrict__ contrib) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t c = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < n_chunks; c += warps) {
    const int64_t i = c * 32 + lane;
    const bool valid = i < n;
    const int64_t off = chunk_off[c];
    const int64_t len = (chunk_off[c + 1] - off) / 32;
    for (int64_t g0 = 0; g0 < len; g0 += G) {
      int32_t col[G];
      double gi[G], gr[G];
#pragma unroll
      for (int e = 0; e < G; ++e) {
        col[e] = (g0 + e < len) ? scol[off + 32 * (g0 + e) + lane] : 0;
        gi[e] = 0.0;
        gr[e] = 0.0;
      }
      for (int q = 0; q < n_nodes; ++q) {
        const double wq = weights[q];
        if (wq == 0.0) continue;  // the end points carry no weight
        double2 l = make_double2(0.0, 0.0);
        if (valid) l = lam_store[(int64_t)bwd_index[q] * ld + i];
        const double lr = wq * l.x, li = wq * l.y;
        const double2* __restrict__ P = psi_store + (int64_t)fwd_index[q] * ld;
#pragma unroll
        for (int e = 0; e < G; ++e) {
          if (g0 + e < len) {
            const double2 x = P[col[e]];
            gi[e] = fma(lr, x.y, fma(-li, x.x, gi[e]));          // Im conj(l) x
            if (!REAL) gr[e] = fma(lr, x.x, fma(li, x.y, gr[e]));  // Re conj(l) x
          }
        }
      }
#pragma unroll
      for (int e = 0; e < G; ++e) {
        if (g0 + e < len) {
          const int64_t sidx = off + 32 * (g0 + e) + lane;
          if (REAL) {
            contrib[sidx] = base[sidx] * gi[e];
          } else {
            const double2 a = reinterpret_cast<const double2*>(base)[sidx];
            contrib[sidx] = fma(a.x, gi[e], a.y * gr[e]);
          }
        }
      }
    }
  }
}

// grad[k] = scale * sum of the contributions of term k's slots (one block per
// term, slots in ascending order, fixed reduction tree).
__global__ void __launch_bounds__(TE_THREADS) bilinear_reduce_kernel(const int64_t* __restrict__ term_ptr,
                                                                     const int64_t* __restrict__ term_slots,
                                                                     const double* __restrict__ contrib, double scale,
                                                                     double* grad) {
  __shared__ double scratch[32];
  const int k = blockIdx.x;
  double acc[1] = {0.0};
  for (int64_t p = term_ptr[k] + threadIdx.x; p < term_ptr[k + 1]; p += blockDim.x) acc[0] += contrib[term_slots[p]];
  te_block_sum<1>(acc, scratch);
  if (threadIdx.x == 0) grad[k] = scale * acc[0];
}

}  // namespace

struct te_adjoint_s {
  int K = 0;
  te_matrix O = nullptr;
  int64_t n = 0;
  std::vector<double> v0;
  double T = 0, tol = 0, interval = 0;
  int m = 40, q = 0;
  std::vector<double> times, weights;  // forward sample times and their quadrature weights
  std::vector<double> tau;             // costate sample times T - s, ascending
  // H(theta) with a fixed pattern: the terms' entries row by row, each entry
  // and SELL slot tagged with its term; theta only rescales the values
  te_matrix Hth = nullptr;
  std::vector<double> theta_now;
  int32_t* d_entry_term = nullptr;  // CSR entries (original order)
  int32_t* d_slot_term = nullptr;   // SELL slots (-1 for padding)
  double* d_entry_base = nullptr;   // theta = 1 values (real: 1 double, complex: 2 per entry)
  double* d_slot_base = nullptr;
  double* d_theta = nullptr;
  int64_t* d_col_ptr = nullptr;     // entries by column (ascending), for the 1-norm
  int32_t* d_col_entry = nullptr;
  double* d_abs = nullptr;          // |theta = 1 value| per entry
  unsigned long long* d_max = nullptr;
  int64_t* d_term_ptr = nullptr;    // SELL slots by term (ascending), for the reduction
  int64_t* d_term_slots = nullptr;
  // evolvers, created on first use and reset for every call
  te_evolver ev_plain = nullptr;  // plain forward: one sample at T
  te_evolver ev_fwd = nullptr;    // forward sampled at the nodes
  te_evolver ev_bwd = nullptr;    // costate sampled at T - nodes
  // device
  double2* store_psi = nullptr;
  double2* store_lam = nullptr;
  double2* lam0 = nullptr;
  double* contrib = nullptr;  // per SELL slot
  double* red = nullptr;      // reduction partials for norms
  unsigned int* counter = nullptr;
  double* d_scalar = nullptr;
  double* d_weights = nullptr;
  int* d_fwd = nullptr;
  int* d_bwd = nullptr;
  double* d_grad = nullptr;
  te_result fwd{}, bwd{};
  int64_t launches = 0;
  double phase_ms[4] = {0, 0, 0, 0};  // theta refresh, forward, costate, bilinear (last call)
};

namespace {

void free_adjoint(te_adjoint a) {
  if (!a) return;
  te_evolver_destroy(a->ev_plain);
  te_evolver_destroy(a->ev_fwd);
  te_evolver_destroy(a->ev_bwd);
  if (a->Hth) te_matrix_destroy(a->Hth);
  for (void* ptr : {(void*)a->d_entry_term, (void*)a->d_slot_term, (void*)a->d_entry_base, (void*)a->d_slot_base,
                    (void*)a->d_theta, (void*)a->d_col_ptr, (void*)a->d_col_entry, (void*)a->d_abs, (void*)a->d_max,
                    (void*)a->d_term_ptr, (void*)a->d_term_slots, (void*)a->store_psi, (void*)a->store_lam,
                    (void*)a->lam0, (void*)a->contrib, (void*)a->red, (void*)a->counter, (void*)a->d_scalar,
                    (void*)a->d_weights, (void*)a->d_fwd, (void*)a->d_bwd, (void*)a->d_grad})
    te_free(ptr);
  delete a;
}

// Host copy of one term in original-order CSR with interleaved complex values.
struct HostTerm {
  std::vector<int32_t> rp, ci;
  std::vector<double> vals;
};

int download_term(te_matrix H, HostTerm& t) {
  const int64_t n = H->n_rows;
  t.rp.resize(n + 1);
  t.ci.resize(H->nnz);
  t.vals.assign(2 * H->nnz, 0.0);
  TE_CUDA(cudaMemcpy(t.rp.data(), H->row_ptr, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost));
  if (!H->nnz) return TE_OK;
  TE_CUDA(cudaMemcpy(t.ci.data(), H->col, sizeof(int32_t) * H->nnz, cudaMemcpyDeviceToHost));
  if (H->is_real) {
    std::vector<double> re(H->nnz);
    TE_CUDA(cudaMemcpy(re.data(), H->val, sizeof(double) * H->nnz, cudaMemcpyDeviceToHost));
    for (int64_t p = 0; p < H->nnz; ++p) t.vals[2 * p] = re[p];
  } else {
    TE_CUDA(cudaMemcpy(t.vals.data(), H->val, sizeof(double) * 2 * H->nnz, cudaMemcpyDeviceToHost));
  }
  return TE_OK;
}

template <class T>
int upload_vec(T** dst, const std::vector<T>& src) {
  TE_CUDA(te_malloc(dst, sizeof(T) * std::max<size_t>(src.size(), 1)));
  if (!src.empty()) TE_CUDA(cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice));
  return TE_OK;
}

// The pattern of H(theta) = sum_k theta_k H_k: the terms' entries row by row
// (term order kept within a row), built once with theta = 1.  Every CSR entry
// and SELL slot remembers its term, so new couplings only rescale values on
// the device; the column lists (1-norm) and the per-term slot lists (gradient
// reduction) are built here too.
int build_pattern(te_adjoint a, const std::vector<HostTerm>& terms) {
  const int64_t n = a->n;
  std::vector<int64_t> rp(n + 1, 0);
  for (const HostTerm& t : terms)
    for (int64_t r = 0; r < n; ++r) rp[r + 1] += t.rp[r + 1] - t.rp[r];
  for (int64_t r = 0; r < n; ++r) rp[r + 1] += rp[r];
  const int64_t nnz = rp[n];
  std::vector<int32_t> ci(nnz), term(nnz);
  std::vector<double> vv(2 * nnz);
  std::vector<int64_t> fill(rp.begin(), rp.end() - 1);
  for (int64_t r = 0; r < n; ++r)
    for (int k = 0; k < a->K; ++k)
      for (int32_t p = terms[k].rp[r]; p < terms[k].rp[r + 1]; ++p) {
        const int64_t d = fill[r]++;
        ci[d] = terms[k].ci[p];
        term[d] = k;
        vv[2 * d] = terms[k].vals[2 * p];
        vv[2 * d + 1] = terms[k].vals[2 * p + 1];
      }
  int rc = te_matrix_create_csr(n, n, nnz, rp.data(), ci.data(), vv.data(), 1, &a->Hth);
  if (rc != TE_OK) return rc;
  te_matrix H = a->Hth;
  if (H->sell.n_long > 0) {  // the bilinear pass walks the SELL slots only
    te_set_error("te_adjoint_create: H has long rows (above max(1024, 32 x mean) entries); not supported");
    return TE_ERR_UNSUPPORTED;
  }
  const int vw = H->is_real ? 1 : 2;
  // SELL slot -> CSR entry (the layout built by te_matrix.cu: chunk c, lane l,
  // k-th entry of row perm[32 c + l] at chunk_off[c] + 32 k + l)
  const TeSell& S = H->sell;
  std::vector<int32_t> perm(n);
  std::vector<int64_t> off(S.n_chunks + 1);
  TE_CUDA(cudaMemcpy(perm.data(), S.perm, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
  TE_CUDA(cudaMemcpy(off.data(), S.chunk_off, sizeof(int64_t) * (S.n_chunks + 1), cudaMemcpyDeviceToHost));
  std::vector<int32_t> sterm(S.slots, -1);
  std::vector<double> sbase(vw * S.slots, 0.0), ebase(vw * nnz);
  for (int64_t c = 0; c < S.n_chunks; ++c) {
    const int64_t len = (off[c + 1] - off[c]) / 32;
    for (int l = 0; l < 32; ++l) {
      const int64_t rnew = c * 32 + l;
      if (rnew >= n) continue;
      const int32_t r = perm[rnew];
      for (int64_t k = 0; k < len && k < rp[r + 1] - rp[r]; ++k) {
        const int64_t sidx = off[c] + 32 * k + l, p = rp[r] + k;
        sterm[sidx] = term[p];
        for (int q = 0; q < vw; ++q) sbase[vw * sidx + q] = vv[2 * p + q];
      }
    }
  }
  for (int64_t p = 0; p < nnz; ++p)
    for (int q = 0; q < vw; ++q) ebase[vw * p + q] = vv[2 * p + q];
  // entries by column, ascending, with |value|
  std::vector<int64_t> cptr(n + 1, 0);
  for (int64_t p = 0; p < nnz; ++p) cptr[ci[p] + 1]++;
  for (int64_t c = 0; c < n; ++c) cptr[c + 1] += cptr[c];
  std::vector<int32_t> centry(nnz);
  std::vector<int64_t> cfill(cptr.begin(), cptr.end() - 1);
  for (int64_t p = 0; p < nnz; ++p) centry[cfill[ci[p]]++] = (int32_t)p;
  std::vector<double> absval(nnz);
  for (int64_t p = 0; p < nnz; ++p) absval[p] = std::hypot(vv[2 * p], vv[2 * p + 1]);
  // slots by term, ascending
  std::vector<int64_t> tptr(a->K + 1, 0);
  for (int64_t sidx = 0; sidx < S.slots; ++sidx)
    if (sterm[sidx] >= 0) tptr[sterm[sidx] + 1]++;
  for (int k = 0; k < a->K; ++k) tptr[k + 1] += tptr[k];
  std::vector<int64_t> tslots(tptr[a->K]), tfill(tptr.begin(), tptr.end() - 1);
  for (int64_t sidx = 0; sidx < S.slots; ++sidx)
    if (sterm[sidx] >= 0) tslots[tfill[sterm[sidx]]++] = sidx;
  if ((rc = upload_vec(&a->d_entry_term, term)) != TE_OK) return rc;
  if ((rc = upload_vec(&a->d_slot_term, sterm)) != TE_OK) return rc;
  if ((rc = upload_vec(&a->d_entry_base, ebase)) != TE_OK) return rc;
  if ((rc = upload_vec(&a->d_slot_base, sbase)) != TE_OK) return rc;
  if ((rc = upload_vec(&a->d_col_ptr, cptr)) != TE_OK) return rc;
  if ((rc = upload_vec(&a->d_col_entry, centry)) != TE_OK) return rc;
  if ((rc = upload_vec(&a->d_abs, absval)) != TE_OK) return rc;
  if ((rc = upload_vec(&a->d_term_ptr, tptr)) != TE_OK) return rc;
  if ((rc = upload_vec(&a->d_term_slots, tslots)) != TE_OK) return rc;
  TE_CUDA(te_malloc(&a->d_theta, sizeof(double) * a->K));
  TE_CUDA(te_malloc(&a->d_max, sizeof(unsigned long long)));
  TE_CUDA(te_malloc(&a->contrib, sizeof(double) * std::max<int64_t>(S.slots, 1)));
  return TE_OK;
}

// Rescale the values of H(theta) and recompute its 1-norm on the device when
// theta differs from the last call's.
int set_theta(te_adjoint a, const double* theta) {
  bool same = a->theta_now.size() == (size_t)a->K;
  for (int k = 0; same && k < a->K; ++k) same = a->theta_now[k] == theta[k];
  if (same) return TE_OK;
  te_matrix H = a->Hth;
  TE_CUDA(cudaMemcpy(a->d_theta, theta, sizeof(double) * a->K, cudaMemcpyHostToDevice));
  TE_CUDA(cudaMemset(a->d_max, 0, sizeof(unsigned long long)));
  const int64_t nnz = H->nnz, slots = H->sell.slots, n = a->n;
  if (H->is_real) {
    refresh_values_kernel<double><<<te_grid_for(slots, 256, 4), 256>>>(slots, a->d_slot_term, a->d_slot_base,
                                                                       a->d_theta, H->sell.val);
    refresh_values_kernel<double><<<te_grid_for(nnz, 256, 4), 256>>>(nnz, a->d_entry_term, a->d_entry_base,
                                                                     a->d_theta, H->val);
  } else {
    refresh_values_kernel<double2><<<te_grid_for(slots, 256, 4), 256>>>(
        slots, a->d_slot_term, reinterpret_cast<const double2*>(a->d_slot_base), a->d_theta,
        reinterpret_cast<double2*>(H->sell.val));
    refresh_values_kernel<double2><<<te_grid_for(nnz, 256, 4), 256>>>(
        nnz, a->d_entry_term, reinterpret_cast<const double2*>(a->d_entry_base), a->d_theta,
        reinterpret_cast<double2*>(H->val));
  }
  norm1_kernel<<<te_grid_for(n, 256, 4), 256>>>(n, a->d_col_ptr, a->d_col_entry, a->d_entry_term, a->d_abs,
                                                a->d_theta, a->d_max);
  unsigned long long bits = 0;
  TE_CUDA(cudaMemcpy(&bits, a->d_max, sizeof(bits), cudaMemcpyDeviceToHost));
  double nrm;
  std::memcpy(&nrm, &bits, sizeof(nrm));
  H->norm1 = nrm;
  if (int rc = te_sell_refresh_fixed(H)) return rc;
  a->theta_now.assign(theta, theta + a->K);
  a->launches += 3;
  return te_cuda_check(cudaGetLastError(), "theta refresh");
}

// Create an evolver of H(theta) over [0, T] sampled only at T (times == null)
// or at the given times with every sampled state stored at store + k n.
int make_evolver(te_adjoint a, double exp_factor, const std::vector<double>* times, double2* store, bool with_obs,
                 te_evolver* out) {
  te_params p{};
  p.t = a->T;
  p.sampling_step = a->T;
  p.exp_factor = exp_factor;
  p.tol = a->tol;
  p.m = a->m;
  te_evolver ev = nullptr;
  int rc = te_evolver_create(a->Hth, a->v0.data(), &p, &ev);
  if (rc != TE_OK) return rc;
  if (times) rc = te_evolver_set_schedule(ev, times->data(), (int64_t)times->size(), store, a->n);
  if (rc == TE_OK && with_obs) rc = te_evolver_add_sparse_observable(ev, a->O);
  if (rc != TE_OK) {
    te_evolver_destroy(ev);
    return rc;
  }
  *out = ev;
  return TE_OK;
}

// Reset an evolver to v (host or device, original order), run it, and read the
// last sample of its observable and/or its last state.
int run_evolver(te_adjoint a, te_evolver ev, const double* v, int v_is_device, te_result* res, double* last_sample,
                double2* last_state_dev) {
  int rc = te_evolver_reset(ev, v, v_is_device);
  if (rc == TE_OK) rc = te_evolver_run(ev, res);
  if (rc == TE_OK && last_sample) {
    const int64_t ns = res->num_samples;
    std::vector<double> smp(std::max<int64_t>(ns, 1));
    rc = te_evolver_samples(ev, 0, smp.data(), ns);
    *last_sample = smp[ns - 1];
  }
  if (rc == TE_OK && last_state_dev) {
    const double* st = nullptr;
    rc = te_evolver_state_device(ev, &st);
    if (rc == TE_OK)
      rc = te_cuda_check(cudaMemcpy(last_state_dev, st, sizeof(double2) * a->n, cudaMemcpyDeviceToDevice),
                         "state copy");
  }
  a->launches += te_evolver_launch_count(ev);
  return rc;
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
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
  a->O = O;
  a->n = n;
  a->v0.assign(v_host, v_host + 2 * n);
  a->T = T;
  a->tol = tol;
  a->m = m;
  a->interval = checkpoint_interval;
  a->q = nodes_per_interval;
  int rc = TE_OK;
  {
    std::vector<HostTerm> host(n_terms);
    for (int k = 0; k < n_terms; ++k)
      if ((rc = download_term(terms[k], host[k])) != TE_OK) return fail(rc);
    if ((rc = build_pattern(a, host)) != TE_OK) return fail(rc);
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
  a->tau.resize(nt);
  for (int64_t i = 0; i < nt; ++i) a->tau[i] = T - a->times[nt - 1 - i];
  a->tau[0] = 0.0;
  for (int64_t i = 1; i < nt; ++i) a->tau[i] = std::min(T, std::max(a->tau[i], a->tau[i - 1]));
  // device buffers
  if ((rc = te_cuda_check(te_malloc(&a->store_psi, sizeof(double2) * n * nt), "psi store")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(te_malloc(&a->store_lam, sizeof(double2) * n * nt), "lambda store")) != TE_OK)
    return fail(rc);
  if ((rc = te_cuda_check(te_malloc(&a->lam0, sizeof(double2) * n * 2), "lambda")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(te_malloc(&a->red, sizeof(double) * 4096), "red")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(te_malloc(&a->counter, sizeof(unsigned int)), "counter")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(cudaMemset(a->counter, 0, sizeof(unsigned int)), "counter")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(te_malloc(&a->d_scalar, sizeof(double)), "scalar")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(te_malloc(&a->d_grad, sizeof(double) * n_terms), "grad")) != TE_OK) return fail(rc);
  std::vector<int> fi(nt), bi(nt);
  for (int64_t i = 0; i < nt; ++i) {
    fi[i] = (int)i;
    bi[i] = (int)(nt - 1 - i);
  }
  if ((rc = upload_vec(&a->d_weights, a->weights)) != TE_OK) return fail(rc);
  if ((rc = upload_vec(&a->d_fwd, fi)) != TE_OK) return fail(rc);
  if ((rc = upload_vec(&a->d_bwd, bi)) != TE_OK) return fail(rc);
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
  a->launches = 0;
  auto t0 = std::chrono::steady_clock::now();
  int rc = set_theta(a, theta);
  a->phase_ms[0] = ms_since(t0);
  if (rc == TE_OK && !a->ev_plain) rc = make_evolver(a, 1.0, nullptr, nullptr, true, &a->ev_plain);
  if (rc != TE_OK) return rc;
  t0 = std::chrono::steady_clock::now();
  rc = run_evolver(a, a->ev_plain, a->v0.data(), 0, &a->fwd, loss, nullptr);
  a->phase_ms[1] = ms_since(t0);
  a->phase_ms[2] = a->phase_ms[3] = 0.0;
  return rc;
}

extern "C" int te_adjoint_run(te_adjoint a, const double* theta, double* loss, double* grad) {
  if (!a || !theta || !loss || !grad) {
    te_set_error("te_adjoint_run: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  const int64_t n = a->n;
  a->launches = 0;
  auto t0 = std::chrono::steady_clock::now();
  int rc = set_theta(a, theta);
  a->phase_ms[0] = ms_since(t0);
  if (rc == TE_OK && !a->ev_fwd) rc = make_evolver(a, 1.0, &a->times, a->store_psi, true, &a->ev_fwd);
  if (rc == TE_OK && !a->ev_bwd) rc = make_evolver(a, -1.0, &a->tau, a->store_lam, false, &a->ev_bwd);
  if (rc != TE_OK) return rc;
  te_matrix H = a->Hth;
  double2* psiT = a->lam0 + n;  // scratch: psi(T) in the original order
  // 1. forward, sampling psi at every node
  t0 = std::chrono::steady_clock::now();
  rc = run_evolver(a, a->ev_fwd, a->v0.data(), 0, &a->fwd, loss, psiT);
  a->phase_ms[1] = ms_since(t0);
  // 2. costate lambda(T) = O psi(T), normalised, evolved with exp(+i H tau)
  t0 = std::chrono::steady_clock::now();
  double lam_norm = 0.0;
  if (rc == TE_OK) rc = te_matrix_spmv(a->O, 1.0, 0.0, (const double*)psiT, (double*)a->lam0, nullptr);
  if (rc == TE_OK) {
    norm2_simple_kernel<<<te_grid_for(n, TE_THREADS, 4), TE_THREADS>>>(n, a->lam0, a->red, a->counter, a->d_scalar);
    double nrm2 = 0.0;
    rc = te_cuda_check(cudaMemcpy(&nrm2, a->d_scalar, sizeof(double), cudaMemcpyDeviceToHost), "norm");
    lam_norm = std::sqrt(nrm2);
    a->launches += 4;
  }
  if (rc == TE_OK && lam_norm > 0.0) {
    scale_kernel<<<te_grid_for(n, TE_THREADS, 4), TE_THREADS>>>(n, a->lam0, 1.0 / lam_norm, a->lam0);
    rc = te_cuda_check(cudaDeviceSynchronize(), "scale");
    a->launches += 1;
    if (rc == TE_OK) rc = run_evolver(a, a->ev_bwd, (const double*)a->lam0, 1, &a->bwd, nullptr, nullptr);
  }
  a->phase_ms[2] = ms_since(t0);
  // 3. bilinear pass over the slots of H(theta), then the per-term sums
  t0 = std::chrono::steady_clock::now();
  if (rc == TE_OK) {
    if (lam_norm > 0.0) {
      const TeSell& S = H->sell;
      const int nt = (int)a->times.size();
      const int grid = te_grid_for(S.n_chunks * 32, TE_THREADS, 8);
      if (H->is_real)
        bilinear_kernel<true, 8><<<grid, TE_THREADS>>>(n, S.n_chunks, S.chunk_off, S.col, a->d_slot_base,
                                                       a->store_psi, a->store_lam, n, a->d_fwd, a->d_bwd,
                                                       a->d_weights, nt, a->contrib);
      else
        bilinear_kernel<false, 8><<<grid, TE_THREADS>>>(n, S.n_chunks, S.chunk_off, S.col, a->d_slot_base,
                                                        a->store_psi, a->store_lam, n, a->d_fwd, a->d_bwd,
                                                        a->d_weights, nt, a->contrib);
      bilinear_reduce_kernel<<<a->K, TE_THREADS>>>(a->d_term_ptr, a->d_term_slots, a->contrib, 2.0 * lam_norm,
                                                   a->d_grad);
      a->launches += 2;
      rc = te_cuda_check(cudaMemcpy(grad, a->d_grad, sizeof(double) * a->K, cudaMemcpyDeviceToHost), "grad");
    } else {
      for (int k = 0; k < a->K; ++k) grad[k] = 0.0;
    }
  }
  a->phase_ms[3] = ms_since(t0);
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

extern "C" int te_adjoint_phase_times(te_adjoint a, double* ms) {
  if (!a || !ms) {
    te_set_error("te_adjoint_phase_times: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  for (int i = 0; i < 4; ++i) ms[i] = a->phase_ms[i];
  return TE_OK;
}
