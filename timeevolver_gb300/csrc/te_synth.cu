// te_synth.cu -- device-side generator of the load-imbalanced synthetic
// workload: a complex Hermitian H = (A + A^H) / 2 whose rows of A have
// Zipf-distributed lengths, scaled to a spectral-norm estimate of 1.
//
// No counterpart in the reference, which only builds Bose-Hubbard and
// black-hole Hamiltonians on the host.  At dimension 1e7 (about 4e8 stored
// entries) a host build would take minutes and ~12 GB of COO, so everything
// is generated on the device from a counter-based hash: every random number is
// a pure function of (seed, row, draw index, stream), which makes the matrix
// independent of the launch shape and reproducible bit for bit by a plain
// numpy restatement at small sizes.
//
//   row length k_r : truncated Zipf on [min_len, max_len], P(k) ~ k^-s, by
//                    inverse CDF of one uniform draw (stream 0);
//   columns of A   : k_r distinct uniform columns; draw t of row r tries the
//                    hash (seed, r, a * 65536 + t, stream 1) mod n for
//                    attempt a = 0, 1, ... until it differs from the row's
//                    earlier columns;
//   values of A    : re + i im, independent N(0, 1) by Box-Muller from the
//                    draws (seed, r, t, 2) and (seed, r, t, 3);
//   H              : (A + A^H) / 2 in CSR with ascending columns per row;
//   scale          : power iteration from a Gaussian start (stream 4), H is
//                    divided by the last |H x| (x normalised).
#include <algorithm>
#include <cmath>
#include <vector>

#include "te_internal.cuh"

namespace {

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__host__ __device__ __forceinline__ uint64_t draw(uint64_t seed, uint64_t row, uint64_t t, uint64_t stream) {
  return mix64(mix64(mix64(seed) ^ row) ^ ((t << 8) | stream));
}

__device__ __forceinline__ double unit_open_right(uint64_t h) { return (double)(h >> 11) * 0x1.0p-53; }  // [0, 1)
__device__ __forceinline__ double unit_open_left(uint64_t h) { return (double)((h >> 11) + 1) * 0x1.0p-53; }  // (0, 1]

__device__ __forceinline__ double2 gaussian_pair(uint64_t h1, uint64_t h2) {
  const double rad = sqrt(-2.0 * log(unit_open_left(h1)));
  double s, c;
  sincospi(2.0 * unit_open_right(h2), &s, &c);
  return make_double2(rad * c, rad * s);
}

const int kMaxAttempts = 64;

__global__ void row_length_kernel(int64_t n, uint64_t seed, const double* __restrict__ cdf, int n_cdf, int min_len,
                                  int32_t* __restrict__ len) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const double u = unit_open_right(draw(seed, r, 0, 0));
    int lo = 0, hi = n_cdf - 1;  // first index with cdf > u (cdf[n_cdf - 1] == 1 > u)
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (cdf[mid] > u)
        hi = mid;
      else
        lo = mid + 1;
    }
    len[r] = min_len + lo;
  }
}

// Entries of A, one thread per row; rows start at rp[r] (int64).
__global__ void entries_kernel(int64_t n, uint64_t seed, const int64_t* __restrict__ rp, const int32_t* __restrict__ len,
                               int32_t* __restrict__ col, double2* __restrict__ val, unsigned int* err) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p0 = rp[r];
    const int k = len[r];
    for (int t = 0; t < k; ++t) {
      int32_t c = 0;
      bool ok = false;
      for (int a = 0; a < kMaxAttempts && !ok; ++a) {
        c = (int32_t)(draw(seed, r, (uint64_t)a * 65536u + t, 1) % (uint64_t)n);
        ok = true;
        for (int q = 0; q < t && ok; ++q) ok = col[p0 + q] != c;
      }
      if (!ok) atomicOr(err, 1u);
      col[p0 + t] = c;
      val[p0 + t] = gaussian_pair(draw(seed, r, t, 2), draw(seed, r, t, 3));
    }
  }
}

__global__ void count_columns_kernel(int64_t nnz, const int32_t* __restrict__ col, int32_t* __restrict__ count) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&count[col[p]], 1);
}

// Row r of A + A^H before sorting: its own entries (tag 0) first, then the
// conjugated entries A_jr of the other rows (tag 1) in arrival order.
__global__ void scatter_kernel(int64_t n, const int64_t* __restrict__ rpa, const int32_t* __restrict__ len,
                               const int32_t* __restrict__ cola, const double2* __restrict__ vala,
                               const int64_t* __restrict__ rps, int32_t* __restrict__ fill, int32_t* __restrict__ tcol,
                               double2* __restrict__ tval, uint8_t* __restrict__ ttag) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p0 = rpa[r];
    const int k = len[r];
    for (int t = 0; t < k; ++t) {
      const int32_t j = cola[p0 + t];
      const double2 a = vala[p0 + t];
      const int64_t own = rps[r] + t;
      tcol[own] = j;
      tval[own] = a;
      ttag[own] = 0;
      const int64_t mirror = rps[j] + len[j] + atomicAdd(&fill[j], 1);
      tcol[mirror] = (int32_t)r;
      tval[mirror] = make_double2(a.x, -a.y);
      ttag[mirror] = 1;
    }
  }
}

// One warp per row: every entry's rank under the key (column, tag), which is
// unique within a row, gives its place in the sorted row.
__global__ void sort_rows_kernel(int64_t n, const int64_t* __restrict__ rps, const int32_t* __restrict__ tcol,
                                 const double2* __restrict__ tval, const uint8_t* __restrict__ ttag,
                                 int32_t* __restrict__ scol, double2* __restrict__ sval, uint8_t* __restrict__ stag) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += warps) {
    const int64_t b = rps[r];
    const int64_t L = rps[r + 1] - b;
    for (int64_t e = lane; e < L; e += 32) {
      const int64_t key = 2 * (int64_t)tcol[b + e] + ttag[b + e];
      int64_t rank = 0;
      for (int64_t f = 0; f < L; ++f) rank += (2 * (int64_t)tcol[b + f] + ttag[b + f]) < key;
      scol[b + rank] = tcol[b + e];
      sval[b + rank] = tval[b + e];
      stag[b + rank] = ttag[b + e];
    }
  }
}

// Entries of row r of H: a column present in both A and A^H appears twice in
// a row (tag 0 then tag 1, adjacent after sorting) and is merged.
__global__ void merged_length_kernel(int64_t n, const int64_t* __restrict__ rps, const int32_t* __restrict__ scol,
                                     int32_t* __restrict__ mlen) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = rps[r], e = rps[r + 1];
    int32_t m = 0;
    for (int64_t q = b; q < e; ++q, ++m)
      if (q + 1 < e && scol[q + 1] == scol[q]) ++q;
    mlen[r] = m;
  }
}

__global__ void merge_rows_kernel(int64_t n, const int64_t* __restrict__ rps, const int32_t* __restrict__ scol,
                                  const double2* __restrict__ sval, const int32_t* __restrict__ rph,
                                  int32_t* __restrict__ hcol, double2* __restrict__ hval) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = rps[r], e = rps[r + 1];
    int64_t out = rph[r];
    for (int64_t q = b; q < e; ++q, ++out) {
      double2 v = sval[q];
      if (q + 1 < e && scol[q + 1] == scol[q]) {
        v.x += sval[q + 1].x;
        v.y += sval[q + 1].y;
        hcol[out] = scol[q];
        ++q;
      } else {
        hcol[out] = scol[q];
      }
      hval[out] = make_double2(0.5 * v.x, 0.5 * v.y);
    }
  }
}

__global__ void start_vector_kernel(int64_t n, uint64_t seed, double2* __restrict__ x) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    x[r] = gaussian_pair(draw(seed, r, 0, 4), draw(seed, r, 1, 4));
}

// Per-block partial sums of |x|^2 (a fixed grid, summed on the host in order).
__global__ void __launch_bounds__(TE_THREADS) norm2_partials_kernel(int64_t n, const double2* __restrict__ x,
                                                                    double* __restrict__ partials) {
  __shared__ double scratch[TE_THREADS / 32];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc = fma(x[i].x, x[i].x, fma(x[i].y, x[i].y, acc));
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < TE_THREADS / 32; ++w) s += scratch[w];
    partials[blockIdx.x] = s;
  }
}

__global__ void scale_kernel(int64_t n, double2* __restrict__ x, double s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = make_double2(s * x[i].x, s * x[i].y);
}

__global__ void scale_real_kernel(int64_t n, double* __restrict__ x, double s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] *= s;
}

template <class T>
struct DevBuf {
  T* p = nullptr;
  ~DevBuf() { te_free(p); }
  int alloc(int64_t count) { return te_cuda_check(te_malloc(&p, sizeof(T) * std::max<int64_t>(count, 1)), "zipf"); }
  T* release() {
    T* q = p;
    p = nullptr;
    return q;
  }
};

int exclusive_scan_host(const std::vector<int32_t>& a, std::vector<int64_t>& out) {
  out.assign(a.size() + 1, 0);
  for (size_t i = 0; i < a.size(); ++i) out[i + 1] = out[i] + a[i];
  return TE_OK;
}

const int kNormGrid = 1024;

int norm2(int64_t n, const double2* x, double* d_partials, double* out) {
  norm2_partials_kernel<<<kNormGrid, TE_THREADS>>>(n, x, d_partials);
  std::vector<double> h(kNormGrid);
  TE_CUDA(cudaMemcpy(h.data(), d_partials, sizeof(double) * kNormGrid, cudaMemcpyDeviceToHost));
  double s = 0.0;
  for (double v : h) s += v;
  *out = s;
  return TE_OK;
}

}  // namespace

extern "C" int te_matrix_create_zipf(int64_t n, double exponent, int32_t min_len, int32_t max_len, uint64_t seed,
                                     int32_t power_iters, double* norm_estimate, te_matrix* out) {
  if (!out || n < 1 || !(exponent > 0.0) || min_len < 1 || max_len < min_len || max_len > 65535 ||
      power_iters < 0 || n < 4 * (int64_t)max_len) {
    te_set_error("te_matrix_create_zipf: invalid arguments (need n >= 4 max_len, 1 <= min_len <= max_len <= 65535)");
    return TE_ERR_INVALID_ARG;
  }
  if (n >= ((int64_t)1 << 31)) {
    te_set_error("te_matrix_create_zipf: n must stay below 2^31 (int32 indices)");
    return TE_ERR_UNSUPPORTED;
  }
  // truncated Zipf CDF (ascending cumulative sums, last entry exactly 1)
  const int K = max_len - min_len + 1;
  std::vector<double> cdf(K);
  double z = 0.0;
  for (int i = 0; i < K; ++i) {
    z += std::pow((double)(min_len + i), -exponent);
    cdf[i] = z;
  }
  for (int i = 0; i < K; ++i) cdf[i] /= z;
  cdf[K - 1] = 1.0;
  const int g = te_grid_fit((const void*)entries_kernel, n, TE_THREADS);
  DevBuf<double> d_cdf;
  DevBuf<int32_t> d_len, d_cnt;
  DevBuf<unsigned int> d_err;
  int rc;
  if ((rc = d_cdf.alloc(K)) != TE_OK || (rc = d_len.alloc(n)) != TE_OK || (rc = d_cnt.alloc(n)) != TE_OK ||
      (rc = d_err.alloc(1)) != TE_OK)
    return rc;
  TE_CUDA(cudaMemcpy(d_cdf.p, cdf.data(), sizeof(double) * K, cudaMemcpyHostToDevice));
  TE_CUDA(cudaMemset(d_err.p, 0, sizeof(unsigned int)));
  TE_CUDA(cudaMemset(d_cnt.p, 0, sizeof(int32_t) * n));
  row_length_kernel<<<g, TE_THREADS>>>(n, seed, d_cdf.p, K, min_len, d_len.p);
  std::vector<int32_t> len(n);
  TE_CUDA(cudaMemcpy(len.data(), d_len.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
  std::vector<int64_t> rpa;
  exclusive_scan_host(len, rpa);
  const int64_t nnz_a = rpa[n];
  if (2 * nnz_a >= ((int64_t)1 << 31)) {
    te_set_error("te_matrix_create_zipf: %lld entries of A + A^H exceed the int32 range", (long long)(2 * nnz_a));
    return TE_ERR_UNSUPPORTED;
  }
  // A
  DevBuf<int64_t> d_rpa, d_rps;
  DevBuf<int32_t> d_cola, d_fill, d_tcol, d_scol, d_mlen;
  DevBuf<double2> d_vala, d_tval, d_sval;
  DevBuf<uint8_t> d_ttag, d_stag;
  if ((rc = d_rpa.alloc(n + 1)) != TE_OK || (rc = d_cola.alloc(nnz_a)) != TE_OK || (rc = d_vala.alloc(nnz_a)) != TE_OK)
    return rc;
  TE_CUDA(cudaMemcpy(d_rpa.p, rpa.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
  entries_kernel<<<g, TE_THREADS>>>(n, seed, d_rpa.p, d_len.p, d_cola.p, d_vala.p, d_err.p);
  count_columns_kernel<<<te_grid_fit((const void*)count_columns_kernel, nnz_a, TE_THREADS), TE_THREADS>>>(
      nnz_a, d_cola.p, d_cnt.p);
  unsigned int err = 0;
  TE_CUDA(cudaMemcpy(&err, d_err.p, sizeof(err), cudaMemcpyDeviceToHost));
  if (err) {
    te_set_error("te_matrix_create_zipf: no distinct column found within %d draws", kMaxAttempts);
    return TE_ERR_INVALID_ARG;
  }
  // A + A^H, unsorted rows: own entries, then mirrored ones
  std::vector<int32_t> cnt(n);
  TE_CUDA(cudaMemcpy(cnt.data(), d_cnt.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
  for (int64_t r = 0; r < n; ++r) cnt[r] += len[r];
  std::vector<int64_t> rps;
  exclusive_scan_host(cnt, rps);
  const int64_t nnz_s = rps[n];  // == 2 nnz_a
  if ((rc = d_rps.alloc(n + 1)) != TE_OK || (rc = d_fill.alloc(n)) != TE_OK || (rc = d_tcol.alloc(nnz_s)) != TE_OK ||
      (rc = d_tval.alloc(nnz_s)) != TE_OK || (rc = d_ttag.alloc(nnz_s)) != TE_OK)
    return rc;
  TE_CUDA(cudaMemcpy(d_rps.p, rps.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
  TE_CUDA(cudaMemset(d_fill.p, 0, sizeof(int32_t) * n));
  scatter_kernel<<<g, TE_THREADS>>>(n, d_rpa.p, d_len.p, d_cola.p, d_vala.p, d_rps.p, d_fill.p, d_tcol.p, d_tval.p,
                                    d_ttag.p);
  te_free(d_cola.release());
  te_free(d_vala.release());
  // sort each row by (column, tag), then merge the pairs
  if ((rc = d_scol.alloc(nnz_s)) != TE_OK || (rc = d_sval.alloc(nnz_s)) != TE_OK || (rc = d_stag.alloc(nnz_s)) != TE_OK)
    return rc;
  sort_rows_kernel<<<te_grid_fit((const void*)sort_rows_kernel, n * 32, TE_THREADS), TE_THREADS>>>(
      n, d_rps.p, d_tcol.p, d_tval.p, d_ttag.p, d_scol.p, d_sval.p, d_stag.p);
  te_free(d_tcol.release());
  te_free(d_tval.release());
  te_free(d_ttag.release());
  if ((rc = d_mlen.alloc(n)) != TE_OK) return rc;
  merged_length_kernel<<<g, TE_THREADS>>>(n, d_rps.p, d_scol.p, d_mlen.p);
  std::vector<int32_t> mlen(n);
  TE_CUDA(cudaMemcpy(mlen.data(), d_mlen.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
  std::vector<int64_t> rph64;
  exclusive_scan_host(mlen, rph64);
  std::vector<int32_t> rph(n + 1);
  for (int64_t r = 0; r <= n; ++r) rph[r] = (int32_t)rph64[r];
  const int64_t nnz_h = rph64[n];
  int32_t *d_rph = nullptr, *d_hcol = nullptr;
  double2* d_hval = nullptr;
  if (te_cuda_check(te_malloc(&d_rph, sizeof(int32_t) * (n + 1)), "zipf") != TE_OK ||
      te_cuda_check(te_malloc(&d_hcol, sizeof(int32_t) * std::max<int64_t>(nnz_h, 1)), "zipf") != TE_OK ||
      te_cuda_check(te_malloc(&d_hval, sizeof(double2) * std::max<int64_t>(nnz_h, 1)), "zipf") != TE_OK) {
    te_free(d_rph);
    te_free(d_hcol);
    te_free(d_hval);
    return TE_ERR_CUDA;
  }
  cudaMemcpy(d_rph, rph.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice);
  merge_rows_kernel<<<g, TE_THREADS>>>(n, d_rps.p, d_scol.p, d_sval.p, d_rph, d_hcol, d_hval);
  rc = te_cuda_check(cudaDeviceSynchronize(), "zipf build");
  if (rc != TE_OK) {
    te_free(d_rph);
    te_free(d_hcol);
    te_free(d_hval);
    return rc;
  }
  te_free(d_scol.release());
  te_free(d_sval.release());
  te_free(d_stag.release());
  te_matrix H = nullptr;
  if ((rc = te_matrix_adopt_device_csr(n, n, rph[n], d_rph, d_hcol, d_hval, &H, NAN)) != TE_OK) return rc;

  // spectral-norm estimate by power iteration, then H /= estimate
  DevBuf<double2> x, y;
  DevBuf<double> partials;
  double est = 1.0;
  if ((rc = x.alloc(n)) == TE_OK && (rc = y.alloc(n)) == TE_OK && (rc = partials.alloc(kNormGrid)) == TE_OK) {
    const int gs = te_grid_fit((const void*)scale_kernel, n, TE_THREADS);
    start_vector_kernel<<<g, TE_THREADS>>>(n, seed, x.p);
    double s2 = 0.0;
    rc = norm2(n, x.p, partials.p, &s2);
    if (rc == TE_OK) scale_kernel<<<gs, TE_THREADS>>>(n, x.p, 1.0 / std::sqrt(s2));
    for (int it = 0; it < power_iters && rc == TE_OK; ++it) {
      rc = te_matrix_spmv(H, 1.0, 0.0, (const double*)x.p, (double*)y.p, nullptr);
      if (rc == TE_OK) rc = norm2(n, y.p, partials.p, &s2);
      if (rc == TE_OK && !(s2 > 0.0)) {
        te_set_error("te_matrix_create_zipf: power iteration reached the zero vector");
        rc = TE_ERR_INVALID_ARG;
      }
      if (rc == TE_OK) {
        est = std::sqrt(s2);
        scale_kernel<<<gs, TE_THREADS>>>(n, y.p, 1.0 / est);
        std::swap(x.p, y.p);
      }
    }
    if (rc == TE_OK && power_iters > 0) {
      const double inv = 1.0 / est;
      const TeSell& S = H->sell;
      if (H->is_real) {  // the values are stored as reals
        scale_real_kernel<<<te_grid_fit((const void*)scale_real_kernel, H->nnz, TE_THREADS), TE_THREADS>>>(
            H->nnz, H->val, inv);
        scale_real_kernel<<<te_grid_fit((const void*)scale_real_kernel, S.slots, TE_THREADS), TE_THREADS>>>(
            S.slots, S.val, inv);
      } else {
        scale_kernel<<<te_grid_fit((const void*)scale_kernel, H->nnz, TE_THREADS), TE_THREADS>>>(
            H->nnz, reinterpret_cast<double2*>(H->val), inv);
        scale_kernel<<<te_grid_fit((const void*)scale_kernel, S.slots, TE_THREADS), TE_THREADS>>>(
            S.slots, reinterpret_cast<double2*>(S.val), inv);
      }
      H->norm1 *= inv;
      rc = te_cuda_check(cudaDeviceSynchronize(), "zipf scale");
    }
  }
  if (rc != TE_OK) {
    te_matrix_destroy(H);
    return rc;
  }
  if (norm_estimate) *norm_estimate = est;
  *out = H;
  return TE_OK;
}
