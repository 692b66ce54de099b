// te_matrix.cu -- sparse matrices on the device and the te_matrix C ABI.
//
// Replaces TE::smatrix with its MKL preparation (core/matrixDataTypes.cpp:264-290,
// :352-396), smatrix::spMV (:325-346) and smatrix::norm1 (:223-235).
//
// Every matrix keeps its original-order CSR (int32 indices) for general
// observables and the public product, and square matrices also get the
// SELL-32 form in length-sorted order used by the Krylov kernels.  On GB300
// the complex-FP64 product is bound by FP64 issue (FP64 runs at 1/58 of the
// FP32 rate, ~1.19 TFLOP/s measured) rather than by HBM, so the layout is
// chosen to spend exactly 2 (real) or 4 (complex) FMAs per stored entry with
// all 32 lanes busy: rows are sorted by length, a warp owns 32 rows of equal
// length, and a real-valued matrix stores real values.
#include <algorithm>
#include <cmath>
#include <complex>
#include <mutex>
#include <numeric>
#include <vector>

#include "te_internal.cuh"
#include "te_rowdot.cuh"
#include "te_sell.cuh"

// ---------------------------------------------------------------- kernels

template <bool REAL>
__global__ void __launch_bounds__(TE_THREADS) sell_spmv_kernel(int64_t n, const int32_t* __restrict__ warp_chunk,
                                                               const int64_t* __restrict__ chunk_off,
                                                               const int32_t* __restrict__ col,
                                                               const double* __restrict__ val, double2 alpha,
                                                               const double2* __restrict__ x,
                                                               double2* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int64_t wid = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int64_t c_end = warp_chunk[wid + 1];
  for (int64_t c = warp_chunk[wid]; c < c_end; ++c) {
    double2 acc = te_sell_row<REAL>(chunk_off, col, val, x, c, lane);
    int64_t r = c * 32 + lane;
    if (r < n) y[r] = make_double2(alpha.x * acc.x - alpha.y * acc.y, alpha.x * acc.y + alpha.y * acc.x);
  }
}

template <bool REAL>
__global__ void __launch_bounds__(TE_THREADS) csr_spmv_kernel(int64_t n, const int32_t* __restrict__ row_ptr,
                                                              const int32_t* __restrict__ col,
                                                              const double* __restrict__ val, double2 alpha,
                                                              const double2* __restrict__ x,
                                                              double2* __restrict__ y) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double2 acc = te_row_dot<REAL>(row_ptr, col, val, x, (int32_t)r);
    y[r] = make_double2(alpha.x * acc.x - alpha.y * acc.y, alpha.x * acc.y + alpha.y * acc.x);
  }
}

// out[i] = in[idx[i]]
__global__ void permute_kernel(int64_t n, const int32_t* __restrict__ idx, const double2* __restrict__ in,
                               double2* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __ldg(in + __ldg(idx + i));
}

void te_launch_sell_spmv(const TeSell& A, bool is_real, double2 alpha, const double2* x_perm, double2* y_perm,
                         cudaStream_t st) {
  if (is_real)
    sell_spmv_kernel<true><<<A.grid, TE_THREADS, 0, st>>>(A.n, A.warp_chunk, A.chunk_off, A.col, A.val, alpha, x_perm,
                                                        y_perm);
  else
    sell_spmv_kernel<false><<<A.grid, TE_THREADS, 0, st>>>(A.n, A.warp_chunk, A.chunk_off, A.col, A.val, alpha, x_perm,
                                                         y_perm);
}

void te_launch_csr_spmv(const te_matrix_s& A, double2 alpha, const double2* x, double2* y, cudaStream_t st) {
  int grid = te_grid_for(A.n_rows, TE_THREADS, 8);
  if (A.is_real)
    csr_spmv_kernel<true><<<grid, TE_THREADS, 0, st>>>(A.n_rows, A.row_ptr, A.col, A.val, alpha, x, y);
  else
    csr_spmv_kernel<false><<<grid, TE_THREADS, 0, st>>>(A.n_rows, A.row_ptr, A.col, A.val, alpha, x, y);
}

void te_launch_permute(int64_t n, const int32_t* idx, const double2* in, double2* out, cudaStream_t st) {
  permute_kernel<<<te_grid_fit((const void*)permute_kernel, n, TE_THREADS), TE_THREADS, 0, st>>>(n, idx, in, out);
}

// ------------------------------------------------------------ host build

namespace {

void free_matrix(te_matrix_s* M) {
  cudaFree(M->row_ptr);
  cudaFree(M->col);
  cudaFree(M->val);
  cudaFree(M->diag_re);
  cudaFree(M->diag_c);
  cudaFree(M->sell.chunk_off);
  cudaFree(M->sell.col);
  cudaFree(M->sell.val);
  cudaFree(M->sell.perm);
  cudaFree(M->sell.iperm);
  cudaFree(M->sell.warp_chunk);
  delete M;
}

template <class T>
int upload(T** dst, const T* src, size_t count) {
  TE_CUDA(cudaMalloc(dst, sizeof(T) * std::max<size_t>(count, 1)));
  if (count) TE_CUDA(cudaMemcpy(*dst, src, sizeof(T) * count, cudaMemcpyHostToDevice));
  return TE_OK;
}

// rp/ci/vv: original-order CSR with interleaved complex values.
int build_matrix(te_matrix_s* M, const std::vector<int32_t>& rp, const std::vector<int32_t>& ci,
                 const std::vector<double>& vv) {
  const int64_t n = M->n_rows, nnz = M->nnz;
  bool real = true;
  for (int64_t i = 0; i < nnz && real; ++i) real = (vv[2 * i + 1] == 0.0);
  bool diag = (M->n_rows == M->n_cols);
  for (int64_t r = 0; r < n && diag; ++r)
    for (int32_t p = rp[r]; p < rp[r + 1]; ++p)
      if (ci[p] != r) {
        diag = false;
        break;
      }
  M->is_real = real;
  M->is_diag = diag;
  // 1-norm as in matrixDataTypes.cpp:223-235 (max absolute column sum)
  std::vector<double> colsum(M->n_cols, 0.0);
  for (int64_t p = 0; p < nnz; ++p) colsum[ci[p]] += std::abs(std::complex<double>(vv[2 * p], vv[2 * p + 1]));
  M->norm1 = *std::max_element(colsum.begin(), colsum.end());

  std::vector<double> vr;
  if (real) {
    vr.resize(nnz);
    for (int64_t i = 0; i < nnz; ++i) vr[i] = vv[2 * i];
  }
  int rc;
  if ((rc = upload(&M->row_ptr, rp.data(), rp.size())) != TE_OK) return rc;
  if ((rc = upload(&M->col, ci.data(), ci.size())) != TE_OK) return rc;
  if ((rc = upload(&M->val, real ? vr.data() : vv.data(), real ? vr.size() : vv.size())) != TE_OK) return rc;
  if (diag) {
    std::vector<double> dre(n, 0.0), dc(2 * n, 0.0);
    for (int64_t r = 0; r < n; ++r)
      for (int32_t p = rp[r]; p < rp[r + 1]; ++p) {
        dre[r] += vv[2 * p];
        dc[2 * r] += vv[2 * p];
        dc[2 * r + 1] += vv[2 * p + 1];
      }
    if ((rc = upload(&M->diag_re, dre.data(), dre.size())) != TE_OK) return rc;
    if ((rc = upload(reinterpret_cast<double**>(&M->diag_c), dc.data(), dc.size())) != TE_OK) return rc;
  }
  if (M->n_rows != M->n_cols) return TE_OK;

  // SELL-32 with rows sorted by length (descending, stable)
  TeSell& S = M->sell;
  S.n = n;
  S.n_chunks = (n + 31) / 32;
  std::vector<int32_t> perm(n), iperm(n);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(),
                   [&](int32_t a, int32_t b) { return (rp[a + 1] - rp[a]) > (rp[b + 1] - rp[b]); });
  for (int64_t i = 0; i < n; ++i) iperm[perm[i]] = (int32_t)i;
  std::vector<int64_t> off(S.n_chunks + 1, 0);
  for (int64_t c = 0; c < S.n_chunks; ++c) {
    int32_t r0 = perm[c * 32];
    int64_t len = rp[r0 + 1] - rp[r0];  // longest row of the chunk comes first
    off[c + 1] = off[c] + 32 * len;
  }
  S.slots = off[S.n_chunks];
  std::vector<int32_t> scol(S.slots);
  std::vector<double> sval((real ? 1 : 2) * S.slots, 0.0);
  for (int64_t c = 0; c < S.n_chunks; ++c) {
    int64_t len = (off[c + 1] - off[c]) / 32;
    for (int lane = 0; lane < 32; ++lane) {
      int64_t rnew = c * 32 + lane;
      int32_t pad_col = (int32_t)std::min<int64_t>(rnew, n - 1);
      int64_t rlen = 0, p0 = 0;
      if (rnew < n) {
        int32_t r = perm[rnew];
        p0 = rp[r];
        rlen = rp[r + 1] - rp[r];
      }
      for (int64_t k = 0; k < len; ++k) {
        int64_t s = off[c] + 32 * k + lane;
        if (k < rlen) {
          scol[s] = iperm[ci[p0 + k]];
          if (real) {
            sval[s] = vv[2 * (p0 + k)];
          } else {
            sval[2 * s] = vv[2 * (p0 + k)];
            sval[2 * s + 1] = vv[2 * (p0 + k) + 1];
          }
        } else {
          scol[s] = pad_col;
        }
      }
    }
  }
  if ((rc = upload(&S.chunk_off, off.data(), off.size())) != TE_OK) return rc;
  if ((rc = upload(&S.col, scol.data(), scol.size())) != TE_OK) return rc;
  if ((rc = upload(&S.val, sval.data(), sval.size())) != TE_OK) return rc;
  if ((rc = upload(&S.perm, perm.data(), perm.size())) != TE_OK) return rc;
  if ((rc = upload(&S.iperm, iperm.data(), iperm.size())) != TE_OK) return rc;
  // static warp schedule: equal FP64 work per warp (te_sell_row issues 2 (real)
  // or 4 (complex) FMAs per slot; the SpMV epilogues about 8 per row)
  const int bps = std::min(te_sell_blocks_per_sm(real),
                           te_kernel_blocks_per_sm(real ? (const void*)sell_spmv_kernel<true>
                                                        : (const void*)sell_spmv_kernel<false>,
                                                   TE_THREADS, 0));
  S.grid = (int)std::min<int64_t>((S.n_chunks * 32 + TE_THREADS - 1) / TE_THREADS, (int64_t)te_num_sms() * bps);
  const int64_t W = (int64_t)S.grid * (TE_THREADS / 32);
  const double w_slot = real ? 2.0 : 4.0, w_chunk = 8.0 * 32;
  auto cost = [&](int64_t c) { return w_slot * (double)off[c] + w_chunk * (double)c; };
  const double total = cost(S.n_chunks);
  std::vector<int32_t> wc(W + 1);
  int64_t c = 0;
  for (int64_t w = 0; w < W; ++w) {
    const double target = total * (double)w / (double)W;
    while (c < S.n_chunks && cost(c) < target) ++c;
    wc[w] = (int32_t)c;
  }
  wc[W] = (int32_t)S.n_chunks;
  if ((rc = upload(&S.warp_chunk, wc.data(), wc.size())) != TE_OK) return rc;
  return TE_OK;
}

int finish_create(int64_t n_rows, int64_t n_cols, const std::vector<int32_t>& rp, const std::vector<int32_t>& ci,
                  const std::vector<double>& vv, te_matrix* out) {
  te_matrix_s* M = new te_matrix_s();
  cudaGetDevice(&M->device);
  M->n_rows = n_rows;
  M->n_cols = n_cols;
  M->nnz = (int64_t)ci.size();
  int rc = build_matrix(M, rp, ci, vv);
  if (rc != TE_OK) {
    free_matrix(M);
    return rc;
  }
  *out = M;
  return TE_OK;
}

}  // namespace

// ------------------------------------------------------------------ C ABI

extern "C" int te_matrix_create_coo(int64_t n_rows, int64_t n_cols, int64_t nnz, const uint64_t* row_index,
                                    const uint64_t* columns, const double* values, te_matrix* out) {
  if (!out || n_rows <= 0 || n_cols <= 0 || nnz < 0 || (nnz > 0 && (!row_index || !columns || !values))) {
    te_set_error("te_matrix_create_coo: invalid arguments");
    return n_rows == 0 || n_cols == 0 ? TE_ERR_EMPTY : TE_ERR_INVALID_ARG;
  }
  if (nnz >= ((int64_t)1 << 31) || n_rows >= ((int64_t)1 << 31) || n_cols >= ((int64_t)1 << 31)) {
    te_set_error("te_matrix_create_coo: sizes must stay below 2^31 (int32 indices)");
    return TE_ERR_UNSUPPORTED;
  }
  for (int64_t i = 0; i < nnz; ++i)
    if (row_index[i] >= (uint64_t)n_rows || columns[i] >= (uint64_t)n_cols) {
      te_set_error("te_matrix_create_coo: entry %lld out of range", (long long)i);
      return TE_ERR_INVALID_ARG;
    }
  // stable COO -> CSR: entries of one row keep their input order
  std::vector<int32_t> rp(n_rows + 1, 0), ci(nnz);
  std::vector<double> vv(2 * nnz);
  for (int64_t i = 0; i < nnz; ++i) rp[row_index[i] + 1]++;
  for (int64_t r = 0; r < n_rows; ++r) rp[r + 1] += rp[r];
  std::vector<int32_t> fill(rp.begin(), rp.end() - 1);
  for (int64_t i = 0; i < nnz; ++i) {
    int32_t p = fill[row_index[i]]++;
    ci[p] = (int32_t)columns[i];
    vv[2 * p] = values[2 * i];
    vv[2 * p + 1] = values[2 * i + 1];
  }
  return finish_create(n_rows, n_cols, rp, ci, vv, out);
}

extern "C" int te_matrix_create_csr(int64_t n_rows, int64_t n_cols, int64_t nnz, const int64_t* row_ptr,
                                    const int32_t* col_idx, const double* values, int values_complex,
                                    te_matrix* out) {
  if (!out || n_rows <= 0 || n_cols <= 0 || nnz < 0 || !row_ptr || (nnz > 0 && (!col_idx || !values))) {
    te_set_error("te_matrix_create_csr: invalid arguments");
    return n_rows == 0 || n_cols == 0 ? TE_ERR_EMPTY : TE_ERR_INVALID_ARG;
  }
  if (nnz >= ((int64_t)1 << 31) || n_rows >= ((int64_t)1 << 31) || n_cols >= ((int64_t)1 << 31)) {
    te_set_error("te_matrix_create_csr: sizes must stay below 2^31 (int32 indices)");
    return TE_ERR_UNSUPPORTED;
  }
  if (row_ptr[0] != 0 || row_ptr[n_rows] != nnz) {
    te_set_error("te_matrix_create_csr: row_ptr must start at 0 and end at nnz");
    return TE_ERR_INVALID_ARG;
  }
  std::vector<int32_t> rp(n_rows + 1);
  for (int64_t r = 0; r <= n_rows; ++r) {
    if (r > 0 && row_ptr[r] < row_ptr[r - 1]) {
      te_set_error("te_matrix_create_csr: row_ptr decreases at row %lld", (long long)r);
      return TE_ERR_INVALID_ARG;
    }
    rp[r] = (int32_t)row_ptr[r];
  }
  std::vector<int32_t> ci(col_idx, col_idx + nnz);
  for (int64_t i = 0; i < nnz; ++i)
    if (ci[i] < 0 || ci[i] >= n_cols) {
      te_set_error("te_matrix_create_csr: column of entry %lld out of range", (long long)i);
      return TE_ERR_INVALID_ARG;
    }
  std::vector<double> vv(2 * nnz, 0.0);
  for (int64_t i = 0; i < nnz; ++i) {
    vv[2 * i] = values_complex ? values[2 * i] : values[i];
    vv[2 * i + 1] = values_complex ? values[2 * i + 1] : 0.0;
  }
  return finish_create(n_rows, n_cols, rp, ci, vv, out);
}

extern "C" int te_matrix_destroy(te_matrix A) {
  if (A) free_matrix(A);
  return TE_OK;
}

extern "C" int te_matrix_info(te_matrix A, int64_t* n_rows, int64_t* n_cols, int64_t* nnz, int* flags,
                              double* norm1) {
  if (!A) {
    te_set_error("te_matrix_info: null matrix");
    return TE_ERR_INVALID_ARG;
  }
  if (n_rows) *n_rows = A->n_rows;
  if (n_cols) *n_cols = A->n_cols;
  if (nnz) *nnz = A->nnz;
  if (flags) *flags = (A->is_real ? 1 : 0) | (A->is_diag ? 2 : 0);
  if (norm1) *norm1 = A->norm1;
  return TE_OK;
}

extern "C" int te_matrix_spmv(te_matrix A, double alpha_re, double alpha_im, const double* in_dev, double* out_dev,
                              void* cuda_stream) {
  if (!A || !in_dev || !out_dev || A->n_rows != A->n_cols) {
    te_set_error("te_matrix_spmv: invalid arguments (square matrix and device buffers required)");
    return TE_ERR_INVALID_ARG;
  }
  cudaStream_t st = (cudaStream_t)cuda_stream;
  const int64_t n = A->n_rows;
  // permute in, SELL product, permute out
  double2 *xp = nullptr, *yp = nullptr;
  TE_CUDA(cudaMallocAsync(&xp, sizeof(double2) * n, st));
  int rc = te_cuda_check(cudaMallocAsync(&yp, sizeof(double2) * n, st), "cudaMallocAsync");
  if (rc == TE_OK) {
    te_launch_permute(n, A->sell.perm, reinterpret_cast<const double2*>(in_dev), xp, st);
    te_launch_sell_spmv(A->sell, A->is_real, make_double2(alpha_re, alpha_im), xp, yp, st);
    te_launch_permute(n, A->sell.iperm, yp, reinterpret_cast<double2*>(out_dev), st);
    rc = te_cuda_check(cudaGetLastError(), "spmv launch");
  }
  cudaFreeAsync(xp, st);
  cudaFreeAsync(yp, st);
  return rc;
}

extern "C" int te_matrix_spmv_host(te_matrix A, double alpha_re, double alpha_im, const double* in_host,
                                   double* out_host) {
  if (!A || !in_host || !out_host) {
    te_set_error("te_matrix_spmv_host: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  const int64_t n = A->n_rows;
  double2 *x = nullptr, *y = nullptr;
  TE_CUDA(cudaMalloc(&x, sizeof(double2) * n));
  int rc = te_cuda_check(cudaMalloc(&y, sizeof(double2) * n), "cudaMalloc");
  if (rc == TE_OK) rc = te_cuda_check(cudaMemcpy(x, in_host, sizeof(double2) * n, cudaMemcpyHostToDevice), "H2D");
  if (rc == TE_OK) rc = te_matrix_spmv(A, alpha_re, alpha_im, (const double*)x, (double*)y, nullptr);
  if (rc == TE_OK) rc = te_cuda_check(cudaDeviceSynchronize(), "spmv");
  if (rc == TE_OK) rc = te_cuda_check(cudaMemcpy(out_host, y, sizeof(double2) * n, cudaMemcpyDeviceToHost), "D2H");
  cudaFree(x);
  cudaFree(y);
  return rc;
}

// ------------------------------------------------- product without allocation
//
// te_matrix_spmv needs two vectors of scratch (the input and the output in the
// matrix's sorted row order) and takes them from cudaMallocAsync on every call.
// Callers that must not allocate -- code recorded into a CUDA graph by stream
// capture, real-time loops whose memory is fixed up front, hosts whose device
// memory budget is preallocated by another framework -- use
// te_matrix_spmv_noalloc instead, which keeps that scratch in the fixed array
// below.  The array is part of the library image, so every GPU that loads the
// library holds it (TE_NOALLOC_MAX_ROWS * 2 * 16 bytes = 8 MiB) until the
// process exits.

#define TE_NOALLOC_MAX_ROWS (1 << 18)

static __device__ __align__(256) double2 g_noalloc_scratch[2 * TE_NOALLOC_MAX_ROWS];

#define TE_NOALLOC_MAX_DEVICES 64

// Device address of g_noalloc_scratch for the current device.  The host-side
// name of the array is only a stand-in; the address is looked up once per
// device (the first call on a device does it, so make that first call before
// any stream capture) and cached.
static int noalloc_scratch(double2** out) {
  static std::mutex mu;
  static double2* addr[TE_NOALLOC_MAX_DEVICES] = {};
  int dev = 0;
  TE_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= TE_NOALLOC_MAX_DEVICES) {
    te_set_error("te_matrix_spmv_noalloc: device %d out of range", dev);
    return TE_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    TE_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    addr[dev] = static_cast<double2*>(p);
  }
  *out = addr[dev];
  return TE_OK;
}

extern "C" int te_matrix_spmv_noalloc(te_matrix A, double alpha_re, double alpha_im, const double* in_dev,
                                      double* out_dev, void* cuda_stream) {
  if (!A || !in_dev || !out_dev || A->n_rows != A->n_cols) {
    te_set_error("te_matrix_spmv_noalloc: invalid arguments (square matrix and device buffers required)");
    return TE_ERR_INVALID_ARG;
  }
  const int64_t n = A->n_rows;
  if (n > TE_NOALLOC_MAX_ROWS) {
    te_set_error("te_matrix_spmv_noalloc: %lld rows exceed the fixed scratch of %d rows; use te_matrix_spmv",
                 (long long)n, TE_NOALLOC_MAX_ROWS);
    return TE_ERR_UNSUPPORTED;
  }
  double2* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc != TE_OK) return rc;
  // both halves are written in full before they are read: nothing to clear
  double2* xp = scratch;
  double2* yp = scratch + TE_NOALLOC_MAX_ROWS;
  cudaStream_t st = (cudaStream_t)cuda_stream;
  te_launch_permute(n, A->sell.perm, reinterpret_cast<const double2*>(in_dev), xp, st);
  te_launch_sell_spmv(A->sell, A->is_real, make_double2(alpha_re, alpha_im), xp, yp, st);
  te_launch_permute(n, A->sell.iperm, yp, reinterpret_cast<double2*>(out_dev), st);
  return te_cuda_check(cudaGetLastError(), "spmv_noalloc launch");
}
