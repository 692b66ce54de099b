// te_matrix.cu -- sparse matrices on the device and the te_matrix C ABI.
//
// Replaces TE::smatrix with its MKL preparation (core/matrixDataTypes.cpp:108-134,
// :196-240), smatrix::spMV (:169-190) and smatrix::norm1 (:67-79).
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
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "te_internal.cuh"
#include "te_rowdot.cuh"
#include "te_sell.cuh"

// ---------------------------------------------------------------- kernels

// K lanes per row as in lanczos_apply_kernel: K = 1 follows the static chunk
// schedule, K = 2, 4 stride over (chunk, part) units.
template <bool REAL, int K>
__global__ void __launch_bounds__(TE_THREADS) sell_spmv_kernel(int64_t n, int64_t n_chunks,
                                                               const int32_t* __restrict__ warp_chunk,
                                                               const int64_t* __restrict__ chunk_off,
                                                               const int32_t* __restrict__ col,
                                                               const double* __restrict__ val, TeLongRows L,
                                                               double2 alpha, const double2* __restrict__ x,
                                                               double2* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int64_t wid = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (K == 1) {
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t sg = wid; sg < L.n_seg; sg += warps) {  // long rows by merge-path segments
      int64_t lr;
      double2 acc;
      if (te_long_segment<REAL>(L, sg, x, lane, &lr, &acc) != 0 && lane == 0)
        y[lr] = make_double2(alpha.x * acc.x - alpha.y * acc.y, alpha.x * acc.y + alpha.y * acc.x);
    }
    const int64_t c_end = warp_chunk[wid + 1];
    for (int64_t c = warp_chunk[wid]; c < c_end; ++c) {
      double2 acc = te_sell_row<REAL>(chunk_off, col, val, x, c, lane);
      int64_t r = c * 32 + lane;
      if (r < n && r >= L.n)
        y[r] = make_double2(alpha.x * acc.x - alpha.y * acc.y, alpha.x * acc.y + alpha.y * acc.x);
    }
  } else {
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t u = wid; u < n_chunks * K; u += warps) {
      const int64_t c = u / K;
      const int part = (int)(u - c * K);
      const double2 acc = te_sell_row_k<REAL, K>(chunk_off, col, val, x, c, part, lane);
      const int64_t r = c * 32 + part * (32 / K) + lane / K;
      if (lane % K == 0 && r < n)
        y[r] = make_double2(alpha.x * acc.x - alpha.y * acc.y, alpha.x * acc.y + alpha.y * acc.x);
    }
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

__global__ void permute_real_kernel(int64_t n, const int32_t* __restrict__ idx, const double* __restrict__ in,
                                    double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __ldg(in + __ldg(idx + i));
}

void te_launch_sell_spmv(const TeSell& A, bool is_real, double2 alpha, const double2* x_perm, double2* y_perm,
                         cudaStream_t st, const TeSegCarry* carry) {
  using K = void (*)(int64_t, int64_t, const int32_t*, const int64_t*, const int32_t*, const double*, TeLongRows,
                     double2, const double2*, double2*);
  static const K table[2][3] = {{sell_spmv_kernel<false, 1>, sell_spmv_kernel<false, 2>, sell_spmv_kernel<false, 4>},
                                {sell_spmv_kernel<true, 1>, sell_spmv_kernel<true, 2>, sell_spmv_kernel<true, 4>}};
  const int li = A.lanes == 4 ? 2 : A.lanes == 2 ? 1 : 0;
  const K k = table[is_real ? 1 : 0][li];
  int grid = A.grid;
  if (A.lanes > 1) {
    const int64_t cap = (int64_t)te_num_sms() * te_kernel_blocks_per_sm((const void*)k, TE_THREADS, 0);
    grid = (int)std::max<int64_t>(1, std::min<int64_t>((A.n_chunks * A.lanes + 7) / 8, cap));
  }
  k<<<grid, TE_THREADS, 0, st>>>(A.n, A.n_chunks, A.warp_chunk, A.chunk_off, A.col, A.val, te_long_rows(A, carry),
                                 alpha, x_perm, y_perm);
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
void te_launch_permute_real(int64_t n, const int32_t* idx, const double* in, double* out, cudaStream_t st) {
  permute_real_kernel<<<te_grid_fit((const void*)permute_real_kernel, n, TE_THREADS), TE_THREADS, 0, st>>>(n, idx, in,
                                                                                                           out);
}

// ------------------------------------------------- device build (kernels)

enum { TE_CSR_BAD_COL = 1, TE_CSR_COMPLEX = 2, TE_CSR_OFFDIAG = 4, TE_CSR_NONFINITE = 8 };

// One thread per row: column range, any imaginary part, any off-diagonal
// entry (flag bits above) and the largest |value| (bit pattern of a
// non-negative double, so the maximum does not depend on the order).
__global__ void csr_scan_kernel(int64_t n_rows, int64_t n_cols, const int32_t* __restrict__ rp,
                                const int32_t* __restrict__ ci, const double2* __restrict__ v, unsigned int* flags,
                                unsigned long long* vmax_bits) {
  unsigned int f = 0;
  double vmax = 0.0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_rows; r += (int64_t)gridDim.x * blockDim.x) {
    for (int32_t p = rp[r]; p < rp[r + 1]; ++p) {
      const int32_t c = ci[p];
      const double2 x = v[p];
      if (c < 0 || c >= n_cols) f |= TE_CSR_BAD_COL;
      if (x.y != 0.0) f |= TE_CSR_COMPLEX;
      if (c != r) f |= TE_CSR_OFFDIAG;
      if (!isfinite(x.x) || !isfinite(x.y)) f |= TE_CSR_NONFINITE;
      vmax = fmax(vmax, hypot(x.x, x.y));
    }
  }
  if (f) atomicOr(flags, f);
  atomicMax(vmax_bits, (unsigned long long)__double_as_longlong(vmax));
}

// Column sums of |value| in 64-bit fixed point (scale 2^e): integer additions
// commute, so the sums do not depend on the order of the atomics.
__global__ void colsum_fixed_kernel(int64_t n_rows, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                    const double2* __restrict__ v, double scale, unsigned long long* colsum) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_rows; r += (int64_t)gridDim.x * blockDim.x)
    for (int32_t p = rp[r]; p < rp[r + 1]; ++p) {
      const double2 x = v[p];
      atomicAdd(&colsum[ci[p]], (unsigned long long)(hypot(x.x, x.y) * scale));
    }
}

__global__ void max_u64_kernel(int64_t n, const unsigned long long* __restrict__ a, unsigned long long* out) {
  unsigned long long m = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = max(m, a[i]);
  atomicMax(out, m);
}

__global__ void real_part_kernel(int64_t n, const double2* __restrict__ v, double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = v[i].x;
}

__global__ void widen_real_kernel(int64_t n, const double* __restrict__ v, double2* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = make_double2(v[i], 0.0);
}

// Diagonal of a diagonal matrix (entries of a row summed in order).
__global__ void diag_sum_kernel(int64_t n, const int32_t* __restrict__ rp, const double2* __restrict__ v,
                                double* __restrict__ dre, double2* __restrict__ dc) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double2 acc = make_double2(0.0, 0.0);
    for (int32_t p = rp[r]; p < rp[r + 1]; ++p) {
      acc.x += v[p].x;
      acc.y += v[p].y;
    }
    dre[r] = acc.x;
    dc[r] = acc;
  }
}

// SELL-32 slots from the CSR: one thread per (chunk, lane), i.e. per sorted
// row index; padding slots point at the row itself with value 0.
template <bool REAL>
__global__ void fill_sell_kernel(int64_t n, int64_t n_long, int64_t n_chunks, const int64_t* __restrict__ off,
                                 const int32_t* __restrict__ perm, const int32_t* __restrict__ iperm,
                                 const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                 const double2* __restrict__ v, int32_t* __restrict__ scol, double* __restrict__ sval) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_chunks * 32;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t >> 5;
    const int lane = (int)(t & 31);
    const int64_t len = (off[c + 1] - off[c]) / 32;
    int64_t p0 = 0, rlen = 0;
    if (t < n && t >= n_long) {  // long rows take no chunk slots
      const int32_t r = perm[t];
      p0 = rp[r];
      rlen = rp[r + 1] - p0;
    }
    const int32_t pad = (int32_t)min(t, n - 1);
    for (int64_t k = 0; k < len; ++k) {
      const int64_t sidx = off[c] + 32 * k + lane;
      if (k < rlen) {
        const double2 x = v[p0 + k];
        scol[sidx] = iperm[ci[p0 + k]];
        if (REAL) {
          sval[sidx] = x.x;
        } else {
          reinterpret_cast<double2*>(sval)[sidx] = x;
        }
      } else {
        scol[sidx] = pad;
        if (REAL) {
          sval[sidx] = 0.0;
        } else {
          reinterpret_cast<double2*>(sval)[sidx] = make_double2(0.0, 0.0);
        }
      }
    }
  }
}

// ------------------------------------------ exclusive prefix sums (setup work)

// Tiles of 2048 elements (256 threads x 8 consecutive): each tile's exclusive
// scan and its total; the totals are scanned by one block, then added back.
constexpr int kScanTile = 2048;

template <typename T>
__device__ __forceinline__ T scan_block_2048(T (&v)[8], T carry, T* warp_tot) {
  T s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += v[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = s;  // inclusive warp scan of the thread sums
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const T y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  T base = carry, total = carry;
  for (int w = 0; w < 8; ++w) {
    if (w < warp) base += warp_tot[w];
    total += warp_tot[w];
  }
  T run = base + x - s;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const T e = v[i];
    v[i] = run;
    run += e;
  }
  __syncthreads();  // warp_tot is reused by the caller's next tile
  return total;
}

template <typename T>
__global__ void __launch_bounds__(256) scan_tiles_kernel(int64_t count, const T* __restrict__ in, T* __restrict__ out,
                                                         T* __restrict__ tile_sums) {
  __shared__ T warp_tot[8];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + threadIdx.x * 8;
  T v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = base + i < count ? in[base + i] : (T)0;
  const T total = scan_block_2048<T>(v, (T)0, warp_tot);
#pragma unroll
  for (int i = 0; i < 8; ++i)
    if (base + i < count) out[base + i] = v[i];
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

template <typename T>
__global__ void __launch_bounds__(256) scan_sums_kernel(int64_t count, T* __restrict__ sums) {
  __shared__ T warp_tot[8];
  T carry = 0;
  for (int64_t t0 = 0; t0 < count; t0 += kScanTile) {
    const int64_t base = t0 + threadIdx.x * 8;
    T v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = base + i < count ? sums[base + i] : (T)0;
    const T total = scan_block_2048<T>(v, carry, warp_tot);
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (base + i < count) sums[base + i] = v[i];
    carry = total;
  }
}

template <typename T>
__global__ void scan_add_kernel(int64_t count, T* __restrict__ out, const T* __restrict__ sums) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    out[i] += sums[i / kScanTile];
}

// out[i] = in[0] + ... + in[i - 1] for i < count (in == out allowed).
template <typename T>
int scan_exclusive(const T* in, T* out, int64_t count) {
  if (count <= 0) return TE_OK;
  const int64_t tiles = (count + kScanTile - 1) / kScanTile;
  T* sums = nullptr;
  int rc = te_cuda_check(te_malloc(&sums, sizeof(T) * tiles), "prefix sums");
  if (rc != TE_OK) return rc;
  scan_tiles_kernel<T><<<(unsigned)tiles, 256>>>(count, in, out, sums);
  if (tiles > 1) {
    scan_sums_kernel<T><<<1, 256>>>(tiles, sums);
    scan_add_kernel<T><<<te_grid_fit((const void*)scan_add_kernel<T>, count, TE_THREADS), TE_THREADS>>>(count, out,
                                                                                                       sums);
  }
  rc = te_cuda_check(cudaGetLastError(), "prefix sums");
  te_free(sums);
  return rc;
}

int te_scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t count) {
  return scan_exclusive<int64_t>(in, out, count);
}

// ------------------------------------------ SELL order on the device

// Sort key of a row for the length-sorted SELL order: 0 for long rows (longer
// than long_min; ordered among themselves on the host), else 1 + long_min - len,
// so longer rows come first.  Keys run from 0 to long_min + 1.
__device__ __forceinline__ int layout_key(const int32_t* __restrict__ rp, int64_t r, int long_min) {
  const int len = rp[r + 1] - rp[r];
  return len > long_min ? 0 : 1 + long_min - len;
}

constexpr int kLayoutTile = 4096;  // rows per tile of the counting sort

// Per-tile key counts, key-major: cnt[key * n_tiles + tile].
__global__ void __launch_bounds__(256) layout_hist_kernel(int64_t n, const int32_t* __restrict__ rp, int long_min,
                                                          int n_keys, int64_t n_tiles, int32_t* __restrict__ cnt) {
  extern __shared__ int hist[];
  for (int k = threadIdx.x; k < n_keys; k += blockDim.x) hist[k] = 0;
  __syncthreads();
  const int64_t r0 = (int64_t)blockIdx.x * kLayoutTile, r1 = min(n, r0 + kLayoutTile);
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) atomicAdd(&hist[layout_key(rp, r, long_min)], 1);
  __syncthreads();
  for (int k = threadIdx.x; k < n_keys; k += blockDim.x) cnt[(int64_t)k * n_tiles + blockIdx.x] = hist[k];
}

// Stable scatter, one warp per tile: the tile's rows in order, 32 at a time.
// Equal keys among the 32 are ranked by lane (match), and a running count per
// key in shared memory carries the rank from one group of 32 to the next, so
// rows of equal key keep their original order.  start = the exclusive scan of
// the key-major counts.
__global__ void __launch_bounds__(32) layout_scatter_kernel(int64_t n, const int32_t* __restrict__ rp, int long_min,
                                                            int n_keys, int64_t n_tiles,
                                                            const int32_t* __restrict__ start,
                                                            int32_t* __restrict__ perm, int32_t* __restrict__ iperm) {
  extern __shared__ int run[];
  const int lane = threadIdx.x;
  for (int k = lane; k < n_keys; k += 32) run[k] = 0;
  __syncwarp();
  const int64_t r0 = (int64_t)blockIdx.x * kLayoutTile, r1 = min(n, r0 + kLayoutTile);
  for (int64_t rb = r0; rb < r1; rb += 32) {
    const int64_t r = rb + lane;
    const bool valid = r < r1;
    const int key = valid ? layout_key(rp, r, long_min) : n_keys;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    int b = 0;
    if (valid && lane == leader) {
      b = run[key];
      run[key] = b + __popc(peers);
    }
    b = __shfl_sync(0xffffffffu, b, leader);
    if (valid) {
      const int pos = start[(int64_t)key * n_tiles + blockIdx.x] + b + __popc(peers & ((1u << lane) - 1u));
      perm[pos] = (int32_t)r;
      iperm[r] = pos;
    }
    __syncwarp();
  }
}

// 32 x the length of the first row of each chunk that is not long (rows are
// sorted), and 0 at index n_chunks: scanned, the chunk offsets.
__global__ void chunk_width_kernel(int64_t n, int64_t n_long, int64_t n_chunks, const int32_t* __restrict__ rp,
                                   const int32_t* __restrict__ perm, int64_t* __restrict__ width) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c <= n_chunks;
       c += (int64_t)gridDim.x * blockDim.x) {
    int64_t w = 0;
    const int64_t i0 = max(c * 32, n_long);
    if (c < n_chunks && i0 < min(n, c * 32 + 32)) {
      const int32_t r = perm[i0];
      w = 32 * (int64_t)(rp[r + 1] - rp[r]);
    }
    width[c] = w;
  }
}

__global__ void long_len_kernel(int64_t n_long, const int32_t* __restrict__ perm, const int32_t* __restrict__ rp,
                                int32_t* __restrict__ len) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_long; i += (int64_t)gridDim.x * blockDim.x)
    len[i] = rp[perm[i] + 1] - rp[perm[i]];
}

__global__ void iperm_set_kernel(int64_t count, const int32_t* __restrict__ perm, int32_t* __restrict__ iperm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    iperm[perm[i]] = (int32_t)i;
}

// The long-row CSR in the sorted basis: block i copies long row i (columns
// through iperm; values as 1 or 2 doubles per entry).
template <bool REAL>
__global__ void long_fill_kernel(int64_t n_long, const int32_t* __restrict__ perm, const int32_t* __restrict__ rp,
                                 const int32_t* __restrict__ ci, const double2* __restrict__ v,
                                 const int32_t* __restrict__ iperm, const int64_t* __restrict__ lp,
                                 int32_t* __restrict__ lcol, double* __restrict__ lval) {
  for (int64_t i = blockIdx.x; i < n_long; i += gridDim.x) {
    const int32_t r = perm[i];
    const int64_t p0 = rp[r], len = rp[r + 1] - p0, q0 = lp[i];
    for (int64_t k = threadIdx.x; k < len; k += blockDim.x) {
      lcol[q0 + k] = iperm[ci[p0 + k]];
      const double2 x = v[p0 + k];
      if (REAL) {
        lval[q0 + k] = x.x;
      } else {
        lval[2 * (q0 + k)] = x.x;
        lval[2 * (q0 + k) + 1] = x.y;
      }
    }
  }
}

enum { TE_COO_BAD = 1, TE_COO_UNSORTED = 2 };

// COO input checks on the device: indices in range (the first bad entry is
// kept) and rows in non-decreasing order.
__global__ void coo_scan_kernel(int64_t nnz, uint64_t n_rows, uint64_t n_cols, const uint64_t* __restrict__ row,
                                const uint64_t* __restrict__ col, unsigned int* flags,
                                unsigned long long* first_bad) {
  unsigned int f = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t r = row[i];
    if (r >= n_rows || col[i] >= n_cols) {
      f |= TE_COO_BAD;
      atomicMin(first_bad, (unsigned long long)i);
    }
    if (i > 0 && row[i - 1] > r) f |= TE_COO_UNSORTED;
  }
  if (f) atomicOr(flags, f);
}

// Row-sorted COO read straight from host memory, on devices that access
// pageable memory through the host's page tables (Grace): the checks of
// coo_scan_kernel, the columns narrowed to int32, the values, and the row
// pointers from the row boundaries (rp[q] = the first entry of a row >= q),
// in one pass over the host arrays.  rp is valid when no flag is raised.
__global__ void __launch_bounds__(TE_THREADS) coo_ingest_kernel(int64_t nnz, uint64_t n_rows, uint64_t n_cols,
                                                                const uint64_t* __restrict__ row,
                                                                const uint64_t* __restrict__ col,
                                                                const double* __restrict__ val,
                                                                int32_t* __restrict__ rp, int32_t* __restrict__ ci,
                                                                double2* __restrict__ v, unsigned int* flags,
                                                                unsigned long long* first_bad) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  unsigned int f = 0;
  for (int64_t base = ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; base < nnz;
       base += warps * 32) {
    const int64_t i = base + lane;
    const bool live = i < nnz;
    const uint64_t r = live ? row[i] : 0, c = live ? col[i] : 0;
    uint64_t prev = __shfl_up_sync(0xffffffffu, r, 1);
    if (lane == 0 && i > 0 && live) prev = row[i - 1];
    if (!live) continue;
    if (r >= n_rows || c >= n_cols) {
      f |= TE_COO_BAD;
      atomicMin(first_bad, (unsigned long long)i);
      continue;
    }
    if (i > 0 && prev > r) f |= TE_COO_UNSORTED;
    ci[i] = (int32_t)c;
    v[i] = make_double2(val[2 * i], val[2 * i + 1]);
    // rows (prev, r] start here (rows 0..r for the first entry)
    const uint64_t q0 = i == 0 ? 0 : prev + 1;
    for (uint64_t q = q0; q <= r; ++q) rp[q] = (int32_t)i;
    if (i == nnz - 1)
      for (uint64_t q = r + 1; q <= n_rows; ++q) rp[q] = (int32_t)nnz;
  }
  if (f) atomicOr(flags, f);
}

__global__ void row_count_kernel(int64_t nnz, const uint64_t* __restrict__ row, int32_t* __restrict__ count) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&count[row[i]], 1);
}

__global__ void narrow_index_kernel(int64_t nnz, const uint64_t* __restrict__ in, int32_t* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int32_t)in[i];
}

// The reference's 1-norm on the device, for real matrices whose |H| is
// symmetric: with every row sorted by column (no duplicates) and every entry
// (r, c) mirrored by (c, r) of the same modulus, column c's entries in row
// order have exactly the moduli of row c in column order, so each row's
// sequential sum equals the entry-order column sum of the row-sorted COO input
// bit for bit.  One thread per row checks the conditions (binary search for
// the mirror entry); flags: 1 a complex value, 2 a row not strictly sorted,
// 4 a missing or different mirror.  The maximum goes to *max_bits.
__global__ void __launch_bounds__(TE_THREADS) mirror_norm1_kernel(int64_t n, const int32_t* __restrict__ rp,
                                                                  const int32_t* __restrict__ ci,
                                                                  const double2* __restrict__ v,
                                                                  unsigned int* flags, unsigned long long* max_bits) {
  unsigned long long smax = 0;  // bit patterns (ordered as the non-negative sums); one atomic per thread
  unsigned int f = 0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    int32_t prev = -1;
    for (int32_t k = rp[r]; k < rp[r + 1]; ++k) {
      const int32_t c = ci[k];
      const double2 a = v[k];
      if (a.y != 0.0) f |= 1u;
      if (c <= prev) f |= 2u;
      prev = c;
      const double m = fabs(a.x);
      s += m;
      int32_t lo = rp[c], hi = rp[c + 1];  // the mirror (c, r) by bisection
      while (lo < hi) {
        const int32_t mid = lo + (hi - lo) / 2;
        if (ci[mid] < (int32_t)r) lo = mid + 1;
        else hi = mid;
      }
      if (lo >= rp[c + 1] || ci[lo] != (int32_t)r || fabs(v[lo].x) != m) f |= 4u;
    }
    smax = max(smax, (unsigned long long)__double_as_longlong(s));
  }
  if (f) atomicOr(flags, f);
  atomicMax(max_bits, smax);
}

// ------------------------------------------------------------ host build

// Static warp schedule of the SpMV passes (equal estimated work per warp:
// 2 (real) or 4 (complex) FMAs per slot, about 8 per row for the epilogues).
int te_seg_carry_alloc(const TeSell& S, TeSegCarry* c) {
  *c = TeSegCarry{};
  if (S.n_split == 0) return TE_OK;
  TE_CUDA(te_malloc(&c->part, sizeof(double2) * S.n_seg));
  int rc = te_cuda_check(te_malloc(&c->cnt, sizeof(unsigned int) * S.n_long), "segment carries");
  if (rc == TE_OK) rc = te_cuda_check(cudaMemset(c->cnt, 0, sizeof(unsigned int) * S.n_long), "segment carries");
  if (rc != TE_OK) te_seg_carry_free(c);
  return rc;
}

void te_seg_carry_free(TeSegCarry* c) {
  te_free(c->part);
  te_free(c->cnt);
  *c = TeSegCarry{};
}

void te_sell_schedule(const std::vector<int64_t>& off, int64_t n_chunks, int blocks_per_sm,
                      bool real, int& grid, bool& saturated, std::vector<int32_t>& wc) {
  const int64_t need = (n_chunks * 32 + TE_THREADS - 1) / TE_THREADS;
  const int64_t cap = (int64_t)te_num_sms() * std::max(blocks_per_sm, 1);
  grid = (int)std::max<int64_t>(1, std::min<int64_t>(need, cap));
  saturated = need > cap;
  const int64_t W = (int64_t)grid * (TE_THREADS / 32);
  const double w_slot = real ? 2.0 : 4.0, w_chunk = 8.0 * 32;
  auto cost = [&](int64_t c) { return w_slot * (double)off[c] + w_chunk * (double)c; };
  const double total = cost(n_chunks);
  wc.assign(W + 1, 0);
  int64_t c = 0;
  for (int64_t w = 0; w < W; ++w) {
    const double target = total * (double)w / (double)W;
    while (c < n_chunks && cost(c) < target) ++c;
    wc[w] = (int32_t)c;
  }
  wc[W] = (int32_t)n_chunks;
}

namespace {

void free_matrix(te_matrix_s* M) {
  te_free(M->row_ptr);
  te_free(M->col);
  te_free(M->val);
  te_free(M->diag_re);
  te_free(M->diag_c);
  te_free(M->sell.chunk_off);
  te_free(M->sell.col);
  te_free(M->sell.val);
  te_free(M->sell.perm);
  te_free(M->sell.iperm);
  te_free(M->sell.warp_chunk);
  te_free(M->sell.long_ptr);
  te_free(M->sell.long_col);
  te_free(M->sell.long_val);
  te_free(M->sell.seg_row);
  te_free(M->sell.seg_begin);
  te_free(M->sell.row_seg);
  te_free(M->sell.seg_part);
  te_free(M->sell.seg_cnt);
  te_sell_free_fixed(M->sell);
  delete M;
}

template <class T>
int upload(T** dst, const T* src, size_t count) {
  TE_CUDA(te_malloc(dst, sizeof(T) * std::max<size_t>(count, 1)));
  if (count) TE_CUDA(cudaMemcpy(*dst, src, sizeof(T) * count, cudaMemcpyHostToDevice));
  return TE_OK;
}

// SELL-32 layout of a square matrix from its row pointers (host): rows sorted
// by length (descending, stable), chunk offsets in slots, and the static warp
// schedule of the SpMV passes (equal FP64 work per warp: te_sell_row issues 2
// (real) or 4 (complex) FMAs per slot, the SpMV epilogues about 8 per row).
// Uploads chunk_off, perm, iperm and warp_chunk; returns perm, iperm and the
// offsets for filling col/val.
// The static warp schedule of the FP64 SELL kernels from the host chunk
// offsets; uploads warp_chunk.
int sell_schedule(TeSell& S, const std::vector<int64_t>& off, bool real) {
  const int bps = std::min(te_sell_blocks_per_sm(real),
                           te_kernel_blocks_per_sm(real ? (const void*)sell_spmv_kernel<true, 1>
                                                        : (const void*)sell_spmv_kernel<false, 1>,
                                                   TE_THREADS, 0));
  std::vector<int32_t> wc;
  te_sell_schedule(off, S.n_chunks, bps, real, S.grid, S.saturated, wc);
  return upload(&S.warp_chunk, wc.data(), wc.size());
}

int sell_layout(te_matrix_s* M, const std::vector<int32_t>& rp, bool real, std::vector<int32_t>& perm,
                std::vector<int32_t>& iperm, std::vector<int64_t>& off) {
  const int64_t n = M->n_rows;
  TeSell& S = M->sell;
  S.n = n;
  S.n_chunks = (n + 31) / 32;
  // stable counting sort by length, longest first
  int32_t max_len = 0;
  for (int64_t r = 0; r < n; ++r) max_len = std::max(max_len, rp[r + 1] - rp[r]);
  std::vector<int64_t> start(max_len + 2, 0);
  for (int64_t r = 0; r < n; ++r) start[max_len - (rp[r + 1] - rp[r]) + 1]++;
  for (int32_t b = 0; b <= max_len; ++b) start[b + 1] += start[b];
  perm.assign(n, 0);
  iperm.assign(n, 0);
  for (int64_t r = 0; r < n; ++r) perm[start[max_len - (rp[r + 1] - rp[r])]++] = (int32_t)r;
  for (int64_t i = 0; i < n; ++i) iperm[perm[i]] = (int32_t)i;
  // long rows: longer than max(1024, 32 x the mean row length); they lead the
  // sorted order and take no chunk slots
  const int64_t nnz = rp[n];
  const int64_t long_min = std::max<int64_t>(1024, 32 * ((nnz + n - 1) / std::max<int64_t>(n, 1)));
  S.n_long = 0;
  while (S.n_long < n && rp[perm[S.n_long] + 1] - rp[perm[S.n_long]] > long_min) ++S.n_long;
  off.assign(S.n_chunks + 1, 0);
  for (int64_t c = 0; c < S.n_chunks; ++c) {
    int64_t len = 0;  // rows are sorted: the first row of the chunk that is not long is the longest
    for (int64_t i = c * 32; i < std::min<int64_t>(n, c * 32 + 32); ++i)
      if (i >= S.n_long) {
        len = rp[perm[i] + 1] - rp[perm[i]];
        break;
      }
    off[c + 1] = off[c] + 32 * len;
  }
  S.slots = off[S.n_chunks];
  int rc;
  if ((rc = upload(&S.chunk_off, off.data(), off.size())) != TE_OK) return rc;
  if ((rc = upload(&S.perm, perm.data(), perm.size())) != TE_OK) return rc;
  if ((rc = upload(&S.iperm, iperm.data(), iperm.size())) != TE_OK) return rc;
  return sell_schedule(S, off, real);
}

// The SELL order of a device CSR without a host copy of its row pointers:
// the same order as sell_layout (stable by length, longest first, long rows
// leading), from a counting sort on the device; the few long rows are
// ordered on the host.  Sets perm, iperm, n_long, chunk_off, slots and the
// schedule.  TE_ERR_UNSUPPORTED (nothing set) when the key range (the long-row
// threshold) is too wide for the sort's shared-memory counters.
int sell_layout_device(te_matrix_s* M, const int32_t* d_rp, bool real) {
  const int64_t n = M->n_rows, nnz = M->nnz;
  TeSell& S = M->sell;
  const int64_t long_min = std::max<int64_t>(1024, 32 * ((nnz + n - 1) / std::max<int64_t>(n, 1)));
  const int64_t n_tiles = (n + kLayoutTile - 1) / kLayoutTile;
  if (long_min + 2 > 8192 || (long_min + 2) * n_tiles > ((int64_t)1 << 27)) return TE_ERR_UNSUPPORTED;
  const int n_keys = (int)long_min + 2;
  S.n = n;
  S.n_chunks = (n + 31) / 32;
  int32_t *cnt = nullptr, *d_len = nullptr;
  auto done = [&](int rc) {
    te_free(cnt);
    te_free(d_len);
    return rc;
  };
  int rc = te_cuda_check(te_malloc(&cnt, sizeof(int32_t) * n_keys * n_tiles), "layout");
  if (rc == TE_OK) rc = te_cuda_check(te_malloc(&S.perm, sizeof(int32_t) * n), "layout");
  if (rc == TE_OK) rc = te_cuda_check(te_malloc(&S.iperm, sizeof(int32_t) * n), "layout");
  if (rc == TE_OK) rc = te_cuda_check(te_malloc(&S.chunk_off, sizeof(int64_t) * (S.n_chunks + 1)), "layout");
  if (rc != TE_OK) return done(rc);
  layout_hist_kernel<<<(unsigned)n_tiles, 256, sizeof(int) * n_keys>>>(n, d_rp, (int)long_min, n_keys, n_tiles, cnt);
  if ((rc = scan_exclusive<int32_t>(cnt, cnt, n_keys * n_tiles)) != TE_OK) return done(rc);
  layout_scatter_kernel<<<(unsigned)n_tiles, 32, sizeof(int) * n_keys>>>(n, d_rp, (int)long_min, n_keys, n_tiles,
                                                                         cnt, S.perm, S.iperm);
  int32_t n_long = 0;  // the rows of key 0: where key 1 starts
  if ((rc = te_cuda_check(cudaMemcpy(&n_long, cnt + n_tiles, sizeof(int32_t), cudaMemcpyDeviceToHost), "layout")) !=
      TE_OK)
    return done(rc);
  S.n_long = n_long;
  if (n_long > 0) {  // long rows: by length, longest first, ties in row order
    std::vector<int32_t> rows(n_long), len(n_long), sorted(n_long);
    if ((rc = te_cuda_check(te_malloc(&d_len, sizeof(int32_t) * n_long), "layout")) != TE_OK) return done(rc);
    long_len_kernel<<<te_grid_fit((const void*)long_len_kernel, n_long, TE_THREADS), TE_THREADS>>>(n_long, S.perm,
                                                                                                   d_rp, d_len);
    if ((rc = te_cuda_check(cudaMemcpy(rows.data(), S.perm, sizeof(int32_t) * n_long, cudaMemcpyDeviceToHost),
                            "layout")) != TE_OK ||
        (rc = te_cuda_check(cudaMemcpy(len.data(), d_len, sizeof(int32_t) * n_long, cudaMemcpyDeviceToHost),
                            "layout")) != TE_OK)
      return done(rc);
    std::vector<int32_t> order(n_long);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return len[a] > len[b]; });
    for (int32_t i = 0; i < n_long; ++i) sorted[i] = rows[order[i]];
    if ((rc = te_cuda_check(cudaMemcpy(S.perm, sorted.data(), sizeof(int32_t) * n_long, cudaMemcpyHostToDevice),
                            "layout")) != TE_OK)
      return done(rc);
    iperm_set_kernel<<<te_grid_fit((const void*)iperm_set_kernel, n_long, TE_THREADS), TE_THREADS>>>(n_long, S.perm,
                                                                                                     S.iperm);
  }
  chunk_width_kernel<<<te_grid_fit((const void*)chunk_width_kernel, S.n_chunks + 1, TE_THREADS), TE_THREADS>>>(
      n, S.n_long, S.n_chunks, d_rp, S.perm, S.chunk_off);
  if ((rc = scan_exclusive<int64_t>(S.chunk_off, S.chunk_off, S.n_chunks + 1)) != TE_OK) return done(rc);
  std::vector<int64_t> off(S.n_chunks + 1);
  if ((rc = te_cuda_check(
           cudaMemcpy(off.data(), S.chunk_off, sizeof(int64_t) * (S.n_chunks + 1), cudaMemcpyDeviceToHost),
           "layout")) != TE_OK)
    return done(rc);
  S.slots = off[S.n_chunks];
  return done(sell_schedule(S, off, real));
}

// Merge-path segments of the long rows (lp: the long-row pointers, host).
// A row of k entries is k + 1 merge items; seg_items is at least 2048 and
// large enough for about two segments per warp of a resident wave over all
// long rows' items, so a row is split only when it alone would hold up the
// pass.  Rows split into equal entry counts per segment.  The matrix-owned
// carries serve te_matrix_spmv_noalloc.
int long_row_segments(TeSell& S, const std::vector<int64_t>& lp) {
  const int64_t nl = S.n_long;
  if (nl == 0) return TE_OK;
  const int64_t items = lp[nl] + nl;
  const int64_t wave_warps = (int64_t)te_num_sms() * 6 * (TE_THREADS / 32);
  S.seg_items = std::max<int64_t>(2048, (items + 2 * wave_warps - 1) / (2 * wave_warps));
  std::vector<int32_t> seg_row, row_seg(nl + 1, 0);
  std::vector<int64_t> seg_begin;
  S.n_split = 0;
  for (int64_t i = 0; i < nl; ++i) {
    const int64_t k = lp[i + 1] - lp[i];
    const int64_t ns = std::max<int64_t>(1, (k + 1 + S.seg_items - 1) / S.seg_items);
    if (ns > 1) ++S.n_split;
    row_seg[i] = (int32_t)seg_row.size();
    for (int64_t t = 0; t < ns; ++t) {
      seg_row.push_back((int32_t)i);
      seg_begin.push_back(lp[i] + k * t / ns);
    }
  }
  row_seg[nl] = (int32_t)seg_row.size();
  seg_begin.push_back(lp[nl]);
  S.n_seg = (int64_t)seg_row.size();
  int rc;
  if ((rc = upload(&S.seg_row, seg_row.data(), seg_row.size())) != TE_OK) return rc;
  if ((rc = upload(&S.seg_begin, seg_begin.data(), seg_begin.size())) != TE_OK) return rc;
  if ((rc = upload(&S.row_seg, row_seg.data(), row_seg.size())) != TE_OK) return rc;
  TeSegCarry c;
  if ((rc = te_seg_carry_alloc(S, &c)) != TE_OK) return rc;
  S.seg_part = c.part;
  S.seg_cnt = c.cnt;
  return TE_OK;
}

// The long-row CSR in the sorted basis from the device CSR (perm and iperm
// final): one device pass after a host prefix over the long rows' lengths.
int long_rows_device(te_matrix_s* M, const int32_t* d_rp, const int32_t* d_ci, const double2* d_v, bool real) {
  TeSell& S = M->sell;
  const int64_t nl = S.n_long;
  if (nl == 0) return TE_OK;
  int32_t* d_len = nullptr;
  std::vector<int32_t> len(nl);
  int rc = te_cuda_check(te_malloc(&d_len, sizeof(int32_t) * nl), "long rows");
  if (rc != TE_OK) return rc;
  long_len_kernel<<<te_grid_fit((const void*)long_len_kernel, nl, TE_THREADS), TE_THREADS>>>(nl, S.perm, d_rp, d_len);
  rc = te_cuda_check(cudaMemcpy(len.data(), d_len, sizeof(int32_t) * nl, cudaMemcpyDeviceToHost), "long rows");
  te_free(d_len);
  if (rc != TE_OK) return rc;
  std::vector<int64_t> lp(nl + 1, 0);
  for (int64_t i = 0; i < nl; ++i) lp[i + 1] = lp[i] + len[i];
  if ((rc = upload(&S.long_ptr, lp.data(), lp.size())) != TE_OK) return rc;
  if ((rc = long_row_segments(S, lp)) != TE_OK) return rc;
  const int64_t ne = std::max<int64_t>(lp[nl], 1);
  if ((rc = te_cuda_check(te_malloc(&S.long_col, sizeof(int32_t) * ne), "long rows")) != TE_OK ||
      (rc = te_cuda_check(te_malloc(&S.long_val, sizeof(double) * (real ? 1 : 2) * ne), "long rows")) != TE_OK)
    return rc;
  const unsigned grid = (unsigned)std::min<int64_t>(nl, 4096);
  if (real)
    long_fill_kernel<true><<<grid, TE_THREADS>>>(nl, S.perm, d_rp, d_ci, d_v, S.iperm, S.long_ptr, S.long_col,
                                                 S.long_val);
  else
    long_fill_kernel<false><<<grid, TE_THREADS>>>(nl, S.perm, d_rp, d_ci, d_v, S.iperm, S.long_ptr, S.long_col,
                                                  S.long_val);
  return te_cuda_check(cudaGetLastError(), "long rows");
}

// The long-row CSR (sorted basis) from host copies of the original CSR.
int build_long_rows(te_matrix_s* M, const std::vector<int32_t>& rp, const std::vector<int32_t>& ci,
                    const std::vector<double>& vv, bool real, const std::vector<int32_t>& perm,
                    const std::vector<int32_t>& iperm) {
  TeSell& S = M->sell;
  if (S.n_long == 0) return TE_OK;
  std::vector<int64_t> lp(S.n_long + 1, 0);
  std::vector<int32_t> lc;
  std::vector<double> lv;
  for (int64_t i = 0; i < S.n_long; ++i) {
    const int32_t r = perm[i];
    for (int32_t p = rp[r]; p < rp[r + 1]; ++p) {
      lc.push_back(iperm[ci[p]]);
      lv.push_back(vv[2 * p]);
      if (!real) lv.push_back(vv[2 * p + 1]);
    }
    lp[i + 1] = (int64_t)lc.size();
  }
  int rc;
  if ((rc = upload(&S.long_ptr, lp.data(), lp.size())) != TE_OK) return rc;
  if ((rc = upload(&S.long_col, lc.data(), lc.size())) != TE_OK) return rc;
  if ((rc = upload(&S.long_val, lv.data(), lv.size())) != TE_OK) return rc;
  return long_row_segments(S, lp);
}

// rp/ci/vv: original-order CSR with interleaved complex values.
int build_matrix(te_matrix_s* M, const std::vector<int32_t>& rp, const std::vector<int32_t>& ci,
                 const std::vector<double>& vv, double norm1_given) {
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
  // 1-norm as in matrixDataTypes.cpp:67-79 (max absolute column sum), unless
  // the caller computed it in its own entry order
  if (std::isnan(norm1_given)) {
    std::vector<double> colsum(M->n_cols, 0.0);
    for (int64_t p = 0; p < nnz; ++p) colsum[ci[p]] += std::abs(std::complex<double>(vv[2 * p], vv[2 * p + 1]));
    M->norm1 = *std::max_element(colsum.begin(), colsum.end());
  } else {
    M->norm1 = norm1_given;
  }

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

  std::vector<int32_t> perm, iperm;
  std::vector<int64_t> off;
  if ((rc = sell_layout(M, rp, real, perm, iperm, off)) != TE_OK) return rc;
  TeSell& S = M->sell;
  std::vector<int32_t> scol(S.slots);
  std::vector<double> sval((real ? 1 : 2) * S.slots, 0.0);
  for (int64_t c = 0; c < S.n_chunks; ++c) {
    int64_t len = (off[c + 1] - off[c]) / 32;
    for (int lane = 0; lane < 32; ++lane) {
      int64_t rnew = c * 32 + lane;
      int32_t pad_col = (int32_t)std::min<int64_t>(rnew, n - 1);
      int64_t rlen = 0, p0 = 0;
      if (rnew < n && rnew >= S.n_long) {
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
  if ((rc = upload(&S.col, scol.data(), scol.size())) != TE_OK) return rc;
  if ((rc = upload(&S.val, sval.data(), sval.size())) != TE_OK) return rc;
  return build_long_rows(M, rp, ci, vv, real, perm, iperm);
}

int finish_create(int64_t n_rows, int64_t n_cols, const std::vector<int32_t>& rp, const std::vector<int32_t>& ci,
                  const std::vector<double>& vv, te_matrix* out, double norm1_given = NAN) {
  for (size_t i = 0; i < vv.size(); ++i)
    if (!std::isfinite(vv[i])) {
      te_set_error("matrix creation: entry %lld is not finite (NaN or Inf)", (long long)(i / 2));
      return TE_ERR_INVALID_ARG;
    }
  te_matrix_s* M = new te_matrix_s();
  cudaGetDevice(&M->device);
  M->n_rows = n_rows;
  M->n_cols = n_cols;
  M->nnz = (int64_t)ci.size();
  int rc = build_matrix(M, rp, ci, vv, norm1_given);
  if (rc != TE_OK) {
    free_matrix(M);
    return rc;
  }
  *out = M;
  return TE_OK;
}

// Device build: the CSR (int32 row pointers, columns, complex values) is
// already on the device and becomes the matrix's own (the caller's buffers
// are adopted: M frees them).  rp_host is a host copy of the row pointers.
// The 1-norm is the maximum column sum of |a| accumulated in 64-bit fixed
// point (relative resolution ~1e-12 of the largest entry), so it does not
// depend on the order of the device atomics.
int build_matrix_device(te_matrix_s* M, int32_t* d_rp, int32_t* d_ci, double2* d_v, double norm1_given) {
  const int64_t n = M->n_rows, nnz = M->nnz;
  M->row_ptr = d_rp;
  M->col = d_ci;
  unsigned int* d_flags = nullptr;
  unsigned long long *d_u64 = nullptr, *d_colsum = nullptr;
  auto cleanup = [&]() {
    te_free(d_flags);
    te_free(d_u64);
    te_free(d_colsum);
  };
  auto fail = [&](int rc) {
    te_free(d_v);
    cleanup();
    return rc;
  };
  if (te_cuda_check(te_malloc(&d_flags, sizeof(unsigned int)), "flags") != TE_OK) return fail(TE_ERR_CUDA);
  if (te_cuda_check(te_malloc(&d_u64, 2 * sizeof(unsigned long long)), "flags") != TE_OK) return fail(TE_ERR_CUDA);
  cudaMemset(d_flags, 0, sizeof(unsigned int));
  cudaMemset(d_u64, 0, 2 * sizeof(unsigned long long));
  const int gr = te_grid_fit((const void*)csr_scan_kernel, n, TE_THREADS);
  csr_scan_kernel<<<gr, TE_THREADS>>>(n, M->n_cols, d_rp, d_ci, d_v, d_flags, d_u64);
  unsigned int flags = 0;
  unsigned long long vmax_bits = 0;
  if (te_cuda_check(cudaMemcpy(&flags, d_flags, sizeof(flags), cudaMemcpyDeviceToHost), "flags") != TE_OK ||
      te_cuda_check(cudaMemcpy(&vmax_bits, d_u64, sizeof(vmax_bits), cudaMemcpyDeviceToHost), "flags") != TE_OK)
    return fail(TE_ERR_CUDA);
  if (flags & TE_CSR_BAD_COL) {
    te_set_error("te_matrix_create_csr_device: a column index is out of range");
    return fail(TE_ERR_INVALID_ARG);
  }
  if (flags & TE_CSR_NONFINITE) {
    te_set_error("matrix creation: an entry is not finite (NaN or Inf)");
    return fail(TE_ERR_INVALID_ARG);
  }
  const bool real = !(flags & TE_CSR_COMPLEX);
  const bool diag = (M->n_rows == M->n_cols) && !(flags & TE_CSR_OFFDIAG);
  M->is_real = real;
  M->is_diag = diag;
  // 1-norm
  double vmax;
  std::memcpy(&vmax, &vmax_bits, sizeof(vmax));
  M->norm1 = std::isnan(norm1_given) ? 0.0 : norm1_given;
  if (std::isnan(norm1_given) && vmax > 0.0 && nnz > 0) {
    const int e = 62 - (int)std::ceil(std::log2(vmax * (double)std::max<int64_t>(n, 1)));
    const double scale = std::ldexp(1.0, e);
    if (te_cuda_check(te_malloc(&d_colsum, sizeof(unsigned long long) * M->n_cols), "colsum") != TE_OK)
      return fail(TE_ERR_CUDA);
    cudaMemset(d_colsum, 0, sizeof(unsigned long long) * M->n_cols);
    colsum_fixed_kernel<<<gr, TE_THREADS>>>(n, d_rp, d_ci, d_v, scale, d_colsum);
    max_u64_kernel<<<te_grid_fit((const void*)max_u64_kernel, M->n_cols, TE_THREADS), TE_THREADS>>>(
        M->n_cols, d_colsum, d_u64 + 1);
    unsigned long long mx = 0;
    if (te_cuda_check(cudaMemcpy(&mx, d_u64 + 1, sizeof(mx), cudaMemcpyDeviceToHost), "norm1") != TE_OK)
      return fail(TE_ERR_CUDA);
    M->norm1 = std::ldexp((double)mx, -e);
  }
  // values: real matrices keep the real parts
  if (real) {
    double* vr = nullptr;
    if (te_cuda_check(te_malloc(&vr, sizeof(double) * std::max<int64_t>(nnz, 1)), "values") != TE_OK)
      return fail(TE_ERR_CUDA);
    real_part_kernel<<<te_grid_fit((const void*)real_part_kernel, nnz, TE_THREADS), TE_THREADS>>>(nnz, d_v, vr);
    M->val = vr;
  } else {
    M->val = reinterpret_cast<double*>(d_v);
  }
  if (diag) {
    if (te_cuda_check(te_malloc(&M->diag_re, sizeof(double) * n), "diag") != TE_OK ||
        te_cuda_check(te_malloc(&M->diag_c, sizeof(double2) * n), "diag") != TE_OK) {
      if (real) te_free(d_v);
      cleanup();
      return TE_ERR_CUDA;
    }
    diag_sum_kernel<<<te_grid_fit((const void*)diag_sum_kernel, n, TE_THREADS), TE_THREADS>>>(n, d_rp, d_v,
                                                                                             M->diag_re, M->diag_c);
  }
  int rc = TE_OK;
  if (M->n_rows == M->n_cols) {
    TeSell& S = M->sell;
    rc = sell_layout_device(M, d_rp, real);
    if (rc == TE_ERR_UNSUPPORTED) {  // a wide key range: the host sort from a copy of the row pointers
      std::vector<int32_t> rp_host(n + 1), perm, iperm;
      std::vector<int64_t> off;
      rc = te_cuda_check(cudaMemcpy(rp_host.data(), d_rp, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost),
                         "layout");
      if (rc == TE_OK) rc = sell_layout(M, rp_host, real, perm, iperm, off);
    }
    if (rc == TE_OK) rc = long_rows_device(M, d_rp, d_ci, d_v, real);
    if (rc == TE_OK) rc = te_cuda_check(te_malloc(&S.col, sizeof(int32_t) * std::max<int64_t>(S.slots, 1)), "sell");
    if (rc == TE_OK)
      rc = te_cuda_check(te_malloc(&S.val, sizeof(double) * (real ? 1 : 2) * std::max<int64_t>(S.slots, 1)), "sell");
    if (rc == TE_OK) {
      const int gf = te_grid_fit(real ? (const void*)fill_sell_kernel<true> : (const void*)fill_sell_kernel<false>,
                                 S.n_chunks * 32, TE_THREADS);
      if (real)
        fill_sell_kernel<true><<<gf, TE_THREADS>>>(n, S.n_long, S.n_chunks, S.chunk_off, S.perm, S.iperm, d_rp, d_ci,
                                                   d_v, S.col, S.val);
      else
        fill_sell_kernel<false><<<gf, TE_THREADS>>>(n, S.n_long, S.n_chunks, S.chunk_off, S.perm, S.iperm, d_rp, d_ci,
                                                    d_v, S.col, S.val);
    }
  }
  if (rc == TE_OK) rc = te_cuda_check(cudaDeviceSynchronize(), "device build");
  if (real) te_free(d_v);
  cleanup();
  return rc;
}

}  // namespace

// Adopt a device CSR (see build_matrix_device); used by the device-side
// workload generators.  On failure the buffers are freed.
int te_matrix_adopt_device_csr(int64_t n_rows, int64_t n_cols, int64_t nnz, int32_t* d_rp, int32_t* d_ci,
                               double2* d_v, te_matrix* out, double norm1) {
  te_matrix_s* M = new te_matrix_s();
  cudaGetDevice(&M->device);
  M->n_rows = n_rows;
  M->n_cols = n_cols;
  M->nnz = nnz;
  int rc = build_matrix_device(M, d_rp, d_ci, d_v, norm1);
  if (rc != TE_OK) {
    free_matrix(M);
    return rc;
  }
  *out = M;
  return TE_OK;
}

// ------------------------------------------------------------------ C ABI

namespace {

// The reference's 1-norm (matrixDataTypes.cpp:67-79): column sums of |a| in the
// order of the COO entries.  Threads own disjoint column ranges and each scans
// all entries, so every column is summed in exactly that order.  Entries with
// an out-of-range column are skipped (the caller rejects them).  |re + i 0| is
// exactly |re| (hypot(x, +-0) = |x|), so real entries skip hypot.
// A set cancel flag (checked every 2^16 entries) abandons the sums (NaN).
double coo_norm1(int64_t n_cols, int64_t nnz, const uint64_t* col, const double* val,
                 const std::atomic<bool>* cancel = nullptr) {
  const int T = (int)std::max<unsigned>(1u, std::min<unsigned>(16u, std::thread::hardware_concurrency()));
  std::vector<double> colsum(n_cols, 0.0);
  auto work = [&](int t) {
    const uint64_t c0 = (uint64_t)(n_cols * t / T), c1 = (uint64_t)(n_cols * (t + 1) / T);
    for (int64_t i = 0; i < nnz; ++i) {
      if (cancel && (i & 0xffff) == 0 && cancel->load(std::memory_order_relaxed)) return;
      const uint64_t c = col[i];
      if (c >= c0 && c < c1) {
        const double re = val[2 * i], im = val[2 * i + 1];
        colsum[c] += im == 0.0 ? std::fabs(re) : std::abs(std::complex<double>(re, im));
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < T; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& th : pool) th.join();
  if (cancel && cancel->load()) return std::nan("");
  return n_cols > 0 ? *std::max_element(colsum.begin(), colsum.end()) : 0.0;
}

// Host conversion: stable COO -> CSR (entries of one row keep their input order).
int create_coo_host(int64_t n_rows, int64_t n_cols, int64_t nnz, const uint64_t* row_index, const uint64_t* columns,
                    const double* values, double norm1, te_matrix* out) {
  for (int64_t i = 0; i < nnz; ++i)
    if (row_index[i] >= (uint64_t)n_rows || columns[i] >= (uint64_t)n_cols) {
      te_set_error("te_matrix_create_coo: entry %lld out of range", (long long)i);
      return TE_ERR_INVALID_ARG;
    }
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
  return finish_create(n_rows, n_cols, rp, ci, vv, out, norm1);
}

// A CPU read of one word in every 4 KiB of the host arrays, on up to 16 threads,
// before the device reads them in place.  The GPU reaches pageable host memory
// through the CPU's page tables; without this pass the same 405 MB read by the
// ingest kernel alternated between 2.8 ms and 60-130 ms from call to call (with
// NUMA balancing off), with it every read took 2.8 ms; the pass itself costs
// about 1.6 ms for those 405 MB.
void touch_host_pages(const void* const* ptrs, const size_t* bytes, int count) {
  const size_t kStride = 4096;
  size_t pages = 0;
  for (int a = 0; a < count; ++a) pages += (bytes[a] + kStride - 1) / kStride;
  const int T = (int)std::max<size_t>(1, std::min<size_t>(16, pages >> 14));  // 16 K pages per thread
  std::atomic<uint64_t> sink(0);
  auto work = [&](int t) {
    uint64_t acc = 0;
    for (int a = 0; a < count; ++a) {
      const unsigned char* p = static_cast<const unsigned char*>(ptrs[a]);
      const size_t np = (bytes[a] + kStride - 1) / kStride;
      for (size_t i = np * t / T; i < np * (t + 1) / T; ++i) acc += *(volatile const unsigned char*)(p + i * kStride);
    }
    sink.fetch_add(acc, std::memory_order_relaxed);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < T; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& th : pool) th.join();
}

// Device conversion of a row-sorted COO (the order TE::Hamiltonian::createMatrix
// produces): the arrays are copied to the GPU as they are, the row pointers come
// from per-row counts, and the layout is built by kernels.  Returns
// TE_ERR_UNSUPPORTED (nothing built, no error set) for unsorted input.
int create_coo_device(int64_t n_rows, int64_t n_cols, int64_t nnz, const uint64_t* row_index, const uint64_t* columns,
                      const double* values, double* norm1_gpu, te_matrix* out, const std::function<void()>& host_done) {
  *norm1_gpu = std::nan("");
  uint64_t *d_row = nullptr, *d_col = nullptr;
  double2* d_v = nullptr;
  int32_t *d_cnt = nullptr, *d_rp = nullptr, *d_ci = nullptr;
  unsigned int* d_flags = nullptr;
  unsigned long long* d_bad = nullptr;
  auto release = [&]() {
    te_free(d_row);
    te_free(d_col);
    te_free(d_cnt);
    te_free(d_flags);
    te_free(d_bad);
  };
  auto fail = [&](int rc) {
    release();
    te_free(d_v);
    te_free(d_rp);
    te_free(d_ci);
    return rc;
  };
  int dev = 0, pageable = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) pageable = 0;
  const char* copy_env = std::getenv("TE_COO_COPY");  // 1: the staging-copy path everywhere
  if (copy_env && copy_env[0] == '1') pageable = 0;
  if (te_cuda_check(te_malloc(&d_v, sizeof(double2) * nnz), "coo") != TE_OK ||
      te_cuda_check(te_malloc(&d_rp, sizeof(int32_t) * (n_rows + 1)), "coo") != TE_OK ||
      te_cuda_check(te_malloc(&d_ci, sizeof(int32_t) * nnz), "coo") != TE_OK ||
      te_cuda_check(te_malloc(&d_flags, sizeof(unsigned int)), "coo") != TE_OK ||
      te_cuda_check(te_malloc(&d_bad, sizeof(unsigned long long)), "coo") != TE_OK)
    return fail(TE_ERR_CUDA);
  const unsigned long long none = ~0ull;
  if (te_cuda_check(cudaMemset(d_flags, 0, sizeof(unsigned int)), "coo") != TE_OK ||
      te_cuda_check(cudaMemcpy(d_bad, &none, sizeof(none), cudaMemcpyHostToDevice), "coo") != TE_OK)
    return fail(TE_ERR_CUDA);
  if (pageable == 1) {
    // the kernel reads the host arrays itself: one pass, no staging copies
    const void* ptrs[3] = {row_index, columns, values};
    const size_t bytes[3] = {sizeof(uint64_t) * nnz, sizeof(uint64_t) * nnz, sizeof(double2) * nnz};
    touch_host_pages(ptrs, bytes, 3);
    coo_ingest_kernel<<<te_grid_fit((const void*)coo_ingest_kernel, nnz, TE_THREADS), TE_THREADS>>>(
        nnz, (uint64_t)n_rows, (uint64_t)n_cols, row_index, columns, values, d_rp, d_ci, d_v, d_flags, d_bad);
  } else {
    if (te_cuda_check(te_malloc(&d_row, sizeof(uint64_t) * nnz), "coo") != TE_OK ||
        te_cuda_check(te_malloc(&d_col, sizeof(uint64_t) * nnz), "coo") != TE_OK)
      return fail(TE_ERR_CUDA);
    if (te_cuda_check(cudaMemcpy(d_row, row_index, sizeof(uint64_t) * nnz, cudaMemcpyHostToDevice), "coo") != TE_OK ||
        te_cuda_check(cudaMemcpy(d_col, columns, sizeof(uint64_t) * nnz, cudaMemcpyHostToDevice), "coo") != TE_OK ||
        te_cuda_check(cudaMemcpy(d_v, values, sizeof(double2) * nnz, cudaMemcpyHostToDevice), "coo") != TE_OK)
      return fail(TE_ERR_CUDA);
    coo_scan_kernel<<<te_grid_fit((const void*)coo_scan_kernel, nnz, TE_THREADS), TE_THREADS>>>(
        nnz, (uint64_t)n_rows, (uint64_t)n_cols, d_row, d_col, d_flags, d_bad);
  }
  unsigned int flags = 0;
  unsigned long long bad = 0;
  if (te_cuda_check(cudaMemcpy(&flags, d_flags, sizeof(flags), cudaMemcpyDeviceToHost), "coo") != TE_OK ||
      te_cuda_check(cudaMemcpy(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost), "coo") != TE_OK)
    return fail(TE_ERR_CUDA);
  host_done();  // the device is done with the host arrays
  if (flags & TE_COO_BAD) {
    te_set_error("te_matrix_create_coo: entry %lld out of range", (long long)bad);
    return fail(TE_ERR_INVALID_ARG);
  }
  if (flags & TE_COO_UNSORTED) return fail(TE_ERR_UNSUPPORTED);
  if (pageable != 1) {
    // row pointers from the per-row counts (rows are sorted, so CSR order = input order)
    const int32_t nnz32 = (int32_t)nnz;
    if (te_cuda_check(te_malloc(&d_cnt, sizeof(int32_t) * n_rows), "coo") != TE_OK ||
        te_cuda_check(cudaMemset(d_cnt, 0, sizeof(int32_t) * n_rows), "coo") != TE_OK)
      return fail(TE_ERR_CUDA);
    row_count_kernel<<<te_grid_fit((const void*)row_count_kernel, nnz, TE_THREADS), TE_THREADS>>>(nnz, d_row, d_cnt);
    if (scan_exclusive<int32_t>(d_cnt, d_rp, n_rows) != TE_OK ||
        te_cuda_check(cudaMemcpy(d_rp + n_rows, &nnz32, sizeof(int32_t), cudaMemcpyHostToDevice), "coo") != TE_OK)
      return fail(TE_ERR_CUDA);
    narrow_index_kernel<<<te_grid_fit((const void*)narrow_index_kernel, nnz, TE_THREADS), TE_THREADS>>>(nnz, d_col,
                                                                                                     d_ci);
  }
  if (n_rows == n_cols) {  // the reference's 1-norm on the device where |H| is symmetric and real
    if (te_cuda_check(cudaMemset(d_flags, 0, sizeof(unsigned int)), "coo") != TE_OK ||
        te_cuda_check(cudaMemset(d_bad, 0, sizeof(unsigned long long)), "coo") != TE_OK)
      return fail(TE_ERR_CUDA);
    mirror_norm1_kernel<<<te_grid_fit((const void*)mirror_norm1_kernel, n_rows, TE_THREADS), TE_THREADS>>>(
        n_rows, d_rp, d_ci, d_v, d_flags, d_bad);
    unsigned int mflags = 0;
    unsigned long long mbits = 0;
    if (te_cuda_check(cudaMemcpy(&mflags, d_flags, sizeof(mflags), cudaMemcpyDeviceToHost), "coo") != TE_OK ||
        te_cuda_check(cudaMemcpy(&mbits, d_bad, sizeof(mbits), cudaMemcpyDeviceToHost), "coo") != TE_OK)
      return fail(TE_ERR_CUDA);
    if (mflags == 0) std::memcpy(norm1_gpu, &mbits, sizeof(double));
  }
  if (te_cuda_check(cudaDeviceSynchronize(), "coo") != TE_OK) return fail(TE_ERR_CUDA);
  release();
  return te_matrix_adopt_device_csr(n_rows, n_cols, nnz, d_rp, d_ci, d_v, out, 0.0);
}

// Below this many entries the host conversion is as fast as the device one.
const int64_t kDeviceCooMinEntries = (int64_t)1 << 18;

}  // namespace

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
  if (nnz < kDeviceCooMinEntries)
    return create_coo_host(n_rows, n_cols, nnz, row_index, columns, values, coo_norm1(n_cols, nnz, columns, values),
                           out);
  // the 1-norm on host threads while the device builds the layout, started
  // once the device has read the host arrays (the two would share host
  // memory bandwidth); the device computes it itself where |H| is real and
  // symmetric (then the host threads are called off)
  double norm1 = 0.0, norm1_gpu = std::nan("");
  std::atomic<bool> cancel(false);
  std::thread norm_thread;
  auto start_norm = [&]() {
    norm_thread = std::thread([&]() { norm1 = coo_norm1(n_cols, nnz, columns, values, &cancel); });
  };
  int rc = create_coo_device(n_rows, n_cols, nnz, row_index, columns, values, &norm1_gpu, out, start_norm);
  if (rc == TE_OK && !std::isnan(norm1_gpu)) cancel.store(true);
  if (norm_thread.joinable()) {
    norm_thread.join();
  } else if (rc == TE_ERR_UNSUPPORTED) {
    norm1 = coo_norm1(n_cols, nnz, columns, values);
  }
  if (rc == TE_OK) {
    (*out)->norm1 = std::isnan(norm1_gpu) ? norm1 : norm1_gpu;
    return TE_OK;
  }
  if (rc != TE_ERR_UNSUPPORTED) return rc;
  return create_coo_host(n_rows, n_cols, nnz, row_index, columns, values, norm1, out);
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

extern "C" int te_matrix_create_csr_device(int64_t n_rows, int64_t n_cols, int64_t nnz, const int32_t* row_ptr_dev,
                                           const int32_t* col_dev, const double* values_dev, int values_complex,
                                           te_matrix* out) {
  if (!out || n_rows <= 0 || n_cols <= 0 || nnz < 0 || !row_ptr_dev || (nnz > 0 && (!col_dev || !values_dev))) {
    te_set_error("te_matrix_create_csr_device: invalid arguments");
    return n_rows == 0 || n_cols == 0 ? TE_ERR_EMPTY : TE_ERR_INVALID_ARG;
  }
  if (nnz >= ((int64_t)1 << 31) || n_rows >= ((int64_t)1 << 31) || n_cols >= ((int64_t)1 << 31)) {
    te_set_error("te_matrix_create_csr_device: sizes must stay below 2^31 (int32 indices)");
    return TE_ERR_UNSUPPORTED;
  }
  std::vector<int32_t> rp(n_rows + 1);
  TE_CUDA(cudaMemcpy(rp.data(), row_ptr_dev, sizeof(int32_t) * (n_rows + 1), cudaMemcpyDeviceToHost));
  if (rp[0] != 0 || rp[n_rows] != nnz) {
    te_set_error("te_matrix_create_csr_device: row_ptr must start at 0 and end at nnz");
    return TE_ERR_INVALID_ARG;
  }
  for (int64_t r = 0; r < n_rows; ++r)
    if (rp[r + 1] < rp[r]) {
      te_set_error("te_matrix_create_csr_device: row_ptr decreases at row %lld", (long long)(r + 1));
      return TE_ERR_INVALID_ARG;
    }
  // private copies (the matrix owns its arrays)
  int32_t *d_rp = nullptr, *d_ci = nullptr;
  double2* d_v = nullptr;
  auto fail = [&](int rc) {
    te_free(d_rp);
    te_free(d_ci);
    te_free(d_v);
    return rc;
  };
  if (te_cuda_check(te_malloc(&d_rp, sizeof(int32_t) * (n_rows + 1)), "csr") != TE_OK ||
      te_cuda_check(te_malloc(&d_ci, sizeof(int32_t) * std::max<int64_t>(nnz, 1)), "csr") != TE_OK ||
      te_cuda_check(te_malloc(&d_v, sizeof(double2) * std::max<int64_t>(nnz, 1)), "csr") != TE_OK)
    return fail(TE_ERR_CUDA);
  if (te_cuda_check(cudaMemcpy(d_rp, row_ptr_dev, sizeof(int32_t) * (n_rows + 1), cudaMemcpyDeviceToDevice), "csr") !=
      TE_OK)
    return fail(TE_ERR_CUDA);
  if (nnz > 0) {
    if (te_cuda_check(cudaMemcpy(d_ci, col_dev, sizeof(int32_t) * nnz, cudaMemcpyDeviceToDevice), "csr") != TE_OK)
      return fail(TE_ERR_CUDA);
    if (values_complex) {
      if (te_cuda_check(cudaMemcpy(d_v, values_dev, sizeof(double2) * nnz, cudaMemcpyDeviceToDevice), "csr") != TE_OK)
        return fail(TE_ERR_CUDA);
    } else {
      widen_real_kernel<<<te_grid_fit((const void*)widen_real_kernel, nnz, TE_THREADS), TE_THREADS>>>(nnz, values_dev,
                                                                                                    d_v);
    }
  }
  return te_matrix_adopt_device_csr(n_rows, n_cols, nnz, d_rp, d_ci, d_v, out, NAN);
}

extern "C" int te_matrix_download_csr(te_matrix A, int32_t* row_ptr, int32_t* col_idx, double* values) {
  if (!A || !row_ptr || (A->nnz > 0 && (!col_idx || !values))) {
    te_set_error("te_matrix_download_csr: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  const int64_t nnz = A->nnz;
  TE_CUDA(cudaMemcpy(row_ptr, A->row_ptr, sizeof(int32_t) * (A->n_rows + 1), cudaMemcpyDeviceToHost));
  if (nnz == 0) return TE_OK;
  TE_CUDA(cudaMemcpy(col_idx, A->col, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost));
  if (A->is_real) {
    std::vector<double> re(nnz);
    TE_CUDA(cudaMemcpy(re.data(), A->val, sizeof(double) * nnz, cudaMemcpyDeviceToHost));
    for (int64_t p = 0; p < nnz; ++p) {
      values[2 * p] = re[p];
      values[2 * p + 1] = 0.0;
    }
  } else {
    TE_CUDA(cudaMemcpy(values, A->val, sizeof(double2) * nnz, cudaMemcpyDeviceToHost));
  }
  return TE_OK;
}

extern "C" int te_matrix_long_segments(te_matrix A, int64_t* segments, int64_t* split_rows, int64_t* segment_items) {
  if (!A || A->n_rows != A->n_cols) {
    te_set_error("te_matrix_long_segments: square matrix required");
    return TE_ERR_INVALID_ARG;
  }
  if (segments) *segments = A->sell.n_seg;
  if (split_rows) *split_rows = A->sell.n_split;
  if (segment_items) *segment_items = A->sell.seg_items;
  return TE_OK;
}

extern "C" int te_matrix_layout(te_matrix A, int64_t* sell_slots, int64_t* long_rows, int64_t* long_entries) {
  if (!A || A->n_rows != A->n_cols) {
    te_set_error("te_matrix_layout: square matrix required");
    return TE_ERR_INVALID_ARG;
  }
  if (sell_slots) *sell_slots = A->sell.slots;
  if (long_rows) *long_rows = A->sell.n_long;
  if (long_entries) {
    int64_t e = 0;
    if (A->sell.n_long > 0)
      TE_CUDA(cudaMemcpy(&e, A->sell.long_ptr + A->sell.n_long, sizeof(int64_t), cudaMemcpyDeviceToHost));
    *long_entries = e;
  }
  return TE_OK;
}

extern "C" int te_matrix_fixed_layout(te_matrix A, int* state, int* n_values, int* scale_shift) {
  if (!A) return TE_ERR_INVALID_ARG;
  const TeSell& S = A->sell;
  if (state) *state = !S.fix_warp_chunk ? 0 : (S.fix_pk ? 2 : (S.fix_nblk > 0 ? 3 : 1));
  if (n_values) *n_values = S.fix_nblk > 0 ? S.fix_nblk : S.fix_nvals;
  if (scale_shift) *scale_shift = S.fix_sh;
  return TE_OK;
}

extern "C" int te_matrix_set_spmv_lanes(te_matrix A, int lanes) {
  if (!A || A->n_rows != A->n_cols || !(lanes == -1 || lanes == 0 || lanes == 1 || lanes == 2 || lanes == 4)) {
    te_set_error("te_matrix_set_spmv_lanes: square matrix and lanes -1 (timed), 0 (by shape), 1, 2 or 4 required");
    return TE_ERR_INVALID_ARG;
  }
  if (lanes > 1 && A->sell.n_long > 0) {
    te_set_error("te_matrix_set_spmv_lanes: a matrix with long rows uses one lane per row");
    return TE_ERR_UNSUPPORTED;
  }
  A->sell.lanes = lanes <= 0 ? 1 : lanes;
  A->sell.lanes_fixed = lanes > 0;
  A->sell.lanes_timed = lanes == -1;
  return TE_OK;
}

extern "C" int te_matrix_spmv_lanes(te_matrix A, int tune_now) {
  if (!A || A->n_rows != A->n_cols) {
    te_set_error("te_matrix_spmv_lanes: square matrix required");
    return TE_ERR_INVALID_ARG;
  }
  if (tune_now) {
    int rc = te_tune_sell_lanes(A);
    if (rc != TE_OK) return rc;
  }
  return A->sell.lanes;
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
  TeSegCarry carry;  // this call's carries of the split long rows (calls may overlap)
  TE_CUDA(cudaMallocAsync(&xp, sizeof(double2) * n, st));
  int rc = te_cuda_check(cudaMallocAsync(&yp, sizeof(double2) * n, st), "cudaMallocAsync");
  if (rc == TE_OK && A->sell.n_split > 0) {
    rc = te_cuda_check(cudaMallocAsync(&carry.part, sizeof(double2) * A->sell.n_seg, st), "cudaMallocAsync");
    if (rc == TE_OK)
      rc = te_cuda_check(cudaMallocAsync(&carry.cnt, sizeof(unsigned int) * A->sell.n_long, st), "cudaMallocAsync");
    if (rc == TE_OK)
      rc = te_cuda_check(cudaMemsetAsync(carry.cnt, 0, sizeof(unsigned int) * A->sell.n_long, st), "memset");
  }
  if (rc == TE_OK) {
    te_launch_permute(n, A->sell.perm, reinterpret_cast<const double2*>(in_dev), xp, st);
    te_launch_sell_spmv(A->sell, A->is_real, make_double2(alpha_re, alpha_im), xp, yp, st,
                        A->sell.n_split > 0 ? &carry : nullptr);
    te_launch_permute(n, A->sell.iperm, yp, reinterpret_cast<double2*>(out_dev), st);
    rc = te_cuda_check(cudaGetLastError(), "spmv launch");
  }
  cudaFreeAsync(xp, st);
  cudaFreeAsync(yp, st);
  if (carry.part) cudaFreeAsync(carry.part, st);
  if (carry.cnt) cudaFreeAsync(carry.cnt, st);
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
  TE_CUDA(te_malloc(&x, sizeof(double2) * n));
  int rc = te_cuda_check(te_malloc(&y, sizeof(double2) * n), "cudaMalloc");
  if (rc == TE_OK) rc = te_cuda_check(cudaMemcpy(x, in_host, sizeof(double2) * n, cudaMemcpyHostToDevice), "H2D");
  if (rc == TE_OK) rc = te_matrix_spmv(A, alpha_re, alpha_im, (const double*)x, (double*)y, nullptr);
  if (rc == TE_OK) rc = te_cuda_check(cudaDeviceSynchronize(), "spmv");
  if (rc == TE_OK) rc = te_cuda_check(cudaMemcpy(out_host, y, sizeof(double2) * n, cudaMemcpyDeviceToHost), "D2H");
  te_free(x);
  te_free(y);
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
