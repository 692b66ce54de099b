// te_model.cu -- number-conserving boson basis and operator matrices built on
// the GPU, in the reference's basis order and with its assembly rules
// (helper/Basis.cpp:37-121, helper/hamiltonian.cpp:318-402).
//
// Basis order.  The reference enumerates the occupations of modes K-1, ..., 1
// in stages: starting from the empty state, the stage of mode m appends, after
// the current list, every element of the list with mode m set to quant,
// 2 quant, ... up to the particles left (mode 0 takes the rest at the end).
// Stage s (mode m = K-1-s) therefore maps list L_s (n_s states) to
//   L_{s+1} = L_s ++ [children of L_s[0]] ++ [children of L_s[1]] ++ ...,
// and a state's index is built stage by stage:
//   r <- r                                   if e[m] = 0,
//   r <- n_s + PS_s[r] + e[m] / quant - 1     otherwise,
// with PS_s the prefix sums of the children counts over L_s.  The device keeps
// every PS_s (their total length is about the dimension), so the index of any
// occupation vector costs K - 1 lookups: no hash table.
//
// Matrix assembly (createMatrix): for every basis row j, every term in order
// is applied to state j; a term that survives gives (column = index of the
// result, value = coef * sqrt factors); equal columns merge in term order; the
// row is sorted by column (stable); values with |v| < DBL_EPSILON are dropped.
// One thread per row, two passes (count, then write).
//
// 1-norm: the reference sums |a| per column in entry order (rows ascending).
// For a Hermitian operator the entries of column c in row order have exactly
// the moduli of row c in column order, so the row sums in column order give
// the same value bit for bit; the builder uses them (for a non-Hermitian
// operator list this is the infinity norm instead).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "te_internal.cuh"

namespace {

#define TE_MODEL_MAX_MODES 64
#define TE_MODEL_MAX_OPS 8
#define TE_MODEL_MAX_TERMS 64  // per-thread row buffers (a row has at most one entry per term)

struct DevTerm {
  double2 coef;
  int n_ops;
  int operation[TE_MODEL_MAX_OPS];
  int mode[TE_MODEL_MAX_OPS];
  int capacity[TE_MODEL_MAX_OPS];
};

struct Stages {
  int K, N, quant;
  const int64_t* n_s;  // K entries: list sizes before each stage (n_s[0] = 1)
  const int64_t* const* ps;  // K - 1 prefix arrays (device pointers)
};

// children counts of list L_s (stage of mode m)
__global__ void stage_count_kernel(int64_t n, const uint8_t* __restrict__ occ, int K, int N, int quant,
                                   int64_t* __restrict__ cnt) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    int tot = 0;
    for (int a = 1; a < K; ++a) tot += occ[l * K + a];
    cnt[l] = (N - tot) / quant;
  }
}

// L_{s+1}: children of element l at n_s + PS[l] + t (mode m = quant (t + 1))
__global__ void stage_expand_kernel(int64_t n, uint8_t* occ, int K, int m, int quant, const int64_t* __restrict__ ps) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cnt = ps[l + 1] - ps[l];
    for (int64_t t = 0; t < cnt; ++t) {
      uint8_t* dst = occ + (n + ps[l] + t) * K;
      for (int a = 0; a < K; ++a) dst[a] = occ[l * K + a];
      dst[m] = (uint8_t)(quant * (t + 1));
    }
  }
}

__global__ void finish_basis_kernel(int64_t n, uint8_t* occ, int K, int N) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    int tot = 0;
    for (int a = 1; a < K; ++a) tot += occ[l * K + a];
    occ[l * K] = (uint8_t)(N - tot);
  }
}

// Index of an occupation vector in the basis, or -1 if it is not a basis state.
__device__ int64_t state_index(const Stages& st, const int* e) {
  int tot = 0;
  for (int a = 0; a < st.K; ++a) {
    if (e[a] < 0) return -1;
    tot += e[a];
  }
  if (tot != st.N) return -1;
  int64_t r = 0;
  for (int s = 0; s < st.K - 1; ++s) {
    const int m = st.K - 1 - s;
    const int o = e[m];
    if (o == 0) continue;
    if (o % st.quant) return -1;
    r = st.n_s[s] + st.ps[s][r] + o / st.quant - 1;
  }
  return r;
}

// Apply one term to the occupations (apply_term of hamiltonian.cpp): false if
// it annihilates the state.
__device__ bool apply_term_dev(const DevTerm& t, int* occ, int K, double2& coef) {
  for (int i = 0; i < t.n_ops; ++i) {
    const int md = t.mode[i];
    const int n = occ[md];
    if (t.operation[i] == 1) {
      const int c = t.capacity[i];
      if (c != 0 && n + 1 > c) return false;
      const double f = sqrt(n + 1.0);
      coef = make_double2(coef.x * f, coef.y * f);
      occ[md] = n + 1;
    } else if (t.operation[i] == -1) {
      if (n == 0) return false;
      const double f = sqrt((double)n);
      coef = make_double2(coef.x * f, coef.y * f);
      occ[md] = n - 1;
    }
  }
  return true;
}

// One row: the merged, column-sorted, filtered entries (count returned; with
// out_col != null they are also written).
__device__ int build_row(const Stages& st, const uint8_t* __restrict__ occ, int64_t j, const DevTerm* __restrict__ terms,
                         int n_terms, int32_t* cols, double2* vals, int32_t* out_col, double2* out_val,
                         double* abs_sum) {
  int e[TE_MODEL_MAX_MODES];
  int cnt = 0;
  for (int ti = 0; ti < n_terms; ++ti) {
    const DevTerm& t = terms[ti];
    for (int a = 0; a < st.K; ++a) e[a] = occ[j * st.K + a];
    double2 c = make_double2(1.0, 0.0);
    if (!apply_term_dev(t, e, st.K, c)) continue;
    // coef = coef * t.coef: the complex product rounded term by term, without
    // contraction into FMAs (as the host build)
    c = make_double2(__dsub_rn(__dmul_rn(c.x, t.coef.x), __dmul_rn(c.y, t.coef.y)),
                     __dadd_rn(__dmul_rn(c.x, t.coef.y), __dmul_rn(c.y, t.coef.x)));
    const int64_t col = state_index(st, e);
    if (col < 0) continue;
    int k = 0;
    while (k < cnt && cols[k] != (int32_t)col) ++k;
    if (k < cnt) {
      vals[k] = make_double2(__dadd_rn(vals[k].x, c.x), __dadd_rn(vals[k].y, c.y));
    } else {
      cols[cnt] = (int32_t)col;
      vals[cnt] = c;
      ++cnt;
    }
  }
  // stable insertion sort by column
  for (int a = 1; a < cnt; ++a) {
    const int32_t kc = cols[a];
    const double2 kv = vals[a];
    int b = a - 1;
    while (b >= 0 && cols[b] > kc) {
      cols[b + 1] = cols[b];
      vals[b + 1] = vals[b];
      --b;
    }
    cols[b + 1] = kc;
    vals[b + 1] = kv;
  }
  int kept = 0;
  double s = 0.0;
  for (int a = 0; a < cnt; ++a) {
    const double mag = hypot(vals[a].x, vals[a].y);
    if (mag < DBL_EPSILON) continue;
    if (out_col) {
      out_col[kept] = cols[a];
      out_val[kept] = vals[a];
    }
    s = __dadd_rn(s, mag);
    ++kept;
  }
  if (abs_sum) *abs_sum = s;
  return kept;
}

// counts (n) -> int64 (n + 1, last 0), for the row-pointer scan
__global__ void widen_counts_kernel(int64_t n, const int32_t* __restrict__ cnt, int64_t* __restrict__ out) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j <= n; j += (int64_t)gridDim.x * blockDim.x)
    out[j] = j < n ? cnt[j] : 0;
}

__global__ void narrow_rp_kernel(int64_t count, const int64_t* __restrict__ in, int32_t* __restrict__ out) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < count; j += (int64_t)gridDim.x * blockDim.x)
    out[j] = (int32_t)in[j];
}

__global__ void row_count_model_kernel(Stages st, const uint8_t* __restrict__ occ, int64_t n,
                                       const DevTerm* __restrict__ terms, int n_terms, int32_t* __restrict__ count) {
  int32_t cols[TE_MODEL_MAX_TERMS];
  double2 vals[TE_MODEL_MAX_TERMS];
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
    count[j] = build_row(st, occ, j, terms, n_terms, cols, vals, nullptr, nullptr, nullptr);
}

__global__ void row_write_model_kernel(Stages st, const uint8_t* __restrict__ occ, int64_t n,
                                       const DevTerm* __restrict__ terms, int n_terms, const int32_t* __restrict__ rp,
                                       int32_t* __restrict__ col, double2* __restrict__ val,
                                       unsigned long long* norm_bits) {
  int32_t cols[TE_MODEL_MAX_TERMS];
  double2 vals[TE_MODEL_MAX_TERMS];
  double mx = 0.0;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    build_row(st, occ, j, terms, n_terms, cols, vals, col + rp[j], val + rp[j], &s);
    mx = fmax(mx, s);
  }
  atomicMax(norm_bits, (unsigned long long)__double_as_longlong(mx));
}

// Exclusive prefix sum of n counts (host round trip: the lists are built once).
int exclusive_scan(const int64_t* d_in, int64_t n, int64_t* d_out, int64_t* total) {
  std::vector<int64_t> h(n), p(n + 1, 0);
  TE_CUDA(cudaMemcpy(h.data(), d_in, sizeof(int64_t) * n, cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < n; ++i) p[i + 1] = p[i] + h[i];
  TE_CUDA(cudaMemcpy(d_out, p.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
  *total = p[n];
  return TE_OK;
}

struct DeviceBasis {
  int K = 0, N = 0, quant = 1;
  int64_t dim = 0;
  uint8_t* occ = nullptr;
  std::vector<int64_t> n_s;
  std::vector<int64_t*> ps;
  int64_t* d_n_s = nullptr;
  int64_t** d_ps = nullptr;
  ~DeviceBasis() {
    cudaFree(occ);
    for (int64_t* p : ps) cudaFree(p);
    cudaFree(d_n_s);
    cudaFree(d_ps);
  }
  Stages stages() const { return Stages{K, N, quant, d_n_s, d_ps}; }
};

int build_basis(int N, int K, int quant, DeviceBasis& B) {
  B.K = K;
  B.N = N;
  B.quant = quant;
  // final size: number of states of modes 1..K-1 with multiples of quant summing to <= N
  // = compositions; computed by running the stage counts on the host in closed form
  // (the list sizes grow stage by stage, so the device list is reallocated once at its final size)
  std::vector<double> ways(N / quant + 1, 0.0);  // ways[q]: states using q quanta over the modes so far
  ways[0] = 1.0;
  for (int s = 0; s < K - 1; ++s) {
    std::vector<double> nw(ways.size(), 0.0);
    for (size_t q = 0; q < ways.size(); ++q)
      for (size_t r = q; r < ways.size(); ++r) nw[r] += ways[q];
    ways.swap(nw);
  }
  double total = 0.0;
  for (double w : ways) total += w;
  if (!(total < 2147483647.0)) {
    te_set_error("te_model: basis dimension %.0f exceeds the int32 index range", total);
    return TE_ERR_UNSUPPORTED;
  }
  const int64_t dim = (int64_t)total;
  TE_CUDA(cudaMalloc(&B.occ, (size_t)dim * K));
  TE_CUDA(cudaMemset(B.occ, 0, (size_t)dim * K));
  int64_t n = 1;
  int64_t* cnt = nullptr;
  TE_CUDA(cudaMalloc(&cnt, sizeof(int64_t) * std::max<int64_t>(dim, 1)));
  int rc = TE_OK;
  for (int s = 0; s < K - 1 && rc == TE_OK; ++s) {
    const int m = K - 1 - s;
    B.n_s.push_back(n);
    int64_t* ps = nullptr;
    if ((rc = te_cuda_check(cudaMalloc(&ps, sizeof(int64_t) * (n + 1)), "basis")) != TE_OK) break;
    B.ps.push_back(ps);
    const int g = te_grid_for(n, 256, 4);
    stage_count_kernel<<<g, 256>>>(n, B.occ, K, N, quant, cnt);
    int64_t added = 0;
    if ((rc = exclusive_scan(cnt, n, ps, &added)) != TE_OK) break;
    if (n + added > dim) {
      te_set_error("te_model: basis enumeration inconsistent");
      rc = TE_ERR_INVALID_ARG;
      break;
    }
    stage_expand_kernel<<<g, 256>>>(n, B.occ, K, m, quant, ps);
    n += added;
  }
  cudaFree(cnt);
  if (rc != TE_OK) return rc;
  B.n_s.push_back(n);
  B.dim = n;
  finish_basis_kernel<<<te_grid_for(n, 256, 4), 256>>>(n, B.occ, K, N);
  TE_CUDA(cudaMalloc(&B.d_n_s, sizeof(int64_t) * B.n_s.size()));
  TE_CUDA(cudaMemcpy(B.d_n_s, B.n_s.data(), sizeof(int64_t) * B.n_s.size(), cudaMemcpyHostToDevice));
  TE_CUDA(cudaMalloc(&B.d_ps, sizeof(int64_t*) * std::max<size_t>(B.ps.size(), 1)));
  if (!B.ps.empty())
    TE_CUDA(cudaMemcpy(B.d_ps, B.ps.data(), sizeof(int64_t*) * B.ps.size(), cudaMemcpyHostToDevice));
  return te_cuda_check(cudaDeviceSynchronize(), "basis");
}

}  // namespace

extern "C" int te_model_create_device(int n_particles, int n_modes, int quant, const te_term* terms, int n_terms,
                                      te_matrix* out, int64_t* dim_out) {
  if (!out || !terms || n_terms < 1 || n_terms > TE_MODEL_MAX_TERMS || n_modes < 1 ||
      n_modes > TE_MODEL_MAX_MODES || n_particles < 0 || n_particles > 255 || quant < 1) {
    te_set_error("te_model_create_device: invalid arguments (1..%d modes, 0..255 particles, 1..%d terms, quant >= 1)",
                 TE_MODEL_MAX_MODES, TE_MODEL_MAX_TERMS);
    return TE_ERR_INVALID_ARG;
  }
  std::vector<DevTerm> dt(n_terms);
  for (int i = 0; i < n_terms; ++i) {
    const te_term& t = terms[i];
    if (t.n_ops < 0 || t.n_ops > TE_MODEL_MAX_OPS) {
      te_set_error("te_model_create_device: term %d has more than %d operations", i, TE_MODEL_MAX_OPS);
      return TE_ERR_INVALID_ARG;
    }
    DevTerm& d = dt[i];
    std::memset(&d, 0, sizeof(d));
    d.coef = make_double2(t.coef_re, t.coef_im);
    d.n_ops = t.n_ops;
    for (int k = 0; k < t.n_ops; ++k) {
      if (t.mode[k] < 0 || t.mode[k] >= n_modes) {
        te_set_error("creationOperator: mode does not exist in vector");
        return TE_ERR_INVALID_ARG;
      }
      d.operation[k] = t.operation[k];
      d.mode[k] = t.mode[k];
      d.capacity[k] = t.capacity[k];
    }
  }
  DeviceBasis B;
  int rc = build_basis(n_particles, n_modes, quant, B);
  if (rc != TE_OK) return rc;
  const int64_t n = B.dim;
  DevTerm* d_terms = nullptr;
  int32_t *d_cnt = nullptr, *d_rp = nullptr, *d_col = nullptr;
  double2* d_val = nullptr;
  unsigned long long* d_norm = nullptr;
  auto fail = [&](int code) {
    cudaFree(d_terms);
    cudaFree(d_cnt);
    cudaFree(d_rp);
    cudaFree(d_col);
    cudaFree(d_val);
    cudaFree(d_norm);
    return code;
  };
  if (te_cuda_check(cudaMalloc(&d_terms, sizeof(DevTerm) * n_terms), "model") != TE_OK ||
      te_cuda_check(cudaMalloc(&d_cnt, sizeof(int32_t) * n), "model") != TE_OK ||
      te_cuda_check(cudaMalloc(&d_norm, sizeof(unsigned long long)), "model") != TE_OK)
    return fail(TE_ERR_CUDA);
  cudaMemcpy(d_terms, dt.data(), sizeof(DevTerm) * n_terms, cudaMemcpyHostToDevice);
  cudaMemset(d_norm, 0, sizeof(unsigned long long));
  const Stages st = B.stages();
  const int g = te_grid_fit((const void*)row_count_model_kernel, n, 128);
  row_count_model_kernel<<<g, 128>>>(st, B.occ, n, d_terms, n_terms, d_cnt);
  // row pointers: a 64-bit scan of the counts on the device (the total must
  // stay below 2^31), narrowed to int32
  int64_t* d_rp64 = nullptr;
  int64_t nnz = 0;
  if (te_cuda_check(cudaMalloc(&d_rp64, sizeof(int64_t) * (n + 1)), "model") != TE_OK) return fail(TE_ERR_CUDA);
  widen_counts_kernel<<<te_grid_fit((const void*)widen_counts_kernel, n + 1, TE_THREADS), TE_THREADS>>>(n, d_cnt,
                                                                                                      d_rp64);
  rc = te_scan_exclusive_i64(d_rp64, d_rp64, n + 1);
  if (rc == TE_OK)
    rc = te_cuda_check(cudaMemcpy(&nnz, d_rp64 + n, sizeof(int64_t), cudaMemcpyDeviceToHost), "model");
  if (rc == TE_OK && nnz >= ((int64_t)1 << 31)) {
    te_set_error("te_model_create_device: more than 2^31 entries");
    rc = TE_ERR_UNSUPPORTED;
  }
  if (rc == TE_OK)
    rc = te_cuda_check(cudaMalloc(&d_rp, sizeof(int32_t) * (n + 1)), "model");
  if (rc == TE_OK)
    narrow_rp_kernel<<<te_grid_fit((const void*)narrow_rp_kernel, n + 1, TE_THREADS), TE_THREADS>>>(n + 1, d_rp64,
                                                                                                   d_rp);
  cudaFree(d_rp64);
  if (rc != TE_OK) return fail(rc);
  if (te_cuda_check(cudaMalloc(&d_col, sizeof(int32_t) * std::max<int64_t>(nnz, 1)), "model") != TE_OK ||
      te_cuda_check(cudaMalloc(&d_val, sizeof(double2) * std::max<int64_t>(nnz, 1)), "model") != TE_OK)
    return fail(TE_ERR_CUDA);
  row_write_model_kernel<<<te_grid_fit((const void*)row_write_model_kernel, n, 128), 128>>>(
      st, B.occ, n, d_terms, n_terms, d_rp, d_col, d_val, d_norm);
  unsigned long long bits = 0;
  if (te_cuda_check(cudaMemcpy(&bits, d_norm, sizeof(bits), cudaMemcpyDeviceToHost), "model") != TE_OK)
    return fail(TE_ERR_CUDA);
  double norm1;
  std::memcpy(&norm1, &bits, sizeof(norm1));
  cudaFree(d_terms);
  cudaFree(d_cnt);
  cudaFree(d_norm);
  d_terms = nullptr;
  d_cnt = nullptr;
  d_norm = nullptr;
  rc = te_matrix_adopt_device_csr(n, n, nnz, d_rp, d_col, d_val, out, norm1);
  if (rc != TE_OK) return rc;  // the matrix freed the arrays
  if (dim_out) *dim_out = n;
  return TE_OK;
}

namespace {

__global__ void state_index_kernel(Stages st, const int* e, int64_t* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *out = state_index(st, e);
}

}  // namespace

extern "C" int te_model_state_index(int n_particles, int n_modes, int quant, const int32_t* occupation,
                                    int64_t* index) {
  if (!occupation || !index || n_modes < 1 || n_modes > TE_MODEL_MAX_MODES || quant < 1 || n_particles < 0 ||
      n_particles > 255) {
    te_set_error("te_model_state_index: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  DeviceBasis B;
  int rc = build_basis(n_particles, n_modes, quant, B);
  if (rc != TE_OK) return rc;
  int* d_e = nullptr;
  int64_t* d_r = nullptr;
  if (te_cuda_check(cudaMalloc(&d_e, sizeof(int) * n_modes), "index") != TE_OK ||
      te_cuda_check(cudaMalloc(&d_r, sizeof(int64_t)), "index") != TE_OK) {
    cudaFree(d_e);
    cudaFree(d_r);
    return TE_ERR_CUDA;
  }
  cudaMemcpy(d_e, occupation, sizeof(int) * n_modes, cudaMemcpyHostToDevice);
  state_index_kernel<<<1, 32>>>(B.stages(), d_e, d_r);
  rc = te_cuda_check(cudaMemcpy(index, d_r, sizeof(int64_t), cudaMemcpyDeviceToHost), "index");
  cudaFree(d_e);
  cudaFree(d_r);
  return rc;
}
