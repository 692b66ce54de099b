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
#define TE_MODEL_MAX_TERMS 128  // per-thread row buffers (a row has at most one entry per term)

struct DevTerm {
  double2 coef;
  int n_ops;
  int operation[TE_MODEL_MAX_OPS];
  int mode[TE_MODEL_MAX_OPS];
  int capacity[TE_MODEL_MAX_OPS];
};

// One basis on the device: the stage lists' sizes and prefix sums, the
// capacity of the qudit modes, and (when every mode is a qudit) the map from
// the staged list to the final list, from which the states whose mode 0
// would exceed the capacity are dropped (Basis.cpp:97-110).
struct Stages {
  int K, N, quant;
  int nq, cap;               // modes K - nq .. K - 1 hold at most cap particles
  const int64_t* n_s;        // K entries: list sizes before each stage (n_s[0] = 1)
  const int64_t* const* ps;  // K - 1 prefix arrays (device pointers)
  const int64_t* keep;       // all modes qudits: final index of each staged state, -1 if dropped; else null
  const uint8_t* occ;        // final list, K occupations per state
  int64_t dim;
};

// A model basis: one basis, or the tensor product of two (tensorBasis,
// Basis.cpp:131-182: index i1 * dim2 + i2, the first set's modes first).
struct ModelBasis {
  Stages a, b;
  int tensor;
  int K;  // modes in all
  int64_t dim;
};

// children counts of list L_s (stage of mode m); qudit stages stop at the capacity
__global__ void stage_count_kernel(int64_t n, const uint8_t* __restrict__ occ, int K, int N, int quant, int cap,
                                   int64_t* __restrict__ cnt) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    int tot = 0;
    for (int a = 1; a < K; ++a) tot += occ[l * K + a];
    const int upper = cap >= 0 ? min(N - tot, cap) : N - tot;
    cnt[l] = upper / quant;
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

// mode 0 takes the missing particles; keep (all-qudit bases) marks the states
// whose mode 0 stays within the capacity
__global__ void finish_basis_kernel(int64_t n, uint8_t* occ, int K, int N, int cap, int64_t* keep) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    int tot = 0;
    for (int a = 1; a < K; ++a) tot += occ[l * K + a];
    occ[l * K] = (uint8_t)(N - tot);
    if (keep) keep[l] = (N - tot <= cap) ? 1 : 0;
  }
}

// keep flags -> exclusive prefix (in place, scanned on the host side) ->
// final index or -1, and the kept states copied into the final list
__global__ void compact_basis_kernel(int64_t n, const uint8_t* __restrict__ occ, int K, const uint8_t* __restrict__ kept,
                                     int64_t* __restrict__ keep, uint8_t* __restrict__ out) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    if (kept[l]) {
      for (int a = 0; a < K; ++a) out[keep[l] * K + a] = occ[l * K + a];
    } else {
      keep[l] = -1;
    }
  }
}

__global__ void keep_flags_kernel(int64_t n, const int64_t* __restrict__ keep, uint8_t* __restrict__ kept) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x)
    kept[l] = (uint8_t)keep[l];
}

// Index of an occupation vector in one basis, or -1 if it is not a basis state.
__device__ int64_t state_index(const Stages& st, const int* e) {
  int tot = 0;
  for (int a = 0; a < st.K; ++a) {
    if (e[a] < 0) return -1;
    tot += e[a];
  }
  if (tot != st.N) return -1;
  for (int a = st.K - st.nq; a < st.K; ++a)
    if (a >= 0 && e[a] > st.cap) return -1;
  int64_t r = 0;
  for (int s = 0; s < st.K - 1; ++s) {
    const int m = st.K - 1 - s;
    const int o = e[m];
    if (o == 0) continue;
    if (o % st.quant) return -1;
    r = st.n_s[s] + st.ps[s][r] + o / st.quant - 1;
  }
  return st.keep ? st.keep[r] : r;
}

__device__ int64_t model_index(const ModelBasis& M, const int* e) {
  if (!M.tensor) return state_index(M.a, e);
  const int64_t i1 = state_index(M.a, e);
  if (i1 < 0) return -1;
  const int64_t i2 = state_index(M.b, e + M.a.K);
  return i2 < 0 ? -1 : i1 * M.b.dim + i2;
}

__device__ void model_occupation(const ModelBasis& M, int64_t j, int* e) {
  if (!M.tensor) {
    for (int a = 0; a < M.K; ++a) e[a] = M.a.occ[j * M.K + a];
    return;
  }
  const int64_t j1 = j / M.b.dim, j2 = j - j1 * M.b.dim;
  for (int a = 0; a < M.a.K; ++a) e[a] = M.a.occ[j1 * M.a.K + a];
  for (int a = 0; a < M.b.K; ++a) e[M.a.K + a] = M.b.occ[j2 * M.b.K + a];
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
__device__ int build_row(const ModelBasis& M, int64_t j, const DevTerm* __restrict__ terms, int n_terms,
                         int32_t* cols, double2* vals, int32_t* out_col, double2* out_val, double* abs_sum) {
  int e[TE_MODEL_MAX_MODES];
  int cnt = 0;
  for (int ti = 0; ti < n_terms; ++ti) {
    const DevTerm& t = terms[ti];
    model_occupation(M, j, e);
    double2 c = make_double2(1.0, 0.0);
    if (!apply_term_dev(t, e, M.K, c)) continue;
    // coef = coef * t.coef: the complex product rounded term by term, without
    // contraction into FMAs (as the host build)
    c = make_double2(__dsub_rn(__dmul_rn(c.x, t.coef.x), __dmul_rn(c.y, t.coef.y)),
                     __dadd_rn(__dmul_rn(c.x, t.coef.y), __dmul_rn(c.y, t.coef.x)));
    const int64_t col = model_index(M, e);
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

__global__ void row_count_model_kernel(ModelBasis M, int64_t n, const DevTerm* __restrict__ terms, int n_terms,
                                       int32_t* __restrict__ count) {
  int32_t cols[TE_MODEL_MAX_TERMS];
  double2 vals[TE_MODEL_MAX_TERMS];
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
    count[j] = build_row(M, j, terms, n_terms, cols, vals, nullptr, nullptr, nullptr);
}

__global__ void row_write_model_kernel(ModelBasis M, int64_t n, const DevTerm* __restrict__ terms, int n_terms,
                                       const int32_t* __restrict__ rp, int32_t* __restrict__ col,
                                       double2* __restrict__ val, unsigned long long* norm_bits) {
  int32_t cols[TE_MODEL_MAX_TERMS];
  double2 vals[TE_MODEL_MAX_TERMS];
  double mx = 0.0;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    build_row(M, j, terms, n_terms, cols, vals, col + rp[j], val + rp[j], &s);
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
  int K = 0, N = 0, quant = 1, nq = 0, cap = 0;
  int64_t dim = 0;
  uint8_t* occ = nullptr;   // final list
  int64_t* keep = nullptr;  // all-qudit bases: staged index -> final index or -1
  std::vector<int64_t> n_s;
  std::vector<int64_t*> ps;
  int64_t* d_n_s = nullptr;
  int64_t** d_ps = nullptr;
  ~DeviceBasis() {
    te_free(occ);
    te_free(keep);
    for (int64_t* p : ps) te_free(p);
    te_free(d_n_s);
    te_free(d_ps);
  }
  Stages stages() const { return Stages{K, N, quant, nq, cap, d_n_s, d_ps, keep, occ, dim}; }
};

// basis(N, K, nq, cap, quant) of helper/Basis.cpp:37-121 on the device.
int build_basis(int N, int K, int nq, int cap, int quant, DeviceBasis& B) {
  B.K = K;
  B.N = N;
  B.quant = quant;
  B.nq = nq;
  B.cap = cap;
  // size of the staged list: states of modes 1..K-1 (multiples of quant, the
  // qudit modes at most cap) with at most N particles, counted per number of
  // quanta used; the final list drops, when every mode is a qudit, the states
  // whose mode 0 would exceed cap
  const int Q = N / quant;
  std::vector<double> ways(Q + 1, 0.0);
  ways[0] = 1.0;
  for (int s = 0; s < K - 1; ++s) {
    const int m = K - 1 - s;
    const int tmax = m >= K - nq ? cap / quant : Q;
    std::vector<double> nw(ways.size(), 0.0);
    for (int q = 0; q <= Q; ++q)
      for (int r = q; r <= Q && r - q <= tmax; ++r) nw[r] += ways[q];
    ways.swap(nw);
  }
  double total = 0.0, kept = 0.0;
  for (int q = 0; q <= Q; ++q) {
    total += ways[q];
    if (K != nq || N - q * quant <= cap) kept += ways[q];
  }
  if (!(total < 2147483647.0)) {
    te_set_error("te_model: basis dimension %.0f exceeds the int32 index range", total);
    return TE_ERR_UNSUPPORTED;
  }
  const int64_t n_full = (int64_t)total;
  uint8_t* occ = nullptr;
  TE_CUDA(te_malloc(&occ, (size_t)std::max<int64_t>(n_full, 1) * K));
  TE_CUDA(cudaMemset(occ, 0, (size_t)std::max<int64_t>(n_full, 1) * K));
  B.occ = occ;
  int64_t n = 1;
  int64_t* cnt = nullptr;
  TE_CUDA(te_malloc(&cnt, sizeof(int64_t) * std::max<int64_t>(n_full, 1)));
  int rc = TE_OK;
  for (int s = 0; s < K - 1 && rc == TE_OK; ++s) {
    const int m = K - 1 - s;
    B.n_s.push_back(n);
    int64_t* ps = nullptr;
    if ((rc = te_cuda_check(te_malloc(&ps, sizeof(int64_t) * (n + 1)), "basis")) != TE_OK) break;
    B.ps.push_back(ps);
    const int g = te_grid_for(n, 256, 4);
    stage_count_kernel<<<g, 256>>>(n, occ, K, N, quant, m >= K - nq ? cap : -1, cnt);
    int64_t added = 0;
    if ((rc = exclusive_scan(cnt, n, ps, &added)) != TE_OK) break;
    if (n + added > n_full) {
      te_set_error("te_model: basis enumeration inconsistent");
      rc = TE_ERR_INVALID_ARG;
      break;
    }
    stage_expand_kernel<<<g, 256>>>(n, occ, K, m, quant, ps);
    n += added;
  }
  te_free(cnt);
  if (rc != TE_OK) return rc;
  if (n != n_full) {
    te_set_error("te_model: basis enumeration inconsistent");
    return TE_ERR_INVALID_ARG;
  }
  B.n_s.push_back(n);
  const bool filter = K == nq;
  if (filter) TE_CUDA(te_malloc(&B.keep, sizeof(int64_t) * (n + 1)));
  finish_basis_kernel<<<te_grid_for(n, 256, 4), 256>>>(n, occ, K, N, cap, B.keep);
  B.dim = n;
  if (filter) {
    uint8_t* flags = nullptr;
    uint8_t* out = nullptr;
    int64_t count = 0;
    TE_CUDA(te_malloc(&flags, n));
    keep_flags_kernel<<<te_grid_for(n, 256, 4), 256>>>(n, B.keep, flags);
    rc = exclusive_scan(B.keep, n, B.keep, &count);
    if (rc == TE_OK && count != (int64_t)kept) {
      te_set_error("te_model: basis filter inconsistent");
      rc = TE_ERR_INVALID_ARG;
    }
    if (rc == TE_OK) rc = te_cuda_check(te_malloc(&out, (size_t)std::max<int64_t>(count, 1) * K), "basis");
    if (rc == TE_OK) compact_basis_kernel<<<te_grid_for(n, 256, 4), 256>>>(n, occ, K, flags, B.keep, out);
    te_free(flags);
    if (rc != TE_OK) {
      te_free(out);
      return rc;
    }
    TE_CUDA(cudaDeviceSynchronize());
    te_free(occ);
    B.occ = out;
    B.dim = count;
  }
  TE_CUDA(te_malloc(&B.d_n_s, sizeof(int64_t) * B.n_s.size()));
  TE_CUDA(cudaMemcpy(B.d_n_s, B.n_s.data(), sizeof(int64_t) * B.n_s.size(), cudaMemcpyHostToDevice));
  TE_CUDA(te_malloc(&B.d_ps, sizeof(int64_t*) * std::max<size_t>(B.ps.size(), 1)));
  if (!B.ps.empty())
    TE_CUDA(cudaMemcpy(B.d_ps, B.ps.data(), sizeof(int64_t*) * B.ps.size(), cudaMemcpyHostToDevice));
  return te_cuda_check(cudaDeviceSynchronize(), "basis");
}

// The basis of a descriptor: one basis, or the tensor product of basis(N1, K1,
// 0, 0) and basis(N2, K2, K2, C2) (Basis.cpp:131-182).
struct DeviceModelBasis {
  DeviceBasis a, b;
  ModelBasis view;
};

int check_desc(const te_basis_desc* d, const char* who) {
  if (!d || d->n_modes < 1 || d->n_particles < 0 || d->n_particles > 255 || d->quant < 1 || d->n_qudits < 0 ||
      d->n_qudits > d->n_modes || d->capacity < 0 || d->n_modes2 < 0 ||
      d->n_modes + d->n_modes2 > TE_MODEL_MAX_MODES) {
    te_set_error("%s: invalid basis (1..%d modes in all, 0..255 particles, 0 <= qudit modes <= modes, "
                 "capacity >= 0, quant >= 1)", who, TE_MODEL_MAX_MODES);
    return TE_ERR_INVALID_ARG;
  }
  if (d->n_modes2 > 0 && (d->n_qudits != 0 || d->quant != 1 || d->n_particles2 < 0 || d->n_particles2 > 255 ||
                          d->capacity2 < 0)) {
    te_set_error("%s: a tensor basis takes a first set without qudit modes and quant 1, and 0..255 particles "
                 "and capacity >= 0 in the second set", who);
    return TE_ERR_INVALID_ARG;
  }
  return TE_OK;
}

int build_model_basis(const te_basis_desc* d, DeviceModelBasis& M) {
  int rc = build_basis(d->n_particles, d->n_modes, d->n_qudits, d->capacity, d->quant, M.a);
  if (rc != TE_OK) return rc;
  M.view.a = M.a.stages();
  M.view.tensor = d->n_modes2 > 0 ? 1 : 0;
  M.view.K = d->n_modes;
  M.view.dim = M.a.dim;
  if (M.view.tensor) {
    if ((rc = build_basis(d->n_particles2, d->n_modes2, d->n_modes2, d->capacity2, 1, M.b)) != TE_OK) return rc;
    if (M.b.dim == 0) {
      te_set_error("te_model: the second set of the tensor basis is empty");
      return TE_ERR_UNSUPPORTED;
    }
    if (!((double)M.a.dim * (double)M.b.dim < 2147483647.0)) {
      te_set_error("te_model: basis dimension exceeds the int32 index range");
      return TE_ERR_UNSUPPORTED;
    }
    M.view.b = M.b.stages();
    M.view.K += d->n_modes2;
    M.view.dim = M.a.dim * M.b.dim;
  } else {
    M.view.b = M.view.a;
  }
  return TE_OK;
}

}  // namespace

extern "C" int te_model_create_device_basis(const te_basis_desc* basis, const te_term* terms, int n_terms,
                                            te_matrix* out, int64_t* dim_out) {
  int rc = check_desc(basis, "te_model_create_device_basis");
  if (rc != TE_OK) return rc;
  if (!out || !terms || n_terms < 1 || n_terms > TE_MODEL_MAX_TERMS) {
    te_set_error("te_model_create_device_basis: invalid arguments (1..%d terms)", TE_MODEL_MAX_TERMS);
    return TE_ERR_INVALID_ARG;
  }
  const int n_modes = basis->n_modes + basis->n_modes2;
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
  DeviceModelBasis MB;
  if ((rc = build_model_basis(basis, MB)) != TE_OK) return rc;
  const int64_t n = MB.view.dim;
  if (n == 0) {
    te_set_error("te_model_create_device_basis: the basis is empty");
    return TE_ERR_DIM;
  }
  DevTerm* d_terms = nullptr;
  int32_t *d_cnt = nullptr, *d_rp = nullptr, *d_col = nullptr;
  double2* d_val = nullptr;
  unsigned long long* d_norm = nullptr;
  auto fail = [&](int code) {
    te_free(d_terms);
    te_free(d_cnt);
    te_free(d_rp);
    te_free(d_col);
    te_free(d_val);
    te_free(d_norm);
    return code;
  };
  if (te_cuda_check(te_malloc(&d_terms, sizeof(DevTerm) * n_terms), "model") != TE_OK ||
      te_cuda_check(te_malloc(&d_cnt, sizeof(int32_t) * n), "model") != TE_OK ||
      te_cuda_check(te_malloc(&d_norm, sizeof(unsigned long long)), "model") != TE_OK)
    return fail(TE_ERR_CUDA);
  cudaMemcpy(d_terms, dt.data(), sizeof(DevTerm) * n_terms, cudaMemcpyHostToDevice);
  cudaMemset(d_norm, 0, sizeof(unsigned long long));
  const ModelBasis st = MB.view;
  const int g = te_grid_fit((const void*)row_count_model_kernel, n, 128);
  row_count_model_kernel<<<g, 128>>>(st, n, d_terms, n_terms, d_cnt);
  // row pointers: a 64-bit scan of the counts on the device (the total must
  // stay below 2^31), narrowed to int32
  int64_t* d_rp64 = nullptr;
  int64_t nnz = 0;
  if (te_cuda_check(te_malloc(&d_rp64, sizeof(int64_t) * (n + 1)), "model") != TE_OK) return fail(TE_ERR_CUDA);
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
    rc = te_cuda_check(te_malloc(&d_rp, sizeof(int32_t) * (n + 1)), "model");
  if (rc == TE_OK)
    narrow_rp_kernel<<<te_grid_fit((const void*)narrow_rp_kernel, n + 1, TE_THREADS), TE_THREADS>>>(n + 1, d_rp64,
                                                                                                   d_rp);
  te_free(d_rp64);
  if (rc != TE_OK) return fail(rc);
  if (te_cuda_check(te_malloc(&d_col, sizeof(int32_t) * std::max<int64_t>(nnz, 1)), "model") != TE_OK ||
      te_cuda_check(te_malloc(&d_val, sizeof(double2) * std::max<int64_t>(nnz, 1)), "model") != TE_OK)
    return fail(TE_ERR_CUDA);
  row_write_model_kernel<<<te_grid_fit((const void*)row_write_model_kernel, n, 128), 128>>>(
      st, n, d_terms, n_terms, d_rp, d_col, d_val, d_norm);
  unsigned long long bits = 0;
  if (te_cuda_check(cudaMemcpy(&bits, d_norm, sizeof(bits), cudaMemcpyDeviceToHost), "model") != TE_OK)
    return fail(TE_ERR_CUDA);
  double norm1;
  std::memcpy(&norm1, &bits, sizeof(norm1));
  te_free(d_terms);
  te_free(d_cnt);
  te_free(d_norm);
  d_terms = nullptr;
  d_cnt = nullptr;
  d_norm = nullptr;
  rc = te_matrix_adopt_device_csr(n, n, nnz, d_rp, d_col, d_val, out, norm1);
  if (rc != TE_OK) return rc;  // the matrix freed the arrays
  if (dim_out) *dim_out = n;
  return TE_OK;
}

extern "C" int te_model_create_device(int n_particles, int n_modes, int quant, const te_term* terms, int n_terms,
                                      te_matrix* out, int64_t* dim_out) {
  te_basis_desc d;
  std::memset(&d, 0, sizeof(d));
  d.n_particles = n_particles;
  d.n_modes = n_modes;
  d.quant = quant;
  return te_model_create_device_basis(&d, terms, n_terms, out, dim_out);
}

namespace {

__global__ void state_index_kernel(ModelBasis M, const int* e, int64_t* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *out = model_index(M, e);
}

}  // namespace

extern "C" int te_model_basis_index(const te_basis_desc* basis, const int32_t* occupation, int64_t* index) {
  int rc = check_desc(basis, "te_model_basis_index");
  if (rc != TE_OK) return rc;
  if (!occupation || !index) {
    te_set_error("te_model_basis_index: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  const int n_modes = basis->n_modes + basis->n_modes2;
  DeviceModelBasis MB;
  if ((rc = build_model_basis(basis, MB)) != TE_OK) return rc;
  int* d_e = nullptr;
  int64_t* d_r = nullptr;
  if (te_cuda_check(te_malloc(&d_e, sizeof(int) * n_modes), "index") != TE_OK ||
      te_cuda_check(te_malloc(&d_r, sizeof(int64_t)), "index") != TE_OK) {
    te_free(d_e);
    te_free(d_r);
    return TE_ERR_CUDA;
  }
  cudaMemcpy(d_e, occupation, sizeof(int) * n_modes, cudaMemcpyHostToDevice);
  state_index_kernel<<<1, 32>>>(MB.view, d_e, d_r);
  rc = te_cuda_check(cudaMemcpy(index, d_r, sizeof(int64_t), cudaMemcpyDeviceToHost), "index");
  te_free(d_e);
  te_free(d_r);
  return rc;
}

extern "C" int te_model_state_index(int n_particles, int n_modes, int quant, const int32_t* occupation,
                                    int64_t* index) {
  te_basis_desc d;
  std::memset(&d, 0, sizeof(d));
  d.n_particles = n_particles;
  d.n_modes = n_modes;
  d.quant = quant;
  return te_model_basis_index(&d, occupation, index);
}
