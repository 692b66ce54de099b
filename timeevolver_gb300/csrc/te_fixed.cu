// te_fixed.cu -- the fixed-point data of a SELL matrix (te_fixed.cuh): the
// scale of its values; a value dictionary with packed slots (real matrices
// with few distinct values) or the limbs of every slot value; and the static
// schedule of the fixed-point apply kernel.  Built once per matrix on first
// use; rebuilt when the values change in place (te_sell_refresh_fixed).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "te_fixed.cuh"
#include "te_internal.cuh"

namespace {

// Largest chunk-row 1-norm (complex: sum of |Re| + |Im|), as the bit pattern
// of a non-negative double.
template <bool REAL>
__global__ void __launch_bounds__(TE_THREADS) fix_rownorm_kernel(int64_t n_chunks, const int64_t* __restrict__ off,
                                                                 const double* __restrict__ val,
                                                                 unsigned long long* max_bits) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t c = t >> 5;
  if (c >= n_chunks) return;  // whole warps
  double s = 0.0;
  for (int64_t q = off[c] + (t & 31); q < off[c + 1]; q += 32)
    s += REAL ? fabs(val[q]) : fabs(val[2 * q]) + fabs(val[2 * q + 1]);
  for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, o));
  if ((t & 31) == 0) atomicMax(max_bits, (unsigned long long)__double_as_longlong(s));
}

__global__ void __launch_bounds__(TE_THREADS) fix_encode_values_kernel(int64_t count, const double* __restrict__ val,
                                                                       int2* __restrict__ out, int sh) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < count; q += (int64_t)gridDim.x * blockDim.x)
    out[q] = te_fix_split(te_fix_encode(val[q], sh));
}

__global__ void __launch_bounds__(TE_THREADS) fix_encode_complex_kernel(int64_t count,
                                                                        const double2* __restrict__ val,
                                                                        int4* __restrict__ out, int sh) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < count; q += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = val[q];
    const int2 re = te_fix_split(te_fix_encode(v.x, sh)), im = te_fix_split(te_fix_encode(v.y, sh));
    out[q] = make_int4(re.x, re.y, im.x, im.y);
  }
}

// Value dictionary: open addressing over the bit patterns of the slot values
// (kDictSlots entries, linear probing); an insertion beyond kDictMax distinct
// values sets the overflow flag, after which every thread stops.
constexpr int kDictMax = 4096;   // values the apply kernel keeps in shared memory (32 KB)
constexpr int kDictSlots = 8192;  // power of two, load factor <= 1/2
constexpr unsigned long long kDictEmpty = ~0ull;

__device__ __forceinline__ unsigned int dict_hash(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  return (unsigned int)k & (kDictSlots - 1);
}

__global__ void __launch_bounds__(TE_THREADS) dict_insert_kernel(int64_t slots, const double* __restrict__ val,
                                                                 unsigned long long* table, int* count,
                                                                 int* overflow) {
  volatile unsigned long long* vt = table;
  volatile int* vo = overflow;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < slots; q += (int64_t)gridDim.x * blockDim.x) {
    if (*vo) return;
    const unsigned long long key = (unsigned long long)__double_as_longlong(val[q]);
    if (key == kDictEmpty) {
      *vo = 1;
      return;
    }
    unsigned int h = dict_hash(key);
    for (int p = 0; p < kDictSlots; ++p) {
      const unsigned long long cur = vt[h];
      if (cur == key) break;
      if (cur == kDictEmpty) {
        const unsigned long long prev = atomicCAS(table + h, kDictEmpty, key);
        if (prev == kDictEmpty) {
          if (atomicAdd(count, 1) >= kDictMax) *vo = 1;
          break;
        }
        if (prev == key) break;
      }
      h = (h + 1) & (kDictSlots - 1);
    }
  }
}

// Packed slot words: column | (index of the slot value << cbits).
__global__ void __launch_bounds__(TE_THREADS) dict_pack_kernel(int64_t slots, const double* __restrict__ val,
                                                               const int32_t* __restrict__ col,
                                                               const unsigned long long* __restrict__ table,
                                                               const int* __restrict__ slot_index, int cbits,
                                                               uint32_t* __restrict__ pk) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < slots; q += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long key = (unsigned long long)__double_as_longlong(val[q]);
    unsigned int h = dict_hash(key);
    int idx = 0;
    for (int p = 0; p < kDictSlots; ++p) {  // every key is present (inserted above)
      if (table[h] == key) {
        idx = slot_index[h];
        break;
      }
      h = (h + 1) & (kDictSlots - 1);
    }
    pk[q] = (uint32_t)col[q] | ((uint32_t)idx << cbits);
  }
}

template <typename T>
void free_ptr(T*& p) {
  cudaFree(p);
  p = nullptr;
}

void free_fixed(TeSell& S) {
  free_ptr(S.fix_val);
  free_ptr(S.fix_val4);
  free_ptr(S.fix_warp_chunk);
  free_ptr(S.fix_pk);
  free_ptr(S.fix_table);
  S.fix_nvals = 0;
  S.fix_cbits = 0;
}

// sh: the largest chunk-row 1-norm maps below 2^61.
int fixed_scale(TeSell& S, bool real) {
  unsigned long long* d_max = nullptr;
  TE_CUDA(cudaMalloc(&d_max, sizeof(unsigned long long)));
  int rc = te_cuda_check(cudaMemset(d_max, 0, sizeof(unsigned long long)), "fixed values");
  const int64_t threads = S.n_chunks * 32;
  const unsigned blocks = (unsigned)((threads + TE_THREADS - 1) / TE_THREADS);
  if (rc == TE_OK && real) fix_rownorm_kernel<true><<<blocks, TE_THREADS>>>(S.n_chunks, S.chunk_off, S.val, d_max);
  if (rc == TE_OK && !real) fix_rownorm_kernel<false><<<blocks, TE_THREADS>>>(S.n_chunks, S.chunk_off, S.val, d_max);
  unsigned long long bits = 0;
  if (rc == TE_OK) rc = te_cuda_check(cudaMemcpy(&bits, d_max, sizeof(bits), cudaMemcpyDeviceToHost), "fixed values");
  cudaFree(d_max);
  if (rc != TE_OK) return rc;
  double rmax;
  std::memcpy(&rmax, &bits, sizeof(rmax));
  if (!(rmax < 1e300)) {
    te_set_error("fixed-point SpMV: matrix row norm not finite");
    return TE_ERR_INVALID_ARG;
  }
  int E = 0;
  if (rmax > 0.0) std::frexp(rmax * (1.0 + 1e-12), &E);
  S.fix_sh = 61 - E;
  return TE_OK;
}

// Packed slots through a value dictionary when the distinct values fit in
// 2^(32 - cbits) indices and in shared memory.  Sets *packed; TE_OK without a
// dictionary is not an error.
int try_dictionary(TeSell& S, bool* packed) {
  *packed = false;
  int cbits = 1;
  while (cbits < 31 && ((int64_t)1 << cbits) < S.n) ++cbits;
  const int limit = (int)std::min<int64_t>(kDictMax, (int64_t)1 << (32 - cbits));
  if (limit < 2) return TE_OK;
  unsigned long long* d_table = nullptr;
  int* d_flags = nullptr;  // count, overflow
  int* d_index = nullptr;
  double* d_vals = nullptr;
  auto cleanup = [&]() {
    cudaFree(d_table);
    cudaFree(d_flags);
    cudaFree(d_index);
    cudaFree(d_vals);
  };
  int rc;
  if ((rc = te_cuda_check(cudaMalloc(&d_table, sizeof(unsigned long long) * kDictSlots), "dictionary")) != TE_OK ||
      (rc = te_cuda_check(cudaMalloc(&d_flags, 2 * sizeof(int)), "dictionary")) != TE_OK ||
      (rc = te_cuda_check(cudaMemset(d_table, 0xff, sizeof(unsigned long long) * kDictSlots), "dictionary")) !=
          TE_OK ||
      (rc = te_cuda_check(cudaMemset(d_flags, 0, 2 * sizeof(int)), "dictionary")) != TE_OK) {
    cleanup();
    return rc;
  }
  dict_insert_kernel<<<te_grid_fit((const void*)dict_insert_kernel, S.slots, TE_THREADS), TE_THREADS>>>(
      S.slots, S.val, d_table, d_flags, d_flags + 1);
  std::vector<unsigned long long> table(kDictSlots);
  int flags[2] = {0, 0};
  if ((rc = te_cuda_check(cudaMemcpy(flags, d_flags, sizeof(flags), cudaMemcpyDeviceToHost), "dictionary")) != TE_OK ||
      (rc = te_cuda_check(
           cudaMemcpy(table.data(), d_table, sizeof(unsigned long long) * kDictSlots, cudaMemcpyDeviceToHost),
           "dictionary")) != TE_OK) {
    cleanup();
    return rc;
  }
  if (flags[1] || flags[0] > limit) {  // too many distinct values: plain limbs
    cleanup();
    return TE_OK;
  }
  // indices in ascending value order (independent of the insertion order)
  std::vector<std::pair<double, int>> vals;
  for (int h = 0; h < kDictSlots; ++h)
    if (table[h] != kDictEmpty) {
      double v;
      std::memcpy(&v, &table[h], sizeof(v));
      vals.push_back({v, h});
    }
  std::sort(vals.begin(), vals.end(), [&](const std::pair<double, int>& a, const std::pair<double, int>& b) {
    if (a.first != b.first) return a.first < b.first;
    return table[a.second] < table[b.second];  // -0.0 and +0.0: by bit pattern
  });
  std::vector<int> index(kDictSlots, 0);
  std::vector<double> sorted(vals.size());
  for (size_t i = 0; i < vals.size(); ++i) {
    index[vals[i].second] = (int)i;
    sorted[i] = vals[i].first;
  }
  const int nv = (int)vals.size();
  if ((rc = te_cuda_check(cudaMalloc(&d_index, sizeof(int) * kDictSlots), "dictionary")) != TE_OK ||
      (rc = te_cuda_check(cudaMalloc(&d_vals, sizeof(double) * std::max(nv, 1)), "dictionary")) != TE_OK ||
      (rc = te_cuda_check(cudaMalloc(&S.fix_table, sizeof(int2) * std::max(nv, 1)), "dictionary")) != TE_OK ||
      (rc = te_cuda_check(cudaMalloc(&S.fix_pk, sizeof(uint32_t) * std::max<int64_t>(S.slots, 1)), "dictionary")) !=
          TE_OK ||
      (rc = te_cuda_check(cudaMemcpy(d_index, index.data(), sizeof(int) * kDictSlots, cudaMemcpyHostToDevice),
                          "dictionary")) != TE_OK ||
      (rc = te_cuda_check(cudaMemcpy(d_vals, sorted.data(), sizeof(double) * nv, cudaMemcpyHostToDevice),
                          "dictionary")) != TE_OK) {
    cleanup();
    return rc;
  }
  dict_pack_kernel<<<te_grid_fit((const void*)dict_pack_kernel, S.slots, TE_THREADS), TE_THREADS>>>(
      S.slots, S.val, S.col, d_table, d_index, cbits, S.fix_pk);
  fix_encode_values_kernel<<<1, TE_THREADS>>>(nv, d_vals, S.fix_table, S.fix_sh);
  rc = te_cuda_check(cudaDeviceSynchronize(), "dictionary");
  cleanup();
  if (rc != TE_OK) return rc;
  S.fix_nvals = nv;
  S.fix_cbits = cbits;
  *packed = true;
  return TE_OK;
}

// Values (dictionary or limbs) at the current sh.
int fixed_values(TeSell& S, bool real) {
  int rc;
  if ((rc = fixed_scale(S, real)) != TE_OK) return rc;
  free_ptr(S.fix_pk);
  free_ptr(S.fix_table);
  S.fix_nvals = 0;
  if (!real) {  // complex: limbs of both parts per slot (no dictionary)
    if (!S.fix_val4 &&
        (rc = te_cuda_check(cudaMalloc(&S.fix_val4, sizeof(int4) * std::max<int64_t>(S.slots, 1)),
                            "fixed values")) != TE_OK)
      return rc;
    fix_encode_complex_kernel<<<te_grid_fit((const void*)fix_encode_complex_kernel, S.slots, TE_THREADS),
                                TE_THREADS>>>(S.slots, reinterpret_cast<const double2*>(S.val), S.fix_val4, S.fix_sh);
    return te_cuda_check(cudaDeviceSynchronize(), "fixed values");
  }
  bool packed = false;
  if ((rc = try_dictionary(S, &packed)) != TE_OK) return rc;
  if (packed) {
    free_ptr(S.fix_val);
    return TE_OK;
  }
  if (!S.fix_val &&
      (rc = te_cuda_check(cudaMalloc(&S.fix_val, sizeof(int2) * std::max<int64_t>(S.slots, 1)), "fixed values")) !=
          TE_OK)
    return rc;
  fix_encode_values_kernel<<<te_grid_fit((const void*)fix_encode_values_kernel, S.slots, TE_THREADS), TE_THREADS>>>(
      S.slots, S.val, S.fix_val, S.fix_sh);
  return te_cuda_check(cudaDeviceSynchronize(), "fixed values");
}

// The static schedule of the fixed-point apply kernel for the current layout.
int fixed_schedule(TeSell& S, bool real) {
  std::vector<int64_t> off(S.n_chunks + 1);
  int rc = te_cuda_check(cudaMemcpy(off.data(), S.chunk_off, sizeof(int64_t) * off.size(), cudaMemcpyDeviceToHost),
                         "fixed schedule");
  if (rc != TE_OK) return rc;
  const int bps = te_apply_fix_blocks_per_sm(real ? (S.fix_pk ? 1 : 0) : 2, sizeof(int2) * S.fix_nvals);
  std::vector<int32_t> wc;
  te_sell_schedule(off, S.n_chunks, bps, real, S.fix_grid, S.fix_saturated, wc);
  int32_t* d_wc = nullptr;
  if ((rc = te_cuda_check(cudaMalloc(&d_wc, sizeof(int32_t) * wc.size()), "fixed schedule")) != TE_OK) return rc;
  rc = te_cuda_check(cudaMemcpy(d_wc, wc.data(), sizeof(int32_t) * wc.size(), cudaMemcpyHostToDevice),
                     "fixed schedule");
  if (rc != TE_OK) {
    cudaFree(d_wc);
    return rc;
  }
  cudaFree(S.fix_warp_chunk);
  S.fix_warp_chunk = d_wc;  // marks the fixed-point data complete
  return TE_OK;
}

}  // namespace

int te_sell_build_fixed(te_matrix_s* A) {
  TeSell& S = A->sell;
  if (S.fix_warp_chunk) return TE_OK;
  if (S.n_chunks < 1) {
    te_set_error("fixed-point SpMV: empty matrix");
    return TE_ERR_INVALID_ARG;
  }
  int rc = fixed_values(S, A->is_real);
  if (rc == TE_OK) rc = fixed_schedule(S, A->is_real);
  if (rc != TE_OK) free_fixed(S);
  return rc;
}

int te_sell_refresh_fixed(te_matrix_s* A) {
  TeSell& S = A->sell;
  if (!S.fix_warp_chunk) return TE_OK;
  const bool was_packed = S.fix_pk != nullptr;
  const int nv = S.fix_nvals;
  int rc = fixed_values(S, A->is_real);
  // the schedule depends on the occupancy, which depends on the table size
  if (rc == TE_OK && (was_packed != (S.fix_pk != nullptr) || nv != S.fix_nvals)) rc = fixed_schedule(S, A->is_real);
  if (rc != TE_OK) free_fixed(S);
  return rc;
}
