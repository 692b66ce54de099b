// te_fixed.cu -- the fixed-point data of a SELL matrix (te_fixed.cuh): the
// scale of its values; a value dictionary with packed slots (real matrices
// with few distinct values) or the limbs of every slot value; and the static
// schedule of the fixed-point apply kernel.  Built once per matrix on first
// use; rebuilt when the values change in place (te_sell_refresh_fixed).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
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

// Column blocks: bounds lo[0] = 0 < lo[1] < ... < lo[nb] = n.
struct BlockDesc {
  int nb;
  int64_t lo[TE_FIX_MAX_BLOCKS + 1];
};

__device__ __forceinline__ int block_of(const BlockDesc& d, int64_t c) {
  int b = 0;
  while (b + 1 < d.nb && c >= d.lo[b + 1]) ++b;
  return b;
}

// The slots of the main layout that carry a value (padding and entries that
// encode to zero contribute nothing and are left out of the blocks).
template <bool REAL>
__device__ __forceinline__ bool slot_has_value(const int2* hv, const int4* hv4, int64_t s) {
  if (REAL) {
    const int2 h = hv[s];
    return (h.x | h.y) != 0;
  }
  const int4 h = hv4[s];
  return (h.x | h.y | h.z | h.w) != 0;
}

// cnt[b n + r]: entries of main row r in column block b.
template <bool REAL>
__global__ void __launch_bounds__(TE_THREADS) block_count_kernel(int64_t n, const int64_t* __restrict__ off,
                                                                 const int32_t* __restrict__ col,
                                                                 const int2* __restrict__ hv,
                                                                 const int4* __restrict__ hv4, BlockDesc d,
                                                                 int32_t* __restrict__ cnt) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    int k[TE_FIX_MAX_BLOCKS] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int64_t c = r >> 5;
    for (int64_t s = off[c] + (r & 31); s < off[c + 1]; s += 32)
      if (slot_has_value<REAL>(hv, hv4, s)) ++k[block_of(d, col[s])];
    for (int b = 0; b < d.nb; ++b) cnt[(int64_t)b * n + r] = k[b];
  }
}

struct BlockFill {
  const int64_t* off[TE_FIX_MAX_BLOCKS];
  int32_t* col[TE_FIX_MAX_BLOCKS];
  int2* hv[TE_FIX_MAX_BLOCKS];
  int4* hv4[TE_FIX_MAX_BLOCKS];
};

// Scatter every valued slot of main row r into its block: block row p =
// pos[b n + r] (present: the row has entries in b), slot off_b[p / 32] +
// p % 32 + 32 k for its k-th entry there (k < its count <= the chunk width).
template <bool REAL>
__global__ void __launch_bounds__(TE_THREADS) block_fill_kernel(int64_t n, const int64_t* __restrict__ off,
                                                                const int32_t* __restrict__ col,
                                                                const int2* __restrict__ hv,
                                                                const int4* __restrict__ hv4, BlockDesc d,
                                                                const int32_t* __restrict__ pos, BlockFill f) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    int k[TE_FIX_MAX_BLOCKS] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int64_t c = r >> 5;
    for (int64_t s = off[c] + (r & 31); s < off[c + 1]; s += 32) {
      if (!slot_has_value<REAL>(hv, hv4, s)) continue;
      const int32_t cl = col[s];
      const int b = block_of(d, cl);
      const int64_t p = pos[(int64_t)b * n + r];
      const int64_t q = f.off[b][p >> 5] + (p & 31) + 32 * (int64_t)k[b]++;
      f.col[b][q] = cl;
      if (REAL)
        f.hv[b][q] = hv[s];
      else
        f.hv4[b][q] = hv4[s];
    }
  }
}

__global__ void fill_i32_kernel(int64_t count, int32_t* __restrict__ out, int32_t v) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < count; q += (int64_t)gridDim.x * blockDim.x)
    out[q] = v;
}

template <typename T>
void free_ptr(T*& p) {
  te_free(p);
  p = nullptr;
}

void free_blocks(TeSell& S) {
  for (int b = 0; b < TE_FIX_MAX_BLOCKS; ++b) {
    TeSell::Block& B = S.fix_blk[b];
    free_ptr(B.chunk_off);
    free_ptr(B.row);
    free_ptr(B.col);
    free_ptr(B.hv);
    free_ptr(B.hv4);
    free_ptr(B.warp_chunk);
    B = TeSell::Block();
  }
  S.fix_nblk = 0;
}

void free_fixed(TeSell& S) {
  free_blocks(S);
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
  TE_CUDA(te_malloc(&d_max, sizeof(unsigned long long)));
  int rc = te_cuda_check(cudaMemset(d_max, 0, sizeof(unsigned long long)), "fixed values");
  const int64_t threads = S.n_chunks * 32;
  const unsigned blocks = (unsigned)((threads + TE_THREADS - 1) / TE_THREADS);
  if (rc == TE_OK && real) fix_rownorm_kernel<true><<<blocks, TE_THREADS>>>(S.n_chunks, S.chunk_off, S.val, d_max);
  if (rc == TE_OK && !real) fix_rownorm_kernel<false><<<blocks, TE_THREADS>>>(S.n_chunks, S.chunk_off, S.val, d_max);
  unsigned long long bits = 0;
  if (rc == TE_OK) rc = te_cuda_check(cudaMemcpy(&bits, d_max, sizeof(bits), cudaMemcpyDeviceToHost), "fixed values");
  te_free(d_max);
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
    te_free(d_table);
    te_free(d_flags);
    te_free(d_index);
    te_free(d_vals);
  };
  int rc;
  if ((rc = te_cuda_check(te_malloc(&d_table, sizeof(unsigned long long) * kDictSlots), "dictionary")) != TE_OK ||
      (rc = te_cuda_check(te_malloc(&d_flags, 2 * sizeof(int)), "dictionary")) != TE_OK ||
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
  if ((rc = te_cuda_check(te_malloc(&d_index, sizeof(int) * kDictSlots), "dictionary")) != TE_OK ||
      (rc = te_cuda_check(te_malloc(&d_vals, sizeof(double) * std::max(nv, 1)), "dictionary")) != TE_OK ||
      (rc = te_cuda_check(te_malloc(&S.fix_table, sizeof(int2) * std::max(nv, 1)), "dictionary")) != TE_OK ||
      (rc = te_cuda_check(te_malloc(&S.fix_pk, sizeof(uint32_t) * std::max<int64_t>(S.slots, 1)), "dictionary")) !=
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
        (rc = te_cuda_check(te_malloc(&S.fix_val4, sizeof(int4) * std::max<int64_t>(S.slots, 1)),
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
      (rc = te_cuda_check(te_malloc(&S.fix_val, sizeof(int2) * std::max<int64_t>(S.slots, 1)), "fixed values")) !=
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
  if ((rc = te_cuda_check(te_malloc(&d_wc, sizeof(int32_t) * wc.size()), "fixed schedule")) != TE_OK) return rc;
  rc = te_cuda_check(cudaMemcpy(d_wc, wc.data(), sizeof(int32_t) * wc.size(), cudaMemcpyHostToDevice),
                     "fixed schedule");
  if (rc != TE_OK) {
    te_free(d_wc);
    return rc;
  }
  te_free(S.fix_warp_chunk);
  S.fix_warp_chunk = d_wc;  // marks the fixed-point data complete
  return TE_OK;
}

// Column blocks when the fixed-point x (16 bytes per row) is larger than this:
// slices of at most kBlockSliceBytes then stay in L2 (126 MB) during their pass.
constexpr int64_t kBlockMinBytes = 96ll << 20;
constexpr int64_t kBlockSliceBytes = 56ll << 20;

int build_blocks(TeSell& S, bool real) {
  const int64_t n = S.n;
  if (S.fix_pk || S.n_long > 0 || S.fix_blocks_req == 1) return TE_OK;
  if (S.fix_blocks_req == 0 && 16 * n <= kBlockMinBytes) return TE_OK;
  const int nb = S.fix_blocks_req >= 2
                     ? (int)std::min<int64_t>(S.fix_blocks_req, std::max<int64_t>(n / 32, 1))
                     : (int)std::min<int64_t>(TE_FIX_MAX_BLOCKS, (16 * n + kBlockSliceBytes - 1) / kBlockSliceBytes);
  if (nb < 2) return TE_OK;
  BlockDesc d{};
  d.nb = nb;
  for (int b = 0; b <= nb; ++b) d.lo[b] = n * b / nb;
  int32_t *d_cnt = nullptr, *d_pos = nullptr;
  auto cleanup = [&]() {
    te_free(d_cnt);
    te_free(d_pos);
  };
  int rc;
  if ((rc = te_cuda_check(te_malloc(&d_cnt, sizeof(int32_t) * nb * n), "column blocks")) != TE_OK) return rc;
  if (real)
    block_count_kernel<true><<<te_grid_fit((const void*)block_count_kernel<true>, n, TE_THREADS), TE_THREADS>>>(
        n, S.chunk_off, S.col, S.fix_val, S.fix_val4, d, d_cnt);
  else
    block_count_kernel<false><<<te_grid_fit((const void*)block_count_kernel<false>, n, TE_THREADS), TE_THREADS>>>(
        n, S.chunk_off, S.col, S.fix_val, S.fix_val4, d, d_cnt);
  std::vector<int32_t> cnt((size_t)nb * n), pos((size_t)nb * n, -1);
  if ((rc = te_cuda_check(cudaMemcpy(cnt.data(), d_cnt, sizeof(int32_t) * nb * n, cudaMemcpyDeviceToHost),
                          "column blocks")) != TE_OK) {
    cleanup();
    return rc;
  }
  const int bps = te_fix_block_blocks_per_sm(real);
  BlockFill fill{};
  S.fix_nblk = nb;  // the arrays below are freed by free_blocks on failure
  for (int b = 0; b < nb && rc == TE_OK; ++b) {
    TeSell::Block& B = S.fix_blk[b];
    const int32_t* cb = cnt.data() + (size_t)b * n;
    // rows by count in the block, descending and stable; block 0 keeps every row
    int32_t maxc = 0;
    for (int64_t r = 0; r < n; ++r) maxc = std::max(maxc, cb[r]);
    std::vector<int64_t> start((size_t)maxc + 2, 0);
    for (int64_t r = 0; r < n; ++r) start[maxc - cb[r] + 1]++;
    for (int32_t k = 0; k <= maxc; ++k) start[k + 1] += start[k];
    const int64_t n_rows = b == 0 ? n : n - (start[maxc + 1] - start[maxc]);  // rows with entries (count 0 last)
    std::vector<int32_t> row(std::max<int64_t>(n_rows, 1));
    int32_t* pb = pos.data() + (size_t)b * n;
    for (int64_t r = 0; r < n; ++r) {
      const int64_t i = start[maxc - cb[r]]++;
      if (i < n_rows) {
        row[i] = (int32_t)r;
        pb[r] = (int32_t)i;
      }
    }
    B.n_rows = n_rows;
    B.n_chunks = (n_rows + 31) / 32;
    std::vector<int64_t> off(B.n_chunks + 1, 0);
    for (int64_t c = 0; c < B.n_chunks; ++c) off[c + 1] = off[c] + 32 * (int64_t)cb[row[c * 32]];
    B.slots = off[B.n_chunks];
    std::vector<int32_t> wc;
    te_sell_schedule(off, B.n_chunks, bps, real, B.grid, B.saturated, wc);
    const int64_t slots = std::max<int64_t>(B.slots, 1);
    if ((rc = te_cuda_check(te_malloc(&B.chunk_off, sizeof(int64_t) * off.size()), "column blocks")) != TE_OK ||
        (rc = te_cuda_check(te_malloc(&B.row, sizeof(int32_t) * row.size()), "column blocks")) != TE_OK ||
        (rc = te_cuda_check(te_malloc(&B.col, sizeof(int32_t) * slots), "column blocks")) != TE_OK ||
        (rc = te_cuda_check(te_malloc(&B.warp_chunk, sizeof(int32_t) * wc.size()), "column blocks")) != TE_OK)
      break;
    if (real)
      rc = te_cuda_check(te_malloc(&B.hv, sizeof(int2) * slots), "column blocks");
    else
      rc = te_cuda_check(te_malloc(&B.hv4, sizeof(int4) * slots), "column blocks");
    if (rc != TE_OK) break;
    cudaMemcpy(B.chunk_off, off.data(), sizeof(int64_t) * off.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(B.row, row.data(), sizeof(int32_t) * row.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(B.warp_chunk, wc.data(), sizeof(int32_t) * wc.size(), cudaMemcpyHostToDevice);
    // padding slots: value 0 at the block's first column
    fill_i32_kernel<<<te_grid_fit((const void*)fill_i32_kernel, slots, TE_THREADS), TE_THREADS>>>(
        slots, B.col, (int32_t)d.lo[b]);
    if (real)
      cudaMemset(B.hv, 0, sizeof(int2) * slots);
    else
      cudaMemset(B.hv4, 0, sizeof(int4) * slots);
    fill.off[b] = B.chunk_off;
    fill.col[b] = B.col;
    fill.hv[b] = B.hv;
    fill.hv4[b] = B.hv4;
  }
  if (rc == TE_OK) rc = te_cuda_check(te_malloc(&d_pos, sizeof(int32_t) * nb * n), "column blocks");
  if (rc == TE_OK)
    rc = te_cuda_check(cudaMemcpy(d_pos, pos.data(), sizeof(int32_t) * nb * n, cudaMemcpyHostToDevice),
                       "column blocks");
  if (rc == TE_OK) {
    if (real)
      block_fill_kernel<true><<<te_grid_fit((const void*)block_fill_kernel<true>, n, TE_THREADS), TE_THREADS>>>(
          n, S.chunk_off, S.col, S.fix_val, S.fix_val4, d, d_pos, fill);
    else
      block_fill_kernel<false><<<te_grid_fit((const void*)block_fill_kernel<false>, n, TE_THREADS), TE_THREADS>>>(
          n, S.chunk_off, S.col, S.fix_val, S.fix_val4, d, d_pos, fill);
    rc = te_cuda_check(cudaDeviceSynchronize(), "column blocks");
  }
  cleanup();
  if (rc != TE_OK) free_blocks(S);
  return rc;
}

}  // namespace

// One build at a time: evolvers on other host threads may share the matrix.
static std::mutex g_fixed_mutex;

int te_sell_build_fixed(te_matrix_s* A) {
  std::lock_guard<std::mutex> lock(g_fixed_mutex);
  TeSell& S = A->sell;
  if (S.fix_warp_chunk) return TE_OK;
  if (S.n_chunks < 1) {
    te_set_error("fixed-point SpMV: empty matrix");
    return TE_ERR_INVALID_ARG;
  }
  int rc = fixed_values(S, A->is_real);
  if (rc == TE_OK) rc = fixed_schedule(S, A->is_real);
  if (rc == TE_OK) rc = build_blocks(S, A->is_real);
  if (rc != TE_OK) free_fixed(S);
  return rc;
}

int te_sell_refresh_fixed(te_matrix_s* A) {
  std::lock_guard<std::mutex> lock(g_fixed_mutex);
  TeSell& S = A->sell;
  if (!S.fix_warp_chunk) return TE_OK;
  const bool was_packed = S.fix_pk != nullptr;
  const int nv = S.fix_nvals;
  int rc = fixed_values(S, A->is_real);
  // the schedule depends on the occupancy, which depends on the table size
  if (rc == TE_OK && (was_packed != (S.fix_pk != nullptr) || nv != S.fix_nvals)) rc = fixed_schedule(S, A->is_real);
  if (rc == TE_OK && S.fix_nblk > 0) {  // the blocks hold copies of the values
    free_blocks(S);
    rc = build_blocks(S, A->is_real);
  }
  if (rc != TE_OK) free_fixed(S);
  return rc;
}

void te_sell_free_fixed(TeSell& S) { free_fixed(S); }

extern "C" int te_matrix_set_fixed_blocks(te_matrix A, int n_blocks) {
  if (!A || n_blocks < 0 || n_blocks > TE_FIX_MAX_BLOCKS) {
    te_set_error("te_matrix_set_fixed_blocks: 0 (automatic), 1 (none) or 2..%d column blocks", TE_FIX_MAX_BLOCKS);
    return TE_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lock(g_fixed_mutex);
  A->sell.fix_blocks_req = n_blocks;
  free_fixed(A->sell);  // rebuilt by the next evolver run that uses it
  return TE_OK;
}
