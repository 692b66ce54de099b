// te_internal.cuh -- shared declarations of the libtegpu CUDA translation units.
//
// Data layout in HBM for one evolution (n = Hilbert dimension, m = Krylov dim):
//   H in SELL-32 form, rows sorted by length (descending, stable) and the basis
//     renumbered in that order: chunk c holds rows 32c..32c+31 of the permuted
//     matrix; slot (c, k, lane) = chunk_off[c] + 32 k + lane holds the k-th
//     entry of row 32c+lane (padding: value 0, column = the row itself);
//     values double (real matrices) or double2 (complex), columns int32;
//   every n-vector (Krylov vectors, w, start vector, sampled state) is kept in
//     the permuted basis, double2 per entry, contiguous;
//   Krylov basis: u_0..u_{m-1}, unnormalised (v_j = s_j u_j, s_j = 1/beta_j);
//   TeDevState: the scalar state of the evolution (coefficients, step
//     control, sampling cursor, reduction counters), written only by kernels.
#pragma once
#include <vector>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/tegpu.h"

#define TE_MMAX 64
#define TE_THREADS 256
#define TE_SCAP 16            // samples scheduled per batch (coefficient slots)
#define TE_NCHEB 256          // largest Chebyshev degree kept for exp(-ixT) e_1
#define TE_TS_KMAX 8          // tanh-sinh refinement levels 0..8
#define TE_TS_KMIN 2
#define TE_TS_NODES 769       // nodes with t >= 0 over levels 0..8
#define TE_FUSED_DIAG 4       // diagonal observables per fused reduction pass
#define TE_FUSED_VEC 2        // vector observables per fused reduction pass
#define TE_FUSED_VALS (TE_FUSED_DIAG + 2 * TE_FUSED_VEC)

// Tanh-sinh and Gauss-Legendre tables (host-computed, uploaded once).
struct TeQuadTables {
  double ts_u[TE_TS_NODES];     // tanh(pi/2 sinh t)
  double ts_w[TE_TS_NODES];     // pi/2 cosh t / cosh^2(pi/2 sinh t)
  double ts_t[TE_TS_NODES];
  int ts_level_begin[TE_TS_KMAX + 2];
  double g15_x[15], g15_w[15];
  double g7_x[7], g7_w[7];
};

// Scalar state of one evolution, resident in device memory.
struct TeDevState {
  // constants
  double t, sampling_step, tol, tol_rate, exp_factor, num_err_est;
  int m_max, n_samples, integ_long, integ_short;
  int max_batch, pad_c0, pad_c1, pad_c2;
  // progress
  double t_now, t_sampling, err, t_step;
  int index_samples, n_steps, m_cur, status;
  int err_code_find, nb_err_roundoff, nb_err_int, fatal;  // fatal: TE_ERR_* raised on the device
  int done, stop_flag, pad_p1, pad_p2;  // stop_flag: k + 1 when a stop condition holds at batch sample k
  // current step
  double err_step, h;
  int breakdown, m_eff, step_code, n_integrals;
  int samples_in_batch, samples_pending, want_w, sample_base;
  // Lanczos coefficients of the current step
  double2 alpha[TE_MMAX];
  double beta[TE_MMAX + 1];
  double s[TE_MMAX + 1];
  // coefficients for psi = sum_j u_j y_j: slot 0 = w(t_step), slots 1.. = samples
  double2 Y[(TE_SCAP + 1) * TE_MMAX];
  double sample_dt[TE_SCAP];
  // Krylov matrix T (real symmetric tridiagonal) and its exponential data
  double d[TE_MMAX], e[TE_MMAX];
  double cheb_c, cheb_rho;
  int cheb_n, eig_valid;      // Chebyshev vectors computed up to degree cheb_n
  double eig_lam[TE_MMAX];    // eigen-decomposition T = Q diag(lam) Q^T (fallback path)
  double eig_Q[TE_MMAX * TE_MMAX];
  double cheb_t[(TE_NCHEB + 1) * TE_MMAX];  // t_n = T_n((T - c)/rho) e_1, row n
  // reduction counters ("last block finishes" pattern)
  unsigned int counter[4];
  double norm2_final;  // ||sampledState||^2 of the final norm check
  // Gram-Schmidt projections of the reorthogonalising mode (two passes)
  double2 proj1[TE_MMAX];
  double2 proj2[TE_MMAX];
  // batched evolutions: the step produced a new start vector (copied into u_0
  // at the beginning of the next step)
  int new_start;
  int pad_tail[3];
  // optional explicit sample times (ascending, sample_times[0] = 0) instead of
  // multiples of sampling_step, and an optional store for every sampled state
  // (sample k at state_store + k * store_ld, in the evolver's row order)
  const double* sample_times;
  double2* state_store;
  int64_t store_ld;
  // 1 / expFactor (0 when expFactor is 0): the folded three-term passes use
  // beta_j^2 / expFactor^2 and alpha_j / expFactor without a division per thread
  double inv_exp_factor;
  // grid barrier of the persistent Lanczos kernel (arrivals, generation)
  unsigned int bar_count, bar_gen;
  // fixed-point SpMV (te_fixed.cuh): u_j is encoded as round(u_j 2^fx_xs[j]);
  // fx_umax[j] is the high word of max |u_j| (a bound), fx_wmax the running
  // high word of max |w'| of the current apply pass
  int fx_xs[TE_MMAX + 1];
  unsigned int fx_umax[TE_MMAX + 1];
  unsigned int fx_wmax, fx_pad;
  // ||u'_j||^2 of the fixed-point copy, exactly: the sum over all rows of the
  // components' squares in units of 2^(2 fx_xs[j] - 62), as a 128-bit integer
  // {low, high} that the update pass's blocks add atomically (the order does
  // not matter) and the next apply pass reads
  unsigned long long fx_nrm[TE_MMAX + 1][2];
  // <u_j, w'> of the fixed-point apply pass j, exactly: each block's FP64 sum
  // (re, im) rounded to a signed 128-bit integer in units of 2^-fx_ak[j] (from
  // an a-priori bound of the sum, so the units are the same in every block)
  // and added atomically {re low, re high, im low, im high}; max|w'| per pass
  unsigned long long fx_alpha[TE_MMAX][4];
  int fx_ak[TE_MMAX];
  unsigned int fx_wmaxj[TE_MMAX];
  // the update pass's coefficient alpha_j s_j / g (alpha_j / expFactor when
  // folded), set with alpha_j by the apply pass
  double upd_gr, upd_gi;
  // limits set by the evolver options that exercise the failure paths (0: the
  // defaults): deepest tanh-sinh level (TE_OPT_TS_MAX_LEVEL), sweeps of the
  // tridiagonal QR (TE_OPT_QR_SWEEP_LIMIT)
  int ts_kmax, qr_sweeps;
};

#define TE_FIX_MAX_BLOCKS 8  // column blocks of the fixed-point SpMV

// SELL-32 matrix in the sorted (permuted) basis.
struct TeSell {
  int64_t n = 0;          // rows = cols
  int64_t n_chunks = 0;
  int64_t slots = 0;      // 32 * sum of chunk lengths
  int64_t* chunk_off = nullptr;
  int32_t* col = nullptr;
  double* val = nullptr;  // real: slots doubles; complex: 2*slots doubles
  int32_t* perm = nullptr;   // permuted index -> original index
  int32_t* iperm = nullptr;  // original index -> permuted index
  // Static schedule of the SpMV passes: warp w of a grid of `grid` blocks of
  // TE_THREADS owns chunks [warp_chunk[w], warp_chunk[w + 1]), contiguous
  // ranges of equal FP64 work (slots plus the per-row epilogue).
  int32_t* warp_chunk = nullptr;
  int grid = 0;
  bool saturated = false;  // the grid is capped at every SM's resident blocks
  // lanes per row of the SpMV passes (1, 2 or 4), chosen by te_tune_sell_lanes
  // or set through te_matrix_set_spmv_lanes; lanes_fixed once chosen
  int lanes = 1;
  bool lanes_fixed = false;
  bool lanes_timed = false;  // chosen by timing the variants (te_matrix_set_spmv_lanes(A, -1))
  // Long rows: rows longer than max(1024, 32 x mean length) -- the first n_long
  // rows of the sorted order -- have no slots in the chunks (one of them would
  // pad its chunk to 32 x its length); their entries form a CSR in the sorted
  // basis that the SpMV passes multiply warp-per-row.
  int64_t n_long = 0;
  int64_t* long_ptr = nullptr;  // n_long + 1
  int32_t* long_col = nullptr;  // sorted-basis columns
  double* long_val = nullptr;   // real: 1, complex: 2 doubles per entry
  // Merge-path segments of the long rows: a long row of k entries is k + 1
  // merge items (its entries and its end); rows of at most seg_items items are
  // one segment (multiplied warp-per-row), longer ones are split into
  // ceil((k + 1) / seg_items) segments of equal entry counts, one warp each.
  // seg_items comes from the long rows' length histogram (at least 2048, and
  // about two segments per warp of a resident wave).  Segment s covers entries
  // [seg_begin[s], seg_begin[s + 1]) of row seg_row[s]; row i owns segments
  // [row_seg[i], row_seg[i + 1]).  n_split rows have more than one segment.
  int64_t n_seg = 0, n_split = 0, seg_items = 0;
  int32_t* seg_row = nullptr;
  int64_t* seg_begin = nullptr;
  int32_t* row_seg = nullptr;
  // carries of the split rows owned by the matrix (te_matrix_spmv_noalloc;
  // evolvers and te_matrix_spmv use their own)
  double2* seg_part = nullptr;
  unsigned int* seg_cnt = nullptr;
  // Fixed-point copy of the chunk values (te_fixed.cuh):
  // slot value round(h 2^fix_sh) as int32 limbs {h0, h1}, built on first use
  // by te_sell_build_fixed, with its own static schedule for the fixed-point
  // apply kernel (whose resident blocks per SM differ).
  int2* fix_val = nullptr;
  int4* fix_val4 = nullptr;  // complex matrices: {Re limbs, Im limbs} per slot
  int fix_sh = 0;
  int32_t* fix_warp_chunk = nullptr;
  int fix_grid = 0;
  bool fix_saturated = false;
  // Value dictionary (matrices with few distinct values, e.g. lattice
  // Hamiltonians): instead of fix_val and col, one word per slot,
  // column | (value index << fix_cbits), and the fix_nvals distinct values
  // (ascending) as fixed-point limbs in fix_table; the apply kernel keeps the
  // table in shared memory.
  uint32_t* fix_pk = nullptr;
  int2* fix_table = nullptr;
  int fix_nvals = 0, fix_cbits = 0;
  // Column blocks (the fixed-point x larger than a share of L2): block b holds
  // the entries with columns in [b n / B, (b + 1) n / B), a slice of x that
  // stays in L2 during its pass.  Each block is a SELL over the rows with
  // entries there (block 0: all rows), sorted by their count in the block;
  // row[i] maps block row i to the main row order.  The passes add their
  // exact int64 row sums into an accumulator, one epilogue pass finishes.
  int fix_nblk = 0;
  int fix_blocks_req = 0;  // te_matrix_set_fixed_blocks: 0 automatic, 1 none, 2.. that many
  struct Block {
    int64_t n_rows = 0, n_chunks = 0, slots = 0;
    int64_t* chunk_off = nullptr;
    int32_t* row = nullptr;
    int32_t* col = nullptr;
    int2* hv = nullptr;   // real values
    int4* hv4 = nullptr;  // complex values
    int32_t* warp_chunk = nullptr;
    int grid = 0;
    bool saturated = false;
  } fix_blk[TE_FIX_MAX_BLOCKS];
};

// Carries of the split long rows for one pass: the partial sum of every
// segment and an arrival count per long row (zero between passes: the warp
// that completes a row resets its count).  Passes that may overlap on the GPU
// need their own.
struct TeSegCarry {
  double2* part = nullptr;    // n_seg
  unsigned int* cnt = nullptr;  // n_long
};
// The long rows of a SELL matrix and their segments, by value for kernels.
struct TeLongRows {
  int64_t n;
  const int64_t* ptr;
  const int32_t* col;
  const double* val;
  int64_t n_seg;
  const int32_t* seg_row;
  const int64_t* seg_begin;
  const int32_t* row_seg;
  double2* part;
  unsigned int* cnt;
};
inline TeLongRows te_long_rows(const TeSell& S, const TeSegCarry* carry = nullptr) {
  return TeLongRows{S.n_long,   S.long_ptr, S.long_col, S.long_val, S.n_seg,
                    S.seg_row,  S.seg_begin, S.row_seg,
                    carry ? carry->part : S.seg_part, carry ? carry->cnt : S.seg_cnt};
}
// Allocate (zeroed) / free carries for the split rows of S (nothing when none).
int te_seg_carry_alloc(const TeSell& S, TeSegCarry* c);
void te_seg_carry_free(TeSegCarry* c);

struct te_matrix_s {
  int64_t n_rows = 0, n_cols = 0, nnz = 0;
  bool is_real = false, is_diag = false;
  double norm1 = 0.0;
  // original-order CSR (general observables, public spmv)
  int32_t* row_ptr = nullptr;
  int32_t* col = nullptr;
  double* val = nullptr;
  double* diag_re = nullptr;  // diagonal matrices: Re of the diagonal, original order
  double2* diag_c = nullptr;  // diagonal matrices: the diagonal, original order
  TeSell sell;                // square matrices only
  int device = 0;
};

// Adopt a device CSR (int32 row pointers, columns, complex values; the matrix
// frees them) -- the device-side build of te_matrix_create_csr_device; nnz =
// d_rp[n_rows].
// norm1: the 1-norm if the caller computed it, NAN to accumulate it on the
// device in fixed point.
// out[i] = in[0] + ... + in[i - 1] for i < count, on the device (in == out
// allowed); synchronous with the default stream.
int te_scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t count);

int te_matrix_adopt_device_csr(int64_t n_rows, int64_t n_cols, int64_t nnz, int32_t* d_rp, int32_t* d_ci,
                               double2* d_v, te_matrix* out, double norm1);

// Programmatic dependent launch: a kernel launched with te_launch_pdl may be
// scheduled while its predecessor in the stream is still finishing (hiding the
// launch and block ramp); it must call te_pdl_wait() before touching anything
// the predecessor writes.  Both are no-ops for a kernel launched normally.
__device__ __forceinline__ void te_pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void te_pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// enable = false launches normally.  Measured on GB300: overlapping the launch
// pays off for kernels whose grid fills every SM's resident slots (L=12 solve
// 3% faster) and costs for smaller grids (dim 92 378: 10% slower), so callers
// enable it only for saturated grids.
template <typename... KArgs, typename... Args>
cudaError_t te_launch_pdl_smem(bool enable, void (*kernel)(KArgs...), int grid, int block, size_t smem,
                               cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
#ifdef TE_NO_PDL  // build option: plain stream-ordered launches
  cfg.numAttrs = 0;
  (void)enable;
#else
  cfg.numAttrs = enable ? 1 : 0;
#endif
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
template <typename... KArgs, typename... Args>
cudaError_t te_launch_pdl(bool enable, void (*kernel)(KArgs...), int grid, int block, cudaStream_t st,
                          Args... args) {
  return te_launch_pdl_smem(enable, kernel, grid, block, 0, st, args...);
}

// error reporting
void te_set_error(const char* fmt, ...);
int te_cuda_check(cudaError_t e, const char* what);

// Allocation through the buffer cache (te_common.cu): te_malloc / te_free
// replace cudaMalloc / cudaFree for every device buffer of the library,
// te_malloc_host / te_free_host cudaMallocHost / cudaFreeHost.
cudaError_t te_malloc_bytes(void** p, size_t bytes);
cudaError_t te_free(void* p);
cudaError_t te_malloc_host_bytes(void** p, size_t bytes);
cudaError_t te_free_host(void* p);
template <class T>
inline cudaError_t te_malloc(T** p, size_t bytes) {
  return te_malloc_bytes(reinterpret_cast<void**>(p), bytes);
}
template <class T>
inline cudaError_t te_malloc_host(T** p, size_t bytes) {
  return te_malloc_host_bytes(reinterpret_cast<void**>(p), bytes);
}
#define TE_CUDA(call)                                      \
  do {                                                     \
    int _rc = te_cuda_check((call), #call);                \
    if (_rc != TE_OK) return _rc;                          \
  } while (0)

// launch shapes
int te_num_sms();
double te_host_sumsq(const double* x, int64_t len);
int te_grid_for(int64_t n_items, int threads, int blocks_per_sm);
// Resident blocks per SM of a kernel at this block size (occupancy query, cached).
int te_kernel_blocks_per_sm(const void* kernel, int threads, size_t dyn_smem);
// Grid of a grid-stride kernel: one block per `threads` items up to one full
// wave (every SM's resident blocks), so that every SM holds the same number
// of blocks once the items exceed a wave.
int te_grid_fit(const void* kernel, int64_t n_items, int threads, size_t dyn_smem = 0);
// True when a grid-stride kernel over n_items would need more blocks than fit at once.
bool te_grid_saturated(const void* kernel, int64_t n_items, int threads, size_t dyn_smem = 0);
// Resident blocks per SM shared by the SELL SpMV passes of a matrix (the
// Lanczos apply variants and the plain SpMV), which run on one static schedule.
int te_sell_blocks_per_sm(bool is_real);

// ---------------------------------------------------------------- launches
// te_matrix.cu
void te_launch_sell_spmv(const TeSell& A, bool is_real, double2 alpha, const double2* x_perm, double2* y_perm,
                         cudaStream_t st, const TeSegCarry* carry = nullptr);
void te_launch_csr_spmv(const te_matrix_s& A, double2 alpha, const double2* x, double2* y, cudaStream_t st);
void te_launch_permute(int64_t n, const int32_t* idx, const double2* in, double2* out, cudaStream_t st);
void te_launch_permute_real(int64_t n, const int32_t* idx, const double* in, double* out, cudaStream_t st);
// te_lanczos.cu
// fold: store w / (expFactor s_j) instead of w (three-term mode with a
// non-zero expFactor; the update kernel then takes the factor into s_{j+1}).
void te_launch_lanczos_apply(const TeSell& A, bool is_real, const double2* u_j, const double2* u_jm1, double2* w,
                             TeDevState* ds, double* partials, int j, bool fold, cudaStream_t st,
                             const TeSegCarry* carry = nullptr);
// X_out (optional): also write the fixed-point copy of u_{j+1} (te_fixed.cuh)
// alpha_acc: alpha_j from the fixed-point apply pass's exact accumulator (the
// fixed-point path; X_out non-null implies it)
void te_launch_lanczos_update(int64_t n, const double2* w, const double2* u_j, double2* u_jp1, TeDevState* ds,
                              double* partials, int j, bool fold, cudaStream_t st, int4* X_out = nullptr,
                              bool alpha_acc = false);
// Fixed-point path of the folded three-term iteration (real matrices, one lane
// per row, te_sell_build_fixed done): te_launch_fix_start encodes u_0 at the
// start of a Krylov step; the apply pass reads the fixed-point copy X of u_j.
int te_sell_build_fixed(te_matrix_s* A);
// Column-blocked fixed-point apply (S.fix_nblk > 0): the block passes into
// acc (n longlong2, exact row sums), then the epilogue pass.
void te_launch_lanczos_apply_fix_blocked(const TeSell& A, bool is_real, const int4* X, longlong2* acc,
                                         const double2* u_j, const double2* u_jm1, double2* w, TeDevState* ds,
                                         double* partials, int j, cudaStream_t st);
int te_fix_block_blocks_per_sm(bool is_real);
// Resident blocks per SM of the fixed-point apply kernel (te_lanczos.cu).
// fmt: 0 real limbs, 1 real value dictionary, 2 complex limbs.
int te_apply_fix_blocks_per_sm(int fmt, size_t dyn_smem);
// Re-encode the fixed-point values after H's SELL values changed in place.
int te_sell_refresh_fixed(te_matrix_s* A);
// Frees the fixed-point form (values, dictionary, schedule, column blocks).
void te_sell_free_fixed(TeSell& S);
void te_launch_fix_start(int64_t n, const double2* u_0, int4* X, TeDevState* ds, double* partials, cudaStream_t st);
void te_launch_lanczos_apply_fix(const TeSell& A, const int4* X, const double2* u_j, const double2* u_jm1,
                                 double2* w, TeDevState* ds, double* partials, int j, cudaStream_t st,
                                 const TeSegCarry* carry = nullptr);
// Static warp schedule of the SpMV passes over the chunk offsets (host): warp w
// of grid blocks owns chunks [wc[w], wc[w + 1]) of equal estimated work.
void te_sell_schedule(const std::vector<int64_t>& off, int64_t n_chunks, int blocks_per_sm,
                      bool real, int& grid, bool& saturated, std::vector<int32_t>& wc);
// All m three-term Lanczos iterations of one Krylov step in one cooperative
// launch (te_lanczos.cu).  Returns false (nothing launched) when the matrix's
// static schedule does not fit the persistent kernel's residency, or the
// device has no cooperative launch; the caller then runs the per-iteration
// passes.  cols[j]: the basis columns of the step.
// spin_limit: polls before a grid-barrier wait gives up (TE_ERR_DEVICE_TIMEOUT);
// extra_arrivals > 0 makes every barrier wait for arrivals that never come
// (the failure-path test of TE_OPT_BARRIER_EXTRA_ARRIVALS).
bool te_launch_lanczos_step(const TeSell& A, bool is_real, double2* const* cols, int m, double2* w, TeDevState* ds,
                            double* partials, cudaStream_t st, unsigned int spin_limit, unsigned int extra_arrivals);
// Device-side stop conditions: after a batch of samples, ds->stop_flag = k + 1
// for the first sample k of the batch at which results[obs][sample] >= threshold
// (direction > 0) or <= threshold (direction < 0) for any condition (te_sample.cu).
#define TE_MAX_STOP_CONDITIONS 4
struct TeStopConds {
  int count;
  int obs[TE_MAX_STOP_CONDITIONS];
  int direction[TE_MAX_STOP_CONDITIONS];
  double threshold[TE_MAX_STOP_CONDITIONS];
};
void te_launch_stop_check(const TeStopConds& c, const double* results, int n_samples_total, TeDevState* ds,
                          cudaStream_t st);
// Re <psi|O|psi> of a dense column-major O on the original ordering (te_sample.cu).
void te_launch_dense_obs(int64_t n, const double2* O, const double2* psi_orig, TeDevState* ds, int sample_in_batch,
                         double* partials, double* results_row, cudaStream_t st);
// Choose the lanes per row of a square matrix's SpMV passes (te_lanczos.cu).
int te_tune_sell_lanes(te_matrix_s* A);
// Gram-Schmidt passes of the reorthogonalising Lanczos mode (te_lanczos.cu)
#define TE_GS_ROWS 2048  // rows per block of the Gram-Schmidt passes
struct TeBasisPtrs {
  const double2* u[TE_MMAX];
};
void te_launch_gs_project(int64_t n, const TeBasisPtrs& V, int nvec, const double2* w, TeDevState* ds,
                          double* partials, cudaStream_t st);
void te_launch_gs_update_project(int64_t n, const TeBasisPtrs& V, int nvec, double2* w, TeDevState* ds,
                                 double* partials, cudaStream_t st);
void te_launch_gs_update_norm(int64_t n, const TeBasisPtrs& V, int nvec, const double2* w, double2* u_next,
                              TeDevState* ds, double* partials, int j, cudaStream_t st);
// te_krylov.cu
int te_upload_quad_tables();
void te_launch_krylov_step(TeDevState* ds, cudaStream_t st);
void te_launch_schedule_samples(TeDevState* ds, cudaStream_t st);
void te_launch_krylov_batch(TeDevState* states, int n_instances, int mode, cudaStream_t st);
// te_sample.cu
// internal: explicit sample times and stored sampled states (te_evolver.cu)
int te_evolver_set_schedule(te_evolver ev, const double* times_host, int64_t count, double2* store_dev,
                            int64_t store_ld);
struct TeCombineArgs {
  const double2* cols[TE_MMAX];
  int m;
  int64_t n;
  double2* w_out;         // new start vector (when the step produced w)
  double2* sample_out;    // batch buffer: sample s at sample_out + s * n
  // optional fixed-point copies of the basis (te_fixed.cuh): X_j at fx + j n,
  // scale 2^fx_xs[j] in the state; the outputs are then formed in integers
  const int4* fx;
};
void te_launch_combine(const TeCombineArgs& a, TeDevState* ds, double2* last_out, cudaStream_t st);
struct TeFusedObs {
  const double* diag[TE_FUSED_DIAG];  // permuted real diagonals
  const double2* vec[TE_FUSED_VEC];   // permuted vectors
  int row_diag[TE_FUSED_DIAG];        // observable index (row of the result table)
  int row_vec[TE_FUSED_VEC];
  int n_diag, n_vec;
};
void te_launch_fused_obs(int64_t n, const double2* psi, const TeFusedObs& f, TeDevState* ds, double* partials,
                         double* results, int n_samples_total, cudaStream_t st);
void te_launch_general_obs(const te_matrix_s& O, const double2* psi_orig, TeDevState* ds, int sample_in_batch,
                           double* partials, double* results_row, cudaStream_t st);
void te_launch_norm2(int64_t n, const double2* x, double* partials, TeDevState* ds, cudaStream_t st);
