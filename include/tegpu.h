/*
 * tegpu.h -- C ABI of the GB300 Krylov real-time evolution library (libtegpu.so).
 *
 * The library computes exp(-i * expFactor * H * t) v on one GPU, with the
 * a-posteriori error bound, step-size control and observable sampling of
 * TimeEvolver's krylovTimeEvolver, entirely in hand-written sm_103a kernels.
 * Every entry point takes plain pointers and sizes; complex numbers are
 * interleaved (re, im) doubles.  Functions return TE_OK (0) or a negative
 * TE_ERR_* code; te_last_error() describes the last failure of the calling
 * thread.  Nothing here calls exit(): the C++ drop-in layer
 * (timeevolver_gb300/host) turns the codes back into the reference's
 * behaviour.
 *
 * Reference interfaces replaced (paths inside the TimeEvolver project):
 *   TE::smatrix + initialize()        core/matrixDataTypes.h:59-99, .cpp:108-134, :196-240
 *   smatrix::spMV                      core/matrixDataTypes.cpp:169-190
 *   smatrix::norm1                     core/matrixDataTypes.cpp:67-79
 *   krylovTimeEvolver(...) ctor        core/krylovTimeEvolver.h:59-60, .cpp:26-94
 *   krylovTimeEvolver::timeEvolve()    core/krylovTimeEvolver.h:61, .cpp:261-512
 *   krylovReturn                       core/krylovTimeEvolver.h:32-51, .cpp:662-676
 *   krylovSpMatrixObservable / krylovVectorObservable::expectation
 *                                      core/krylovObservables.cpp:173-236
 *   krylovBasicObservable::expectation (user subclasses, host callback)
 *                                      core/krylovObservables.h:42
 */
#ifndef TEGPU_H
#define TEGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TEGPU_ABI_VERSION 1

/* ------------------------------------------------------------ error codes */
#define TE_OK 0
#define TE_ERR_INVALID_ARG (-1)     /* bad pointer, size or parameter */
#define TE_ERR_CUDA (-2)            /* a CUDA runtime call failed */
#define TE_ERR_EMPTY (-3)           /* "Invalid Hilbertspace dimension" (krylovTimeEvolver.cpp:39-43) */
#define TE_ERR_NOT_NORMALIZED (-4)  /* "Initial vector is not normalized" (krylovTimeEvolver.cpp:45-48) */
#define TE_ERR_NO_STEP (-5)         /* 20 halvings did not meet the tolerance (krylovTimeEvolver.cpp:203-207) */
#define TE_ERR_EIGEN (-6)           /* Krylov eigensolver did not converge (the LAPACK error of :365-370) */
#define TE_ERR_DIM (-7)             /* "Incompatible dimensions" (krylovObservables.cpp:180-184) */
#define TE_ERR_OUT_OF_MEMORY (-8)
#define TE_ERR_UNSUPPORTED (-9)     /* e.g. Krylov dimension above TE_MAX_KRYLOV */
#define TE_ERR_DEVICE_TIMEOUT (-10) /* a bounded device-side wait gave up */

#define TE_MAX_KRYLOV 64            /* largest Krylov dimension m */

/* status codes of krylovReturn::statusCode (krylovTimeEvolver.h:41-45) */
#define TE_STATUS_OK 0
#define TE_STATUS_LUCKY_BREAKDOWN 1
#define TE_STATUS_BELOW_ROUNDOFF 2
#define TE_STATUS_STOPPED 3
#define TE_STATUS_ROUNDOFF 10
#define TE_STATUS_ROUNDOFF_TOTAL 11
#define TE_STATUS_INTEGRATION 20
#define TE_STATUS_NORM 30
#define TE_STATUS_MULTIPLE 100

typedef struct te_matrix_s* te_matrix;   /* device-resident sparse matrix */
typedef struct te_evolver_s* te_evolver; /* one time evolution (krylovTimeEvolver) */

/* Description of the last error raised on the calling thread. */
const char* te_last_error(void);
int te_abi_version(void);

/* Select the CUDA device used by subsequently created objects. */
int te_set_device(int device);

/* Buffer cache.  Device buffers of at least 1 MiB (and small pinned host
 * buffers) that the library releases are kept and reused by a later request
 * of exactly the same size on the same device, so that repeated evolutions
 * of one dimension skip the driver's allocation and release.  A block is
 * cached only once the device is idle.  te_set_buffer_cache_limit caps the
 * cached device bytes (default 8 GiB; 0 disables the cache and frees what it
 * holds), te_release_buffers frees every cached block, te_buffer_cache_bytes
 * reports the cached device bytes.  A failed allocation releases the cache
 * and tries again. */
int te_set_buffer_cache_limit(int64_t device_bytes);
int te_release_buffers(void);
int64_t te_buffer_cache_bytes(void);

/* --------------------------------------------------------------- matrices */

/* Upload a COO matrix (the storage of TE::smatrix: values, columns and
 * rowIndex arrays of length nnz, size_t indices) and convert it to device
 * CSR with int32 column indices.  Entries of one row are kept in input order;
 * duplicates are kept (they add, as in the reference's COO loop).  A matrix
 * whose imaginary parts are all zero is stored with real values (same
 * results, half the value bytes and FP64 work).  Replaces smatrix(...) +
 * initialize() (matrixDataTypes.cpp:108-134, :196-240).
 * A row-sorted COO of at least 2^18 entries (the order createMatrix produces)
 * is converted on the device: where the device accesses pageable host memory
 * (Grace hosts) one kernel reads the three arrays in place, elsewhere they are
 * copied first (environment TE_COO_COPY=1 forces the copies everywhere).
 * Other input is converted on the host.  The 1-norm is the reference's
 * (column sums in entry order) either way. */
int te_matrix_create_coo(int64_t n_rows, int64_t n_cols, int64_t nnz, const uint64_t* row_index,
                         const uint64_t* columns, const double* values, te_matrix* out);

/* Upload a CSR matrix with int32 indices (row_ptr of length n_rows + 1).
 * values_complex != 0: values are nnz interleaved complex doubles, else nnz
 * real doubles. */
int te_matrix_create_csr(int64_t n_rows, int64_t n_cols, int64_t nnz, const int64_t* row_ptr,
                         const int32_t* col_idx, const double* values, int values_complex, te_matrix* out);

/* Same from a CSR already in device memory (row_ptr_dev: n_rows + 1 int32;
 * col_dev: nnz int32; values_dev: nnz complex or real doubles); the arrays are
 * copied.  The layout is built on the device; the 1-norm is accumulated in
 * 64-bit fixed point (independent of the order of the device's atomics,
 * resolution ~1e-12 of the largest |entry|) instead of the reference's
 * floating-point column sums.  No counterpart in the reference (which builds
 * every matrix on the host). */
int te_matrix_create_csr_device(int64_t n_rows, int64_t n_cols, int64_t nnz, const int32_t* row_ptr_dev,
                                const int32_t* col_dev, const double* values_dev, int values_complex,
                                te_matrix* out);

/* Synthetic load-imbalanced workload, generated on the device (no
 * counterpart in the reference): H = (A + A^H) / 2 where row r of A has k_r
 * distinct uniformly random columns, k_r drawn from the Zipf law
 * P(k) ~ k^-exponent truncated to [min_len, max_len], and entries with
 * independent N(0, 1) real and imaginary parts; H is then divided by a
 * spectral-norm estimate from power_iters power iterations (returned in
 * *norm_estimate; power_iters = 0 leaves H unscaled).  Every random number is
 * a counter-based hash of (seed, row, draw, stream), so the matrix does not
 * depend on the launch shape.  Needs n >= 4 max_len. */
int te_matrix_create_zipf(int64_t n, double exponent, int32_t min_len, int32_t max_len, uint64_t seed,
                          int32_t power_iters, double* norm_estimate, te_matrix* out);

/* Layout of a square matrix: SELL-32 slots (stored entries plus padding), and
 * the rows kept out of the chunks because they are longer than
 * max(1024, 32 x the mean row length) (multiplied warp-per-row) with their
 * entries.  No counterpart in the reference. */
int te_matrix_layout(te_matrix A, int64_t* sell_slots, int64_t* long_rows, int64_t* long_entries);

/* Merge-path segments of the long rows (no counterpart in the reference,
 * whose spMV is MKL's or a serial COO loop, matrixDataTypes.cpp:169-190): a
 * long row of k entries is k + 1 merge items; segment_items (from the long
 * rows' length histogram: at least 2048, about two segments per warp of a
 * resident wave) bounds a segment.  Rows within it are multiplied
 * warp-per-row; longer rows (split_rows of them) are split into segments of
 * equal entry counts, one warp each, whose partial sums are added in segment
 * order by the warp that finishes last (the sum does not depend on which
 * warp ran which segment).  segments = all segments of all long rows. */
int te_matrix_long_segments(te_matrix A, int64_t* segments, int64_t* split_rows, int64_t* segment_items);

/* Lanes per row of the matrix's SELL-32 SpMV passes (no counterpart in the
 * reference).  1: one lane per row (the layout's native form); 2 or 4: each
 * row's entries are split over 2 or 4 lanes of a warp, which multiplies the
 * warps in flight for matrices too small to fill the GPU.  0 (the default):
 * chosen from the matrix's shape on first use -- 2 when the matrix has at
 * least 2048 chunks of 32 rows, fewer chunks than the GPU has resident warps
 * and no long rows, else 1 -- so that the same matrix always gets the same
 * choice (it changes the summation order of a row, so results differ by
 * rounding between choices).  -1: the autotuner -- time the Lanczos pass for
 * 1, 2 and 4 on the matrix on first use and keep 2 or 4 only when more than
 * 10% faster (two copies of a matrix near that margin may be tuned
 * differently).  Setting 1, 2 or 4 pins it. */
int te_matrix_set_spmv_lanes(te_matrix A, int lanes);
/* Fixed-point form of a matrix for TE_OPT_FIXED_SPMV (no counterpart in the
 * reference), built by the first evolver that uses it: *state 0 not built,
 * 1 limbs of every slot value (8 bytes per slot for real, 16 for complex
 * values, plus the 4-byte column), 2 a value dictionary (real matrices: one
 * 4-byte word per slot, column and value index; at most 4096 distinct values
 * and 2^(32 - column bits)), 3 limbs split into column blocks (matrices
 * whose fixed-point vector, 16 bytes per row, exceeds 96 MB: each block's
 * slice of it stays in L2 during its pass); *n_values the dictionary size
 * (state 2) or the number of blocks (state 3); *scale_shift the sh of
 * round(h 2^sh). */
int te_matrix_fixed_layout(te_matrix A, int* state, int* n_values, int* scale_shift);
/* Column blocks of the fixed-point form (no counterpart in the reference):
 * 0 (default) automatic (blocks of at most 56 MB of the fixed-point vector
 * when it exceeds 96 MB), 1 none, 2..8 that many (matrices with a value
 * dictionary or long rows are never blocked).  Drops an existing fixed-point
 * form; the next evolver run that uses it builds it again. */
int te_matrix_set_fixed_blocks(te_matrix A, int n_blocks);
/* Current lanes per row (1, 2, 4), making the shape-based choice first if
 * tune_now != 0 and it is still open; a negative value is an error code. */
int te_matrix_spmv_lanes(te_matrix A, int tune_now);

/* ------------------------------------------------- models built on the GPU */

/* One operator term, as TE::opTerm (helper/hamiltonian.h): coefficient times
 * a sequence of n_ops ladder operations applied in order to the state,
 * operation +1 (creation, blocked above capacity when capacity != 0) or -1
 * (annihilation) on mode[k]; up to 8 operations. */
typedef struct te_term {
  double coef_re, coef_im;
  int32_t n_ops;
  int32_t operation[8];
  int32_t mode[8];
  int32_t capacity[8];
} te_term;

/* Matrix of sum_terms on the number-conserving basis basis(n_particles,
 * n_modes, 0, 0, quant) of helper/Basis.cpp, built on the GPU in the
 * reference's basis order and with createMatrix's rules
 * (helper/hamiltonian.cpp:318-402: terms applied per row in order, equal
 * columns merged in term order, columns ascending, |v| < DBL_EPSILON dropped),
 * so the result equals the host builder's entry for entry.  The 1-norm is the
 * reference's for Hermitian term lists.  Up to 64 modes, 255 particles, 128
 * terms; *dim receives the dimension. */
int te_model_create_device(int n_particles, int n_modes, int quant, const te_term* terms, int n_terms,
                           te_matrix* out, int64_t* dim);
/* Index of an occupation vector (n_modes ints) in that basis, -1 if it is not
 * a basis state. */
int te_model_state_index(int n_particles, int n_modes, int quant, const int32_t* occupation, int64_t* index);

/* A basis for the device builder, given by the constructor arguments of the
 * reference's bases:
 *   n_modes2 == 0: basis(n_particles, n_modes, n_qudits, capacity, quant)
 *     (helper/Basis.cpp:37-121): modes n_modes - n_qudits .. n_modes - 1 hold
 *     at most `capacity` particles; when every mode is a qudit, states whose
 *     mode 0 would exceed it are dropped;
 *   n_modes2 > 0: tensorBasis(n_particles, n_modes, n_particles2, n_modes2,
 *     capacity2) (helper/Basis.cpp:131-182): basis(n_particles, n_modes, 0, 0)
 *     times basis(n_particles2, n_modes2, n_modes2, capacity2), the first set's
 *     modes first, index i1 * dim2 + i2 (n_qudits 0 and quant 1 required). */
typedef struct te_basis_desc {
  int32_t n_particles, n_modes, n_qudits, capacity, quant;
  int32_t n_particles2, n_modes2, capacity2;
} te_basis_desc;
/* te_model_create_device on any such basis (same rules, up to 64 modes in
 * all); an empty second set of a tensor basis is rejected. */
int te_model_create_device_basis(const te_basis_desc* basis, const te_term* terms, int n_terms, te_matrix* out,
                                 int64_t* dim);
/* Index of an occupation vector (all modes) in that basis, -1 if absent. */
int te_model_basis_index(const te_basis_desc* basis, const int32_t* occupation, int64_t* index);

/* Copy a matrix's original-order CSR to host buffers: row_ptr (n_rows + 1),
 * col_idx (nnz), values (nnz interleaved complex doubles). */
int te_matrix_download_csr(te_matrix A, int32_t* row_ptr, int32_t* col_idx, double* values);

int te_matrix_destroy(te_matrix A);

/* n_rows, n_cols, nnz, flags (bit0 real values, bit1 diagonal), and the
 * reference's 1-norm (max absolute column sum, matrixDataTypes.cpp:67-79). */
int te_matrix_info(te_matrix A, int64_t* n_rows, int64_t* n_cols, int64_t* nnz, int* flags, double* norm1);

/* out = alpha * A * in on device buffers (complex n), on a CUDA stream
 * (NULL = the library's stream).  Replaces smatrix::spMV
 * (matrixDataTypes.cpp:169-190). */
int te_matrix_spmv(te_matrix A, double alpha_re, double alpha_im, const double* in_dev, double* out_dev,
                   void* cuda_stream);

/* Same with host buffers (copies in and out, synchronous). */
int te_matrix_spmv_host(te_matrix A, double alpha_re, double alpha_im, const double* in_host,
                        double* out_host);

/* te_matrix_spmv without any device allocation, for callers that cannot call
 * cudaMalloc (work recorded into CUDA graphs by stream capture, real-time
 * loops, hosts whose device memory is preallocated by another framework).
 * No counterpart in the reference.  Its scratch is a fixed array inside the
 * library (8 MiB on every GPU that loads it), so matrices are limited to
 * 262144 rows (TE_ERR_UNSUPPORTED beyond); the first call on a device looks
 * the array up and should come before any stream capture; calls whose
 * executions overlap on the GPU share the array and race. */
int te_matrix_spmv_noalloc(te_matrix A, double alpha_re, double alpha_im, const double* in_dev, double* out_dev,
                           void* cuda_stream);

/* ----------------------------------------------------------------- evolver */

/* Parameters of krylovTimeEvolver (krylovTimeEvolver.h:59; defaults of the
 * 5-argument constructor, .cpp:93-94: exp_factor 1, tol 1e-6, m 40,
 * fast_integration 0). */
typedef struct te_params {
  double t;              /* total evolution time */
  double sampling_step;  /* time between samples */
  double exp_factor;     /* exp(-i exp_factor H t) */
  double tol;            /* error bound on the final state (2-norm) */
  int32_t m;             /* Krylov dimension (clamped to the Hilbert dimension) */
  int32_t fast_integration; /* Gauss 15/7 instead of tanh-sinh */
  int32_t progress_bar;  /* accepted for API parity; the GPU path prints nothing */
  int32_t reorth;        /* 0: the reference's three-term Lanczos recurrence
                            (krylovTimeEvolver.cpp:537-546); 1: classical
                            Gram-Schmidt against all previous basis vectors
                            plus one reorthogonalisation pass (no counterpart
                            in the reference; numerically stable basis) */
} te_params;

/* Result record of one evolution (krylovReturn, krylovTimeEvolver.h:32-51). */
typedef struct te_result {
  double err;            /* accumulated analytic error bound */
  double evolved_time;   /* t_now at the end (krylovReturn::evolvedTime) */
  int64_t num_samples;   /* samples taken */
  int64_t n_steps;       /* Krylov steps */
  int64_t dim;           /* Hilbert-space dimension */
  int64_t krylov_dim;    /* Krylov dimension at the end (reduced by a lucky breakdown) */
  int32_t status;        /* TE_STATUS_* */
  int32_t nb_err_roundoff;
  int32_t nb_err_int;
  int32_t reserved;
} te_result;

/* Host callback for observables that are neither sparse matrices nor
 * vectors (user subclasses of krylovBasicObservable).  Receives the sampled
 * state on the host (complex dim) and writes the value to store; returns 0,
 * or 1 to request the stop of the evolution (requestStopException, status 3). */
typedef int (*te_observable_fn)(void* user, const double* state, int64_t dim, double* value_out);

/* Create an evolution of v (host, complex n, copied) under H.  H stays owned
 * by the caller and must outlive the evolver.  Replaces the constructor
 * (krylovTimeEvolver.cpp:26-84); returns TE_ERR_EMPTY / TE_ERR_NOT_NORMALIZED
 * where the reference exits. */
int te_evolver_create(te_matrix H, const double* v_host, const te_params* params, te_evolver* out);
int te_evolver_destroy(te_evolver ev);

/* Device-side stop condition (the requestStopException of an observable,
 * krylovTimeEvolver.cpp:423-436, without a host round trip): the evolution
 * stops at the first sample at which observable obs_index (in the order the
 * observables were added) is >= threshold (direction > 0) or <= threshold
 * (direction < 0); that sample is not counted, status 3 (0 at t = 0), as for
 * a stop requested by a callback.  Up to 4 conditions; any one stops. */
int te_evolver_add_stop_condition(te_evolver ev, int obs_index, double threshold, int direction);

/* Dense observable Re <psi|O|psi> for a complex n x n O stored column-major
 * (values: 2 n^2 doubles, the layout of TE::matrix), evaluated on the GPU for
 * every sample (krylovMatrixObservable, krylovObservables.cpp:119-138, whose
 * constructor the reference keeps private; 4 n^2 FMAs per sample, so meant for
 * small n).  O is copied to the device. */
int te_evolver_add_dense_observable(te_evolver ev, const double* values, int64_t n);

/* Observables, sampled in the order added (krylovObservables.cpp).  A
 * sparse observable stores Re <psi|O|psi>; a vector observable stores
 * |<psi|o>|^2.  O stays owned by the caller. */
int te_evolver_add_sparse_observable(te_evolver ev, te_matrix O);
int te_evolver_add_vector_observable(te_evolver ev, const double* o_host);
int te_evolver_add_callback_observable(te_evolver ev, te_observable_fn fn, void* user);

/* Run timeEvolve() (krylovTimeEvolver.cpp:261-512). */
int te_evolver_run(te_evolver ev, te_result* result);

/* Sampled values of observable obs_index (count doubles; the number of
 * samples is floor(t / sampling_step) + 1, entries past num_samples are 0). */
int te_evolver_samples(te_evolver ev, int obs_index, double* out_host, int64_t count);

/* The returned state: the last sampled state (krylovReturn::evolvedState,
 * krylovTimeEvolver.cpp:665), complex dim, to host or device memory. */
int te_evolver_state(te_evolver ev, double* out_host);
int te_evolver_state_device(te_evolver ev, const double** out_dev);

/* Per-step record, for tests and tracing: t_now, t_step, err_step, h,
 * m_eff, breakdown flag, findMaximalStepSize code, integrals evaluated. */
typedef struct te_step_record {
  double t_now, t_step, err_step, h;
  int32_t m_eff, breakdown, code, n_integrals;
} te_step_record;
int te_evolver_trace(te_evolver ev, te_step_record* out, int64_t max_records, int64_t* n_records);

/* Kernel launches issued by the last te_evolver_run (for launch accounting). */
int64_t te_evolver_launch_count(te_evolver ev);

/* The Krylov matrix of the last Krylov step, for tests and tracing (no
 * counterpart in the reference, whose Hessenberg matrix H is internal,
 * krylovTimeEvolver.cpp:523-571): the real symmetric tridiagonal T with
 * H_k = D(-iT)D^-1 (diag: m doubles, offdiag: m - 1), *m_out = m, and
 * *eig_used = 1 when that step evaluated exp(-ixT) through the eigen-
 * decomposition of T (tridiagonal QR; arguments beyond the Chebyshev-Bessel
 * series), whose m eigenvalues (unordered) are then written to eigenvalues.
 * Buffers may be NULL; m <= TE_MAX_KRYLOV. */
int te_evolver_krylov_matrix(te_evolver ev, double* diag, double* offdiag, double* eigenvalues, int32_t* m_out,
                             int32_t* eig_used);

/* Evolver options (no counterpart in the reference).
 * TE_OPT_FUSED_LANCZOS: run the three-term Lanczos iterations of a Krylov step
 * as one persistent cooperative kernel with grid barriers instead of two
 * launches per iteration (same step sequence; the norm sums round
 * differently).  0: never; 1 (default): for matrices of fewer than 2048
 * 32-row chunks, where launch costs dominate (measured on GB300: 20% faster
 * at dim 6435, equal at dim 92378, slower from dim 352716); 2: always, where
 * a cooperative launch of the matrix's schedule is possible. */
#define TE_OPT_FUSED_LANCZOS 1
/* TE_OPT_FIXED_SPMV: the SpMV of the three-term Lanczos passes in integer
 * arithmetic instead of FP64 FMAs (GB300 issues FP64 at 1/58 of its FP32
 * rate).  H's values are held as round(h 2^sh) with the largest row 1-norm R
 * (complex: of |Re h| + |Im h|) below 2^61, each Krylov vector as
 * round(u 2^xs) with a bound U on max|u| below 2^61; a row sum is accumulated
 * in int64 from int32 limb products and rounded to double once.  Error of a
 * row of k entries below (1.25 k 2^-56 + (k + 1) 2^-61) R U + 2^-53 |y| for
 * real H, (5 k 2^-56 + (2 k + 1) 2^-61) R U + 2^-53 |y| for complex H, against
 * FP64's k 2^-53 sum|h||u|.  The recurrence and all reductions stay FP64.
 * Applies to the per-iteration passes of matrices of at least 2048 32-row
 * chunks (smaller ones run the persistent FP64 kernel); see
 * te_matrix_fixed_layout for the forms (value dictionary, column blocks).
 * 0: FP64 SpMV; 1 (default): fixed point. */
#define TE_OPT_FIXED_SPMV 2
/* Options that bound or exercise the failure paths (no counterpart in the
 * reference, which exits or keeps going where these return an error):
 * TE_OPT_BARRIER_SPIN_LIMIT: polls (each a load and a short sleep) before a
 * grid-barrier wait of the persistent Lanczos kernel gives up; the run then
 * returns TE_ERR_DEVICE_TIMEOUT and the evolver can be reset and run again.
 * Default 2^22 (seconds; a co-resident grid arrives in microseconds).
 * TE_OPT_BARRIER_EXTRA_ARRIVALS: 1 makes every barrier of that kernel wait
 * for one arrival more than the grid has, so every wait gives up after the
 * spin limit: a test of the timeout path that faults nothing (default 0).
 * TE_OPT_TS_MAX_LEVEL: the deepest tanh-sinh level of the error integral
 * (2..8, default 8).  With fewer levels the quadrature misses its 1e-3
 * relative accuracy, and a step whose integral matters for the bound gets
 * code 20 (status TE_STATUS_INTEGRATION), the reference's response to a
 * quadrature that did not converge (krylovTimeEvolver.cpp:584-618).
 * TE_OPT_QR_SWEEP_LIMIT: sweeps of the tridiagonal QR eigensolve before it
 * reports TE_ERR_EIGEN (the LAPACK failure of zhseqr, matrixDataTypes.h:135-156);
 * 0 (default) 40 m + 40. */
#define TE_OPT_BARRIER_SPIN_LIMIT 3
#define TE_OPT_BARRIER_EXTRA_ARRIVALS 4
#define TE_OPT_TS_MAX_LEVEL 5
#define TE_OPT_QR_SWEEP_LIMIT 6
int te_evolver_set_option(te_evolver ev, int option, int value);

/* Prepare another run of the same evolution (same H, parameters and
 * observables, device buffers reused) from the start vector v (complex n):
 * v_is_device != 0 reads v from device memory, else from host memory.  No
 * counterpart in the reference (an evolver there runs once); it lets a caller
 * repeat evolutions without reallocating the Krylov basis. */
int te_evolver_reset(te_evolver ev, const double* v, int v_is_device);

/* The CUDA stream every kernel of this evolver is launched on (cudaStream_t). */
void* te_evolver_stream(te_evolver ev);

/* Per-kernel timing with CUDA events on the evolver's stream, accumulated over
 * the runs made while enabled.  kind: 0 Lanczos apply (SpMV + fused epilogue),
 * 1 Lanczos update, 2 Krylov-space step kernel, 3 combine (V y), 4 observable
 * reductions. */
int te_evolver_profile(te_evolver ev, int enable);
int te_evolver_kernel_time(te_evolver ev, int kind, double* total_ms, int64_t* launches);

/* ------------------------------------------------------- batched evolutions */

/* Many independent evolutions of uneven dimension advanced together: each
 * instance is a krylovTimeEvolver (own H, v, t, sampling step, tolerance,
 * Krylov dimension, step size and status), all instances share every kernel
 * launch of a Krylov step (segmented SELL-32 matrix over the concatenated
 * rows, per-instance reductions, one Krylov-space block per instance), and the
 * launches of one step are replayed as a CUDA graph.  No counterpart in the
 * reference (which runs one evolution per krylovTimeEvolver); per instance
 * the results equal those of te_evolver_run with the same inputs.
 * Restrictions: reorth 0, up to 4 diagonal observables per instance. */
typedef struct te_batch_s* te_batch;

/* H[i] (square, caller-owned, must outlive the batch), v_host[i] (complex
 * n_i, copied) and params[i] for i < n_instances. */
int te_batch_create(int n_instances, const te_matrix* H, const double* const* v_host, const te_params* params,
                    te_batch* out);
int te_batch_destroy(te_batch b);
/* A diagonal observable of one instance (Re <psi|O|psi>, krylovSpMatrixObservable). */
int te_batch_add_observable(te_batch b, int instance, te_matrix O);
/* Run every instance to its final time; results[i] as te_evolver_run (may be NULL).
 * A batch can be run again (same inputs). */
int te_batch_run(te_batch b, te_result* results);
int te_batch_samples(te_batch b, int instance, int obs_index, double* out_host, int64_t count);
int te_batch_state(te_batch b, int instance, double* out_host);
int64_t te_batch_launch_count(te_batch b);
void* te_batch_stream(te_batch b);
/* Global steps of the last te_batch_run (each: one Krylov step of every
 * running instance).  No counterpart in the reference. */
int64_t te_batch_global_steps(te_batch b);

/* Batch options (no counterpart in the reference).
 * TE_BATCH_OPT_PERSISTENT: 0 (default) replays the launches of one global step
 *   as a CUDA graph and waits for each; 1 runs the whole batch in one
 *   persistent cooperative launch (one 1024-thread block per SM, the passes
 *   separated by grid barriers with bounded waits), which gives the same
 *   results bit for bit and waits once per run.
 * TE_BATCH_OPT_BARRIER_SPIN_LIMIT: polls before a grid-barrier wait of the
 *   persistent kernel gives up (te_batch_run then returns
 *   TE_ERR_DEVICE_TIMEOUT); default 2^22. */
#define TE_BATCH_OPT_PERSISTENT 1
#define TE_BATCH_OPT_BARRIER_SPIN_LIMIT 2
/* TE_BATCH_OPT_BARRIER_EXTRA_ARRIVALS: 1 makes every grid barrier of the
 *   persistent kernel wait for one block more than the grid has, so that the
 *   first wait runs out (a test of the timeout path); default 0. */
#define TE_BATCH_OPT_BARRIER_EXTRA_ARRIVALS 3
int te_batch_set_option(te_batch b, int option, int value);

/* ------------------------------------------------------------------ adjoint */

/* Gradient of L(theta) = <psi(T)|O|psi(T)>, psi(T) = exp(-i H(theta) T) v,
 * H(theta) = sum_k theta_k H_k, by the adjoint method:
 * dL/dtheta_k = 2 Im int_0^T <lambda(s)|H_k|psi(s)> ds with the costate
 * lambda(s) = exp(+i H (T - s)) O psi(T) evolved backward on the GPU, the time
 * integral by Gauss-Legendre with nodes_per_interval nodes on every
 * checkpoint interval of length checkpoint_interval, and the bilinear forms of
 * all terms in one fused pass.  The forward evolution is krylovTimeEvolver's
 * algorithm (expFactor 1, tolerance tol, Krylov dimension m); no counterpart
 * in the reference, which has no differentiation.  The terms are copied at
 * creation; O (caller-owned) must outlive the object; v (complex n) is copied. */
typedef struct te_adjoint_s* te_adjoint;
int te_adjoint_create(int n_terms, const te_matrix* terms, te_matrix O, const double* v_host, double T, double tol,
                      int m, double checkpoint_interval, int nodes_per_interval, te_adjoint* out);
int te_adjoint_destroy(te_adjoint a);
/* loss and gradient (n_terms doubles) at theta */
int te_adjoint_run(te_adjoint a, const double* theta, double* loss, double* grad);
/* loss only: one plain forward evolution sampled at 0 and T */
int te_adjoint_forward(te_adjoint a, const double* theta, double* loss);
/* results of the last forward / backward evolutions, kernel launches of the last call, sample nodes */
int te_adjoint_stats(te_adjoint a, te_result* forward, te_result* backward, int64_t* launches, int64_t* n_nodes);
/* host wall time (ms) of the last call's phases: ms[0] coupling refresh, ms[1]
 * forward evolution, ms[2] costate evolution, ms[3] bilinear pass */
int te_adjoint_phase_times(te_adjoint a, double* ms);

#ifdef __cplusplus
}
#endif
#endif /* TEGPU_H */
