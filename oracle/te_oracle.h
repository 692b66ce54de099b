/*
 * te_oracle.h -- C ABI of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * The oracle is a plain C++ restatement of TimeEvolver's Krylov real-time
 * evolution (core/krylovTimeEvolver.cpp, core/matrixDataTypes.cpp,
 * core/krylovObservables.cpp).  It exists to check the CUDA path: only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it.
 * The product library never links or calls it.
 *
 * Parity pin: the full pipeline reproduces the reference's golden outputs
 * (output/ResultBlackHole_N20_*.h5, output/ResultBlackHole_N1_*.h5) within
 * the reference's own 1e-8 test tolerance (test/testBlackHole.cpp:39-44).
 *
 * Complex arrays are interleaved (re, im) doubles.
 */
#ifndef TE_ORACLE_H
#define TE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Observable kinds understood by oracle_evolve. */
enum { ORACLE_OBS_SPARSE = 0, ORACLE_OBS_VECTOR = 1, ORACLE_OBS_STOP = 2 };

typedef struct oracle_obs {
  int kind;              /* ORACLE_OBS_* */
  int64_t nnz;           /* sparse: number of COO entries */
  const int64_t* row;    /* sparse: COO rows */
  const int64_t* col;    /* sparse: COO columns */
  const double* val;     /* sparse: complex values; vector: complex vector of length n */
  int64_t stop_at;       /* stop: throw the stop request when sampling this sample index */
} oracle_obs;

typedef struct oracle_result {
  double err;
  double evolved_time;
  int64_t num_samples;
  int64_t n_steps;
  int64_t dim;
  int64_t krylov_dim;
  int32_t status;
  int32_t nb_err_roundoff;
  int32_t nb_err_int;
  int32_t pad;
} oracle_result;

/* One record per Krylov step. */
typedef struct oracle_step {
  double t_now;        /* time at the start of the step */
  double t_step;
  double err_step;
  double h;            /* last Lanczos norm */
  int32_t m_eff;       /* Krylov dimension used (m_hbd on breakdown) */
  int32_t breakdown;
  int32_t code;        /* findMaximalStepSize return code */
  int32_t n_integrals; /* error integrals evaluated */
} oracle_step;

/* Full evolution, restating krylovTimeEvolver(...) + timeEvolve().
 * reorth != 0 replaces the three-term Lanczos update by classical
 * Gram-Schmidt with one reorthogonalisation pass (the GPU's stable mode).
 * samples: n_obs * n_samples_total doubles (row per observable), may be NULL.
 * state_out: complex n (the last sampled state), may be NULL.
 * trace: up to max_trace step records (may be NULL); *n_trace receives the count.
 * Returns 0 on success, a negative code on invalid input (the reference
 * would exit(1) there). */
int oracle_evolve(int64_t n, int64_t nnz, const int64_t* row, const int64_t* col, const double* val,
                  const double* v, double t, double sampling_step, double exp_factor, double tol,
                  int m, int fast_integration, int reorth, int n_obs, const oracle_obs* obs, double* samples,
                  double* state_out, oracle_result* result, oracle_step* trace, int64_t max_trace,
                  int64_t* n_trace, int n_threads);

/* out = alpha * H * in for a COO matrix (core/matrixDataTypes.cpp:182-188). */
int oracle_spmv(int64_t n, int64_t nnz, const int64_t* row, const int64_t* col, const double* val,
                double alpha_re, double alpha_im, const double* in, double* out);

/* Maximum absolute column sum (core/matrixDataTypes.cpp:67-79). */
double oracle_norm1(int64_t n, int64_t nnz, const int64_t* col, const double* val);

/* One Lanczos pass (core/krylovTimeEvolver.cpp:523-571) from the normalised
 * start vector v.  H_out: complex m*m col-major; V_out: complex n*m
 * col-major (may be NULL).  Returns 1 on lucky breakdown, 0 otherwise. */
int oracle_lanczos(int64_t n, int64_t nnz, const int64_t* row, const int64_t* col, const double* val,
                   const double* v, double exp_factor, double tol_rate, int m, double* H_out,
                   double* V_out, double* h_out, int64_t* m_hbd_out);

/* Eigen-decomposition of the m*m Krylov matrix H (complex col-major):
 * eigenvalues (complex m) and eigenvectors Z (complex m*m col-major). */
int oracle_krylov_eig(int m, const double* H, double* eigenvalues, double* Z);

/* Error integral of core/krylovTimeEvolver.cpp:584-618 for a decomposed
 * Krylov matrix.  method 0/1 = Gauss 15/7, 2 = tanh-sinh.  Returns the
 * integral; *success receives the accuracy flag. */
double oracle_integrate_error(int m, const double* eigenvalues, const double* Z, double h, double a,
                              double b, int method, double tol_rate, double tol, int* success);

/* findMaximalStepSize (core/krylovTimeEvolver.cpp:153-254).  w_out: complex m. */
int oracle_find_step(int m, const double* eigenvalues, const double* Z, double h, double tol_rate,
                     double t_step_suggestion, double t_step_max, int n_substeps,
                     double numerical_error_estimate, int increase_step, int fast_integration,
                     double tol, double* t_step_out, double* w_out, double* err_step_out,
                     int* n_integrals_out);

/* Tanh-sinh quadrature of a built-in test integrand (kind 0: x^p, 1: cos(p x),
 * 2: exp(p x)) -- checks the quadrature rule in isolation. */
double oracle_ts_test(int kind, double p, double a, double b, double tol, double* err, double* l1,
                      int* levels);

/* Last tanh-sinh level (2..8, default 8) of every later integral; below 8 the
 * rule gives up earlier, which the failure-path tests use to reach status 20. */
void oracle_set_ts_max_level(int level);

#ifdef __cplusplus
}
#endif
#endif
