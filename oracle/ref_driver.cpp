/*
 * ref_driver.cpp -- C entry point over the reference's own krylovTimeEvolver
 * (TEST INFRASTRUCTURE ONLY).
 *
 * ref_recipe.py compiles this file together with the reference's unmodified
 * core/krylovTimeEvolver.cpp, core/matrixDataTypes.cpp,
 * core/krylovObservables.cpp and core/krylovLogger.cpp (read where they lie in
 * the reference tree) against the stand-in headers of ref_shim/ into
 * oracle/_ref/libteref.so.  With -DUSE_OPENBLAS the reference takes its own
 * serial COO loop for smatrix::spMV (core/matrixDataTypes.cpp:182-188) and
 * its own loops for expV/mulV (core/matrixDataTypes.h:108-130); BLAS-1/2 and
 * zhseqr come from numpy's OpenBLAS, the quadrature from te_quadrature.h.
 * The tests use it to check the restatement in te_oracle.cpp.
 *
 * The reference exits the process on fatal conditions
 * (krylovTimeEvolver.cpp:39-48, :203-207); this entry point rejects the
 * input conditions it can see before constructing the evolver.
 */
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "krylovTimeEvolver.h"

typedef std::complex<double> cd;

static std::unique_ptr<smatrix> coo_matrix(int64_t n, int64_t nnz, const int64_t* row, const int64_t* col,
                                           const double* val) {
  std::vector<size_t> r(nnz), c(nnz);
  std::vector<cd> x(nnz);
  for (int64_t i = 0; i < nnz; ++i) {
    r[i] = (size_t)row[i];
    c[i] = (size_t)col[i];
    x[i] = cd(val[2 * i], val[2 * i + 1]);
  }
  return std::make_unique<smatrix>(x.data(), c.data(), r.data(), (size_t)nnz, (unsigned)n, (unsigned)n);
}

/* One evolution with the reference's krylovTimeEvolver (10-argument
 * constructor, progress bar off).  Complex arrays are interleaved doubles.
 * Observable i: obs_kind[i] 0 sparse (COO obs_row/obs_col/obs_val, obs_nnz[i]
 * entries) or 1 vector (obs_val[i], n complex).  samples: n_obs x cap
 * doubles; scalars: err, evolved_time; counts: num_samples, n_steps,
 * krylov_dim, status.  Returns 0, -1 for invalid arguments, -2 for a start
 * vector that is not normalized (where the reference would exit). */
extern "C" int teref_evolve(int64_t n, int64_t nnz, const int64_t* row, const int64_t* col, const double* val,
                            const double* v, double t, double sampling_step, double exp_factor, double tol, int m,
                            int fast_integration, int n_obs, const int* obs_kind, const int64_t* obs_nnz,
                            const int64_t* const* obs_row, const int64_t* const* obs_col,
                            const double* const* obs_val, double* samples, int64_t cap, double* state,
                            double* scalars, int64_t* counts) {
  if (n <= 0 || nnz <= 0 || !row || !col || !val || !v || n_obs < 0 || m < 1) return -1;
  double nrm = 0.0;
  for (int64_t i = 0; i < 2 * n; ++i) nrm += v[i] * v[i];
  if (!(std::fabs(std::sqrt(nrm) - 1.0) <= tol)) return -2;
  std::vector<cd> vin(n);
  for (int64_t i = 0; i < n; ++i) vin[i] = cd(v[2 * i], v[2 * i + 1]);
  std::vector<std::unique_ptr<krylovBasicObservable>> obs;
  for (int k = 0; k < n_obs; ++k) {
    const std::string name = "obs" + std::to_string(k);
    if (obs_kind[k] == 0) {
      obs.push_back(std::make_unique<krylovSpMatrixObservable>(
          name, coo_matrix(n, obs_nnz[k], obs_row[k], obs_col[k], obs_val[k])));
    } else if (obs_kind[k] == 1) {
      std::vector<cd> o(n);
      for (int64_t i = 0; i < n; ++i) o[i] = cd(obs_val[k][2 * i], obs_val[k][2 * i + 1]);
      obs.push_back(std::make_unique<krylovVectorObservable>(name, o.data(), (size_t)n));
    } else {
      return -1;
    }
  }
  krylovTimeEvolver ev(t, vin.data(), sampling_step, std::move(obs), coo_matrix(n, nnz, row, col, val), exp_factor,
                       tol, m, fast_integration != 0, false);
  ev.changeLogLevel(krylovLogger::WARNING);
  std::unique_ptr<krylovReturn> ret(ev.timeEvolve());
  for (int64_t i = 0; i < n; ++i) {
    state[2 * i] = ret->evolvedState[i].real();
    state[2 * i + 1] = ret->evolvedState[i].imag();
  }
  for (int k = 0; k < n_obs; ++k) {
    const double* x = ret->observableList[k]->retExpectationValues();
    const int64_t ns = std::min<int64_t>(cap, (int64_t)ret->numSamples);
    for (int64_t s = 0; s < ns; ++s) samples[k * cap + s] = x[s];
  }
  scalars[0] = ret->err;
  scalars[1] = ret->evolvedTime;
  counts[0] = (int64_t)ret->numSamples;
  counts[1] = (int64_t)ret->n_steps;
  counts[2] = (int64_t)ret->krylovDim;
  counts[3] = ret->statusCode;
  return 0;
}
