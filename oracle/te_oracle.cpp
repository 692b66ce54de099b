/*
 * te_oracle.cpp -- CPU oracle for the Krylov real-time evolution exp(-iHt)v.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C++, the algorithm
 * of TimeEvolver's krylovTimeEvolver (core/krylovTimeEvolver.cpp) together
 * with the pieces of core/matrixDataTypes.cpp and core/krylovObservables.cpp
 * that the evolution calls.  The tests, the smoke check and the benchmark's
 * CPU-baseline leg use it to check and time the CUDA path; the product never
 * links it.
 *
 * The reference delegates three pieces of arithmetic to third-party
 * libraries that are not available here; the oracle restates them from the
 * published mathematics:
 *   - LAPACKE_zhseqr on the m x m Krylov matrix (core/matrixDataTypes.h:135-156)
 *     -> cyclic complex Jacobi on the Hermitian matrix i*H_k (the Krylov matrix
 *        of the anti-Hermitian operator -i*expFactor*H is anti-Hermitian up to
 *        rounding, so its Schur form is its eigen-decomposition);
 *   - Boost.Math tanh_sinh<double> (Boost 1.83 in the reference's CI)
 *     -> a tanh-sinh (Takahasi-Mori double-exponential) rule with level
 *        halving, tolerance test err <= tol * L1 (rule below);
 *   - Boost.Math gauss<double,15/7> -> Gauss-Legendre nodes by Newton
 *     iteration on the Legendre recurrence.
 * Parity is pinned end-to-end by the reference's golden HDF5 outputs (tests
 * compare at the reference's 1e-8 test tolerance).
 *
 * Reductions use fixed 1024-element blocks summed in order, so results do not
 * depend on the number of OpenMP threads.
 */
#include "te_oracle.h"
#include "te_quadrature.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef std::complex<double> cd;

namespace {

using namespace te_quad;
int g_ts_kmax = TS_KMAX;  // oracle_set_ts_max_level: a lower last level makes the rule miss its tolerance
const int N_BLOCK = 1024;

/* --------------------------------------------------------------- BLAS-1 */

struct CSR {
  int64_t n = 0;
  std::vector<int64_t> rowptr, col;
  std::vector<cd> val;
};

// COO -> CSR, keeping the order of entries within each row so that the
// row-parallel product equals the reference's serial COO loop
// (core/matrixDataTypes.cpp:183-188) for row-sorted input.
CSR make_csr(int64_t n, int64_t nnz, const int64_t* row, const int64_t* col, const double* val) {
  CSR A;
  A.n = n;
  A.rowptr.assign(n + 1, 0);
  for (int64_t i = 0; i < nnz; ++i) A.rowptr[row[i] + 1]++;
  for (int64_t i = 0; i < n; ++i) A.rowptr[i + 1] += A.rowptr[i];
  A.col.resize(nnz);
  A.val.resize(nnz);
  std::vector<int64_t> fill(A.rowptr.begin(), A.rowptr.end() - 1);
  for (int64_t i = 0; i < nnz; ++i) {
    int64_t p = fill[row[i]]++;
    A.col[p] = col[i];
    A.val[p] = cd(val[2 * i], val[2 * i + 1]);
  }
  return A;
}

void spmv(const CSR& A, cd alpha, const cd* in, cd* out) {
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < A.n; ++r) {
    cd acc = 0;
    for (int64_t p = A.rowptr[r]; p < A.rowptr[r + 1]; ++p) acc += alpha * A.val[p] * in[A.col[p]];
    out[r] = acc;
  }
}

// sum_i conj(x_i) y_i
cd zdotc(int64_t n, const cd* x, const cd* y) {
  int64_t nb = (n + N_BLOCK - 1) / N_BLOCK;
  std::vector<cd> part(nb);
#pragma omp parallel for schedule(static)
  for (int64_t b = 0; b < nb; ++b) {
    cd s = 0;
    int64_t e = std::min<int64_t>(n, (b + 1) * N_BLOCK);
    for (int64_t i = b * N_BLOCK; i < e; ++i) s += std::conj(x[i]) * y[i];
    part[b] = s;
  }
  cd s = 0;
  for (int64_t b = 0; b < nb; ++b) s += part[b];
  return s;
}

double dznrm2(int64_t n, const cd* x) {
  int64_t nb = (n + N_BLOCK - 1) / N_BLOCK;
  std::vector<double> part(nb);
#pragma omp parallel for schedule(static)
  for (int64_t b = 0; b < nb; ++b) {
    double s = 0;
    int64_t e = std::min<int64_t>(n, (b + 1) * N_BLOCK);
    for (int64_t i = b * N_BLOCK; i < e; ++i) s += std::norm(x[i]);
    part[b] = s;
  }
  double s = 0;
  for (int64_t b = 0; b < nb; ++b) s += part[b];
  return std::sqrt(s);
}

void zaxpy(int64_t n, cd a, const cd* x, cd* y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) y[i] += a * x[i];
}

// y = V * x, V is n x m col-major (cblas_zgemv NoTrans)
void zgemv_n(int64_t n, int m, const cd* V, const cd* x, cd* y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    cd s = 0;
    for (int j = 0; j < m; ++j) s += V[i + (int64_t)j * n] * x[j];
    y[i] = s;
  }
}

/* ------------------------------------------------------- Krylov eigen */

// Eigen-decomposition of the Krylov matrix H (m x m col-major).  The matrix
// B = i*H is Hermitian up to rounding; its Hermitian part is diagonalised by
// cyclic complex Jacobi rotations.  eigenvalues of H = -i * eig(B), with the
// same eigenvectors (columns of Z).
void krylov_eig(int m, const cd* H, cd* lambda, cd* Z) {
  std::vector<cd> B(m * m);
  const cd I(0, 1);
  for (int c = 0; c < m; ++c)
    for (int r = 0; r < m; ++r) {
      cd a = I * H[r + c * m];
      cd b = std::conj(I * H[c + r * m]);
      B[r + c * m] = 0.5 * (a + b);
    }
  for (int r = 0; r < m; ++r) B[r + r * m] = cd(B[r + r * m].real(), 0.0);
  for (int i = 0; i < m * m; ++i) Z[i] = 0;
  for (int i = 0; i < m; ++i) Z[i + i * m] = 1;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0, diag = 0;
    for (int c = 0; c < m; ++c)
      for (int r = 0; r < m; ++r) {
        if (r == c)
          diag += std::norm(B[r + c * m]);
        else
          off += std::norm(B[r + c * m]);
      }
    if (off <= 1e-34 * diag || off == 0.0) break;
    for (int p = 0; p < m - 1; ++p)
      for (int q = p + 1; q < m; ++q) {
        cd bpq = B[p + q * m];
        double r = std::abs(bpq);
        if (r == 0.0) continue;
        double app = B[p + p * m].real(), aqq = B[q + q * m].real();
        if (r < 1e-300) continue;
        cd ph = bpq / r;  // e^{i phi}
        double theta = (aqq - app) / (2.0 * r);
        double tt = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double cs = 1.0 / std::sqrt(tt * tt + 1.0), sn = tt * cs;
        // G = [[c, s], [-s e^{-i phi}, c e^{-i phi}]] acting on coordinates (p, q)
        cd g00 = cs, g01 = sn, g10 = -sn * std::conj(ph), g11 = cs * std::conj(ph);
        for (int k = 0; k < m; ++k) {  // columns: B <- B G
          cd bp = B[k + p * m], bq = B[k + q * m];
          B[k + p * m] = bp * g00 + bq * g10;
          B[k + q * m] = bp * g01 + bq * g11;
          cd zp = Z[k + p * m], zq = Z[k + q * m];
          Z[k + p * m] = zp * g00 + zq * g10;
          Z[k + q * m] = zp * g01 + zq * g11;
        }
        for (int k = 0; k < m; ++k) {  // rows: B <- G^H B
          cd bp = B[p + k * m], bq = B[q + k * m];
          B[p + k * m] = std::conj(g00) * bp + std::conj(g10) * bq;
          B[q + k * m] = std::conj(g01) * bp + std::conj(g11) * bq;
        }
        B[p + q * m] = 0;
        B[q + p * m] = 0;
        B[p + p * m] = cd(B[p + p * m].real(), 0);
        B[q + q * m] = cd(B[q + q * m].real(), 0);
      }
  }
  const cd mI(0, -1);
  for (int k = 0; k < m; ++k) lambda[k] = mI * B[k + k * m].real();
}

/* ----------------------------------------------------------- evolver */

struct Evolver {
  // inputs
  CSR H;
  double t, samplingStep, tol;
  cd expFactor;
  size_t m, Hsize;
  bool fastIntegration;
  int reorth = 0;  // 1: classical Gram-Schmidt + one reorthogonalisation pass
  double matrixNorm;
  // observables
  struct Obs {
    int kind;
    CSR O;
    std::vector<cd> vec;
    int64_t stop_at;
    std::vector<double> values;
    size_t sampleIndex = 0;
  };
  std::vector<Obs> obs;
  // state
  std::vector<cd> currentVec, sampledState, tmpBlasVec;
  size_t n_samples, index_samples = 0;
  double t_now = 0, t_sampling = 0, err = 0;
  int n_steps = 0, statusCode = 0;
  double termination = 1e-3;
  int integrationMethodLong = 2, integrationMethodShort = 2;
  int n_integrals = 0;
  std::vector<oracle_step>* trace = nullptr;

  // expKrylov (core/krylovTimeEvolver.cpp:685-702): Z (e^{x lambda} .* Z^H e1)
  void expKrylov(double x, const cd* Z, const cd* lambda, cd* out) const {
    std::vector<cd> tmp(m);
    for (size_t k = 0; k < m; ++k) tmp[k] = std::exp(lambda[k] * x) * std::conj(Z[0 + k * m]);
    for (size_t j = 0; j < m; ++j) {
      cd s = 0;
      for (size_t k = 0; k < m; ++k) s += Z[j + k * m] * tmp[k];
      out[j] = s;
    }
  }

  // integrateError (core/krylovTimeEvolver.cpp:584-618)
  double integrateError(double a, double b, const cd* Z, const cd* lambda, double h, int method,
                        double tolRate, bool& successful) {
    ++n_integrals;
    std::vector<cd> buf(m);
    auto f = [&](double x) {
      expKrylov(x, Z, lambda, buf.data());
      return h * std::abs(buf[m - 1]);
    };
    double ret, error = 0;
    bool success = true;
    if (method == 0) {
      ret = gauss_rule(gauss15(), f, a, b);
    } else if (method == 1) {
      ret = gauss_rule(gauss7(), f, a, b);
    } else {
      TSResult r = tanh_sinh(f, a, b, termination, g_ts_kmax);
      if (r.nonfinite) {
        // the reference replaces a failed quadrature by 10*tol (:601-605)
        ret = tol * 10;
        error = 0;
      } else {
        ret = r.value;
        error = r.err;
      }
      if (error / ret > termination && ret > termination * (b - a) * tolRate) success = false;
    }
    successful = successful && success;
    return ret;
  }

  // findMaximalStepSize (core/krylovTimeEvolver.cpp:153-254); returns -1 when
  // GO_MAX halvings did not meet the tolerance (the reference exits there).
  int findMaximalStepSize(const cd* T, const cd* spectrumH, double h, double tolRate, double t_stepSuggestion,
                          double t_step_max, int n_substeps, double numericalErrorEstimate, bool increaseStep,
                          double* t_stepRet, cd* w_KrylovRet, double* err_stepRet) {
    const unsigned GO_MAX = 20;
    unsigned nbReductions = 0;
    double t_step = t_stepSuggestion;
    int code = 0;
    bool ok = true;
    bool skipSubsteps = false;
    if (t_step > t_step_max) {
      t_step = t_step_max;
      skipSubsteps = true;
    }
    double err_step = integrateError(0, t_step, T, spectrumH, h, integrationMethodLong, tolRate, ok);
    if (increaseStep && !skipSubsteps) {
      double err_new = err_step, t_new = t_step;
      while (err_new < tolRate * t_new && t_step < t_step_max) {
        t_step = t_new;
        err_step = err_new;
        if (t_step >= t_step_max) {
          skipSubsteps = true;
          break;
        }
        t_new *= 2;
        if (t_new > t_step_max) t_new = t_step_max;
        err_new = integrateError(0, t_new, T, spectrumH, h, integrationMethodLong, tolRate, ok);
      }
    }
    while (err_step > tolRate * t_step) {
      nbReductions++;
      t_step = t_step / 2.0;
      err_step = integrateError(0, t_step, T, spectrumH, h, integrationMethodLong, tolRate, ok);
      if (nbReductions == GO_MAX) return -1;
      skipSubsteps = false;
    }
    double s = t_step / n_substeps;
    int n_s = 0;
    double deltaError = 0;
    if (!skipSubsteps) {
      while (err_step + deltaError < tolRate * (t_step + n_s * s)) {
        err_step += deltaError;
        n_s++;
        if (t_step + (n_s - 1) * s >= t_step_max) break;
        deltaError = integrateError(t_step + (n_s - 1) * s, t_step + n_s * s, T, spectrumH, h,
                                    integrationMethodShort, tolRate, ok);
      }
      t_step += (n_s - 1) * s;
    }
    if (err_step < numericalErrorEstimate) {
      if (!skipSubsteps || err_step > 0.1 * tolRate * t_step) code += 1;
    }
    if (!ok) code += 20;
    *t_stepRet = t_step;
    *err_stepRet = err_step;
    expKrylov(t_step, T, spectrumH, w_KrylovRet);
    return code;
  }

  // arnoldiAlgorithm (core/krylovTimeEvolver.cpp:523-571); with reorth != 0
  // the three-term update is replaced by classical Gram-Schmidt against all
  // previous vectors plus one reorthogonalisation pass (CGS2), keeping the
  // tridiagonal coefficients H[j,j] = p1_j + p2_j and beta = ||w||.
  bool lanczos(double tolRate, std::vector<cd>& Hm, std::vector<cd>& V, double* hRet, size_t* mRet) {
    const int64_t n = (int64_t)Hsize;
    std::copy(currentVec.begin(), currentVec.end(), V.begin());
    for (size_t j = 0; j < m; ++j) {
      cd* vj = V.data() + j * n;
      spmv(H, expFactor, vj, tmpBlasVec.data());
      if (reorth) {
        std::vector<cd> p1(j + 1), p2(j + 1);
        for (size_t i = 0; i <= j; ++i) p1[i] = zdotc(n, V.data() + i * n, tmpBlasVec.data());
        for (size_t i = 0; i <= j; ++i) zaxpy(n, -p1[i], V.data() + i * n, tmpBlasVec.data());
        for (size_t i = 0; i <= j; ++i) p2[i] = zdotc(n, V.data() + i * n, tmpBlasVec.data());
        for (size_t i = 0; i <= j; ++i) zaxpy(n, -p2[i], V.data() + i * n, tmpBlasVec.data());
        Hm[j + j * m] = p1[j] + p2[j];
      } else {
      if (j != 0) {
        cd negH = -1.0 * Hm[j - 1 + j * m];
        zaxpy(n, negH, V.data() + (j - 1) * n, tmpBlasVec.data());
      }
      Hm[j + j * m] = zdotc(n, vj, tmpBlasVec.data());
      zaxpy(n, -1.0 * Hm[j + j * m], vj, tmpBlasVec.data());
      }
      double normy = dznrm2(n, tmpBlasVec.data());
      if (normy < tolRate) {
        *mRet = j + 1;
        *hRet = normy;
        return true;
      }
      if (j + 1 != m) {
        Hm[j + (j + 1) * m] = cd(-normy, Hm[j + (j + 1) * m].imag());
        Hm[j + 1 + j * m] = cd(normy, Hm[j + 1 + j * m].imag());
        double inv = 1.0 / normy;
        cd* vn = V.data() + (j + 1) * n;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) vn[i] = tmpBlasVec[i] * inv;
      } else {
        *hRet = normy;
      }
    }
    *mRet = m;
    return false;
  }

  // sample (core/krylovTimeEvolver.cpp:120-126) with the observable kinds of
  // core/krylovObservables.cpp:173-236.  Returns false when an observable
  // requested the stop (requestStopException).
  bool sample() {
    const int64_t n = (int64_t)Hsize;
    for (auto& o : obs) {
      if (o.kind == ORACLE_OBS_STOP) {
        if ((int64_t)index_samples == o.stop_at) return false;
        continue;
      }
      cd val;
      if (o.kind == ORACLE_OBS_SPARSE) {
        spmv(o.O, cd(1, 0), sampledState.data(), tmpBlasVec.data());
        val = zdotc(n, sampledState.data(), tmpBlasVec.data());
        if (o.sampleIndex < o.values.size()) o.values[o.sampleIndex] = val.real();
      } else {
        cd d = zdotc(n, sampledState.data(), o.vec.data());
        if (o.sampleIndex < o.values.size()) o.values[o.sampleIndex] = std::norm(d);
      }
      o.sampleIndex++;
    }
    index_samples++;
    return true;
  }

  // timeEvolve (core/krylovTimeEvolver.cpp:261-512)
  int timeEvolve(int* nbErrRoundOffOut, int* nbErrIntOut) {
    const int N_SUBSTEPS = 50;
    const double INITIAL_STEP_FRACTION = 0.97;
    if (fastIntegration) {
      integrationMethodLong = 0;
      integrationMethodShort = 1;
    } else {
      integrationMethodLong = integrationMethodShort = 2;
    }
    double t_step = 1.0 / 10.0;
    double tolRate = tol / t;
    double numericalErrorEstimate = Hsize * matrixNorm * DBL_EPSILON;
    double numericalErrorEstimateTotal = 0;
    size_t m_hbd = m;
    int errorCodeFindSubstep = 0;
    int nbErrRoundOff = 0, nbErrInt = 0, nbErrors = 0;
    *nbErrRoundOffOut = *nbErrIntOut = 0;

    if (!sample()) return 0;  // stop requested at t = 0: status stays 0 (:306-313)

    const int64_t n = (int64_t)Hsize;
    std::vector<cd> Hm(m * m), V(n * m), eig(m), Z(m * m), w1(m), w2(m);
    double h = 0;
    while (index_samples < n_samples) {
      n_steps++;
      double err_step = 0;
      n_integrals = 0;
      double t_now_step = t_now;
      std::fill(Hm.begin(), Hm.end(), cd(0, 0));
      bool hbd = lanczos(tolRate, Hm, V, &h, &m_hbd);
      if (hbd) {
        t_step = t - t_now;
        std::vector<cd> Ht(m_hbd * m_hbd);
        for (size_t c = 0; c < m_hbd; ++c)
          for (size_t r = 0; r < m_hbd; ++r) Ht[r + c * m_hbd] = Hm[r + c * m];
        Hm = Ht;
        V.resize(n * m_hbd);
        m = m_hbd;
        eig.resize(m);
        Z.resize(m * m);
        w1.resize(m);
        w2.resize(m);
        statusCode = 1;
      }
      krylov_eig((int)m, Hm.data(), eig.data(), Z.data());
      if (!hbd) {
        double s_0 = INITIAL_STEP_FRACTION * t_step;
        errorCodeFindSubstep = findMaximalStepSize(Z.data(), eig.data(), h, tolRate, s_0, t - t_now, N_SUBSTEPS,
                                                   numericalErrorEstimate, t_now == 0, &t_step, w1.data(),
                                                   &err_step);
        if (errorCodeFindSubstep < 0) return -3;
        zgemv_n(n, (int)m, V.data(), w1.data(), currentVec.data());
      }
      switch (errorCodeFindSubstep) {
        case 1: nbErrRoundOff++; break;
        case 20: nbErrInt++; break;
        case 21: nbErrInt++; nbErrRoundOff++; break;
        default: break;
      }
      if (trace) {
        oracle_step rec;
        rec.t_now = t_now_step;
        rec.t_step = t_step;
        rec.err_step = err_step;
        rec.h = h;
        rec.m_eff = (int32_t)m;
        rec.breakdown = hbd ? 1 : 0;
        rec.code = hbd ? 0 : errorCodeFindSubstep;
        rec.n_integrals = n_integrals;
        trace->push_back(rec);
      }
      // sampling (:405-437)
      while (index_samples < n_samples &&
             (t_sampling + samplingStep <= t_now + t_step ||
              (index_samples == n_samples - 1 && std::fabs(t_now + t_step - t) <= DBL_EPSILON))) {
        t_sampling += samplingStep;
        for (size_t k = 0; k < m; ++k) w1[k] = std::exp(eig[k] * (t_sampling - t_now));
        for (size_t k = 0; k < m; ++k) w2[k] = std::conj(Z[0 + k * m]) * w1[k];
        for (size_t j = 0; j < m; ++j) {
          cd s = 0;
          for (size_t k = 0; k < m; ++k) s += Z[j + k * m] * w2[k];
          w1[j] = s;
        }
        zgemv_n(n, (int)m, V.data(), w1.data(), sampledState.data());
        if (!sample()) {
          statusCode = 3;
          *nbErrRoundOffOut = nbErrRoundOff;
          *nbErrIntOut = nbErrInt;
          return 0;
        }
      }
      t_now += t_step;
      err += err_step;
    }
    if (std::fabs(dznrm2(n, sampledState.data()) - 1.0) > tol) {
      nbErrors++;
      statusCode = 30;
    }
    numericalErrorEstimateTotal = numericalErrorEstimate * n_steps;
    if (nbErrRoundOff != 0) {
      nbErrors++;
      statusCode = 10;
    }
    if (nbErrInt != 0) {
      nbErrors++;
      statusCode = 20;
    }
    if (numericalErrorEstimateTotal > err && nbErrRoundOff == 0) {
      if (numericalErrorEstimateTotal > tol) {
        statusCode = 11;
        nbErrors++;
      } else if (statusCode != 1) {
        statusCode = 2;
      }
    }
    if (nbErrors > 1) statusCode = 100;
    *nbErrRoundOffOut = nbErrRoundOff;
    *nbErrIntOut = nbErrInt;
    return 0;
  }
};

double norm1_coo(int64_t n, int64_t nnz, const int64_t* col, const double* val) {
  std::vector<double> colVal(n, 0.0);
  for (int64_t i = 0; i < nnz; ++i) colVal[col[i]] += std::abs(cd(val[2 * i], val[2 * i + 1]));
  return n ? *std::max_element(colVal.begin(), colVal.end()) : 0.0;
}

}  // namespace

/* ------------------------------------------------------------- C ABI */

extern "C" int oracle_evolve(int64_t n, int64_t nnz, const int64_t* row, const int64_t* col, const double* val,
                             const double* v, double t, double sampling_step, double exp_factor, double tol,
                             int m, int fast_integration, int reorth, int n_obs, const oracle_obs* obs,
                             double* samples, double* state_out, oracle_result* result, oracle_step* trace,
                             int64_t max_trace, int64_t* n_trace, int n_threads) {
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#else
  (void)n_threads;
#endif
  if (n <= 0) return -1;  // "Invalid Hilbertspace dimension" (:39-43)
  const cd* vin = reinterpret_cast<const cd*>(v);
  if (std::fabs(dznrm2(n, vin) - 1.0) > tol) return -2;  // "Initial vector is not normalized" (:45-48)
  Evolver E;
  E.H = make_csr(n, nnz, row, col, val);
  E.t = t;
  E.samplingStep = sampling_step;
  E.tol = tol;
  E.expFactor = cd(0, -1 * exp_factor);
  E.fastIntegration = fast_integration != 0;
  E.reorth = reorth;
  E.matrixNorm = norm1_coo(n, nnz, col, val);
  E.Hsize = (size_t)n;
  E.m = std::min<size_t>((size_t)m, E.Hsize);
  E.n_samples = (size_t)std::floor(t / sampling_step) + 1;
  E.currentVec.assign(vin, vin + n);
  E.sampledState.assign(vin, vin + n);
  E.tmpBlasVec.assign(n, cd(0, 0));
  for (int i = 0; i < n_obs; ++i) {
    Evolver::Obs o;
    o.kind = obs[i].kind;
    o.stop_at = obs[i].stop_at;
    if (o.kind == ORACLE_OBS_SPARSE) {
      o.O = make_csr(n, obs[i].nnz, obs[i].row, obs[i].col, obs[i].val);
    } else if (o.kind == ORACLE_OBS_VECTOR) {
      const cd* p = reinterpret_cast<const cd*>(obs[i].val);
      o.vec.assign(p, p + n);
    }
    if (o.kind != ORACLE_OBS_STOP) o.values.assign(E.n_samples, 0.0);
    E.obs.push_back(std::move(o));
  }
  std::vector<oracle_step> tr;
  if (trace) E.trace = &tr;
  int rcErr = 0, rcInt = 0;
  int rc = E.timeEvolve(&rcErr, &rcInt);
  if (rc != 0) return rc;
  if (samples) {
    int oi = 0;
    for (auto& o : E.obs) {
      if (o.kind == ORACLE_OBS_STOP) continue;
      std::memcpy(samples + (size_t)oi * E.n_samples, o.values.data(), sizeof(double) * E.n_samples);
      ++oi;
    }
  }
  if (state_out) std::memcpy(state_out, E.sampledState.data(), sizeof(cd) * n);
  if (result) {
    result->err = E.err;
    result->evolved_time = E.t_now;
    result->num_samples = (int64_t)E.index_samples;
    result->n_steps = E.n_steps;
    result->dim = n;
    result->krylov_dim = (int64_t)E.m;
    result->status = E.statusCode;
    result->nb_err_roundoff = rcErr;
    result->nb_err_int = rcInt;
    result->pad = 0;
  }
  if (trace) {
    int64_t k = std::min<int64_t>(max_trace, (int64_t)tr.size());
    std::memcpy(trace, tr.data(), sizeof(oracle_step) * k);
    if (n_trace) *n_trace = (int64_t)tr.size();
  } else if (n_trace) {
    *n_trace = 0;
  }
  return 0;
}

extern "C" int oracle_spmv(int64_t n, int64_t nnz, const int64_t* row, const int64_t* col, const double* val,
                           double alpha_re, double alpha_im, const double* in, double* out) {
  CSR A = make_csr(n, nnz, row, col, val);
  spmv(A, cd(alpha_re, alpha_im), reinterpret_cast<const cd*>(in), reinterpret_cast<cd*>(out));
  return 0;
}

extern "C" double oracle_norm1(int64_t n, int64_t nnz, const int64_t* col, const double* val) {
  return norm1_coo(n, nnz, col, val);
}

extern "C" int oracle_lanczos(int64_t n, int64_t nnz, const int64_t* row, const int64_t* col, const double* val,
                              const double* v, double exp_factor, double tol_rate, int m, double* H_out,
                              double* V_out, double* h_out, int64_t* m_hbd_out) {
  Evolver E;
  E.H = make_csr(n, nnz, row, col, val);
  E.expFactor = cd(0, -1 * exp_factor);
  E.Hsize = (size_t)n;
  E.m = (size_t)m;
  const cd* vin = reinterpret_cast<const cd*>(v);
  E.currentVec.assign(vin, vin + n);
  E.tmpBlasVec.assign(n, cd(0, 0));
  std::vector<cd> Hm(m * m, cd(0, 0)), V((size_t)n * m);
  double h = 0;
  size_t mh = m;
  bool hbd = E.lanczos(tol_rate, Hm, V, &h, &mh);
  std::memcpy(H_out, Hm.data(), sizeof(cd) * m * m);
  if (V_out) std::memcpy(V_out, V.data(), sizeof(cd) * V.size());
  *h_out = h;
  *m_hbd_out = (int64_t)mh;
  return hbd ? 1 : 0;
}

extern "C" int oracle_krylov_eig(int m, const double* H, double* eigenvalues, double* Z) {
  krylov_eig(m, reinterpret_cast<const cd*>(H), reinterpret_cast<cd*>(eigenvalues), reinterpret_cast<cd*>(Z));
  return 0;
}

extern "C" double oracle_integrate_error(int m, const double* eigenvalues, const double* Z, double h, double a,
                                         double b, int method, double tol_rate, double tol, int* success) {
  Evolver E;
  E.m = (size_t)m;
  E.tol = tol;
  bool ok = true;
  double r = E.integrateError(a, b, reinterpret_cast<const cd*>(Z), reinterpret_cast<const cd*>(eigenvalues), h,
                              method, tol_rate, ok);
  *success = ok ? 1 : 0;
  return r;
}

extern "C" int oracle_find_step(int m, const double* eigenvalues, const double* Z, double h, double tol_rate,
                                double t_step_suggestion, double t_step_max, int n_substeps,
                                double numerical_error_estimate, int increase_step, int fast_integration,
                                double tol, double* t_step_out, double* w_out, double* err_step_out,
                                int* n_integrals_out) {
  Evolver E;
  E.m = (size_t)m;
  E.tol = tol;
  E.fastIntegration = fast_integration != 0;
  E.integrationMethodLong = fast_integration ? 0 : 2;
  E.integrationMethodShort = fast_integration ? 1 : 2;
  int code = E.findMaximalStepSize(reinterpret_cast<const cd*>(Z), reinterpret_cast<const cd*>(eigenvalues), h,
                                   tol_rate, t_step_suggestion, t_step_max, n_substeps, numerical_error_estimate,
                                   increase_step != 0, t_step_out, reinterpret_cast<cd*>(w_out), err_step_out);
  if (n_integrals_out) *n_integrals_out = E.n_integrals;
  return code;
}

extern "C" double oracle_ts_test(int kind, double p, double a, double b, double tol, double* err, double* l1,
                                 int* levels) {
  auto f = [&](double x) {
    if (kind == 0) return std::pow(x, p);
    if (kind == 1) return std::cos(p * x);
    return std::exp(p * x);
  };
  TSResult r = tanh_sinh(f, a, b, tol, g_ts_kmax);
  if (err) *err = r.err;
  if (l1) *l1 = r.l1;
  if (levels) *levels = r.levels;
  return r.value;
}

// Last tanh-sinh level (2..8) of every later integral; the failure-path tests
// set it low so that the quadrature reports a miss (status 20).
extern "C" void oracle_set_ts_max_level(int level) {
  g_ts_kmax = level < TS_KMIN ? TS_KMIN : level > TS_KMAX ? TS_KMAX : level;
}
