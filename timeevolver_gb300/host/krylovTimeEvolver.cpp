// krylovTimeEvolver.cpp -- C++ drop-in over the GPU evolution.
//
// Constructor: core/krylovTimeEvolver.cpp:26-94 (argument handling, the
// exit(1) checks of :39-48, n_samples of :57, observable result arrays).
// timeEvolve: hands H, v and the observables to te_evolver_* (tegpu.h) and
// rebuilds krylovReturn (:662-676).  Sparse-matrix and vector observables are
// evaluated on the GPU; any other observable is called back on the host with
// the sampled state, and a requestStopException it throws stops the evolution
// (status 3, as :423-436).
#include "krylovTimeEvolver.h"

#include <cmath>
#include <cstdlib>

krylovReturn::krylovReturn(unsigned int Hsize, int status) {
  err = 0;
  n_steps = 0;
  krylovDim = 0;
  dim = Hsize;
  statusCode = status;
  evolvedTime = 0;
  numSamples = 0;
  evolvedState = new std::complex<double>[Hsize];
}

krylovReturn::~krylovReturn() { delete[] evolvedState; }

krylovTimeEvolver::krylovTimeEvolver(double t, std::complex<double>* v, double samplingStep,
                                     std::vector<std::unique_ptr<krylovBasicObservable>> observables,
                                     std::unique_ptr<smatrix> Ham, double expFactor, double tol, int mm,
                                     bool fastIntegration, bool progressBar) {
  this->t = t;
  this->samplingStep = samplingStep;
  this->tol = tol;
  this->progressBar = progressBar;
  this->Ham = std::move(Ham);
  this->expFactor = std::complex<double>(0, -1 * expFactor);
  this->fastIntegration = fastIntegration;
  this->nbObservables = (int)observables.size();
  this->Hsize = this->Ham->m;
  this->m = std::min<size_t>(mm, Hsize);
  if (Hsize == 0) {
    logger.log_message(krylovLogger::FATAL, "Invalid Hilbertspace dimension");
    exit(1);
  }
  double nrm = 0;
  for (size_t i = 0; i < Hsize; ++i) nrm += std::norm(v[i]);
  if (std::abs(std::sqrt(nrm) - 1.0) > tol) {
    logger.log_message(krylovLogger::FATAL, "Initial vector is not normalized");
    exit(1);
  }
  this->Ham->initialize();
  n_samples = (size_t)floor(t / samplingStep) + 1;
  initial.assign(v, v + Hsize);
  obsVector = std::move(observables);
  for (auto& o : obsVector) o->initializeResultArray(n_samples);
}

krylovTimeEvolver::krylovTimeEvolver(double t, std::complex<double>* v, double samplingStep,
                                     std::vector<std::unique_ptr<krylovBasicObservable>> observables,
                                     std::unique_ptr<smatrix> Ham)
    : krylovTimeEvolver(t, v, samplingStep, std::move(observables), std::move(Ham), 1.0, 1e-6, 40, false, false) {}

krylovTimeEvolver::~krylovTimeEvolver() { obsVector.clear(); }

void krylovTimeEvolver::changeLogLevel(krylovLogger::loggingLevel level) { logger.set_loggingLevel(level); }

namespace {

struct CallbackCtx {
  krylovBasicObservable* obs;
  std::vector<std::complex<double>> buf;
};

// host observable: the reference calls expectation(sampledState, Hsize); a
// requestStopException becomes a stop request
int host_observable(void* user, const double* state, int64_t dim, double* value_out) {
  CallbackCtx* c = static_cast<CallbackCtx*>(user);
  const std::complex<double>* s = reinterpret_cast<const std::complex<double>*>(state);
  c->buf.assign(s, s + dim);
  try {
    std::complex<double> r = c->obs->expectation(c->buf.data(), (int)dim);
    *value_out = r.real();
  } catch (requestStopException&) {
    return 1;
  }
  return 0;
}

}  // namespace

krylovReturn* krylovTimeEvolver::timeEvolve() {
  if (fastIntegration)
    logger.log_message(krylovLogger::WARNING,
                       "Please note that a less accurate method for evaluating the error integral was used. We "
                       "recommend recomputing with accurate integration to establish the validity of the result.");
  te_matrix H = Ham->device();
  if (!H) {
    logger.log_message(krylovLogger::FATAL, "spMV error ");
    exit(1);
  }
  te_params p{};
  p.t = t;
  p.sampling_step = samplingStep;
  p.exp_factor = -expFactor.imag();
  p.tol = tol;
  p.m = (int32_t)m;
  p.fast_integration = fastIntegration ? 1 : 0;
  p.progress_bar = progressBar ? 1 : 0;
  te_evolver ev = nullptr;
  int rc = te_evolver_create(H, reinterpret_cast<const double*>(initial.data()), &p, &ev);
  if (rc != TE_OK) {
    logger.log_message(krylovLogger::FATAL, te_last_error());
    exit(1);
  }
  // observables in order; the GPU-evaluated ones store their values after the run
  std::vector<CallbackCtx> ctx(obsVector.size());
  std::vector<int> gpu_kind(obsVector.size(), 0);  // 1 = values come from the GPU table
  for (size_t i = 0; i < obsVector.size(); ++i) {
    krylovBasicObservable* o = obsVector[i].get();
    if (auto* sp = dynamic_cast<krylovSpMatrixObservable*>(o)) {
      te_matrix Od = sp->matrixPtr()->device();
      rc = Od ? te_evolver_add_sparse_observable(ev, Od) : TE_ERR_INVALID_ARG;
      gpu_kind[i] = 1;
    } else if (auto* vo = dynamic_cast<krylovVectorObservable*>(o)) {
      rc = te_evolver_add_vector_observable(ev, reinterpret_cast<const double*>(vo->data()));
      gpu_kind[i] = 1;
    } else {
      ctx[i].obs = o;
      rc = te_evolver_add_callback_observable(ev, host_observable, &ctx[i]);
    }
    if (rc != TE_OK) {
      logger.log_message(krylovLogger::FATAL, std::string("Incompatible dimensions: ") + te_last_error());
      exit(1);
    }
  }
  te_result res{};
  rc = te_evolver_run(ev, &res);
  if (rc != TE_OK) {
    logger.log_message(krylovLogger::FATAL, std::string("Error: ") + te_last_error());
    exit(1);
  }
  krylovReturn* ret = new krylovReturn((unsigned int)Hsize, res.status);
  te_evolver_state(ev, reinterpret_cast<double*>(ret->evolvedState));
  std::vector<double> buf(n_samples);
  for (size_t i = 0; i < obsVector.size(); ++i) {
    krylovBasicObservable* o = obsVector[i].get();
    if (gpu_kind[i]) {
      te_evolver_samples(ev, (int)i, buf.data(), (int64_t)n_samples);
      for (size_t k = 0; k < n_samples; ++k) o->expectationValues[k] = buf[k];
      o->sampleIndex = (size_t)res.num_samples;
    }
  }
  switch (res.status) {
    case 10:
    case 100:
      logger.log_message(krylovLogger::WARNING,
                         "CRITICAL WARNING: The computed error bound was smaller than the estimate of the numerical "
                         "error in " + std::to_string(res.nb_err_roundoff) + " Krylov spaces.");
      break;
    case 20:
      logger.log_message(krylovLogger::WARNING,
                         "CRITICAL WARNING: The error of numerical integration did not meet the required accuracy "
                         "in " + std::to_string(res.nb_err_int) + " Krylov spaces.");
      break;
    case 30:
      logger.log_message(krylovLogger::WARNING, "CRITICAL WARNING: Norm of state vector is not inside specified tolerance.");
      break;
    default:
      break;
  }
  ret->n_steps = (size_t)res.n_steps;
  ret->err = res.err;
  ret->dim = Hsize;
  ret->krylovDim = (size_t)res.krylov_dim;
  m = (size_t)res.krylov_dim;
  ret->evolvedTime = res.evolved_time;
  ret->numSamples = (size_t)res.num_samples;
  te_evolver_destroy(ev);
  ret->observableList = std::move(obsVector);
  ret->hamiltonianMatrix = std::move(Ham);
  return ret;
}
