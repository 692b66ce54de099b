// te_evolver.cu -- host orchestration of one time evolution and its C ABI.
//
// Replaces the krylovTimeEvolver constructor (core/krylovTimeEvolver.cpp:26-84)
// and timeEvolve() (:261-512).  The control flow of the reference's main loop
// runs on the device (Lanczos coefficients, step-size search, sampling cursor
// and status counters live in TeDevState); the host only enqueues one Krylov
// step at a time (2m Lanczos passes, one Krylov-space kernel, one combine
// pass, one observable pass), reads back a few scalars and decides whether a
// further sample batch or step is needed.  Observables that cannot be fused
// (non-diagonal sparse matrices, host callbacks) are evaluated per sample.
#include <cfloat>
#include <cstddef>
#include <cmath>
#include <cstring>
#include <vector>

#include "te_internal.cuh"

namespace {

struct HostObs {
  int kind;  // 0 fused diagonal, 1 fused vector, 2 general sparse, 3 callback, 4 dense
  te_matrix O = nullptr;
  double2* dense = nullptr;      // dense: column-major n x n (original order)
  double* diag_perm = nullptr;   // fused diagonal (permuted, Re)
  double2* vec_perm = nullptr;   // fused vector (permuted)
  te_observable_fn fn = nullptr;
  void* user = nullptr;
};

// Scalars read back after every batch (prefix of TeDevState).
struct Summary {
  double t, sampling_step, tol, tol_rate, exp_factor, num_err_est;
  int m_max, n_samples, integ_long, integ_short;
  int max_batch, pad_c0, pad_c1, pad_c2;
  double t_now, t_sampling, err, t_step;
  int index_samples, n_steps, m_cur, status;
  int err_code_find, nb_err_roundoff, nb_err_int, fatal;
  int done, stop_flag, pad_p1, pad_p2;
  double err_step, h;
  int breakdown, m_eff, step_code, n_integrals;
  int samples_in_batch, samples_pending, want_w, sample_base;
};
static_assert(sizeof(Summary) == offsetof(TeDevState, alpha), "summary must mirror the TeDevState prefix");

}  // namespace

struct te_evolver_s {
  te_matrix H = nullptr;
  int device = 0;
  cudaStream_t st = nullptr;
  te_params p{};
  int64_t n = 0;
  int m = 0;
  int64_t n_samples = 0;
  TeDevState* ds = nullptr;
  Summary* sum = nullptr;  // pinned
  double2* slab = nullptr;  // m basis columns + spare start vector + w + sampled state
  double2* cols[TE_MMAX + 1] = {};
  double2* spare = nullptr;
  double2* w = nullptr;
  double2* sampled = nullptr;
  double2* batch = nullptr;  // max_batch samples
  double2* orig_tmp = nullptr;  // original-order copy for general/callback observables
  double* partials = nullptr;
  double* results = nullptr;  // n_obs x n_samples
  int max_batch = 1;
  int fused_lanczos = 1;  // TE_OPT_FUSED_LANCZOS: 0 never, 1 automatic, 2 always
  int fixed_spmv = 1;     // TE_OPT_FIXED_SPMV: 0 FP64 SpMV, 1 fixed-point SpMV
  unsigned int barrier_spins = 1u << 22;  // TE_OPT_BARRIER_SPIN_LIMIT (~seconds of polling)
  unsigned int barrier_extra = 0;         // TE_OPT_BARRIER_EXTRA_ARRIVALS
  int ts_max_level = 0;                   // TE_OPT_TS_MAX_LEVEL (0: 8)
  int qr_sweeps = 0;                      // TE_OPT_QR_SWEEP_LIMIT (0: 40 m + 40)
  int4* X = nullptr;      // fixed-point copies of the Krylov vectors (m x n rows)
  longlong2* fx_acc = nullptr;  // column-blocked fixed-point SpMV: exact row sums (n rows)
  TeSegCarry seg;               // carries of H's split long rows (this evolver's passes)
  int batch_cap = 0;         // states the batch buffer holds
  size_t results_cap = 0;    // doubles the results buffer holds
  std::vector<HostObs> obs;
  TeStopConds stops{};  // device-side stop conditions
  std::vector<te_step_record> trace;
  te_result res{};
  bool ran = false;
  int64_t launches = 0;
  double2* host_state = nullptr;  // pinned buffer for callbacks
  double* sample_times = nullptr;  // explicit sample times (device), optional
  double2* state_store = nullptr;  // store for every sampled state (caller-owned), optional
  int64_t store_ld = 0;
  // per-kernel event timing
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, int>> pending;  // (kind, first event index) of recorded pairs
  size_t ev_used = 0;
  double kernel_ms[5] = {0, 0, 0, 0, 0};
  int64_t kernel_n[5] = {0, 0, 0, 0, 0};
};

namespace {

const size_t kPartials = (size_t)TE_SCAP * TE_FUSED_VALS * 8 * 1024;

// Event pair around one launch when profiling (no-op otherwise).
struct ProfScope {
  te_evolver ev;
  int kind;
  int idx = -1;
  ProfScope(te_evolver e, int k) : ev(e), kind(k) {
    if (!ev->profiling) return;
    while (ev->ev_pool.size() < ev->ev_used + 2) {
      cudaEvent_t x;
      cudaEventCreate(&x);
      ev->ev_pool.push_back(x);
    }
    idx = (int)ev->ev_used;
    ev->ev_used += 2;
    cudaEventRecord(ev->ev_pool[idx], ev->st);
  }
  ~ProfScope() {
    if (idx < 0) return;
    cudaEventRecord(ev->ev_pool[idx + 1], ev->st);
    ev->pending.emplace_back(kind, idx);
  }
};

// Fold the completed event pairs into the per-kind totals (after a sync).
void collect_profile(te_evolver ev) {
  for (auto& p : ev->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ev->ev_pool[p.second], ev->ev_pool[p.second + 1]) == cudaSuccess) {
      ev->kernel_ms[p.first] += ms;
      ev->kernel_n[p.first] += 1;
    }
  }
  ev->pending.clear();
  ev->ev_used = 0;
}

int read_summary(te_evolver ev) {
  TE_CUDA(cudaMemcpyAsync(ev->sum, ev->ds, sizeof(Summary), cudaMemcpyDeviceToHost, ev->st));
  TE_CUDA(cudaStreamSynchronize(ev->st));
  if (ev->profiling) collect_profile(ev);
  return TE_OK;
}

// Observables of the current batch: fused reductions on the device, then the
// per-sample general / callback observables.  *stop_at receives the batch
// index of a stop request (or -1).
int process_batch(te_evolver ev, int* stop_at, bool synced) {
  *stop_at = -1;
  // fused passes (up to TE_FUSED_DIAG diagonal + TE_FUSED_VEC vector observables per pass)
  std::vector<const HostObs*> dg, vc;
  std::vector<int> dgi, vci;
  for (size_t i = 0; i < ev->obs.size(); ++i) {
    if (ev->obs[i].kind == 0) {
      dg.push_back(&ev->obs[i]);
      dgi.push_back((int)i);
    } else if (ev->obs[i].kind == 1) {
      vc.push_back(&ev->obs[i]);
      vci.push_back((int)i);
    }
  }
  size_t id = 0, iv = 0;
  while (id < dg.size() || iv < vc.size()) {
    TeFusedObs f{};
    while (id < dg.size() && f.n_diag < TE_FUSED_DIAG) {
      f.diag[f.n_diag] = dg[id]->diag_perm;
      f.row_diag[f.n_diag++] = dgi[id];
      ++id;
    }
    while (iv < vc.size() && f.n_vec < TE_FUSED_VEC) {
      f.vec[f.n_vec] = vc[iv]->vec_perm;
      f.row_vec[f.n_vec++] = vci[iv];
      ++iv;
    }
    {
      ProfScope ps(ev, 4);
      te_launch_fused_obs(ev->n, ev->batch, f, ev->ds, ev->partials, ev->results, (int)ev->n_samples, ev->st);
    }
    ++ev->launches;
  }
  bool need_host = false;
  for (auto& o : ev->obs) need_host |= (o.kind == 2 || o.kind == 3 || o.kind == 4);
  if (!need_host) {
    if (ev->stops.count) {
      te_launch_stop_check(ev->stops, ev->results, (int)ev->n_samples, ev->ds, ev->st);
      ++ev->launches;
    }
    return TE_OK;
  }
  if (!synced) {
    int rc = read_summary(ev);
    if (rc != TE_OK) return rc;
  }
  const int S = ev->sum->samples_in_batch;
  for (int s = 0; s < S; ++s) {
    te_launch_permute(ev->n, ev->H->sell.iperm, ev->batch + (int64_t)s * ev->n, ev->orig_tmp, ev->st);
    ++ev->launches;
    for (size_t i = 0; i < ev->obs.size(); ++i) {
      HostObs& o = ev->obs[i];
      if (o.kind == 2) {
        te_launch_general_obs(*o.O, ev->orig_tmp, ev->ds, s, ev->partials, ev->results + i * ev->n_samples, ev->st);
        ++ev->launches;
      } else if (o.kind == 4) {
        te_launch_dense_obs(ev->n, o.dense, ev->orig_tmp, ev->ds, s, ev->partials, ev->results + i * ev->n_samples,
                            ev->st);
        ++ev->launches;
      } else if (o.kind == 3) {
        TE_CUDA(cudaMemcpyAsync(ev->host_state, ev->orig_tmp, sizeof(double2) * ev->n, cudaMemcpyDeviceToHost,
                                ev->st));
        TE_CUDA(cudaStreamSynchronize(ev->st));
        double value = 0.0;
        int stop = o.fn(o.user, reinterpret_cast<const double*>(ev->host_state), ev->n, &value);
        if (stop) {
          *stop_at = s;
          return TE_OK;
        }
        TE_CUDA(cudaMemcpyAsync(ev->results + i * ev->n_samples + ev->sum->sample_base + s, &value, sizeof(double),
                                cudaMemcpyHostToDevice, ev->st));
        TE_CUDA(cudaStreamSynchronize(ev->st));
      }
    }
  }
  if (ev->stops.count) {
    te_launch_stop_check(ev->stops, ev->results, (int)ev->n_samples, ev->ds, ev->st);
    ++ev->launches;
  }
  return TE_OK;
}

void free_evolver(te_evolver ev) {
  if (!ev) return;
  te_free(ev->ds);
  te_free_host(ev->sum);
  te_free_host(ev->host_state);
  te_free(ev->slab);
  te_free(ev->X);
  te_seg_carry_free(&ev->seg);
  te_free(ev->fx_acc);
  te_free(ev->batch);
  te_free(ev->orig_tmp);
  te_free(ev->partials);
  te_free(ev->results);
  te_free(ev->sample_times);
  for (auto& o : ev->obs) {
    te_free(o.diag_perm);
    te_free(o.vec_perm);
    te_free(o.dense);
  }
  for (auto e : ev->ev_pool) cudaEventDestroy(e);
  if (ev->st) cudaStreamDestroy(ev->st);
  delete ev;
}

// Sample results, zeroed for every run; the buffer is kept while it is large enough.
int alloc_results(te_evolver ev) {
  size_t count = std::max<size_t>(1, ev->obs.size()) * (size_t)ev->n_samples;
  if (count > ev->results_cap) {
    te_free(ev->results);
    ev->results = nullptr;
    ev->results_cap = 0;
    TE_CUDA(te_malloc(&ev->results, sizeof(double) * count));
    ev->results_cap = count;
  }
  TE_CUDA(cudaMemsetAsync(ev->results, 0, sizeof(double) * count, ev->st));
  return TE_OK;
}

int run(te_evolver ev, te_result* out) {
  const int64_t n = ev->n;
  cudaStream_t st = ev->st;
  ev->launches = 0;
  ev->trace.clear();
  bool need_host = false;
  for (auto& o : ev->obs) need_host |= (o.kind == 2 || o.kind == 3 || o.kind == 4);
  ev->max_batch = need_host ? 1 : (int)std::max<int64_t>(1, std::min<int64_t>(TE_SCAP, ((int64_t)256 << 20) / (16 * n)));
  if (ev->max_batch > ev->batch_cap) {  // kept across runs while large enough
    te_free(ev->batch);
    ev->batch = nullptr;
    ev->batch_cap = 0;
    TE_CUDA(te_malloc(&ev->batch, sizeof(double2) * n * ev->max_batch));
    ev->batch_cap = ev->max_batch;
  }
  int rc = alloc_results(ev);
  if (rc != TE_OK) return rc;

  // ---- initial device state (constructor + the first lines of timeEvolve)
  TeDevState* hs = new TeDevState();
  std::memset(hs, 0, sizeof(TeDevState));
  hs->t = ev->p.t;
  hs->sampling_step = ev->p.sampling_step;
  hs->tol = ev->p.tol;
  hs->tol_rate = ev->p.tol / ev->p.t;                                            // :287
  hs->exp_factor = ev->p.exp_factor;
  hs->inv_exp_factor = ev->p.exp_factor != 0.0 ? 1.0 / ev->p.exp_factor : 0.0;
  hs->num_err_est = (double)n * ev->H->norm1 * DBL_EPSILON;                      // :289
  hs->m_max = ev->m;
  hs->n_samples = (int)ev->n_samples;
  hs->integ_long = ev->p.fast_integration ? 0 : 2;                               // :269-277
  hs->integ_short = ev->p.fast_integration ? 1 : 2;
  hs->max_batch = ev->max_batch;
  hs->t_step = 0.1;                                                              // :285
  hs->m_cur = ev->m;
  hs->m_eff = ev->m;
  hs->s[0] = 1.0;
  // initial sample (:306-313): psi = v, one output with coefficient 1 on u_0
  hs->samples_in_batch = 1;
  hs->sample_base = 0;
  hs->index_samples = 1;
  hs->want_w = 0;
  hs->Y[1 * TE_MMAX + 0] = make_double2(1.0, 0.0);
  hs->n_steps = ev->n_samples > 1 ? 1 : 0;
  hs->done = ev->n_samples > 1 ? 0 : 1;
  hs->sample_times = ev->sample_times;
  hs->state_store = ev->state_store;
  hs->store_ld = ev->store_ld;
  hs->ts_kmax = ev->ts_max_level;
  hs->qr_sweeps = ev->qr_sweeps;
  rc = te_cuda_check(cudaMemcpyAsync(ev->ds, hs, sizeof(TeDevState), cudaMemcpyHostToDevice, st), "state upload");
  TE_CUDA(cudaStreamSynchronize(st));
  delete hs;
  if (rc != TE_OK) return rc;

  TeCombineArgs ca{};
  ca.n = n;
  ca.w_out = ev->spare;
  ca.sample_out = ev->batch;
  ca.m = 1;
  ca.cols[0] = ev->cols[0];
  te_launch_combine(ca, ev->ds, ev->sampled, st);
  ++ev->launches;
  int stop_at = -1;
  rc = process_batch(ev, &stop_at, false);
  if (rc != TE_OK) return rc;
  TE_CUDA(cudaGetLastError());
  rc = read_summary(ev);
  if (rc != TE_OK) return rc;
  Summary* S = ev->sum;
  if (stop_at < 0 && S->stop_flag) stop_at = S->stop_flag - 1;
  te_result r{};
  r.dim = n;
  if (stop_at >= 0) {  // stop requested at t = 0: plain return, status 0 (:309-313)
    r.krylov_dim = ev->m;
    r.num_samples = 0;
    *out = r;
    return TE_OK;
  }

  int m = ev->m;
  double err_prev = 0.0, t_prev = 0.0;
  int64_t guard = 0;
  // fixed-point SpMV in the folded three-term passes (te_fixed.cuh) for
  // matrices large enough for the per-iteration passes
  // (its own schedule, one lane per row); otherwise the FP64 passes, whose
  // lanes per row are tuned once per matrix on first use
  bool fix = ev->fixed_spmv != 0 && ev->p.reorth == 0 && ev->p.exp_factor != 0.0 &&
             ev->H->sell.n_chunks >= 2048 && ev->fused_lanczos != 2;
  if (fix) {
    // the fixed-point form and its vectors; without memory for them the
    // evolution runs the FP64 passes instead
    rc = te_sell_build_fixed(ev->H);
    if (rc == TE_OK && !ev->X) rc = te_cuda_check(te_malloc(&ev->X, sizeof(int4) * n * ev->m), "fixed-point basis");
    if (rc == TE_OK && ev->H->sell.fix_nblk > 0 && !ev->fx_acc)
      rc = te_cuda_check(te_malloc(&ev->fx_acc, sizeof(longlong2) * n), "fixed-point sums");
    if (rc == TE_ERR_OUT_OF_MEMORY) {
      cudaGetLastError();
      fix = false;
    } else if (rc != TE_OK) {
      return rc;
    }
  }
  if (!fix && (rc = te_tune_sell_lanes(ev->H)) != TE_OK) return rc;
  while (!S->done) {
    if (S->fatal) break;
    if (++guard > ((int64_t)1 << 40)) break;
    t_prev = S->t_now;
    err_prev = S->err;
    // STEP 1: Lanczos (:338)
    const bool cgs2 = ev->p.reorth != 0;
    const bool fold = !cgs2 && ev->p.exp_factor != 0.0;
    bool fused = false;
    // all m iterations in one persistent launch: measured faster than the
    // per-iteration passes only while launch costs dominate (dim 6435: -20%;
    // dim 92378: equal; dim >= 352716: slower), hence the automatic size rule
    const bool want_fused = ev->fused_lanczos == 2 || (ev->fused_lanczos == 1 && ev->H->sell.n_chunks < 2048);
    if (fold && want_fused) {
      ProfScope ps(ev, 0);
      fused = te_launch_lanczos_step(ev->H->sell, ev->H->is_real, ev->cols, m, ev->w, ev->ds, ev->partials, st,
                                     ev->barrier_spins, ev->barrier_extra);
      if (fused) ++ev->launches;
    }
    const bool fix_step = fix && fold && !fused;
    if (fix_step) {
      ProfScope ps(ev, 3);
      te_launch_fix_start(n, ev->cols[0], ev->X, ev->ds, ev->partials, st);
      ev->launches += 2;
    }
    for (int j = 0; j < m && !fused; ++j) {
      {
        ProfScope ps(ev, 0);
        if (fix_step && ev->H->sell.fix_nblk > 0) {
          te_launch_lanczos_apply_fix_blocked(ev->H->sell, ev->H->is_real, ev->X + (int64_t)j * n, ev->fx_acc,
                                              ev->cols[j], j > 0 ? ev->cols[j - 1] : nullptr, ev->w, ev->ds,
                                              ev->partials, j, st);
          ev->launches += ev->H->sell.fix_nblk;  // the block passes before the epilogue
        } else if (fix_step) {
          te_launch_lanczos_apply_fix(ev->H->sell, ev->X + (int64_t)j * n, ev->cols[j],
                                      j > 0 ? ev->cols[j - 1] : nullptr, ev->w, ev->ds, ev->partials, j, st, &ev->seg);
        }
        else
          te_launch_lanczos_apply(ev->H->sell, ev->H->is_real, ev->cols[j],
                                  (j > 0 && !cgs2) ? ev->cols[j - 1] : nullptr, ev->w, ev->ds, ev->partials, j, fold,
                                  st, &ev->seg);
      }
      if (!cgs2) {
        ProfScope ps(ev, 1);
        te_launch_lanczos_update(n, ev->w, ev->cols[j], j + 1 < m ? ev->cols[j + 1] : nullptr, ev->ds, ev->partials,
                                 j, fold, st, fix_step && j + 1 < m ? ev->X + (int64_t)(j + 1) * n : nullptr,
                                 fix_step);
        ev->launches += 2;
      } else {
        // classical Gram-Schmidt against u_0..u_j, then one reorthogonalisation pass
        TeBasisPtrs V{};
        for (int i = 0; i <= j; ++i) V.u[i] = ev->cols[i];
        ProfScope ps(ev, 1);
        te_launch_gs_project(n, V, j + 1, ev->w, ev->ds, ev->partials, st);
        te_launch_gs_update_project(n, V, j + 1, ev->w, ev->ds, ev->partials, st);
        te_launch_gs_update_norm(n, V, j + 1, ev->w, j + 1 < m ? ev->cols[j + 1] : nullptr, ev->ds, ev->partials, j,
                                 st);
        ev->launches += 4;
      }
    }
    // STEP 1b-3: Krylov-space kernel (eigen data, step search, w, first batch)
    {
      ProfScope ps(ev, 2);
      te_launch_krylov_step(ev->ds, st);
    }
    ++ev->launches;
    for (int j = 0; j < m; ++j) ca.cols[j] = ev->cols[j];
    ca.m = m;
    ca.w_out = ev->spare;
    ca.fx = fix_step ? ev->X : nullptr;  // the basis's fixed-point copies, this step
    {
      ProfScope ps(ev, 3);
      te_launch_combine(ca, ev->ds, ev->sampled, st);
    }
    ++ev->launches;
    rc = process_batch(ev, &stop_at, false);
    if (rc != TE_OK) return rc;
    rc = read_summary(ev);
    if (rc != TE_OK) return rc;
    if (stop_at < 0 && S->stop_flag) stop_at = S->stop_flag - 1;
    if (S->fatal) break;
    // the combine pass above used the step's own m (m_eff on a breakdown)
    te_step_record rec{};
    rec.t_now = t_prev;
    rec.t_step = S->t_step;
    rec.err_step = S->err_step;
    rec.h = S->h;
    rec.m_eff = S->m_eff;
    rec.breakdown = S->breakdown;
    rec.code = S->breakdown ? 0 : S->err_code_find;
    rec.n_integrals = S->n_integrals;
    ev->trace.push_back(rec);
    const bool produced_w = S->want_w != 0;
    while (stop_at < 0 && S->samples_pending && !S->fatal) {
      {
        ProfScope ps(ev, 2);
        te_launch_schedule_samples(ev->ds, st);
      }
      ++ev->launches;
      ca.w_out = ev->spare;
      {
        ProfScope ps(ev, 3);
        te_launch_combine(ca, ev->ds, ev->sampled, st);
      }
      ++ev->launches;
      rc = process_batch(ev, &stop_at, false);
      if (rc != TE_OK) return rc;
      rc = read_summary(ev);
      if (rc != TE_OK) return rc;
      if (stop_at < 0 && S->stop_flag) stop_at = S->stop_flag - 1;
    }
    if (S->fatal) break;
    if (stop_at >= 0) {
      // stopped by an observable (:423-436): status 3, time and error of the step start
      r.err = err_prev;
      r.evolved_time = t_prev;
      r.num_samples = S->sample_base + stop_at;
      r.n_steps = S->n_steps;
      r.krylov_dim = S->m_cur;
      r.status = TE_STATUS_STOPPED;
      r.nb_err_roundoff = S->nb_err_roundoff;
      r.nb_err_int = S->nb_err_int;
      *out = r;
      return TE_OK;
    }
    if (produced_w) std::swap(ev->cols[0], ev->spare);
    m = S->m_cur;
  }
  if (S->fatal) {
    te_set_error("device-side failure %d during the evolution (%s)", S->fatal,
                 S->fatal == TE_ERR_NO_STEP              ? "no small enough time step found to meet the tolerance"
                 : S->fatal == TE_ERR_EIGEN              ? "Krylov eigensolver did not converge"
                 : S->fatal == TE_ERR_DEVICE_TIMEOUT     ? "a grid-barrier wait of the persistent Lanczos kernel gave up"
                                                         : "step search limit");
    return S->fatal;
  }
  // final checks (:445-504)
  te_launch_norm2(n, ev->sampled, ev->partials, ev->ds, st);
  ++ev->launches;
  double norm2 = 0.0;
  TE_CUDA(cudaMemcpyAsync(&norm2, &ev->ds->norm2_final, sizeof(double), cudaMemcpyDeviceToHost, st));
  TE_CUDA(cudaStreamSynchronize(st));
  int status = S->status;
  int nbErrors = 0;
  if (std::fabs(std::sqrt(norm2) - 1.0) > ev->p.tol) {
    nbErrors++;
    status = TE_STATUS_NORM;
  }
  const double numErrTotal = S->num_err_est * S->n_steps;
  if (S->nb_err_roundoff != 0) {
    nbErrors++;
    status = TE_STATUS_ROUNDOFF;
  }
  if (S->nb_err_int != 0) {
    nbErrors++;
    status = TE_STATUS_INTEGRATION;
  }
  if (numErrTotal > S->err && S->nb_err_roundoff == 0) {
    if (numErrTotal > ev->p.tol) {
      status = TE_STATUS_ROUNDOFF_TOTAL;
      nbErrors++;
    } else if (status != TE_STATUS_LUCKY_BREAKDOWN) {
      status = TE_STATUS_BELOW_ROUNDOFF;
    }
  }
  if (nbErrors > 1) status = TE_STATUS_MULTIPLE;
  r.err = S->err;
  r.evolved_time = S->t_now;
  r.num_samples = S->index_samples;
  r.n_steps = S->n_steps;
  r.krylov_dim = S->m_cur;
  r.status = status;
  r.nb_err_roundoff = S->nb_err_roundoff;
  r.nb_err_int = S->nb_err_int;
  *out = r;
  return TE_OK;
}

}  // namespace

// ------------------------------------------------------------------ C ABI

extern "C" int te_evolver_create(te_matrix H, const double* v_host, const te_params* params, te_evolver* out) {
  if (!H || !v_host || !params || !out) {
    te_set_error("te_evolver_create: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  if (H->n_rows == 0) {
    te_set_error("Invalid Hilbertspace dimension");
    return TE_ERR_EMPTY;
  }
  if (H->n_rows != H->n_cols) {
    te_set_error("te_evolver_create: the Hamiltonian must be square");
    return TE_ERR_INVALID_ARG;
  }
  const te_params& p = *params;
  if (!(p.t > 0.0) || !(p.sampling_step > 0.0) || !(p.tol > 0.0) || p.m < 1 || !std::isfinite(p.exp_factor) ||
      p.reorth < 0 || p.reorth > 1) {
    te_set_error("te_evolver_create: t, sampling_step, tol must be positive, m >= 1, reorth 0 or 1");
    return TE_ERR_INVALID_ARG;
  }
  const int64_t n = H->n_rows;
  const int m = (int)std::min<int64_t>(p.m, n);  // :35
  if (m > TE_MMAX) {
    te_set_error("te_evolver_create: Krylov dimension %d above the supported %d", m, TE_MMAX);
    return TE_ERR_UNSUPPORTED;
  }
  // normalisation check (:45-48), host-side on the caller's vector
  const double nrm = te_host_sumsq(v_host, 2 * n);
  if (!(std::fabs(std::sqrt(nrm) - 1.0) <= p.tol)) {  // a NaN entry fails too
    te_set_error("Initial vector is not normalized");
    return TE_ERR_NOT_NORMALIZED;
  }
  const double ns = std::floor(p.t / p.sampling_step) + 1.0;  // :57
  if (!(ns < 2e9)) {
    te_set_error("te_evolver_create: too many samples");
    return TE_ERR_UNSUPPORTED;
  }
  int rc = te_upload_quad_tables();
  if (rc != TE_OK) return rc;
  te_evolver ev = new te_evolver_s();
  ev->H = H;
  ev->p = p;
  ev->n = n;
  ev->m = m;
  ev->n_samples = (int64_t)ns;
  cudaGetDevice(&ev->device);
  auto fail = [&](int code) {
    free_evolver(ev);
    return code;
  };
  if ((rc = te_cuda_check(cudaStreamCreateWithFlags(&ev->st, cudaStreamNonBlocking), "stream")) != TE_OK)
    return fail(rc);
  if ((rc = te_cuda_check(te_malloc(&ev->ds, sizeof(TeDevState)), "state")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(cudaMemset(ev->ds, 0, sizeof(TeDevState)), "state")) != TE_OK) return fail(rc);
  if ((rc = te_cuda_check(te_malloc_host(&ev->sum, sizeof(Summary)), "pinned")) != TE_OK) return fail(rc);
  if ((rc = te_seg_carry_alloc(H->sell, &ev->seg)) != TE_OK) return fail(rc);
  // basis columns, spare start vector, w, sampled state
  if ((rc = te_cuda_check(te_malloc(&ev->slab, sizeof(double2) * n * (m + 3)), "Krylov basis")) != TE_OK)
    return fail(rc);
  for (int j = 0; j < m; ++j) ev->cols[j] = ev->slab + (int64_t)j * n;
  ev->spare = ev->slab + (int64_t)m * n;
  ev->w = ev->slab + (int64_t)(m + 1) * n;
  ev->sampled = ev->slab + (int64_t)(m + 2) * n;
  if ((rc = te_cuda_check(te_malloc(&ev->partials, sizeof(double) * kPartials), "partials")) != TE_OK)
    return fail(rc);
  if ((rc = te_cuda_check(te_malloc(&ev->orig_tmp, sizeof(double2) * n), "tmp")) != TE_OK) return fail(rc);
  // v (original order) -> permuted start vector
  if ((rc = te_cuda_check(cudaMemcpy(ev->orig_tmp, v_host, sizeof(double2) * n, cudaMemcpyHostToDevice), "H2D")) !=
      TE_OK)
    return fail(rc);
  te_launch_permute(n, H->sell.perm, ev->orig_tmp, ev->cols[0], ev->st);
  if ((rc = te_cuda_check(cudaStreamSynchronize(ev->st), "permute")) != TE_OK) return fail(rc);
  *out = ev;
  return TE_OK;
}

extern "C" int te_evolver_destroy(te_evolver ev) {
  free_evolver(ev);
  return TE_OK;
}

extern "C" int te_evolver_add_sparse_observable(te_evolver ev, te_matrix O) {
  if (!ev || !O) {
    te_set_error("te_evolver_add_sparse_observable: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  if (O->n_rows != ev->n || O->n_cols != ev->n) {
    te_set_error("Incompatible dimensions");
    return TE_ERR_DIM;
  }
  HostObs o;
  if (O->is_diag) {
    o.kind = 0;
    TE_CUDA(te_malloc(&o.diag_perm, sizeof(double) * ev->n));
    // permuted Re(diagonal): gather through the permutation of H
    te_launch_permute_real(ev->n, ev->H->sell.perm, O->diag_re, o.diag_perm, ev->st);
    if (int rc = te_cuda_check(cudaStreamSynchronize(ev->st), "diagonal observable")) {
      te_free(o.diag_perm);
      return rc;
    }
  } else {
    o.kind = 2;
    o.O = O;
  }
  ev->obs.push_back(o);
  return TE_OK;
}

extern "C" int te_evolver_add_dense_observable(te_evolver ev, const double* values_host, int64_t n) {
  if (!ev || !values_host) {
    te_set_error("te_evolver_add_dense_observable: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  if (n != ev->n) {
    te_set_error("Incompatible dimensions");
    return TE_ERR_DIM;
  }
  HostObs o;
  o.kind = 4;
  TE_CUDA(te_malloc(&o.dense, sizeof(double2) * n * n));
  const cudaError_t e = cudaMemcpy(o.dense, values_host, sizeof(double2) * n * n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    te_free(o.dense);
    return te_cuda_check(e, "dense observable upload");
  }
  ev->obs.push_back(o);
  return TE_OK;
}

extern "C" int te_evolver_add_stop_condition(te_evolver ev, int obs_index, double threshold, int direction) {
  if (!ev || obs_index < 0 || obs_index >= (int)ev->obs.size() || direction == 0 || !std::isfinite(threshold)) {
    te_set_error("te_evolver_add_stop_condition: an existing observable index, a finite threshold and a non-zero "
                 "direction are required");
    return TE_ERR_INVALID_ARG;
  }
  if (ev->stops.count >= TE_MAX_STOP_CONDITIONS) {
    te_set_error("te_evolver_add_stop_condition: at most %d conditions", TE_MAX_STOP_CONDITIONS);
    return TE_ERR_UNSUPPORTED;
  }
  const int k = ev->stops.count++;
  ev->stops.obs[k] = obs_index;
  ev->stops.direction[k] = direction > 0 ? 1 : -1;
  ev->stops.threshold[k] = threshold;
  return TE_OK;
}

extern "C" int te_evolver_add_vector_observable(te_evolver ev, const double* o_host) {
  if (!ev || !o_host) {
    te_set_error("te_evolver_add_vector_observable: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  HostObs o;
  o.kind = 1;
  TE_CUDA(te_malloc(&o.vec_perm, sizeof(double2) * ev->n));
  TE_CUDA(cudaMemcpy(ev->orig_tmp, o_host, sizeof(double2) * ev->n, cudaMemcpyHostToDevice));
  te_launch_permute(ev->n, ev->H->sell.perm, ev->orig_tmp, o.vec_perm, ev->st);
  TE_CUDA(cudaStreamSynchronize(ev->st));
  ev->obs.push_back(o);
  return TE_OK;
}

extern "C" int te_evolver_add_callback_observable(te_evolver ev, te_observable_fn fn, void* user) {
  if (!ev || !fn) {
    te_set_error("te_evolver_add_callback_observable: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  if (!ev->host_state) TE_CUDA(te_malloc_host(&ev->host_state, sizeof(double2) * ev->n));
  HostObs o;
  o.kind = 3;
  o.fn = fn;
  o.user = user;
  ev->obs.push_back(o);
  return TE_OK;
}

extern "C" int te_evolver_run(te_evolver ev, te_result* result) {
  if (!ev) {
    te_set_error("te_evolver_run: null evolver");
    return TE_ERR_INVALID_ARG;
  }
  if (ev->ran) {
    te_set_error("te_evolver_run: call te_evolver_reset before running an evolver again");
    return TE_ERR_INVALID_ARG;
  }
  ev->ran = true;
  te_result r{};
  int rc = run(ev, &r);
  if (ev->profiling) collect_profile(ev);
  if (rc == TE_OK) rc = te_cuda_check(cudaGetLastError(), "evolution");
  if (rc != TE_OK) return rc;
  ev->res = r;
  if (result) *result = r;
  return TE_OK;
}

extern "C" int te_evolver_samples(te_evolver ev, int obs_index, double* out_host, int64_t count) {
  if (!ev || !out_host || obs_index < 0 || obs_index >= (int)ev->obs.size() || count < 0) {
    te_set_error("te_evolver_samples: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  if (!ev->results) {
    te_set_error("te_evolver_samples: the evolver has not run");
    return TE_ERR_INVALID_ARG;
  }
  const int64_t k = std::min<int64_t>(count, ev->n_samples);
  TE_CUDA(cudaMemcpy(out_host, ev->results + (int64_t)obs_index * ev->n_samples, sizeof(double) * k,
                     cudaMemcpyDeviceToHost));
  for (int64_t i = k; i < count; ++i) out_host[i] = 0.0;
  return TE_OK;
}

extern "C" int te_evolver_state(te_evolver ev, double* out_host) {
  if (!ev || !out_host) {
    te_set_error("te_evolver_state: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  // last sampled state, back to the caller's ordering
  te_launch_permute(ev->n, ev->H->sell.iperm, ev->sampled, ev->orig_tmp, ev->st);
  TE_CUDA(cudaMemcpyAsync(out_host, ev->orig_tmp, sizeof(double2) * ev->n, cudaMemcpyDeviceToHost, ev->st));
  TE_CUDA(cudaStreamSynchronize(ev->st));
  return TE_OK;
}

extern "C" int te_evolver_state_device(te_evolver ev, const double** out_dev) {
  if (!ev || !out_dev) {
    te_set_error("te_evolver_state_device: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  te_launch_permute(ev->n, ev->H->sell.iperm, ev->sampled, ev->orig_tmp, ev->st);
  TE_CUDA(cudaStreamSynchronize(ev->st));
  *out_dev = reinterpret_cast<const double*>(ev->orig_tmp);
  return TE_OK;
}

extern "C" int te_evolver_trace(te_evolver ev, te_step_record* out, int64_t max_records, int64_t* n_records) {
  if (!ev) {
    te_set_error("te_evolver_trace: null evolver");
    return TE_ERR_INVALID_ARG;
  }
  const int64_t k = std::min<int64_t>(max_records, (int64_t)ev->trace.size());
  if (out && k > 0) std::memcpy(out, ev->trace.data(), sizeof(te_step_record) * k);
  if (n_records) *n_records = (int64_t)ev->trace.size();
  return TE_OK;
}

extern "C" int64_t te_evolver_launch_count(te_evolver ev) { return ev ? ev->launches : 0; }

extern "C" int te_evolver_krylov_matrix(te_evolver ev, double* diag, double* offdiag, double* eigenvalues,
                                        int32_t* m_out, int32_t* eig_used) {
  if (!ev || !ev->ds) {
    te_set_error("te_evolver_krylov_matrix: null evolver");
    return TE_ERR_INVALID_ARG;
  }
  TE_CUDA(cudaStreamSynchronize(ev->st));
  int32_t m = 0, valid = 0;
  TE_CUDA(cudaMemcpy(&m, (const char*)ev->ds + offsetof(TeDevState, m_eff), sizeof(int32_t), cudaMemcpyDeviceToHost));
  TE_CUDA(cudaMemcpy(&valid, (const char*)ev->ds + offsetof(TeDevState, eig_valid), sizeof(int32_t),
                     cudaMemcpyDeviceToHost));
  m = std::max(0, std::min(m, (int32_t)TE_MMAX));
  if (diag) TE_CUDA(cudaMemcpy(diag, ev->ds->d, sizeof(double) * m, cudaMemcpyDeviceToHost));
  if (offdiag && m > 1) TE_CUDA(cudaMemcpy(offdiag, ev->ds->e, sizeof(double) * (m - 1), cudaMemcpyDeviceToHost));
  if (eigenvalues && valid) TE_CUDA(cudaMemcpy(eigenvalues, ev->ds->eig_lam, sizeof(double) * m, cudaMemcpyDeviceToHost));
  if (m_out) *m_out = m;
  if (eig_used) *eig_used = valid;
  return TE_OK;
}

// Sample at the given ascending times (times[0] = 0, times[count-1] <= t)
// instead of multiples of sampling_step, and optionally store every sampled
// state (evolver row order) at store_dev + k * store_ld.
int te_evolver_set_schedule(te_evolver ev, const double* times_host, int64_t count, double2* store_dev,
                            int64_t store_ld) {
  if (!ev || count < 1 || !times_host || times_host[0] != 0.0) {
    te_set_error("te_evolver_set_schedule: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  for (int64_t i = 1; i < count; ++i)
    if (!(times_host[i] >= times_host[i - 1]) || times_host[i] > ev->p.t) {
      te_set_error("te_evolver_set_schedule: sample times must ascend within [0, t]");
      return TE_ERR_INVALID_ARG;
    }
  te_free(ev->sample_times);
  ev->sample_times = nullptr;
  TE_CUDA(te_malloc(&ev->sample_times, sizeof(double) * count));
  TE_CUDA(cudaMemcpy(ev->sample_times, times_host, sizeof(double) * count, cudaMemcpyHostToDevice));
  ev->n_samples = count;
  ev->state_store = store_dev;
  ev->store_ld = store_ld;
  return TE_OK;
}

extern "C" int te_evolver_reset(te_evolver ev, const double* v, int v_is_device) {
  if (!ev || !v) {
    te_set_error("te_evolver_reset: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  const int64_t n = ev->n;
  if (!v_is_device) {
    const double nrm = te_host_sumsq(v, 2 * n);
    if (!(std::fabs(std::sqrt(nrm) - 1.0) <= ev->p.tol)) {
      te_set_error("Initial vector is not normalized");
      return TE_ERR_NOT_NORMALIZED;
    }
  }
  TE_CUDA(cudaMemcpyAsync(ev->orig_tmp, v, sizeof(double2) * n,
                          v_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ev->st));
  // the Krylov basis columns were rotated by earlier runs: restore the slab order
  for (int j = 0; j < ev->m; ++j) ev->cols[j] = ev->slab + (int64_t)j * n;
  ev->spare = ev->slab + (int64_t)ev->m * n;
  te_launch_permute(n, ev->H->sell.perm, ev->orig_tmp, ev->cols[0], ev->st);
  ev->ran = false;
  return te_cuda_check(cudaGetLastError(), "te_evolver_reset");
}

extern "C" int te_evolver_set_option(te_evolver ev, int option, int value) {
  if (!ev) return TE_ERR_INVALID_ARG;
  switch (option) {
    case TE_OPT_FUSED_LANCZOS:
      if (value < 0 || value > 2) {
        te_set_error("te_evolver_set_option: TE_OPT_FUSED_LANCZOS takes 0, 1 or 2");
        return TE_ERR_INVALID_ARG;
      }
      ev->fused_lanczos = value;
      return TE_OK;
    case TE_OPT_FIXED_SPMV:
      if (value < 0 || value > 1) {
        te_set_error("te_evolver_set_option: TE_OPT_FIXED_SPMV takes 0 or 1");
        return TE_ERR_INVALID_ARG;
      }
      ev->fixed_spmv = value;
      return TE_OK;
    case TE_OPT_BARRIER_SPIN_LIMIT:
      if (value < 1) {
        te_set_error("te_evolver_set_option: TE_OPT_BARRIER_SPIN_LIMIT takes a positive poll count");
        return TE_ERR_INVALID_ARG;
      }
      ev->barrier_spins = (unsigned int)value;
      return TE_OK;
    case TE_OPT_BARRIER_EXTRA_ARRIVALS:
      if (value < 0 || value > 1) {
        te_set_error("te_evolver_set_option: TE_OPT_BARRIER_EXTRA_ARRIVALS takes 0 or 1");
        return TE_ERR_INVALID_ARG;
      }
      ev->barrier_extra = (unsigned int)value;
      return TE_OK;
    case TE_OPT_TS_MAX_LEVEL:
      if (value < 2 || value > 8) {
        te_set_error("te_evolver_set_option: TE_OPT_TS_MAX_LEVEL takes 2..8");
        return TE_ERR_INVALID_ARG;
      }
      ev->ts_max_level = value == 8 ? 0 : value;
      return TE_OK;
    case TE_OPT_QR_SWEEP_LIMIT:
      if (value < 0) {
        te_set_error("te_evolver_set_option: TE_OPT_QR_SWEEP_LIMIT takes 0 (automatic) or a sweep count");
        return TE_ERR_INVALID_ARG;
      }
      ev->qr_sweeps = value;
      return TE_OK;
    default:
      te_set_error("te_evolver_set_option: unknown option %d", option);
      return TE_ERR_INVALID_ARG;
  }
}

extern "C" void* te_evolver_stream(te_evolver ev) { return ev ? (void*)ev->st : nullptr; }

extern "C" int te_evolver_profile(te_evolver ev, int enable) {
  if (!ev) return TE_ERR_INVALID_ARG;
  ev->profiling = enable != 0;
  for (int k = 0; k < 5; ++k) {
    ev->kernel_ms[k] = 0.0;
    ev->kernel_n[k] = 0;
  }
  ev->pending.clear();
  ev->ev_used = 0;
  return TE_OK;
}

extern "C" int te_evolver_kernel_time(te_evolver ev, int kind, double* total_ms, int64_t* launches) {
  if (!ev || kind < 0 || kind > 4) return TE_ERR_INVALID_ARG;
  if (total_ms) *total_ms = ev->kernel_ms[kind];
  if (launches) *launches = ev->kernel_n[kind];
  return TE_OK;
}
