// te_batch.cu -- many independent evolutions of uneven dimension at once.
//
// Every instance runs the algorithm of krylovTimeEvolver::timeEvolve
// (core/krylovTimeEvolver.cpp:261-512) with its own H, v, t, tolerance, step
// size, Krylov dimension and status; the instances advance together, one
// Krylov step of every active instance per global step:
//   * one segmented SELL-32 matrix over the concatenated (length-sorted) rows of
//     all instances; a chunk of 32 rows never straddles two instances, so a warp
//     always works for one instance and reads its scalars once;
//   * each Lanczos iteration is one apply pass and one update pass over every
//     active instance's rows on a per-step warp schedule of equal FP64 cost;
//     per-(warp, instance) partials are summed per instance in a fixed order
//     by the warp that writes the instance's last one (deterministic);
//   * the Krylov-space work (exponential, error integrals, step size, sample
//     schedule) runs one thread block per instance;
//   * the whole sequence of one global step (2 m_max Lanczos kernels, Krylov
//     kernel, combine, observables, flag gather) is captured once as a CUDA
//     graph and replayed; the host syncs once per global step.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "te_batch.cuh"
#include "te_internal.cuh"

namespace {

// Per-pass kernels of the graph path: one hardware warp per schedule warp.
__global__ void batch_active_kernel(int64_t n_chunks, const int32_t* __restrict__ chunk_inst,
                                    const TeDevState* states, int32_t* active, int* count) {
  batch_active_body(n_chunks, chunk_inst, states, active, count, (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                    (int64_t)gridDim.x * blockDim.x);
}

__global__ void __launch_bounds__(1024) batch_schedule_kernel(BatchGeom g, const TeDevState* states, int n_inst,
                                                              int n_warps, double w_slot, double* inst_cost,
                                                              int32_t* warp_begin, int32_t* inst_w0,
                                                              int32_t* inst_nseg, int32_t* seg_base,
                                                              int32_t* next_run, int32_t* inst_nwrite) {
  __shared__ double total;
  batch_schedule_body(g, states, n_inst, n_warps, w_slot, inst_cost, warp_begin, inst_w0, inst_nseg, seg_base,
                      next_run, inst_nwrite, &total);
}

template <bool REAL, bool HAS_PREV>
__global__ void __launch_bounds__(TE_THREADS, REAL ? 6 : 5) batch_apply_kernel(BatchGeom g, BatchSched sc,
                                                                 const double2* __restrict__ V,
                                                                 double2* __restrict__ w, TeDevState* states,
                                                                 double* seg_partials, int j) {
  batch_apply_warp<REAL, HAS_PREV, false>(g, sc, V, w, states, seg_partials, j,
                                          blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5));
}

__global__ void __launch_bounds__(TE_THREADS) batch_update_kernel(BatchGeom g, BatchSched sc,
                                                                  double2* __restrict__ V,
                                                                  const double2* __restrict__ w, TeDevState* states,
                                                                  double* seg_partials, int j) {
  batch_update_warp<false>(g, sc, V, w, states, seg_partials, j, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5));
}

__global__ void __launch_bounds__(TE_THREADS) batch_new_start_kernel(BatchGeom g, double2* __restrict__ V,
                                                                     const double2* __restrict__ spare,
                                                                     const TeDevState* states) {
  batch_new_start_body<false>(g, V, spare, states, (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5),
                       (int64_t)gridDim.x * (blockDim.x >> 5));
}

// Clear the new-start flags once the copies are done (one thread per instance).
__global__ void batch_clear_start_kernel(TeDevState* states, int n_inst) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_inst; i += gridDim.x * blockDim.x)
    states[i].new_start = 0;
}

__global__ void __launch_bounds__(TE_THREADS) batch_combine_kernel(BatchGeom g, const double2* __restrict__ V,
                                                                   double2* spare, double2* sampled,
                                                                   const TeDevState* states, int m_override) {
  batch_combine_body<false>(g, V, spare, sampled, states, m_override,
                     (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5),
                     (int64_t)gridDim.x * (blockDim.x >> 5));
}

struct BlockSync {
  __device__ void operator()() const { __syncthreads(); }
};

// Diagonal observables, one block per instance.
__global__ void __launch_bounds__(TE_THREADS) batch_obs_kernel(BatchGeom g, const double2* __restrict__ sampled,
                                                               const double* __restrict__ diag, const int* n_obs,
                                                               const int64_t* result_off, double* results,
                                                               TeDevState* states) {
  __shared__ double scratch[TE_BATCH_MAX_OBS * 32];
  batch_obs_inst<false>(g, sampled, diag, n_obs, result_off, results, states, blockIdx.x, threadIdx.x, blockDim.x, scratch,
                 BlockSync());
}

// ||sampled||^2 of every instance, one block per instance.
__global__ void __launch_bounds__(TE_THREADS) batch_norm_kernel(BatchGeom g, const double2* __restrict__ sampled,
                                                                TeDevState* states) {
  __shared__ double scratch[32];
  batch_norm_inst<false>(g, sampled, states, blockIdx.x, threadIdx.x, blockDim.x, scratch, BlockSync());
}

__global__ void batch_flags_kernel(const TeDevState* states, int n_inst, int* flags) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_inst; i += gridDim.x * blockDim.x)
    flags[i] = batch_flag(states[i]);
}

// global = local + offset (columns of one instance into the concatenated rows)
__global__ void offset_copy_kernel(const int32_t* __restrict__ in, int32_t* __restrict__ out, int64_t count,
                                   int32_t offset) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = in[i] + offset;
}

__global__ void real_to_complex_kernel(const double* __restrict__ in, double2* __restrict__ out, int64_t count) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = make_double2(in[i], 0.0);
}

__global__ void scatter_permuted_kernel(int64_t n, const int32_t* __restrict__ perm, const double2* __restrict__ in,
                                        double2* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = in[perm[i]];
}

__global__ void gather_diag_kernel(int64_t n, const int32_t* __restrict__ perm, const double2* __restrict__ dc,
                                   double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = dc[perm[i]].x;
}

}  // namespace

struct te_batch_s {
  int B = 0;
  int m_max = 0;
  bool is_real = true;
  cudaStream_t st = nullptr;
  std::vector<te_matrix> H;
  std::vector<te_params> p;
  std::vector<int64_t> inst_row, inst_chunk, n_samples;
  std::vector<int32_t> inst_n;
  int64_t ld = 0, n_chunks = 0, slots = 0;
  // device
  int32_t* d_chunk_inst = nullptr;
  int64_t* d_chunk_off = nullptr;
  int32_t* d_col = nullptr;
  double* d_val = nullptr;
  int64_t* d_inst_row = nullptr;
  int32_t* d_inst_n = nullptr;
  int64_t* d_inst_chunk = nullptr;
  TeDevState* ds = nullptr;
  double2* V = nullptr;
  double2* spare = nullptr;
  double2* w = nullptr;
  double2* sampled = nullptr;
  double2* v0 = nullptr;  // start vectors (permuted), kept for reruns
  double* diag = nullptr;  // TE_BATCH_MAX_OBS x ld
  int* d_nobs = nullptr;
  int64_t* d_result_off = nullptr;
  double* results = nullptr;
  int* d_flags = nullptr;
  int* h_flags = nullptr;  // pinned
  int32_t* d_active = nullptr;  // chunks of the running instances
  int* d_active_count = nullptr;
  // Lanczos schedule of the current global step (batch_schedule_kernel)
  int n_warps = 0;
  int32_t* d_warp_begin = nullptr;
  int32_t* d_inst_w0 = nullptr;
  int32_t* d_inst_nseg = nullptr;
  int32_t* d_seg_base = nullptr;
  int32_t* d_next_run = nullptr;
  int32_t* d_inst_nwrite = nullptr;
  unsigned int* d_arrivals = nullptr;  // 2 per instance
  double* d_inst_cost = nullptr;
  double* seg_partials = nullptr;
  std::vector<int> nobs;
  std::vector<int64_t> result_off;
  cudaGraphExec_t g_step = nullptr, g_batch = nullptr;
  int64_t launches = 0;
  bool ran = false;
  // TE_BATCH_OPT_PERSISTENT: 0 graph replay per global step, 1 one persistent launch
  int persistent = 0;
  unsigned int spin_limit = 1u << 22;  // TE_BATCH_OPT_BARRIER_SPIN_LIMIT
  unsigned int extra_arrivals = 0;     // TE_BATCH_OPT_BARRIER_EXTRA_ARRIVALS
  unsigned int* d_bar = nullptr;       // grid barrier: count, generation
  int* d_err = nullptr;                // error raised on the device by the persistent kernel
  int64_t* d_steps = nullptr;          // global steps the persistent kernel completed
  int64_t global_steps = 0;
};

namespace {

BatchGeom geom(const te_batch_s* b) {
  BatchGeom g;
  g.n_chunks = b->n_chunks;
  g.chunk_inst = b->d_chunk_inst;
  g.chunk_off = b->d_chunk_off;
  g.col = b->d_col;
  g.val = b->d_val;
  g.inst_row = b->d_inst_row;
  g.inst_n = b->d_inst_n;
  g.inst_chunk = b->d_inst_chunk;
  g.ld = b->ld;
  g.active = b->d_active;
  g.active_count = b->d_active_count;
  return g;
}

BatchGeom geom_all_chunks(const te_batch_s* b) {
  BatchGeom g = geom(b);
  g.active = nullptr;
  g.active_count = nullptr;
  return g;
}

void free_batch(te_batch b) {
  if (!b) return;
  if (b->g_step) cudaGraphExecDestroy(b->g_step);
  if (b->g_batch) cudaGraphExecDestroy(b->g_batch);
  te_free(b->d_chunk_inst);
  te_free(b->d_chunk_off);
  te_free(b->d_col);
  te_free(b->d_val);
  te_free(b->d_inst_row);
  te_free(b->d_inst_n);
  te_free(b->d_inst_chunk);
  te_free(b->ds);
  te_free(b->V);
  te_free(b->spare);
  te_free(b->w);
  te_free(b->sampled);
  te_free(b->v0);
  te_free(b->diag);
  te_free(b->d_nobs);
  te_free(b->d_result_off);
  te_free(b->results);
  te_free(b->d_flags);
  te_free_host(b->h_flags);
  te_free(b->d_active);
  te_free(b->d_active_count);
  te_free(b->d_warp_begin);
  te_free(b->d_inst_w0);
  te_free(b->d_inst_nseg);
  te_free(b->d_seg_base);
  te_free(b->d_bar);
  te_free(b->d_err);
  te_free(b->d_steps);
  te_free(b->d_next_run);
  te_free(b->d_inst_nwrite);
  te_free(b->d_arrivals);
  te_free(b->d_inst_cost);
  te_free(b->seg_partials);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
}

// One resident wave of the chunk-strided kernels (new start, combine).
int grid_chunks(const te_batch_s* b) {
  const void* k[] = {(const void*)batch_new_start_kernel, (const void*)batch_combine_kernel};
  int bps = 8;
  for (const void* f : k) bps = std::min(bps, te_kernel_blocks_per_sm(f, TE_THREADS, 0));
  return (int)std::min<int64_t>((b->n_chunks * 32 + TE_THREADS - 1) / TE_THREADS, (int64_t)te_num_sms() * bps);
}

// Logical warps of the Lanczos schedule: one resident wave of the apply/update
// kernels.  The graph path launches one hardware warp for each; the persistent
// kernel's warps loop over them, so both sum the same segments in the same
// order.
int lanczos_warps(const te_batch_s* b) {
  const void* k[] = {(const void*)batch_apply_kernel<true, true>,  (const void*)batch_apply_kernel<true, false>,
                     (const void*)batch_apply_kernel<false, true>, (const void*)batch_apply_kernel<false, false>,
                     (const void*)batch_update_kernel};
  int bps = 8;
  for (const void* f : k) bps = std::min(bps, te_kernel_blocks_per_sm(f, TE_THREADS, 0));
  const int64_t blocks = std::min<int64_t>((b->n_chunks * 32 + TE_THREADS - 1) / TE_THREADS,
                                           (int64_t)te_num_sms() * bps);
  return (int)std::max<int64_t>(blocks, 1) * (TE_THREADS / 32);
}

BatchSched sched(const te_batch_s* b) {
  BatchSched sc;
  sc.warp_begin = b->d_warp_begin;
  sc.inst_w0 = b->d_inst_w0;
  sc.inst_nseg = b->d_inst_nseg;
  sc.seg_base = b->d_seg_base;
  sc.next_run = b->d_next_run;
  sc.inst_nwrite = b->d_inst_nwrite;
  sc.arrivals = b->d_arrivals;
  return sc;
}

// Record the kernels of one global step (or of one extra sample batch).
int enqueue_step(te_batch b, bool full_step) {
  const BatchGeom g = geom(b);
  cudaStream_t st = b->st;
  const int gc = grid_chunks(b);
  int64_t k = 0;
  if (full_step) {
    TE_CUDA(cudaMemsetAsync(b->d_active_count, 0, sizeof(int), st));
    batch_active_kernel<<<te_grid_fit((const void*)batch_active_kernel, b->n_chunks, 256), 256, 0, st>>>(
        b->n_chunks, b->d_chunk_inst, b->ds, b->d_active, b->d_active_count);
    batch_new_start_kernel<<<gc, TE_THREADS, 0, st>>>(g, b->V, b->spare, b->ds);
    batch_clear_start_kernel<<<(b->B + 255) / 256, 256, 0, st>>>(b->ds, b->B);
    k += 2;
    const BatchSched sc = sched(b);
    const int gl = b->n_warps / (TE_THREADS / 32);
    batch_schedule_kernel<<<1, 1024, 0, st>>>(g, b->ds, b->B, b->n_warps, b->is_real ? 2.0 : 4.0, b->d_inst_cost,
                                              b->d_warp_begin, b->d_inst_w0, b->d_inst_nseg, b->d_seg_base,
                                              b->d_next_run, b->d_inst_nwrite);
    k += 1;
    for (int j = 0; j < b->m_max; ++j) {
      if (b->is_real) {
        if (j > 0)
          batch_apply_kernel<true, true><<<gl, TE_THREADS, 0, st>>>(g, sc, b->V, b->w, b->ds, b->seg_partials, j);
        else
          batch_apply_kernel<true, false><<<gl, TE_THREADS, 0, st>>>(g, sc, b->V, b->w, b->ds, b->seg_partials, j);
      } else {
        if (j > 0)
          batch_apply_kernel<false, true><<<gl, TE_THREADS, 0, st>>>(g, sc, b->V, b->w, b->ds, b->seg_partials, j);
        else
          batch_apply_kernel<false, false><<<gl, TE_THREADS, 0, st>>>(g, sc, b->V, b->w, b->ds, b->seg_partials, j);
      }
      batch_update_kernel<<<gl, TE_THREADS, 0, st>>>(g, sc, b->V, b->w, b->ds, b->seg_partials, j);
      k += 2;
    }
  }
  te_launch_krylov_batch(b->ds, b->B, full_step ? 0 : 1, st);
  batch_combine_kernel<<<gc, TE_THREADS, 0, st>>>(g, b->V, b->spare, b->sampled, b->ds, 0);
  batch_obs_kernel<<<b->B, TE_THREADS, 0, st>>>(g, b->sampled, b->diag, b->d_nobs, b->d_result_off, b->results,
                                                b->ds);
  batch_flags_kernel<<<(b->B + 255) / 256, 256, 0, st>>>(b->ds, b->B, b->d_flags);
  k += 4;
  TE_CUDA(cudaMemcpyAsync(b->h_flags, b->d_flags, sizeof(int) * b->B, cudaMemcpyDeviceToHost, st));
  b->launches += 0;  // counted per replay
  (void)k;
  return te_cuda_check(cudaGetLastError(), "batch enqueue");
}

int64_t kernels_per_replay(const te_batch_s* b, bool full_step) {
  return (full_step ? 4 + 2 * (int64_t)b->m_max : 0) + 4;
}

int capture(te_batch b, bool full_step, cudaGraphExec_t* exec) {
  cudaGraph_t graph = nullptr;
  TE_CUDA(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_step(b, full_step);
  cudaError_t e = cudaStreamEndCapture(b->st, &graph);
  if (rc != TE_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  TE_CUDA(e);
  rc = te_cuda_check(cudaGraphInstantiate(exec, graph, 0), "graph instantiate");
  cudaGraphDestroy(graph);
  return rc;
}

// The whole run in one persistent launch (after reset_states).
int run_persistent(te_batch b, int grid) {
  TeBatchPersist a;
  a.g = geom(b);
  a.sc = sched(b);
  a.inst_cost = b->d_inst_cost;
  a.warp_begin = b->d_warp_begin;
  a.inst_w0 = b->d_inst_w0;
  a.inst_nseg = b->d_inst_nseg;
  a.seg_base = b->d_seg_base;
  a.next_run = b->d_next_run;
  a.inst_nwrite = b->d_inst_nwrite;
  a.active = b->d_active;
  a.active_count = b->d_active_count;
  a.V = b->V;
  a.w = b->w;
  a.spare = b->spare;
  a.sampled = b->sampled;
  a.states = b->ds;
  a.seg_partials = b->seg_partials;
  a.diag = b->diag;
  a.n_obs = b->d_nobs;
  a.result_off = b->d_result_off;
  a.results = b->results;
  a.n_inst = b->B;
  a.m_max = b->m_max;
  a.n_warps = b->n_warps;
  a.is_real = b->is_real;
  a.w_slot = b->is_real ? 2.0 : 4.0;
  a.bar_count = b->d_bar;
  a.bar_gen = b->d_bar + 1;
  a.err = b->d_err;
  a.spin_limit = b->spin_limit;
  a.arrivals = (unsigned int)grid + b->extra_arrivals;
  a.max_global_steps = (int64_t)1 << 40;
  a.steps_done = b->d_steps;
  TE_CUDA(cudaMemsetAsync(b->d_bar, 0, 2 * sizeof(unsigned int), b->st));
  TE_CUDA(cudaMemsetAsync(b->d_err, 0, sizeof(int), b->st));
  TE_CUDA(cudaMemsetAsync(b->d_steps, 0, sizeof(int64_t), b->st));
  int rc = te_launch_batch_persistent(a, grid, b->st);
  if (rc != TE_OK) return rc;
  b->launches += 1;
  int err = 0;
  TE_CUDA(cudaMemcpyAsync(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, b->st));
  TE_CUDA(cudaMemcpyAsync(&b->global_steps, b->d_steps, sizeof(int64_t), cudaMemcpyDeviceToHost, b->st));
  TE_CUDA(cudaStreamSynchronize(b->st));
  if (err) {
    te_set_error("te_batch_run: a grid-barrier wait of the persistent batched kernel gave up");
    return err;
  }
  return TE_OK;
}

int reset_states(te_batch b) {
  const BatchGeom g = geom_all_chunks(b);
  std::vector<TeDevState> hs(b->B);
  for (int i = 0; i < b->B; ++i) {
    TeDevState& s = hs[i];
    std::memset(&s, 0, sizeof(TeDevState));
    const te_params& p = b->p[i];
    const int m = (int)std::min<int64_t>(p.m, b->inst_n[i]);
    s.t = p.t;
    s.sampling_step = p.sampling_step;
    s.tol = p.tol;
    s.tol_rate = p.tol / p.t;
    s.exp_factor = p.exp_factor;
    s.inv_exp_factor = p.exp_factor != 0.0 ? 1.0 / p.exp_factor : 0.0;
    s.num_err_est = (double)b->inst_n[i] * b->H[i]->norm1 * DBL_EPSILON;
    s.m_max = m;
    s.n_samples = (int)b->n_samples[i];
    s.integ_long = p.fast_integration ? 0 : 2;
    s.integ_short = p.fast_integration ? 1 : 2;
    s.max_batch = 1;
    s.t_step = 0.1;
    s.m_cur = m;
    s.m_eff = m;
    s.s[0] = 1.0;
    s.samples_in_batch = 1;  // the sample at t = 0 (:306-313)
    s.sample_base = 0;
    s.index_samples = 1;
    s.Y[1 * TE_MMAX + 0] = make_double2(1.0, 0.0);
    s.n_steps = b->n_samples[i] > 1 ? 1 : 0;
    s.done = b->n_samples[i] > 1 ? 0 : 1;
  }
  TE_CUDA(cudaMemcpyAsync(b->ds, hs.data(), sizeof(TeDevState) * b->B, cudaMemcpyHostToDevice, b->st));
  TE_CUDA(cudaMemsetAsync(b->d_arrivals, 0, sizeof(unsigned int) * 2 * b->B, b->st));
  TE_CUDA(cudaMemcpyAsync(b->V, b->v0, sizeof(double2) * b->ld, cudaMemcpyDeviceToDevice, b->st));
  batch_combine_kernel<<<grid_chunks(b), TE_THREADS, 0, b->st>>>(g, b->V, b->spare, b->sampled, b->ds, 1);
  batch_obs_kernel<<<b->B, TE_THREADS, 0, b->st>>>(g, b->sampled, b->diag, b->d_nobs, b->d_result_off, b->results,
                                                   b->ds);
  b->launches += 2;
  TE_CUDA(cudaStreamSynchronize(b->st));
  return TE_OK;
}

}  // namespace

// ------------------------------------------------------------------ C ABI

extern "C" int te_batch_create(int n_instances, const te_matrix* H, const double* const* v_host,
                               const te_params* params, te_batch* out) {
  if (n_instances <= 0 || !H || !v_host || !params || !out) {
    te_set_error("te_batch_create: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  int rc = te_upload_quad_tables();
  if (rc != TE_OK) return rc;
  te_batch b = new te_batch_s();
  auto fail = [&](int code) {
    free_batch(b);
    return code;
  };
  b->B = n_instances;
  for (int i = 0; i < n_instances; ++i) {
    const te_params& p = params[i];
    if (!H[i] || !v_host[i] || H[i]->n_rows != H[i]->n_cols || !(p.t > 0.0) || !(p.sampling_step > 0.0) ||
        !(p.tol > 0.0) || p.m < 1 || p.reorth != 0 || p.exp_factor == 0.0 || !std::isfinite(p.exp_factor)) {
      te_set_error("te_batch_create: instance %d: invalid matrix or parameters (reorth and expFactor 0 are not "
                   "batched)", i);
      return fail(TE_ERR_INVALID_ARG);
    }
    if (H[i]->sell.n_long > 0) {
      te_set_error("te_batch_create: instance %d: matrices with long rows (above max(1024, 32 x mean) entries) are "
                   "not batched", i);
      return fail(TE_ERR_UNSUPPORTED);
    }
    const int64_t n = H[i]->n_rows;
    const double nrm = te_host_sumsq(v_host[i], 2 * n);
    if (!(std::fabs(std::sqrt(nrm) - 1.0) <= p.tol)) {
      te_set_error("te_batch_create: instance %d: Initial vector is not normalized", i);
      return fail(TE_ERR_NOT_NORMALIZED);
    }
    const int m = (int)std::min<int64_t>(p.m, n);
    if (m > TE_MMAX) {
      te_set_error("te_batch_create: instance %d: Krylov dimension above %d", i, TE_MMAX);
      return fail(TE_ERR_UNSUPPORTED);
    }
    b->m_max = std::max(b->m_max, m);
    b->H.push_back(H[i]);
    b->p.push_back(p);
    b->is_real = b->is_real && H[i]->is_real;
    b->n_samples.push_back((int64_t)std::floor(p.t / p.sampling_step) + 1);
  }
  // geometry: instance rows padded to whole chunks
  b->inst_row.resize(n_instances + 1);
  b->inst_chunk.resize(n_instances + 1);
  b->inst_n.resize(n_instances);
  int64_t rows = 0, chunks = 0, slots = 0;
  std::vector<int64_t> slot_begin(n_instances);
  for (int i = 0; i < n_instances; ++i) {
    b->inst_row[i] = rows;
    b->inst_chunk[i] = chunks;
    b->inst_n[i] = (int32_t)b->H[i]->n_rows;
    slot_begin[i] = slots;
    rows += b->H[i]->sell.n_chunks * 32;
    chunks += b->H[i]->sell.n_chunks;
    slots += b->H[i]->sell.slots;
  }
  b->inst_row[n_instances] = rows;
  b->inst_chunk[n_instances] = chunks;
  b->ld = rows;
  b->n_chunks = chunks;
  b->slots = slots;
  if (rows >= ((int64_t)1 << 31)) {
    te_set_error("te_batch_create: the instances together exceed 2^31 rows");
    return fail(TE_ERR_UNSUPPORTED);
  }
  if ((rc = te_cuda_check(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking), "stream")) != TE_OK)
    return fail(rc);
  cudaStream_t st = b->st;
  std::vector<int64_t> off(chunks + 1);
  std::vector<int32_t> cinst(chunks);
  for (int i = 0; i < n_instances; ++i) {
    const TeSell& S = b->H[i]->sell;
    std::vector<int64_t> loc(S.n_chunks + 1);
    if ((rc = te_cuda_check(cudaMemcpy(loc.data(), S.chunk_off, sizeof(int64_t) * (S.n_chunks + 1),
                                       cudaMemcpyDeviceToHost), "chunk_off")) != TE_OK)
      return fail(rc);
    for (int64_t c = 0; c < S.n_chunks; ++c) {
      off[b->inst_chunk[i] + c] = slot_begin[i] + loc[c];
      cinst[b->inst_chunk[i] + c] = i;
    }
  }
  off[chunks] = slots;
  auto alloc = [&](void** p, size_t bytes) { return te_cuda_check(te_malloc(p, std::max<size_t>(bytes, 16)), "alloc"); };
  const int vw = b->is_real ? 1 : 2;
  if ((rc = alloc((void**)&b->d_chunk_off, sizeof(int64_t) * (chunks + 1))) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_chunk_inst, sizeof(int32_t) * chunks)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_col, sizeof(int32_t) * slots)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_val, sizeof(double) * vw * slots)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_inst_row, sizeof(int64_t) * (n_instances + 1))) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_inst_chunk, sizeof(int64_t) * (n_instances + 1))) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_inst_n, sizeof(int32_t) * n_instances)) != TE_OK) return fail(rc);
  TE_CUDA(cudaMemcpy(b->d_chunk_off, off.data(), sizeof(int64_t) * (chunks + 1), cudaMemcpyHostToDevice));
  TE_CUDA(cudaMemcpy(b->d_chunk_inst, cinst.data(), sizeof(int32_t) * chunks, cudaMemcpyHostToDevice));
  TE_CUDA(cudaMemcpy(b->d_inst_row, b->inst_row.data(), sizeof(int64_t) * (n_instances + 1), cudaMemcpyHostToDevice));
  TE_CUDA(cudaMemcpy(b->d_inst_chunk, b->inst_chunk.data(), sizeof(int64_t) * (n_instances + 1),
                     cudaMemcpyHostToDevice));
  TE_CUDA(cudaMemcpy(b->d_inst_n, b->inst_n.data(), sizeof(int32_t) * n_instances, cudaMemcpyHostToDevice));
  for (int i = 0; i < n_instances; ++i) {
    const TeSell& S = b->H[i]->sell;
    const int gr = te_grid_for(S.slots, 256, 4);
    offset_copy_kernel<<<gr, 256, 0, st>>>(S.col, b->d_col + slot_begin[i], S.slots, (int32_t)b->inst_row[i]);
    if (b->is_real)
      TE_CUDA(cudaMemcpyAsync(b->d_val + slot_begin[i], S.val, sizeof(double) * S.slots, cudaMemcpyDeviceToDevice, st));
    else if (b->H[i]->is_real)
      real_to_complex_kernel<<<gr, 256, 0, st>>>(S.val, reinterpret_cast<double2*>(b->d_val) + slot_begin[i],
                                                 S.slots);
    else
      TE_CUDA(cudaMemcpyAsync(b->d_val + 2 * slot_begin[i], S.val, sizeof(double2) * S.slots,
                              cudaMemcpyDeviceToDevice, st));
  }
  const int64_t ld = b->ld;
  if ((rc = alloc((void**)&b->ds, sizeof(TeDevState) * n_instances)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->V, sizeof(double2) * ld * b->m_max)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->spare, sizeof(double2) * ld)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->w, sizeof(double2) * ld)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->sampled, sizeof(double2) * ld)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->v0, sizeof(double2) * ld)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->diag, sizeof(double) * TE_BATCH_MAX_OBS * ld)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_nobs, sizeof(int) * n_instances)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_result_off, sizeof(int64_t) * n_instances)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_flags, sizeof(int) * n_instances)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_active, sizeof(int32_t) * std::max<int64_t>(chunks, 1))) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_active_count, sizeof(int))) != TE_OK) return fail(rc);
  b->n_warps = lanczos_warps(b);
  if ((rc = alloc((void**)&b->d_warp_begin, sizeof(int32_t) * (b->n_warps + 1))) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_inst_w0, sizeof(int32_t) * n_instances)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_inst_nseg, sizeof(int32_t) * n_instances)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_seg_base, sizeof(int32_t) * n_instances)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_next_run, sizeof(int32_t) * n_instances)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_inst_nwrite, sizeof(int32_t) * n_instances)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_arrivals, sizeof(unsigned int) * 2 * n_instances)) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_inst_cost, sizeof(double) * (n_instances + 1))) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_bar, 2 * sizeof(unsigned int))) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_err, sizeof(int))) != TE_OK) return fail(rc);
  if ((rc = alloc((void**)&b->d_steps, sizeof(int64_t))) != TE_OK) return fail(rc);
  // segments: every warp has at most one per instance it touches
  if ((rc = alloc((void**)&b->seg_partials, sizeof(double) * 2 * ((int64_t)b->n_warps + n_instances + 1))) != TE_OK)
    return fail(rc);
  TE_CUDA(te_malloc_host(&b->h_flags, sizeof(int) * n_instances));
  TE_CUDA(cudaMemsetAsync(b->V, 0, sizeof(double2) * ld * b->m_max, st));
  TE_CUDA(cudaMemsetAsync(b->spare, 0, sizeof(double2) * ld, st));
  TE_CUDA(cudaMemsetAsync(b->w, 0, sizeof(double2) * ld, st));
  TE_CUDA(cudaMemsetAsync(b->v0, 0, sizeof(double2) * ld, st));
  TE_CUDA(cudaMemsetAsync(b->diag, 0, sizeof(double) * TE_BATCH_MAX_OBS * ld, st));
  // start vectors into the instances' sorted order
  double2* tmp = nullptr;
  int64_t nmax = 0;
  for (int i = 0; i < n_instances; ++i) nmax = std::max<int64_t>(nmax, b->inst_n[i]);
  if ((rc = alloc((void**)&tmp, sizeof(double2) * nmax)) != TE_OK) return fail(rc);
  for (int i = 0; i < n_instances; ++i) {
    TE_CUDA(cudaMemcpyAsync(tmp, v_host[i], sizeof(double2) * b->inst_n[i], cudaMemcpyHostToDevice, st));
    scatter_permuted_kernel<<<te_grid_for(b->inst_n[i], 256, 4), 256, 0, st>>>(b->inst_n[i], b->H[i]->sell.perm, tmp,
                                                                              b->v0 + b->inst_row[i]);
    TE_CUDA(cudaStreamSynchronize(st));
  }
  te_free(tmp);
  b->nobs.assign(n_instances, 0);
  TE_CUDA(cudaMemcpy(b->d_nobs, b->nobs.data(), sizeof(int) * n_instances, cudaMemcpyHostToDevice));
  *out = b;
  return TE_OK;
}

extern "C" int te_batch_add_observable(te_batch b, int instance, te_matrix O) {
  if (!b || !O || instance < 0 || instance >= b->B) {
    te_set_error("te_batch_add_observable: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  if (O->n_rows != b->inst_n[instance] || O->n_cols != b->inst_n[instance]) {
    te_set_error("Incompatible dimensions");
    return TE_ERR_DIM;
  }
  if (!O->is_diag || b->nobs[instance] >= TE_BATCH_MAX_OBS) {
    te_set_error("te_batch_add_observable: batched evolutions take up to %d diagonal observables per instance",
                 TE_BATCH_MAX_OBS);
    return TE_ERR_UNSUPPORTED;
  }
  const int k = b->nobs[instance]++;
  gather_diag_kernel<<<te_grid_for(b->inst_n[instance], 256, 4), 256, 0, b->st>>>(
      b->inst_n[instance], b->H[instance]->sell.perm, O->diag_c, b->diag + (int64_t)k * b->ld + b->inst_row[instance]);
  TE_CUDA(cudaStreamSynchronize(b->st));
  TE_CUDA(cudaMemcpy(b->d_nobs, b->nobs.data(), sizeof(int) * b->B, cudaMemcpyHostToDevice));
  return TE_OK;
}

extern "C" int te_batch_run(te_batch b, te_result* results) {
  if (!b) {
    te_set_error("te_batch_run: null batch");
    return TE_ERR_INVALID_ARG;
  }
  b->launches = 0;
  // result table
  if (!b->results) {
    b->result_off.assign(b->B, 0);
    int64_t tot = 0;
    for (int i = 0; i < b->B; ++i) {
      b->result_off[i] = tot;
      tot += (int64_t)std::max(1, b->nobs[i]) * b->n_samples[i];
    }
    TE_CUDA(te_malloc(&b->results, sizeof(double) * std::max<int64_t>(tot, 1)));
    TE_CUDA(cudaMemset(b->results, 0, sizeof(double) * std::max<int64_t>(tot, 1)));
    TE_CUDA(cudaMemcpy(b->d_result_off, b->result_off.data(), sizeof(int64_t) * b->B, cudaMemcpyHostToDevice));
  }
  int rc = reset_states(b);
  if (rc != TE_OK) return rc;
  b->global_steps = 0;
  if (b->persistent) {
    const int grid = te_batch_persistent_grid(b->is_real);
    if (grid <= 0) {
      te_set_error("te_batch_run: the persistent batched kernel cannot be co-resident on this device");
      return TE_ERR_UNSUPPORTED;
    }
    if ((rc = run_persistent(b, grid)) != TE_OK) return rc;
  } else {
  if (!b->g_step) {
    if ((rc = capture(b, true, &b->g_step)) != TE_OK) return rc;
    if ((rc = capture(b, false, &b->g_batch)) != TE_OK) return rc;
  }
  const int64_t per_step = kernels_per_replay(b, true), per_batch = kernels_per_replay(b, false);
  for (int64_t guard = 0; guard < ((int64_t)1 << 30); ++guard) {
    TE_CUDA(cudaGraphLaunch(b->g_step, b->st));
    TE_CUDA(cudaStreamSynchronize(b->st));
    b->launches += per_step;
    bool pending = false, all_done = true, fatal = false;
    for (int i = 0; i < b->B; ++i) {
      pending |= (b->h_flags[i] & 2) != 0;
      all_done &= (b->h_flags[i] & 1) != 0;
      fatal |= (b->h_flags[i] & 4) != 0;
    }
    while (pending && !fatal) {
      TE_CUDA(cudaGraphLaunch(b->g_batch, b->st));
      TE_CUDA(cudaStreamSynchronize(b->st));
      b->launches += per_batch;
      pending = false;
      all_done = true;
      for (int i = 0; i < b->B; ++i) {
        pending |= (b->h_flags[i] & 2) != 0;
        all_done &= (b->h_flags[i] & 1) != 0;
        fatal |= (b->h_flags[i] & 4) != 0;
      }
    }
    ++b->global_steps;
    if (fatal || all_done) break;
  }
  batch_norm_kernel<<<b->B, TE_THREADS, 0, b->st>>>(geom(b), b->sampled, b->ds);
  b->launches += 1;
  }
  std::vector<TeDevState> hs(b->B);
  TE_CUDA(cudaMemcpyAsync(hs.data(), b->ds, sizeof(TeDevState) * b->B, cudaMemcpyDeviceToHost, b->st));
  TE_CUDA(cudaStreamSynchronize(b->st));
  int first_fatal = 0;
  for (int i = 0; i < b->B; ++i) {
    const TeDevState& S = hs[i];
    if (S.fatal && !first_fatal) first_fatal = S.fatal;
    // final checks of :445-504
    int status = S.status, nbErrors = 0;
    if (std::fabs(std::sqrt(S.norm2_final) - 1.0) > b->p[i].tol) {
      nbErrors++;
      status = TE_STATUS_NORM;
    }
    const double numErrTotal = S.num_err_est * S.n_steps;
    if (S.nb_err_roundoff != 0) {
      nbErrors++;
      status = TE_STATUS_ROUNDOFF;
    }
    if (S.nb_err_int != 0) {
      nbErrors++;
      status = TE_STATUS_INTEGRATION;
    }
    if (numErrTotal > S.err && S.nb_err_roundoff == 0) {
      if (numErrTotal > b->p[i].tol) {
        status = TE_STATUS_ROUNDOFF_TOTAL;
        nbErrors++;
      } else if (status != TE_STATUS_LUCKY_BREAKDOWN) {
        status = TE_STATUS_BELOW_ROUNDOFF;
      }
    }
    if (nbErrors > 1) status = TE_STATUS_MULTIPLE;
    if (results) {
      te_result& r = results[i];
      r = te_result{};
      r.err = S.err;
      r.evolved_time = S.t_now;
      r.num_samples = S.index_samples;
      r.n_steps = S.n_steps;
      r.dim = b->inst_n[i];
      r.krylov_dim = S.m_cur;
      r.status = S.fatal ? S.fatal : status;
      r.nb_err_roundoff = S.nb_err_roundoff;
      r.nb_err_int = S.nb_err_int;
    }
  }
  b->ran = true;
  if (first_fatal) {
    te_set_error("device-side failure %d in a batched evolution", first_fatal);
    return first_fatal;
  }
  return TE_OK;
}

extern "C" int te_batch_samples(te_batch b, int instance, int obs_index, double* out_host, int64_t count) {
  if (!b || !b->ran || instance < 0 || instance >= b->B || obs_index < 0 || obs_index >= b->nobs[instance] ||
      !out_host || count < 0) {
    te_set_error("te_batch_samples: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  const int64_t k = std::min<int64_t>(count, b->n_samples[instance]);
  TE_CUDA(cudaMemcpy(out_host, b->results + b->result_off[instance] + (int64_t)obs_index * b->n_samples[instance],
                     sizeof(double) * k, cudaMemcpyDeviceToHost));
  for (int64_t i = k; i < count; ++i) out_host[i] = 0.0;
  return TE_OK;
}

extern "C" int te_batch_state(te_batch b, int instance, double* out_host) {
  if (!b || !b->ran || instance < 0 || instance >= b->B || !out_host) {
    te_set_error("te_batch_state: invalid arguments");
    return TE_ERR_INVALID_ARG;
  }
  const int64_t n = b->inst_n[instance];
  double2* tmp = nullptr;
  TE_CUDA(te_malloc(&tmp, sizeof(double2) * n));
  te_launch_permute(n, b->H[instance]->sell.iperm, b->sampled + b->inst_row[instance], tmp, b->st);
  int rc = te_cuda_check(cudaMemcpyAsync(out_host, tmp, sizeof(double2) * n, cudaMemcpyDeviceToHost, b->st), "D2H");
  if (rc == TE_OK) rc = te_cuda_check(cudaStreamSynchronize(b->st), "sync");
  te_free(tmp);
  return rc;
}

extern "C" int64_t te_batch_launch_count(te_batch b) { return b ? b->launches : 0; }

extern "C" int64_t te_batch_global_steps(te_batch b) { return b ? b->global_steps : 0; }

extern "C" int te_batch_set_option(te_batch b, int option, int value) {
  if (!b) {
    te_set_error("te_batch_set_option: null batch");
    return TE_ERR_INVALID_ARG;
  }
  switch (option) {
    case TE_BATCH_OPT_PERSISTENT:
      if (value != 0 && value != 1) break;
      b->persistent = value;
      return TE_OK;
    case TE_BATCH_OPT_BARRIER_SPIN_LIMIT:
      if (value < 1) break;
      b->spin_limit = (unsigned int)value;
      return TE_OK;
    case TE_BATCH_OPT_BARRIER_EXTRA_ARRIVALS:
      if (value != 0 && value != 1) break;
      b->extra_arrivals = (unsigned int)value;
      return TE_OK;
    default:
      te_set_error("te_batch_set_option: unknown option %d", option);
      return TE_ERR_INVALID_ARG;
  }
  te_set_error("te_batch_set_option: value %d out of range for option %d", value, option);
  return TE_ERR_INVALID_ARG;
}

extern "C" void* te_batch_stream(te_batch b) { return b ? (void*)b->st : nullptr; }

extern "C" int te_batch_destroy(te_batch b) {
  free_batch(b);
  return TE_OK;
}
