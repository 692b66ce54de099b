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

#include "te_internal.cuh"
#include "te_reduce.cuh"
#include "te_sell.cuh"

#define TE_BATCH_MAX_OBS 4

namespace {

struct BatchGeom {
  int64_t n_chunks;
  const int32_t* chunk_inst;  // instance of every chunk
  const int64_t* chunk_off;   // global SELL slot offsets (n_chunks + 1)
  const int32_t* col;         // global row indices
  const double* val;
  const int64_t* inst_row;    // first global row of each instance
  const int32_t* inst_n;      // dimension of each instance
  const int64_t* inst_chunk;  // first chunk of each instance (n_inst + 1)
  int64_t ld;                 // leading dimension of the basis (total padded rows)
  // chunks of the instances still running at the start of the global step
  // (null: every chunk); late global steps, when few instances are left, then
  // cost no more than those instances' work
  const int32_t* active;
  const int* active_count;
};

// The i-th chunk of a pass and the number of chunks to visit.
__device__ __forceinline__ int64_t batch_chunk_count(const BatchGeom& g) {
  return g.active ? (int64_t)*g.active_count : g.n_chunks;
}
__device__ __forceinline__ int64_t batch_chunk(const BatchGeom& g, int64_t i) {
  return g.active ? (int64_t)__ldg(g.active + i) : i;
}

// Compact the chunks of the running instances (one thread per chunk, one
// atomic per warp) for the once-per-step passes (new start vector, combine).
// The order of the list does not matter: those passes write rows, not sums.
__global__ void batch_active_kernel(int64_t n_chunks, const int32_t* __restrict__ chunk_inst,
                                    const TeDevState* states, int32_t* active, int* count) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n_chunks; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = base + threadIdx.x;
    bool keep = false;
    if (c < n_chunks) {
      const TeDevState* ds = states + chunk_inst[c];
      keep = !ds->done && !ds->fatal;
    }
    const unsigned mask = __ballot_sync(0xffffffffu, keep);
    int pos = 0;
    if (lane == 0 && mask) pos = atomicAdd(count, __popc(mask));
    pos = __shfl_sync(0xffffffffu, pos, 0);
    if (keep) active[pos + __popc(mask & ((1u << lane) - 1u))] = (int32_t)c;
  }
}

__device__ __forceinline__ bool lanczos_skip(const TeDevState* ds, int j) {
  return ds->fatal != 0 || ds->done != 0 || ds->breakdown != 0 || j >= ds->m_cur;
}

// ---------------------------------------------------------------------------
// Lanczos passes over the segmented layout.
//
// A schedule, recomputed on the device at the start of every global step,
// gives warp w the contiguous chunk range [warp_begin[w], warp_begin[w + 1])
// of equal FP64 cost over the running instances (finished instances inside a
// range are skipped whole).  A warp accumulates per lane across the chunks of
// one instance and reduces once per (warp, instance) segment; segment s of
// instance i goes to slot seg_base[i] + (w - inst_w0[i]), so the per-instance
// sum runs over consecutive slots in a fixed order (deterministic).  The
// recurrence is folded as in the single-instance passes: the apply pass
// stores w' = w / (e s_j), the update forms u'_{j+1} = w' - (alpha_j / e) u_j
// and sets s_{j+1} = e s_j / beta_{j+1}.

struct BatchSched {
  const int32_t* warp_begin;  // W + 1 global chunk indices
  const int32_t* inst_w0;     // first warp covering each instance
  const int32_t* inst_nseg;   // segments (warps) covering each running instance, 0 otherwise
  const int32_t* seg_base;    // first segment slot of each instance
  const int32_t* next_run;    // the next running instance after each instance (n_inst: none)
  const int32_t* inst_nwrite; // segments of each instance that are written (non-empty warps)
  unsigned int* arrivals;     // per instance: segments written so far (apply pass, update pass)
};

// Where a warp continues after the chunks of instance inst that it must skip:
// past every finished instance at once, or past this instance only.
__device__ __forceinline__ int64_t batch_skip_to(const BatchGeom& g, const BatchSched& sc, const TeDevState* ds,
                                                 int inst, int64_t cend) {
  const int64_t nxt = (ds->done || ds->fatal) ? (int64_t)g.inst_chunk[sc.next_run[inst]]
                                              : (int64_t)g.inst_chunk[inst + 1];
  return min(nxt, cend);
}

// One block: per-instance costs, warp boundaries by binary search, segment bases.
__global__ void __launch_bounds__(1024) batch_schedule_kernel(BatchGeom g, const TeDevState* states, int n_inst,
                                                              int n_warps, double w_slot, double* inst_cost,
                                                              int32_t* warp_begin, int32_t* inst_w0,
                                                              int32_t* inst_nseg, int32_t* seg_base,
                                                              int32_t* next_run, int32_t* inst_nwrite) {
  const double w_chunk = 8.0 * 32.0;
  __shared__ double total;
  for (int i = threadIdx.x; i < n_inst; i += blockDim.x) {
    const TeDevState& d = states[i];
    const int64_t c0 = g.inst_chunk[i], c1 = g.inst_chunk[i + 1];
    const bool run = !d.done && !d.fatal;
    inst_cost[i + 1] = run ? w_slot * (double)(g.chunk_off[c1] - g.chunk_off[c0]) + w_chunk * (double)(c1 - c0) : 0.0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // exclusive prefix over instances (n_inst is small)
    inst_cost[0] = 0.0;
    for (int i = 0; i < n_inst; ++i) inst_cost[i + 1] += inst_cost[i];
    total = inst_cost[n_inst];
  }
  __syncthreads();
  for (int w = threadIdx.x; w <= n_warps; w += blockDim.x) {
    int32_t c;
    const double target = total * (double)w / (double)n_warps;
    if (w == n_warps || !(total > 0.0)) {
      c = (int32_t)g.n_chunks;
    } else {
      int lo = 0, hi = n_inst - 1;  // instance k: inst_cost[k] <= target < inst_cost[k + 1]
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (inst_cost[mid] <= target)
          lo = mid;
        else
          hi = mid - 1;
      }
      int k = lo;
      while (k < n_inst - 1 && !(inst_cost[k + 1] > target)) ++k;  // step over empty (finished) instances
      const double rem = target - inst_cost[k];
      const int64_t c0 = g.inst_chunk[k], c1 = g.inst_chunk[k + 1];
      int64_t a = c0, b = c1;  // first chunk whose cost prefix within the instance reaches rem
      while (a < b) {
        const int64_t mid = (a + b) >> 1;
        const double cm = w_slot * (double)(g.chunk_off[mid] - g.chunk_off[c0]) + w_chunk * (double)(mid - c0);
        if (cm < rem)
          a = mid + 1;
        else
          b = mid;
      }
      c = (int32_t)a;
    }
    warp_begin[w] = c;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n_inst; i += blockDim.x) {
    const TeDevState& d = states[i];
    const int64_t c0 = g.inst_chunk[i], c1 = g.inst_chunk[i + 1];
    int nseg = 0, w0 = 0;
    if (!d.done && !d.fatal && c1 > c0) {
      auto last_warp_at_or_before = [&](int64_t c) {  // last w with warp_begin[w] <= c
        int lo = 0, hi = n_warps;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (warp_begin[mid] <= c)
            lo = mid;
          else
            hi = mid - 1;
        }
        return lo;
      };
      w0 = last_warp_at_or_before(c0);
      nseg = last_warp_at_or_before(c1 - 1) - w0 + 1;
    }
    inst_w0[i] = w0;
    inst_nseg[i] = nseg;
    int nw = 0;
    for (int s = 0; s < nseg; ++s) nw += warp_begin[w0 + s] < warp_begin[w0 + s + 1];
    inst_nwrite[i] = nw;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int32_t base = 0;
    for (int i = 0; i < n_inst; ++i) {
      seg_base[i] = base;
      base += inst_nseg[i];
    }
  } else if (threadIdx.x == 32) {
    int32_t nxt = n_inst;  // next running instance after i
    for (int i = n_inst - 1; i >= 0; --i) {
      next_run[i] = nxt;
      if (!states[i].done && !states[i].fatal) nxt = i;
    }
  }
}

// Lane 0 has written this warp's segment partial(s) of instance inst; the warp
// that completes the instance's count sums its written segments in slot order
// (the same order whichever warp comes last) and returns true with the sums in
// every lane.  NV values per segment at seg_partials[NV * slot + k].
template <int NV>
__device__ __forceinline__ bool batch_segment_done(const BatchSched& sc, int inst, int which,
                                                   const double* seg_partials, double (&tot)[NV]) {
  const int lane = threadIdx.x & 31;
  unsigned int prev = 0;
  if (lane == 0) {
    __threadfence();
    prev = atomicAdd(&sc.arrivals[2 * inst + which], 1u);
  }
  prev = __shfl_sync(0xffffffffu, prev, 0);
  if (prev + 1 != (unsigned int)sc.inst_nwrite[inst]) return false;
  __threadfence();
  const int64_t s0 = sc.seg_base[inst];
  const int w0 = sc.inst_w0[inst], ns = sc.inst_nseg[inst];
#pragma unroll
  for (int k = 0; k < NV; ++k) tot[k] = 0.0;
  for (int s = lane; s < ns; s += 32) {
    if (!(sc.warp_begin[w0 + s] < sc.warp_begin[w0 + s + 1])) continue;  // an empty warp wrote nothing
#pragma unroll
    for (int k = 0; k < NV; ++k) tot[k] += __ldcg(seg_partials + NV * (s0 + s) + k);
  }
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    tot[k] = te_warp_sum(tot[k]);
    tot[k] = __shfl_sync(0xffffffffu, tot[k], 0);
  }
  if (lane == 0) sc.arrivals[2 * inst + which] = 0u;  // ready for the next pass
  return true;
}

template <bool REAL, bool HAS_PREV>
__global__ void __launch_bounds__(TE_THREADS, REAL ? 6 : 5) batch_apply_kernel(BatchGeom g, BatchSched sc,
                                                                 const double2* __restrict__ V,
                                                                 double2* __restrict__ w, TeDevState* states,
                                                                 double* seg_partials, int j) {
  const int lane = threadIdx.x & 31;
  const int wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const double2* __restrict__ u_j = V + (int64_t)j * g.ld;
  const double2* __restrict__ u_jm1 = HAS_PREV ? V + (int64_t)(j - 1) * g.ld : nullptr;
  int64_t c = sc.warp_begin[wid];
  const int64_t cend = sc.warp_begin[wid + 1];
  while (c < cend) {
    const int inst = __ldg(g.chunk_inst + c);
    const TeDevState* ds = states + inst;
    const int64_t c1 = min((int64_t)__ldg(g.inst_chunk + inst + 1), cend);
    if (lanczos_skip(ds, j)) {
      c = batch_skip_to(g, sc, ds, inst, cend);
      continue;
    }
    const double sj = ds->s[j];
    const double gg = ds->exp_factor * sj;
    double cw = 0.0;
    if (HAS_PREV) {
      const double bie = ds->beta[j] * ds->inv_exp_factor;
      cw = bie * bie;
    }
    const int64_t row0 = __ldg(g.inst_row + inst);
    const int n_i = __ldg(g.inst_n + inst);
    double a0 = 0.0, a1 = 0.0;
    for (; c < c1; ++c) {
      const double2 y = te_sell_row<REAL>(g.chunk_off, g.col, g.val, u_j, c, lane);
      const int64_t r = c * 32 + lane;
      double2 wr = make_double2(0.0, 0.0);
      if (r - row0 < n_i) {
        if (HAS_PREV) {
          const double2 up = u_jm1[r];
          wr.x = fma(cw, up.x, y.y);
          wr.y = fma(cw, up.y, -y.x);
        } else {
          wr.x = y.y;
          wr.y = -y.x;
        }
        const double2 uj = u_j[r];
        a0 = fma(uj.x, wr.x, fma(uj.y, wr.y, a0));
        a1 = fma(uj.x, wr.y, fma(-uj.y, wr.x, a1));
      }
      w[r] = wr;
    }
    a0 = te_warp_sum(a0);
    a1 = te_warp_sum(a1);
    if (lane == 0) {
      const int64_t seg = sc.seg_base[inst] + (wid - sc.inst_w0[inst]);
      seg_partials[2 * seg] = a0;
      seg_partials[2 * seg + 1] = a1;
    }
    double tot[2];
    if (batch_segment_done<2>(sc, inst, 0, seg_partials, tot) && lane == 0) {
      const double f = sj * gg;  // alpha_j = s_j g <u_j, w'>
      states[inst].alpha[j] = make_double2(f * tot[0], f * tot[1]);
    }
  }
}

__global__ void __launch_bounds__(TE_THREADS) batch_update_kernel(BatchGeom g, BatchSched sc,
                                                                  double2* __restrict__ V,
                                                                  const double2* __restrict__ w, TeDevState* states,
                                                                  double* seg_partials, int j) {
  const int lane = threadIdx.x & 31;
  const int wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const double2* __restrict__ u_j = V + (int64_t)j * g.ld;
  double2* __restrict__ u_jp1 = V + (int64_t)(j + 1) * g.ld;
  int64_t c = sc.warp_begin[wid];
  const int64_t cend = sc.warp_begin[wid + 1];
  while (c < cend) {
    const int inst = __ldg(g.chunk_inst + c);
    const TeDevState* ds = states + inst;
    const int64_t c1 = min((int64_t)__ldg(g.inst_chunk + inst + 1), cend);
    if (lanczos_skip(ds, j)) {
      c = batch_skip_to(g, sc, ds, inst, cend);
      continue;
    }
    const double2 al = ds->alpha[j];
    const double q = ds->inv_exp_factor;  // alpha_j s_j / (e s_j)
    const double gr = al.x * q, gi = al.y * q;
    const bool store = j + 1 < ds->m_cur;
    const int64_t row0 = __ldg(g.inst_row + inst);
    const int n_i = __ldg(g.inst_n + inst);
    double nrm = 0.0;
    for (; c < c1; ++c) {
      const int64_t r = c * 32 + lane;
      double2 o = make_double2(0.0, 0.0);
      if (r - row0 < n_i) {
        const double2 wv = w[r], u = u_j[r];
        o.x = fma(-gr, u.x, fma(gi, u.y, wv.x));
        o.y = fma(-gr, u.y, fma(-gi, u.x, wv.y));
        nrm = fma(o.x, o.x, fma(o.y, o.y, nrm));
      }
      if (store) u_jp1[r] = o;
    }
    nrm = te_warp_sum(nrm);
    if (lane == 0) seg_partials[sc.seg_base[inst] + (wid - sc.inst_w0[inst])] = nrm;
    double tot[1];
    if (batch_segment_done<1>(sc, inst, 1, seg_partials, tot) && lane == 0) {
      TeDevState* dw = states + inst;
      const double g = dw->exp_factor * dw->s[j];
      const double beta = fabs(g) * sqrt(tot[0]);
      const int m = dw->m_cur;
      if (beta < dw->tol_rate) {  // lucky breakdown (:551-555)
        dw->breakdown = 1;
        dw->m_eff = j + 1;
        dw->h = beta;
      } else if (j + 1 != m) {
        dw->beta[j + 1] = beta;
        dw->s[j + 1] = g / beta;
      } else {
        dw->h = beta;
        dw->m_eff = m;
      }
    }
  }
}

// Start vector of the next step: u_0 = the w of the previous step.
__global__ void __launch_bounds__(TE_THREADS) batch_new_start_kernel(BatchGeom g, double2* __restrict__ V,
                                                                     const double2* __restrict__ spare,
                                                                     const TeDevState* states) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t n_visit = batch_chunk_count(g);
  for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n_visit; i += warps) {
    const int64_t c = batch_chunk(g, i);
    const int inst = __ldg(g.chunk_inst + c);
    const TeDevState* ds = states + inst;
    if (!ds->new_start || ds->fatal || ds->done) continue;
    const int64_t r = c * 32 + lane;
    V[r] = spare[r];
  }
}

// Clear the new-start flags once the copies are done (one thread per instance).
__global__ void batch_clear_start_kernel(TeDevState* states, int n_inst) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_inst; i += gridDim.x * blockDim.x)
    states[i].new_start = 0;
}

// psi = sum_j u_j Y[slot][j] for each instance's outputs of this batch:
// slot 0 (w) -> spare, slot 1 (the sample; batches hold one sample) -> sampled.
template <int G>
__device__ __forceinline__ void batch_combine_rows(const double2* __restrict__ V, int64_t ld, int64_t r, int m,
                                                   const double2* Y, const int* slots, double2* spare,
                                                   double2* sampled) {
  double2 acc[G];
#pragma unroll
  for (int o = 0; o < G; ++o) acc[o] = make_double2(0.0, 0.0);
  for (int j = 0; j < m; ++j) {
    const double2 u = V[(int64_t)j * ld + r];
#pragma unroll
    for (int o = 0; o < G; ++o) {
      const double2 y = Y[slots[o] * TE_MMAX + j];
      acc[o].x = fma(u.x, y.x, fma(-u.y, y.y, acc[o].x));
      acc[o].y = fma(u.x, y.y, fma(u.y, y.x, acc[o].y));
    }
  }
#pragma unroll
  for (int o = 0; o < G; ++o) {
    if (slots[o] == 0)
      spare[r] = acc[o];
    else
      sampled[r] = acc[o];
  }
}

__global__ void __launch_bounds__(TE_THREADS) batch_combine_kernel(BatchGeom g, const double2* __restrict__ V,
                                                                   double2* spare, double2* sampled,
                                                                   const TeDevState* states, int m_override) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t n_visit = batch_chunk_count(g);
  for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n_visit; i += warps) {
    const int64_t c = batch_chunk(g, i);
    const int inst = __ldg(g.chunk_inst + c);
    const TeDevState* ds = states + inst;
    if (ds->fatal) continue;
    const int want_w = ds->want_w, S = ds->samples_in_batch;
    const int nout = want_w + S;
    if (nout == 0) continue;
    const int m = m_override > 0 ? m_override : ds->m_eff;
    const int64_t r = c * 32 + lane;
    int slots[2];
    slots[0] = want_w ? 0 : 1;
    slots[1] = 1;
    if (nout == 1)
      batch_combine_rows<1>(V, g.ld, r, m, ds->Y, slots, spare, sampled);
    else
      batch_combine_rows<2>(V, g.ld, r, m, ds->Y, slots, spare, sampled);
  }
}

// Diagonal observables of every instance with a sample in this batch
// (one block per instance): Re sum_i O_ii |psi_i|^2.
__global__ void __launch_bounds__(TE_THREADS) batch_obs_kernel(BatchGeom g, const double2* __restrict__ sampled,
                                                               const double* __restrict__ diag, const int* n_obs,
                                                               const int64_t* result_off, double* results,
                                                               TeDevState* states) {
  __shared__ double scratch[TE_BATCH_MAX_OBS * 32];
  const int inst = blockIdx.x;
  TeDevState* ds = states + inst;
  const int no = n_obs[inst];
  if (ds->fatal || ds->samples_in_batch == 0 || no == 0) return;
  const int64_t r0 = g.inst_row[inst];
  const int n = g.inst_n[inst];
  double acc[TE_BATCH_MAX_OBS] = {0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double2 p = sampled[r0 + i];
    const double p2 = fma(p.x, p.x, p.y * p.y);
    for (int k = 0; k < no; ++k) acc[k] = fma(diag[(int64_t)k * g.ld + r0 + i], p2, acc[k]);
  }
  te_block_sum<TE_BATCH_MAX_OBS>(acc, scratch);
  if (threadIdx.x == 0) {
    const int s = ds->sample_base;
    for (int k = 0; k < no; ++k) results[result_off[inst] + (int64_t)k * ds->n_samples + s] = acc[k];
  }
}

// ||sampled||^2 of every instance (final norm check of :446).
__global__ void __launch_bounds__(TE_THREADS) batch_norm_kernel(BatchGeom g, const double2* __restrict__ sampled,
                                                                TeDevState* states) {
  __shared__ double scratch[32];
  const int inst = blockIdx.x;
  const int64_t r0 = g.inst_row[inst];
  const int n = g.inst_n[inst];
  double acc[1] = {0.0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double2 p = sampled[r0 + i];
    acc[0] = fma(p.x, p.x, fma(p.y, p.y, acc[0]));
  }
  te_block_sum<1>(acc, scratch);
  if (threadIdx.x == 0) states[inst].norm2_final = acc[0];
}

// One flag word per instance: bit0 done, bit1 samples pending, bit2 fatal.
__global__ void batch_flags_kernel(const TeDevState* states, int n_inst, int* flags) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_inst; i += gridDim.x * blockDim.x) {
    const TeDevState& d = states[i];
    flags[i] = (d.done ? 1 : 0) | (d.samples_pending && !d.done ? 2 : 0) | (d.fatal ? 4 : 0);
  }
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
  cudaFree(b->d_chunk_inst);
  cudaFree(b->d_chunk_off);
  cudaFree(b->d_col);
  cudaFree(b->d_val);
  cudaFree(b->d_inst_row);
  cudaFree(b->d_inst_n);
  cudaFree(b->d_inst_chunk);
  cudaFree(b->ds);
  cudaFree(b->V);
  cudaFree(b->spare);
  cudaFree(b->w);
  cudaFree(b->sampled);
  cudaFree(b->v0);
  cudaFree(b->diag);
  cudaFree(b->d_nobs);
  cudaFree(b->d_result_off);
  cudaFree(b->results);
  cudaFree(b->d_flags);
  cudaFreeHost(b->h_flags);
  cudaFree(b->d_active);
  cudaFree(b->d_active_count);
  cudaFree(b->d_warp_begin);
  cudaFree(b->d_inst_w0);
  cudaFree(b->d_inst_nseg);
  cudaFree(b->d_seg_base);
  cudaFree(b->d_next_run);
  cudaFree(b->d_inst_nwrite);
  cudaFree(b->d_arrivals);
  cudaFree(b->d_inst_cost);
  cudaFree(b->seg_partials);
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

// Warps of the Lanczos passes: one resident wave of the apply/update kernels.
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
    double nrm = 0.0;
    for (int64_t k = 0; k < 2 * n; ++k) nrm += v_host[i][k] * v_host[i][k];
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
  auto alloc = [&](void** p, size_t bytes) { return te_cuda_check(cudaMalloc(p, std::max<size_t>(bytes, 16)), "alloc"); };
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
  // segments: every warp has at most one per instance it touches
  if ((rc = alloc((void**)&b->seg_partials, sizeof(double) * 2 * ((int64_t)b->n_warps + n_instances + 1))) != TE_OK)
    return fail(rc);
  TE_CUDA(cudaMallocHost(&b->h_flags, sizeof(int) * n_instances));
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
  cudaFree(tmp);
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
    TE_CUDA(cudaMalloc(&b->results, sizeof(double) * std::max<int64_t>(tot, 1)));
    TE_CUDA(cudaMemset(b->results, 0, sizeof(double) * std::max<int64_t>(tot, 1)));
    TE_CUDA(cudaMemcpy(b->d_result_off, b->result_off.data(), sizeof(int64_t) * b->B, cudaMemcpyHostToDevice));
  }
  int rc = reset_states(b);
  if (rc != TE_OK) return rc;
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
    if (fatal || all_done) break;
  }
  batch_norm_kernel<<<b->B, TE_THREADS, 0, b->st>>>(geom(b), b->sampled, b->ds);
  b->launches += 1;
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
  TE_CUDA(cudaMalloc(&tmp, sizeof(double2) * n));
  te_launch_permute(n, b->H[instance]->sell.iperm, b->sampled + b->inst_row[instance], tmp, b->st);
  int rc = te_cuda_check(cudaMemcpyAsync(out_host, tmp, sizeof(double2) * n, cudaMemcpyDeviceToHost, b->st), "D2H");
  if (rc == TE_OK) rc = te_cuda_check(cudaStreamSynchronize(b->st), "sync");
  cudaFree(tmp);
  return rc;
}

extern "C" int64_t te_batch_launch_count(te_batch b) { return b ? b->launches : 0; }

extern "C" void* te_batch_stream(te_batch b) { return b ? (void*)b->st : nullptr; }

extern "C" int te_batch_destroy(te_batch b) {
  free_batch(b);
  return TE_OK;
}
