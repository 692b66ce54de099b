// te_batch.cuh -- device bodies of the batched evolution passes, shared by the
// per-pass kernels of te_batch.cu (replayed as a CUDA graph per global step)
// and by the persistent batched kernel of te_krylov.cu (one cooperative launch
// for a whole batch run), so both run the same arithmetic in the same order.
//
// Segmented layout: one SELL-32 matrix over the concatenated (length-sorted)
// rows of all instances; a chunk of 32 rows never straddles two instances, so
// a warp always works for one instance and reads its scalars once.
//
// Every multiply-add here is an explicit fma(): the bodies are compiled into
// two translation units (te_krylov.cu without implicit contraction), and
// results must not depend on where the compiler fuses.
//
// XCG (persistent kernel): vectors that the launch itself rewrites at every
// global step are read with L2-only loads, never through the read-only cache
// or an L1 copy that may predate the last write; te_krylov.cu, which holds the
// persistent kernel, is compiled with L2-only default loads for the same
// reason (the instance states, the schedule, the active-chunk list).
#pragma once
#include "te_internal.cuh"
#include "te_reduce.cuh"
#include "te_sell.cuh"

#define TE_BATCH_MAX_OBS 4

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

// The Lanczos schedule of one global step (batch_schedule_body).
struct BatchSched {
  const int32_t* warp_begin;  // W + 1 global chunk indices
  const int32_t* inst_w0;     // first warp covering each instance
  const int32_t* inst_nseg;   // segments (warps) covering each running instance, 0 otherwise
  const int32_t* seg_base;    // first segment slot of each instance
  const int32_t* next_run;    // the next running instance after each instance (n_inst: none)
  const int32_t* inst_nwrite; // segments of each instance that are written (non-empty warps)
  unsigned int* arrivals;     // per instance: segments written so far (apply pass, update pass)
};

// Arguments of the persistent batched kernel (te_krylov.cu).
#define TE_BATCH_PTHREADS 1024
struct TeBatchPersist {
  BatchGeom g;    // with the active-chunk list
  BatchSched sc;  // read side of the schedule
  // write side of the schedule (block 0 rebuilds it every global step)
  double* inst_cost;
  int32_t *warp_begin, *inst_w0, *inst_nseg, *seg_base, *next_run, *inst_nwrite;
  int32_t* active;
  int* active_count;
  double2 *V, *w, *spare, *sampled;
  TeDevState* states;
  double* seg_partials;
  const double* diag;
  const int* n_obs;
  const int64_t* result_off;
  double* results;
  int n_inst, m_max, n_warps;
  bool is_real;
  double w_slot;
  // grid barrier: arrival count, generation, error word, polls before giving up
  unsigned int* bar_count;
  unsigned int* bar_gen;
  int* err;
  unsigned int spin_limit;
  unsigned int arrivals;  // arrivals that complete a barrier (the grid; one more only to test the timeout)
  int64_t max_global_steps;
  int64_t* steps_done;
};
// Blocks of one co-resident wave of the persistent kernel (0: not available).
int te_batch_persistent_grid(bool is_real);
int te_launch_batch_persistent(const TeBatchPersist& a, int grid, cudaStream_t st);

namespace {

// Loads of data that the persistent kernel itself rewrites (other SMs, before
// a grid barrier, again and again over the global steps): L2-only loads there
// (this SM's L1 may hold a copy from an earlier step), never the read-only
// path that a const __restrict__ pointer would allow.
template <bool XCG, typename T>
__device__ __forceinline__ T bload(const T* p) {
  if (XCG) return __ldcg(p);
  return *p;
}


// The i-th chunk of a pass and the number of chunks to visit.
__device__ __forceinline__ int64_t batch_chunk_count(const BatchGeom& g) {
  return g.active ? (int64_t)*g.active_count : g.n_chunks;
}
__device__ __forceinline__ int64_t batch_chunk(const BatchGeom& g, int64_t i) {
  return g.active ? (int64_t)g.active[i] : i;
}

// Compact the chunks of the running instances (thread t of T takes chunks
// t, t + T, ... in warp-aligned groups; one atomic per warp) for the
// once-per-step passes (new start vector, combine).  The order of the list
// does not matter: those passes write rows, not sums.
__device__ __forceinline__ void batch_active_body(int64_t n_chunks, const int32_t* __restrict__ chunk_inst,
                                                  const TeDevState* states, int32_t* active, int* count,
                                                  int64_t t0, int64_t T) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = t0 - lane; base < n_chunks; base += T) {
    const int64_t c = base + lane;
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
// and sets s_{j+1} = e s_j / beta_{j+1}.  "Warps" of the schedule are logical:
// the graph path launches one hardware warp per schedule warp, the persistent
// kernel loops its warps over them.


// Where a warp continues after the chunks of instance inst that it must skip:
// past every finished instance at once, or past this instance only.
__device__ __forceinline__ int64_t batch_skip_to(const BatchGeom& g, const BatchSched& sc, const TeDevState* ds,
                                                 int inst, int64_t cend) {
  const int64_t nxt = (ds->done || ds->fatal) ? (int64_t)g.inst_chunk[sc.next_run[inst]]
                                              : (int64_t)g.inst_chunk[inst + 1];
  return min(nxt, cend);
}

// Per-instance costs, warp boundaries by binary search, segment bases (one
// block; *total is a shared-memory double).
__device__ __forceinline__ void batch_schedule_body(const BatchGeom& g, const TeDevState* states, int n_inst,
                                                    int n_warps, double w_slot, double* inst_cost,
                                                    int32_t* warp_begin, int32_t* inst_w0, int32_t* inst_nseg,
                                                    int32_t* seg_base, int32_t* next_run, int32_t* inst_nwrite,
                                                    double* total) {
  const double w_chunk = 8.0 * 32.0;
  for (int i = threadIdx.x; i < n_inst; i += blockDim.x) {
    const TeDevState& d = states[i];
    const int64_t c0 = g.inst_chunk[i], c1 = g.inst_chunk[i + 1];
    const bool run = !d.done && !d.fatal;
    inst_cost[i + 1] =
        run ? fma(w_slot, (double)(g.chunk_off[c1] - g.chunk_off[c0]), w_chunk * (double)(c1 - c0)) : 0.0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // exclusive prefix over instances (n_inst is small)
    inst_cost[0] = 0.0;
    for (int i = 0; i < n_inst; ++i) inst_cost[i + 1] += inst_cost[i];
    *total = inst_cost[n_inst];
  }
  __syncthreads();
  const double tot = *total;
  for (int w = threadIdx.x; w <= n_warps; w += blockDim.x) {
    int32_t c;
    const double target = tot * (double)w / (double)n_warps;
    if (w == n_warps || !(tot > 0.0)) {
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
        const double cm = fma(w_slot, (double)(g.chunk_off[mid] - g.chunk_off[c0]), w_chunk * (double)(mid - c0));
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

// Apply pass of schedule warp wid: w' = -i H u_j + (beta_j / e)^2 u_{j-1} over
// its chunks, alpha_j = s_j g <u_j, w'> per instance.
template <bool REAL, bool HAS_PREV, bool XCG>
__device__ __forceinline__ void batch_apply_warp(const BatchGeom& g, const BatchSched& sc,
                                                 const double2* __restrict__ V, double2* __restrict__ w,
                                                 TeDevState* states, double* seg_partials, int j, int wid) {
  const int lane = threadIdx.x & 31;
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
      const double2 y = te_sell_row<REAL, XCG ? 2 : 0>(g.chunk_off, g.col, g.val, u_j, c, lane);
      const int64_t r = c * 32 + lane;
      double2 wr = make_double2(0.0, 0.0);
      if (r - row0 < n_i) {
        if (HAS_PREV) {
          const double2 up = bload<XCG>(u_jm1 + r);
          wr.x = fma(cw, up.x, y.y);
          wr.y = fma(cw, up.y, -y.x);
        } else {
          wr.x = y.y;
          wr.y = -y.x;
        }
        const double2 uj = bload<XCG>(u_j + r);
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

// Update pass of schedule warp wid: u'_{j+1} = w' - (alpha_j / e) u_j,
// beta_{j+1} = |e s_j| ||u'_{j+1}|| per instance, breakdown test.
template <bool XCG>
__device__ __forceinline__ void batch_update_warp(const BatchGeom& g, const BatchSched& sc, double2* __restrict__ V,
                                                  const double2* __restrict__ w, TeDevState* states,
                                                  double* seg_partials, int j, int wid) {
  const int lane = threadIdx.x & 31;
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
        const double2 wv = bload<XCG>(w + r), u = bload<XCG>(u_j + r);
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
      const double ge = dw->exp_factor * dw->s[j];
      const double beta = fabs(ge) * sqrt(tot[0]);
      const int m = dw->m_cur;
      if (beta < dw->tol_rate) {  // lucky breakdown (:551-555)
        dw->breakdown = 1;
        dw->m_eff = j + 1;
        dw->h = beta;
      } else if (j + 1 != m) {
        dw->beta[j + 1] = beta;
        dw->s[j + 1] = ge / beta;
      } else {
        dw->h = beta;
        dw->m_eff = m;
      }
    }
  }
}

// Start vector of the next step: u_0 = the w of the previous step (warp wi of
// nw over the visited chunks).
template <bool XCG>
__device__ __forceinline__ void batch_new_start_body(const BatchGeom& g, double2* __restrict__ V,
                                                     const double2* __restrict__ spare, const TeDevState* states,
                                                     int64_t wi, int64_t nw) {
  const int lane = threadIdx.x & 31;
  const int64_t n_visit = batch_chunk_count(g);
  for (int64_t i = wi; i < n_visit; i += nw) {
    const int64_t c = batch_chunk(g, i);
    const int inst = __ldg(g.chunk_inst + c);
    const TeDevState* ds = states + inst;
    if (!ds->new_start || ds->fatal || ds->done) continue;
    const int64_t r = c * 32 + lane;
    V[r] = bload<XCG>(spare + r);
  }
}

// psi = sum_j u_j Y[slot][j] for each instance's outputs of this batch:
// slot 0 (w) -> spare, slot 1 (the sample; batches hold one sample) -> sampled.
template <int G, bool XCG>
__device__ __forceinline__ void batch_combine_rows(const double2* __restrict__ V, int64_t ld, int64_t r, int m,
                                                   const double2* Y, const int* slots, double2* spare,
                                                   double2* sampled) {
  double2 acc[G];
#pragma unroll
  for (int o = 0; o < G; ++o) acc[o] = make_double2(0.0, 0.0);
  for (int j = 0; j < m; ++j) {
    const double2 u = bload<XCG>(V + (int64_t)j * ld + r);
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

template <bool XCG>
__device__ __forceinline__ void batch_combine_body(const BatchGeom& g, const double2* __restrict__ V, double2* spare,
                                                   double2* sampled, const TeDevState* states, int m_override,
                                                   int64_t wi, int64_t nw) {
  const int lane = threadIdx.x & 31;
  const int64_t n_visit = batch_chunk_count(g);
  for (int64_t i = wi; i < n_visit; i += nw) {
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
      batch_combine_rows<1, XCG>(V, g.ld, r, m, ds->Y, slots, spare, sampled);
    else
      batch_combine_rows<2, XCG>(V, g.ld, r, m, ds->Y, slots, spare, sampled);
  }
}

// Sum of NV values over a group of nthreads = 32 k threads (thread tid of the
// group; result in tid 0) in the order of te_block_sum over a block of that
// size: warp trees, then warp 0 adds the warps' sums.  sync() synchronises the
// group; scratch holds NV * 32 doubles of the group.
template <int NV, typename Sync>
__device__ __forceinline__ void batch_group_sum(double (&v)[NV], double* scratch, int tid, int nthreads, Sync sync) {
  const int lane = tid & 31, warp = tid >> 5, nw = nthreads >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = te_warp_sum(v[k]);
  sync();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) scratch[k * 32 + warp] = v[k];
  }
  sync();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = lane < nw ? scratch[k * 32 + lane] : 0.0;
      v[k] = te_warp_sum(x);
    }
  }
  sync();
}

// Diagonal observables of instance inst with a sample in this batch, by a
// group of nthreads threads: Re sum_i O_ii |psi_i|^2 into the results table.
template <bool XCG, typename Sync>
__device__ __forceinline__ void batch_obs_inst(const BatchGeom& g, const double2* __restrict__ sampled,
                                               const double* __restrict__ diag, const int* n_obs,
                                               const int64_t* result_off, double* results, TeDevState* states,
                                               int inst, int tid, int nthreads, double* scratch, Sync sync) {
  TeDevState* ds = states + inst;
  const int no = n_obs[inst];
  if (ds->fatal || ds->samples_in_batch == 0 || no == 0) return;
  const int64_t r0 = g.inst_row[inst];
  const int n = g.inst_n[inst];
  double acc[TE_BATCH_MAX_OBS] = {0.0, 0.0, 0.0, 0.0};
  for (int i = tid; i < n; i += nthreads) {
    const double2 p = bload<XCG>(sampled + r0 + i);
    const double p2 = fma(p.x, p.x, p.y * p.y);
    for (int k = 0; k < no; ++k) acc[k] = fma(diag[(int64_t)k * g.ld + r0 + i], p2, acc[k]);
  }
  batch_group_sum<TE_BATCH_MAX_OBS>(acc, scratch, tid, nthreads, sync);
  if (tid == 0) {
    const int s = ds->sample_base;
    for (int k = 0; k < no; ++k) results[result_off[inst] + (int64_t)k * ds->n_samples + s] = acc[k];
  }
}

// ||sampled||^2 of instance inst (final norm check of :446), by a group.
template <bool XCG, typename Sync>
__device__ __forceinline__ void batch_norm_inst(const BatchGeom& g, const double2* __restrict__ sampled,
                                                TeDevState* states, int inst, int tid, int nthreads, double* scratch,
                                                Sync sync) {
  const int64_t r0 = g.inst_row[inst];
  const int n = g.inst_n[inst];
  double acc[1] = {0.0};
  for (int i = tid; i < n; i += nthreads) {
    const double2 p = bload<XCG>(sampled + r0 + i);
    acc[0] = fma(p.x, p.x, fma(p.y, p.y, acc[0]));
  }
  batch_group_sum<1>(acc, scratch, tid, nthreads, sync);
  if (tid == 0) states[inst].norm2_final = acc[0];
}

// One flag word per instance: bit0 done, bit1 samples pending, bit2 fatal.
__device__ __forceinline__ int batch_flag(const TeDevState& d) {
  return (d.done ? 1 : 0) | (d.samples_pending && !d.done ? 2 : 0) | (d.fatal ? 4 : 0);
}

}  // namespace
