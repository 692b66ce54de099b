// te_krylov.cu -- the Krylov-space part of one time step, on one thread block.
//
// Replaces, per Krylov step of krylovTimeEvolver::timeEvolve
// (core/krylovTimeEvolver.cpp:261-512):
//   LAPACKE_zhseqr on the m x m Krylov matrix (:365, matrixDataTypes.h:135-156),
//   expKrylov (:685-702), integrateError (:584-618),
//   findMaximalStepSize (:153-254), and the sampling schedule of :405-421.
//
// Krylov matrix.  Lanczos on A = -i expFactor H gives H_k with diagonal
// alpha_j (imaginary up to rounding) and off-diagonals +-beta_j.  With
// D = diag(i^j), H_k = D (-i T) D^{-1} where T is the real symmetric
// tridiagonal matrix with T_jj = -Im(alpha_j), T_{j,j+1} = beta_{j+1}; so
// exp(x H_k) e_1 = D exp(-i x T) e_1 (the rounding-level real parts of
// alpha_j are dropped).
//
// Exponential.  On GB300 FP64 issue is the scarce resource (a warp FP64
// instruction costs the same with 1 or 32 lanes active), so the dense
// eigensolve of the reference is replaced on the hot path by the
// Chebyshev-Bessel (Jacobi-Anger) expansion
//   exp(-i x T) e_1 = e^{-ixc} sum_n eps_n (-i)^n J_n(x rho) t_n,
//   t_n = T_n((T - c)/rho) e_1,   [c - rho, c + rho] = Gershgorin interval,
// with the vectors t_n built once per step by the three-term recurrence and
// the Bessel values J_n by Miller's backward recurrence (one lane per
// abscissa, all lanes busy).  The error integrand h |e_m^T exp(-ixT) e_1|
// only involves n >= m-1 (t_n has support 0..n), so it is evaluated without
// the cancellation of the eigenvector form.  Arguments x rho beyond the
// stored degree (lucky-breakdown steps that jump to the final time, very long
// step candidates) use the eigen-decomposition T = Q diag(lam) Q^T computed
// by implicit symmetric QR with Wilkinson shifts on one warp.
//
// Quadrature.  Tanh-sinh with the level rule shared with the CPU oracle
// (nodes t in [-3, 3], level k adds odd multiples of 2^-k, stop at the first
// level k >= 2 with |I_k - I_{k-1}| <= 1e-3 L1_k, at most level 8); levels
// 0..4 are evaluated together (97 abscissae).  Gauss-Legendre 15/7 for
// fastIntegration.  The step-size search runs the reference's control flow
// with every integral block-parallel; all threads follow the same branches.
#include <cfloat>
#include <cmath>
#include <vector>

#include "te_batch.cuh"
#include "te_internal.cuh"

__constant__ TeQuadTables c_quad;

#define TE_KBUF 8  // outputs per coefficient group

struct KSmem {
  double tc[(TE_NCHEB + 1) * TE_MMAX];  // Chebyshev vectors, row n
  double fp[TE_TS_NODES], fm[TE_TS_NODES];
  double Q[TE_MMAX * TE_MMAX];          // eigenvectors (col-major), fallback path
  double J[TE_KBUF][TE_NCHEB + 8];      // Bessel values per output
  double lam[TE_MMAX];
  double d[TE_MMAX], e[TE_MMAX], dd[TE_MMAX], ee[TE_MMAX];
  double gs[TE_NCHEB + 8];              // signed, doubled last components of t_n
  double rc[TE_MMAX], rs[TE_MMAX];      // rotations of one QR sweep
  double red[64];
  double bc[16];
  int ibc[16];
};

static_assert(sizeof(KSmem) + 4096 <= 232448, "Krylov kernel shared memory exceeds the per-block limit");

__device__ __forceinline__ double warp_sum_all(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Miller start index (multiple of 4) for accurate J_n(z), n <= max(m, z).
__device__ __forceinline__ int bessel_start(double z, int m) {
  double a = fmax((double)m, z);
  double k0 = a + 25.0 + 2.0 * sqrt(a);
  if (!(k0 < 1e6)) return 1 << 30;
  return 4 * (int)ceil(k0 * 0.25);
}

__device__ __forceinline__ bool needs_rescale(double v) {
  int hi = __double2hiint(v);
  return ((hi >> 20) & 0x7ff) > 1023 + 600;
}

struct KCtx {
  TeDevState* ds;
  KSmem* sm;
  int m;
  double h, rho, c;
  int cheb_n;     // Chebyshev vectors available up to this degree
  bool eig_ok;    // eigen-decomposition available
  int fatal;
};

// ------------------------------------------------------------ Chebyshev

// Extend t_n (and the signed last components gs) up to degree K
// (block-cooperative; K >= 2).
__device__ void ensure_cheb(KCtx& C, int K) {
  if (K <= C.cheb_n) return;
  KSmem* S = C.sm;
  const int m = C.m;
  const int j = threadIdx.x;
  const int old = C.cheb_n;
  int n0 = old;
  if (old < 0) {
    if (j < TE_MMAX) S->tc[j] = (j == 0) ? 1.0 : 0.0;
    __syncthreads();
    if (j < TE_MMAX) {
      double v = 0.0;
      if (j < m) {
        v = 0.5 * S->dd[j] * S->tc[j];
        if (j > 0) v = fma(0.5 * S->ee[j - 1], S->tc[j - 1], v);
        if (j + 1 < m) v = fma(0.5 * S->ee[j], S->tc[j + 1], v);
      }
      S->tc[TE_MMAX + j] = v;
    }
    __syncthreads();
    n0 = 1;
  }
  for (int n = n0; n < K; ++n) {
    if (j < TE_MMAX) {
      const double* tn = S->tc + n * TE_MMAX;
      const double* tp = S->tc + (n - 1) * TE_MMAX;
      double v = 0.0;
      if (j < m) {
        v = fma(S->dd[j], tn[j], -tp[j]);
        if (j > 0) v = fma(S->ee[j - 1], tn[j - 1], v);
        if (j + 1 < m) v = fma(S->ee[j], tn[j + 1], v);
      }
      S->tc[(n + 1) * TE_MMAX + j] = v;
    }
    __syncthreads();
  }
  // signed doubled last components: R uses even n, I odd n
  for (int n = old + 1 + threadIdx.x; n <= K; n += blockDim.x) {
    const double g = S->tc[n * TE_MMAX + (m - 1)];
    const int r = n & 3;
    S->gs[n] = (n == 0) ? g : ((r == 0 || r == 3) ? 2.0 * g : -2.0 * g);
  }
  C.cheb_n = K;
  __syncthreads();
}

// Integrand h |e_m^T exp(-i x T) e_1| by Chebyshev-Bessel, K iterations.
__device__ double integrand_cheb(const KCtx& C, double x, int K) {
  const double z = x * C.rho;
  const double* gs = C.sm->gs;
  if (!(z > 1e-200)) return (C.m == 1) ? C.h * fabs(gs[0]) : 0.0;
  const double inv2z = 2.0 / z;
  double jp1 = 0.0, jk = 1e-200;
  double R = 0.0, I = 0.0, nrm = 0.0;
  double f = (double)K * inv2z;
  for (int k = K; k >= 4; k -= 4) {
    // k = 4q
    R = fma(gs[k], jk, R);
    nrm = fma(2.0, jk, nrm);
    double jm = fma(f, jk, -jp1);
    f -= inv2z;
    jp1 = jk;
    jk = jm;
    // k - 1
    I = fma(gs[k - 1], jk, I);
    jm = fma(f, jk, -jp1);
    f -= inv2z;
    jp1 = jk;
    jk = jm;
    // k - 2
    R = fma(gs[k - 2], jk, R);
    nrm = fma(2.0, jk, nrm);
    jm = fma(f, jk, -jp1);
    f -= inv2z;
    jp1 = jk;
    jk = jm;
    // k - 3
    I = fma(gs[k - 3], jk, I);
    jm = fma(f, jk, -jp1);
    f -= inv2z;
    jp1 = jk;
    jk = jm;
    if (needs_rescale(jk)) {
      const double sc = 0x1p-600;
      jk *= sc;
      jp1 *= sc;
      R *= sc;
      I *= sc;
      nrm *= sc;
    }
  }
  // jk = J_0 (unnormalised)
  nrm += jk;
  R = fma(gs[0], jk, R);
  return C.h * hypot(R, I) / fabs(nrm);
}

// Bessel values J_0..J_K(z), normalised, into out[] (one thread).
__device__ void bessel_table(double z, int K, double* out) {
  if (!(z > 1e-200)) {
    for (int k = 0; k <= K; ++k) out[k] = (k == 0) ? 1.0 : 0.0;
    return;
  }
  const double inv2z = 2.0 / z;
  double jp1 = 0.0, jk = 1e-200, nrm = 0.0;
  double f = (double)K * inv2z;
  out[K] = jk;
  for (int k = K; k >= 1; --k) {
    if ((k & 1) == 0) nrm = fma(2.0, jk, nrm);
    double jm = fma(f, jk, -jp1);
    f -= inv2z;
    jp1 = jk;
    jk = jm;
    out[k - 1] = jk;
    if (needs_rescale(jk)) {
      const double sc = 0x1p-600;
      for (int q = k - 1; q <= K; ++q) out[q] *= sc;
      jk = out[k - 1];
      jp1 *= sc;
      nrm *= sc;
    }
  }
  nrm += jk;
  const double inv = 1.0 / nrm;
  for (int k = 0; k <= K; ++k) out[k] *= inv;
}

// ------------------------------------------------------------ eigen path

// Implicit symmetric tridiagonal QR with Wilkinson shifts, warp 0 only.
// Q (col-major, ld TE_MMAX) must hold the identity on entry.  Returns 0 on
// success, 1 if the sweep limit was reached.
__device__ int tridiag_qr_warp(int m, double* d, double* e, double* Q, double* rc, double* rs, int max_sweeps) {
  const int lane = threadIdx.x & 31;
  int q = m - 1;
  int sweeps = 0;
  while (true) {
    int p_out = 0, q_out = 0;
    if (lane == 0) {
      for (int i = 0; i < q; ++i)
        if (fabs(e[i]) <= DBL_EPSILON * (fabs(d[i]) + fabs(d[i + 1]))) e[i] = 0.0;
      while (q > 0 && e[q - 1] == 0.0) --q;
      int p = q;
      if (q > 0) {
        p = q - 1;
        while (p > 0 && e[p - 1] != 0.0) --p;
        // Wilkinson shift from the trailing 2x2 block
        double dl = d[q - 1], dq = d[q], eq = e[q - 1];
        double delta = 0.5 * (dl - dq);
        double rr = hypot(delta, eq);
        double den = delta + (delta >= 0.0 ? rr : -rr);
        double mu = (den != 0.0) ? dq - eq * eq / den : dq - fabs(eq);
        double x = d[p] - mu, zz = e[p];
        for (int k = p; k < q; ++k) {
          double r = hypot(x, zz);
          double cs = 1.0, sn = 0.0;
          if (r != 0.0) {
            cs = x / r;
            sn = zz / r;
          }
          if (k > p) e[k - 1] = r;
          double a = d[k], b = e[k], dd2 = d[k + 1];
          double cc = cs * cs, ss = sn * sn, csn = cs * sn;
          d[k] = cc * a + 2.0 * csn * b + ss * dd2;
          d[k + 1] = ss * a - 2.0 * csn * b + cc * dd2;
          e[k] = csn * (dd2 - a) + (cc - ss) * b;
          if (k + 1 < q) {
            double bulge = sn * e[k + 1];
            e[k + 1] = cs * e[k + 1];
            x = e[k];
            zz = bulge;
          }
          rc[k] = cs;
          rs[k] = sn;
        }
      }
      p_out = p;
      q_out = q;
    }
    q = __shfl_sync(0xffffffffu, q_out, 0);
    int p = __shfl_sync(0xffffffffu, p_out, 0);
    if (q == 0) break;
    __syncwarp();
    for (int row = lane; row < m; row += 32) {
      double a = Q[p * TE_MMAX + row];
      for (int k = p; k < q; ++k) {
        double b = Q[(k + 1) * TE_MMAX + row];
        double cs = rc[k], sn = rs[k];
        Q[k * TE_MMAX + row] = cs * a + sn * b;
        a = -sn * a + cs * b;
      }
      Q[q * TE_MMAX + row] = a;
    }
    __syncwarp();
    if (++sweeps > max_sweeps) return 1;
  }
  return 0;
}

// Eigen-decomposition of T into sm->lam / sm->Q (block-cooperative call).
__device__ void ensure_eig(KCtx& C) {
  if (C.eig_ok) return;
  KSmem* S = C.sm;
  __shared__ double dtmp[TE_MMAX], etmp[TE_MMAX];
  const int m = C.m;
  for (int i = threadIdx.x; i < TE_MMAX * TE_MMAX; i += blockDim.x) {
    int r = i % TE_MMAX, c = i / TE_MMAX;
    S->Q[i] = (r == c) ? 1.0 : 0.0;
  }
  if (threadIdx.x < TE_MMAX) {
    dtmp[threadIdx.x] = threadIdx.x < m ? S->d[threadIdx.x] : 0.0;
    etmp[threadIdx.x] = threadIdx.x + 1 < m ? S->e[threadIdx.x] : 0.0;
  }
  __syncthreads();
  int fail = 0;
  const int max_sweeps = C.ds->qr_sweeps > 0 ? C.ds->qr_sweeps : 40 * m + 40;
  if (threadIdx.x < 32) fail = tridiag_qr_warp(m, dtmp, etmp, S->Q, S->rc, S->rs, max_sweeps);
  if (threadIdx.x == 0) S->ibc[0] = fail;
  __syncthreads();
  if (S->ibc[0] && threadIdx.x == 0) C.ds->fatal = TE_ERR_EIGEN;
  if (threadIdx.x < m) S->lam[threadIdx.x] = dtmp[threadIdx.x];
  C.eig_ok = true;
  __syncthreads();
}

__device__ double integrand_eig(const KCtx& C, double x) {
  const KSmem* S = C.sm;
  const int m = C.m;
  double re = 0.0, im = 0.0;
  for (int k = 0; k < m; ++k) {
    double ck = S->Q[k * TE_MMAX + (m - 1)] * S->Q[k * TE_MMAX];
    double sn, cs;
    sincos(x * S->lam[k], &sn, &cs);
    re = fma(ck, cs, re);
    im = fma(-ck, sn, im);
  }
  return C.h * hypot(re, im);
}

// ------------------------------------------------------------ quadrature

struct IntResult {
  double value, err;
  bool nonfinite;
};

// Evaluate the integrand at the abscissae of nodes [n0, n1) of the tanh-sinh
// table on [a, b] into sm->fp / sm->fm (block-cooperative).
__device__ void eval_ts_nodes(KCtx& C, double a, double b, int n0, int n1, bool use_eig, int K) {
  KSmem* S = C.sm;
  const double c = 0.5 * (a + b), d = 0.5 * (b - a);
  const int nev = 2 * (n1 - n0);
  for (int e = threadIdx.x; e < nev; e += blockDim.x) {
    const int node = n0 + (e >> 1);
    const bool minus = e & 1;
    if (minus && node == 0) continue;  // t = 0 is evaluated once
    const double u = c_quad.ts_u[node];
    const double x = minus ? c - d * u : c + d * u;
    const double f = use_eig ? integrand_eig(C, x) : integrand_cheb(C, x, K);
    if (minus)
      S->fm[node] = f;
    else
      S->fp[node] = f;
  }
  __syncthreads();
}

// Tanh-sinh integral of the error integrand on [a, b].
__device__ IntResult ts_integrate(KCtx& C, double a, double b) {
  KSmem* S = C.sm;
  IntResult res = {0.0, 0.0, false};
  if (!(b > a)) return res;
  const double zmax = fmax(fabs(a), fabs(b)) * C.rho;
  int K = bessel_start(zmax, C.m);
  const bool use_eig = K > TE_NCHEB;
  if (use_eig)
    ensure_eig(C);
  else
    ensure_cheb(C, K);
  const double d = 0.5 * (b - a);
  const int* lb = c_quad.ts_level_begin;
  // levels 0..4 at once
  eval_ts_nodes(C, a, b, 0, lb[5], use_eig, K);
  double sum = 0.0, sum_abs = 0.0, prev = 0.0;
  bool nonfinite = false;
  int evaluated = 4;
  const int kmax = C.ds->ts_kmax >= TE_TS_KMIN && C.ds->ts_kmax < TE_TS_KMAX ? C.ds->ts_kmax : TE_TS_KMAX;
  for (int k = 0; k <= kmax; ++k) {
    if (k > evaluated) {
      eval_ts_nodes(C, a, b, lb[k], lb[k + 1], use_eig, K);
      evaluated = k;
    }
    // level sum on warp 0, broadcast through shared memory
    if (threadIdx.x < 32) {
      double s = 0.0, sa = 0.0;
      bool bad = false;
      for (int node = lb[k] + (int)threadIdx.x; node < lb[k + 1]; node += 32) {
        const double w = c_quad.ts_w[node];
        if (node == 0) {
          double fv = S->fp[0];
          s = fma(w, fv, s);
          sa = fma(w, fabs(fv), sa);
          bad |= !isfinite(fv);
        } else {
          double f1 = S->fp[node], f2 = S->fm[node];
          s = fma(w, f1 + f2, s);
          sa = fma(w, fabs(f1) + fabs(f2), sa);
          bad |= !isfinite(f1) || !isfinite(f2);
        }
      }
      s = warp_sum_all(s);
      sa = warp_sum_all(sa);
      bad = __any_sync(0xffffffffu, bad);
      if (threadIdx.x == 0) {
        S->bc[0] = s;
        S->bc[1] = sa;
        S->ibc[1] = bad ? 1 : 0;
      }
    }
    __syncthreads();
    sum += S->bc[0];
    sum_abs += S->bc[1];
    nonfinite |= S->ibc[1] != 0;
    __syncthreads();
    const double hk = ldexp(1.0, -k);
    const double Ik = d * hk * sum;
    const double L1 = d * hk * sum_abs;
    res.value = Ik;
    if (k >= 1) {
      res.err = fabs(Ik - prev);
      if (k >= TE_TS_KMIN && res.err <= 1e-3 * L1) break;
    }
    prev = Ik;
  }
  res.nonfinite = nonfinite;
  return res;
}

__device__ double gauss_integrate(KCtx& C, double a, double b, int npts) {
  KSmem* S = C.sm;
  const double* xs = npts == 15 ? c_quad.g15_x : c_quad.g7_x;
  const double* ws = npts == 15 ? c_quad.g15_w : c_quad.g7_w;
  const double c = 0.5 * (a + b), d = 0.5 * (b - a);
  const double zmax = fmax(fabs(a), fabs(b)) * C.rho;
  int K = bessel_start(zmax, C.m);
  const bool use_eig = K > TE_NCHEB;
  if (use_eig)
    ensure_eig(C);
  else
    ensure_cheb(C, K);
  if (threadIdx.x < 32) {
    double s = 0.0;
    if ((int)threadIdx.x < npts) {
      double x = c + d * xs[threadIdx.x];
      double f = use_eig ? integrand_eig(C, x) : integrand_cheb(C, x, K);
      s = ws[threadIdx.x] * f;
    }
    s = warp_sum_all(s);
    if (threadIdx.x == 0) S->bc[0] = s;
  }
  __syncthreads();
  double r = d * S->bc[0];
  __syncthreads();
  return r;
}

// integrateError (core/krylovTimeEvolver.cpp:584-618); uniform across the block.
__device__ double integrate_error(KCtx& C, double a, double b, int method, double tolRate, bool& successful) {
  TeDevState* ds = C.ds;
  if (threadIdx.x == 0) ds->n_integrals++;
  double ret, error = 0.0;
  bool success = true;
  if (method == 0) {
    ret = gauss_integrate(C, a, b, 15);
  } else if (method == 1) {
    ret = gauss_integrate(C, a, b, 7);
  } else {
    IntResult r = ts_integrate(C, a, b);
    if (r.nonfinite) {
      ret = ds->tol * 10.0;  // the reference's response to a failed quadrature (:601-605)
      error = 0.0;
    } else {
      ret = r.value;
      error = r.err;
    }
    if (error / ret > 1e-3 && ret > 1e-3 * (b - a) * tolRate) success = false;
  }
  successful = successful && success;
  return ret;
}

// findMaximalStepSize (core/krylovTimeEvolver.cpp:153-254).  Returns the
// code (0/1/20/21) or -1 when 20 halvings did not suffice.
__device__ int find_step(KCtx& C, double tolRate, double t_stepSuggestion, double t_step_max, int n_substeps,
                         double numericalErrorEstimate, bool increaseStep, double* t_stepRet, double* err_stepRet) {
  TeDevState* ds = C.ds;
  const int mlong = ds->integ_long, mshort = ds->integ_short;
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
  double err_step = integrate_error(C, 0.0, t_step, mlong, tolRate, ok);
  if (increaseStep && !skipSubsteps) {
    double err_new = err_step, t_new = t_step;
    int guard = 0;
    while (err_new < tolRate * t_new && t_step < t_step_max && guard++ < 4096) {
      t_step = t_new;
      err_step = err_new;
      if (t_step >= t_step_max) {
        skipSubsteps = true;
        break;
      }
      t_new *= 2;
      if (t_new > t_step_max) t_new = t_step_max;
      err_new = integrate_error(C, 0.0, t_new, mlong, tolRate, ok);
    }
  }
  while (err_step > tolRate * t_step) {
    nbReductions++;
    t_step = t_step / 2.0;
    err_step = integrate_error(C, 0.0, t_step, mlong, tolRate, ok);
    if (nbReductions == GO_MAX) return -1;
    skipSubsteps = false;
  }
  const double s = t_step / n_substeps;
  int n_s = 0;
  double deltaError = 0.0;
  if (!skipSubsteps) {
    while (err_step + deltaError < tolRate * (t_step + n_s * s)) {
      err_step += deltaError;
      n_s++;
      if (t_step + (n_s - 1) * s >= t_step_max) break;
      if (n_s > (1 << 22)) return -2;
      deltaError = integrate_error(C, t_step + (n_s - 1) * s, t_step + n_s * s, mshort, tolRate, ok);
    }
    t_step += (n_s - 1) * s;
  }
  if (err_step < numericalErrorEstimate) {
    if (!skipSubsteps || err_step > 0.1 * tolRate * t_step) code += 1;
  }
  if (!ok) code += 20;
  *t_stepRet = t_step;
  *err_stepRet = err_step;
  return code;
}

// ------------------------------------------------------- coefficient vectors

// Y[slot] = s_j i^j [exp(-i dt T) e_1]_j for the listed outputs
// (block-cooperative; at most TE_KBUF outputs per call).
__device__ void output_coefficients(KCtx& C, const double* dts, const int* slots, int count) {
  KSmem* S = C.sm;
  TeDevState* ds = C.ds;
  const int m = C.m;
  double zmax = 0.0;
  for (int o = 0; o < count; ++o) zmax = fmax(zmax, fabs(dts[o]) * C.rho);
  const int K = bessel_start(zmax, m);
  const bool use_eig = K > TE_NCHEB;
  if (use_eig)
    ensure_eig(C);
  else
    ensure_cheb(C, K);
  if (!use_eig) {
    if ((int)threadIdx.x < count) bessel_table(dts[threadIdx.x] * C.rho, K, S->J[threadIdx.x]);
    __syncthreads();
    // signed coefficients a_n = eps_n sigma_n J_n (sigma: + for n%4 in {0,3}, - otherwise)
    for (int i = threadIdx.x; i < count * (K + 1); i += blockDim.x) {
      int o = i / (K + 1), n = i % (K + 1);
      int r = n & 3;
      double sg = (r == 0 || r == 3) ? 1.0 : -1.0;
      S->J[o][n] *= (n == 0) ? 1.0 : 2.0 * sg;
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < count * m; i += blockDim.x) {
    const int o = i / m, j = i % m;
    const double dt = dts[o];
    double re = 0.0, im = 0.0;
    if (!use_eig) {
      const double* a = S->J[o];
      for (int n = 0; n + 1 <= K; n += 2) {
        re = fma(a[n], S->tc[n * TE_MMAX + j], re);
        im = fma(a[n + 1], S->tc[(n + 1) * TE_MMAX + j], im);
      }
      if ((K & 1) == 0) re = fma(a[K], S->tc[K * TE_MMAX + j], re);
      // times e^{-i dt c}
      double sn, cs;
      sincos(dt * C.c, &sn, &cs);
      double r2 = re * cs + im * sn;
      double i2 = im * cs - re * sn;
      re = r2;
      im = i2;
    } else {
      for (int k = 0; k < m; ++k) {
        double q = S->Q[k * TE_MMAX + j] * S->Q[k * TE_MMAX];
        double sn, cs;
        sincos(dt * S->lam[k], &sn, &cs);
        re = fma(q, cs, re);
        im = fma(-q, sn, im);
      }
    }
    // times i^j, then the column scale s_j of the unnormalised basis
    double yr, yi;
    switch (j & 3) {
      case 0: yr = re; yi = im; break;
      case 1: yr = -im; yi = re; break;
      case 2: yr = -re; yi = -im; break;
      default: yr = im; yi = -re; break;
    }
    const double sj = ds->s[j];
    ds->Y[slots[o] * TE_MMAX + j] = make_double2(yr * sj, yi * sj);
  }
  __syncthreads();
}

// Schedule the next batch of samples of the current Krylov space (the
// while-condition of :405) and compute their coefficients.  When the batch
// exhausts the step, advance t_now and err (:440-441) and open the next step.
__device__ void schedule_batch(KCtx& C) {
  TeDevState* ds = C.ds;
  KSmem* S = C.sm;
  __shared__ double dts[TE_SCAP];
  __shared__ int cnt_s, pending_s;
  if (threadIdx.x == 0) {
    const double t = ds->t, ss = ds->sampling_step, t_now = ds->t_now, t_step = ds->t_step;
    const int ns = ds->n_samples;
    int idx = ds->index_samples;
    double ts = ds->t_sampling;
    int cnt = 0;
    ds->sample_base = idx;
    const double* times = ds->sample_times;
    auto cond = [&](int i, double tsv) {
      if (i >= ns) return false;
      const double next = times ? times[i] : tsv + ss;
      return next <= t_now + t_step || (i == ns - 1 && fabs(t_now + t_step - t) <= DBL_EPSILON);
    };
    while (cnt < ds->max_batch && cond(idx, ts)) {
      ts = times ? times[idx] : ts + ss;
      dts[cnt] = ts - t_now;
      ++cnt;
      ++idx;
    }
    const bool pending = cond(idx, ts);
    ds->t_sampling = ts;
    ds->index_samples = idx;
    ds->samples_in_batch = cnt;
    ds->samples_pending = pending ? 1 : 0;
    cnt_s = cnt;
    pending_s = pending ? 1 : 0;
  }
  __syncthreads();
  const int cnt = cnt_s;
  for (int o0 = 0; o0 < cnt; o0 += TE_KBUF) {
    int slots[TE_KBUF];
    const int k = min(TE_KBUF, cnt - o0);
    for (int o = 0; o < k; ++o) slots[o] = 1 + o0 + o;
    output_coefficients(C, dts + o0, slots, k);
  }
  if (threadIdx.x == 0 && !pending_s) {
    ds->t_now += ds->t_step;
    ds->err += ds->err_step;
    if (ds->index_samples < ds->n_samples) {
      ds->n_steps++;
      ds->breakdown = 0;
    } else {
      ds->done = 1;
    }
  }
  (void)S;
  __syncthreads();
}

// Load T from the Lanczos coefficients and set up the Chebyshev data.
__device__ void setup_krylov_matrix(KCtx& C) {
  TeDevState* ds = C.ds;
  KSmem* S = C.sm;
  const int m = C.m;
  if (threadIdx.x < TE_MMAX) {
    int j = threadIdx.x;
    S->d[j] = j < m ? -ds->alpha[j].y : 0.0;
    S->e[j] = j + 1 < m ? ds->beta[j + 1] : 0.0;
    ds->d[j] = S->d[j];
    ds->e[j] = S->e[j];
  }
  __syncthreads();
  // Gershgorin interval on warp 0
  if (threadIdx.x < 32) {
    double lo = INFINITY, hi = -INFINITY;
    for (int j = threadIdx.x; j < m; j += 32) {
      double r = fabs(S->e[j]) + (j > 0 ? fabs(S->e[j - 1]) : 0.0);
      lo = fmin(lo, S->d[j] - r);
      hi = fmax(hi, S->d[j] + r);
    }
    for (int o = 16; o > 0; o >>= 1) {
      lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (threadIdx.x == 0) {
      double c = 0.5 * (hi + lo), rho = 0.5 * (hi - lo);
      if (!(rho > 1e-300 * fmax(1.0, fabs(c)))) rho = 1.0;
      S->bc[2] = c;
      S->bc[3] = rho;
    }
  }
  __syncthreads();
  C.c = S->bc[2];
  C.rho = S->bc[3];
  if (threadIdx.x < TE_MMAX) {
    int j = threadIdx.x;
    S->dd[j] = j < m ? 2.0 * (S->d[j] - C.c) / C.rho : 0.0;
    S->ee[j] = j + 1 < m ? 2.0 * S->e[j] / C.rho : 0.0;
  }
  __syncthreads();
  C.cheb_n = -1;
  C.eig_ok = false;
}

// Persist Chebyshev / eigen data for the later batch launches.
__device__ void save_krylov_data(KCtx& C) {
  TeDevState* ds = C.ds;
  KSmem* S = C.sm;
  for (int i = threadIdx.x; i < (C.cheb_n + 1) * TE_MMAX; i += blockDim.x) ds->cheb_t[i] = S->tc[i];
  if (C.eig_ok) {
    for (int i = threadIdx.x; i < TE_MMAX * TE_MMAX; i += blockDim.x) ds->eig_Q[i] = S->Q[i];
    if (threadIdx.x < TE_MMAX) ds->eig_lam[threadIdx.x] = S->lam[threadIdx.x];
  }
  if (threadIdx.x == 0) {
    ds->cheb_c = C.c;
    ds->cheb_rho = C.rho;
    ds->cheb_n = C.cheb_n;
    ds->eig_valid = C.eig_ok ? 1 : 0;
  }
  __syncthreads();
}

__device__ void load_krylov_data(KCtx& C) {
  TeDevState* ds = C.ds;
  KSmem* S = C.sm;
  C.c = ds->cheb_c;
  C.rho = ds->cheb_rho;
  C.cheb_n = ds->cheb_n;
  C.eig_ok = ds->eig_valid != 0;
  if (threadIdx.x < TE_MMAX) {
    S->d[threadIdx.x] = ds->d[threadIdx.x];
    S->e[threadIdx.x] = ds->e[threadIdx.x];
    S->dd[threadIdx.x] = threadIdx.x < C.m ? 2.0 * (S->d[threadIdx.x] - C.c) / C.rho : 0.0;
    S->ee[threadIdx.x] = threadIdx.x + 1 < C.m ? 2.0 * S->e[threadIdx.x] / C.rho : 0.0;
    if (C.eig_ok) S->lam[threadIdx.x] = ds->eig_lam[threadIdx.x];
  }
  for (int i = threadIdx.x; i < (C.cheb_n + 1) * TE_MMAX; i += blockDim.x) S->tc[i] = ds->cheb_t[i];
  if (C.eig_ok)
    for (int i = threadIdx.x; i < TE_MMAX * TE_MMAX; i += blockDim.x) S->Q[i] = ds->eig_Q[i];
  __syncthreads();
  if (C.cheb_n >= 0) {
    // rebuild the signed last components
    const int K = C.cheb_n;
    for (int n = threadIdx.x; n <= K; n += blockDim.x) {
      const double g = S->tc[n * TE_MMAX + (C.m - 1)];
      const int r = n & 3;
      S->gs[n] = (n == 0) ? g : ((r == 0 || r == 3) ? 2.0 * g : -2.0 * g);
    }
  }
  __syncthreads();
}

// One Krylov-space step of one evolution (block-cooperative).
// mode 0: full step (matrix setup, step search, w, first sample batch);
// mode 1: next sample batch of the same Krylov space.
__device__ void krylov_step_body(TeDevState* ds, int mode, KSmem* S) {
  if (ds->fatal != 0) return;
  if ((mode == 0 && ds->done != 0) || (mode == 1 && ds->samples_pending == 0)) {
    // nothing to do for this evolution: make the combine/observable passes skip it
    if (threadIdx.x == 0) {
      ds->samples_in_batch = 0;
      ds->want_w = 0;
    }
    return;
  }
  KCtx C;
  C.ds = ds;
  C.sm = S;
  C.m = ds->m_eff;
  C.h = ds->h;
  C.fatal = 0;
  if (mode == 1) {
    load_krylov_data(C);
    if (threadIdx.x == 0) ds->want_w = 0;
    schedule_batch(C);
    save_krylov_data(C);
    return;
  }
  if (threadIdx.x == 0) ds->n_integrals = 0;
  setup_krylov_matrix(C);
  const bool hbd = ds->breakdown != 0;
  if (hbd) {
    // lucky breakdown (:342-363): the remaining time in one step, m reduced for good
    if (threadIdx.x == 0) {
      ds->t_step = ds->t - ds->t_now;
      ds->err_step = 0.0;
      ds->m_cur = C.m;
      ds->status = TE_STATUS_LUCKY_BREAKDOWN;
      ds->want_w = 0;
      ds->new_start = 0;
    }
  } else {
    const double s0 = 0.97 * ds->t_step;
    double t_step = 0.0, err_step = 0.0;
    int code = find_step(C, ds->tol_rate, s0, ds->t - ds->t_now, 50, ds->num_err_est, ds->t_now == 0.0, &t_step,
                         &err_step);
    if (code < 0) {
      if (threadIdx.x == 0) ds->fatal = code == -1 ? TE_ERR_NO_STEP : TE_ERR_UNSUPPORTED;
      return;
    }
    if (threadIdx.x == 0) {
      ds->t_step = t_step;
      ds->err_step = err_step;
      ds->err_code_find = code;
      ds->want_w = 1;
      ds->new_start = 1;
    }
    __syncthreads();
    double dts[1] = {t_step};
    int slots[1] = {0};
    output_coefficients(C, dts, slots, 1);
  }
  if (threadIdx.x == 0) {
    switch (ds->err_code_find) {  // :386-399 (a breakdown step re-counts the previous code)
      case 1: ds->nb_err_roundoff++; break;
      case 20: ds->nb_err_int++; break;
      case 21:
        ds->nb_err_int++;
        ds->nb_err_roundoff++;
        break;
      default: break;
    }
  }
  __syncthreads();
  if (ds->fatal != 0) return;
  schedule_batch(C);
  save_krylov_data(C);
}

// One block (one per SM at most: the shared memory of KSmem), so the whole
// register file is available; at the default budget of 64 registers the
// kernel spilled 260 bytes.
__global__ void __launch_bounds__(TE_THREADS, 1) krylov_kernel(TeDevState* ds, int mode) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  krylov_step_body(ds, mode, reinterpret_cast<KSmem*>(smem_raw));
}

// Batched evolutions: block b runs the step of instance b.
__global__ void __launch_bounds__(TE_THREADS, 1) krylov_batch_kernel(TeDevState* states, int mode) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  krylov_step_body(states + blockIdx.x, mode, reinterpret_cast<KSmem*>(smem_raw));
}

// ---------------------------------------------------------------------------
// Batched evolutions in one persistent launch: the whole run of a batch (every
// global step: active list, new start vectors, schedule, the m Lanczos
// iterations, the Krylov-space step of every instance, combine, observables,
// extra sample batches, and the final norms) in one cooperative kernel of one
// 1024-thread block per SM, the passes separated by bounded grid barriers.
// The passes are the device bodies of te_batch.cuh, called with the same
// logical schedule warps as the per-pass kernels (hardware warps loop over
// them) and with 256-thread groups for the per-instance reductions, so the
// results equal the graph path's bit for bit; the host waits once per run
// instead of once per global step.
__device__ __forceinline__ void batch_flags_all(const TeDevState* states, int n_inst, int& pending, int& all_done,
                                                int& fatal) {
  int p = 0, d = 1, f = 0;
  for (int i = threadIdx.x; i < n_inst; i += blockDim.x) {
    const int fl = batch_flag(states[i]);
    p |= (fl & 2) != 0;
    d &= (fl & 1) != 0;
    f |= (fl & 4) != 0;
  }
  pending = __syncthreads_or(p);
  all_done = __syncthreads_and(d);
  fatal = __syncthreads_or(f);
}

template <bool REAL>
__global__ void __launch_bounds__(TE_BATCH_PTHREADS, 1) batch_persistent_kernel(TeBatchPersist a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  KSmem* S = reinterpret_cast<KSmem*>(smem_raw);
  // outside the Krylov phase the start of the shared memory serves the group
  // reductions and the schedule's total
  const int ngrp = blockDim.x / TE_THREADS, grp = threadIdx.x / TE_THREADS, gtid = threadIdx.x % TE_THREADS;
  double* gscratch = reinterpret_cast<double*>(smem_raw) + grp * (TE_BATCH_MAX_OBS * 32);
  double* total = reinterpret_cast<double*>(smem_raw) + ngrp * (TE_BATCH_MAX_OBS * 32);
  auto gsync = [grp]() { asm volatile("bar.sync %0, %1;" ::"r"(grp + 1), "r"(TE_THREADS) : "memory"); };
  const int G = gridDim.x;
  auto bar = [&]() { return te_grid_barrier(a.bar_count, a.bar_gen, a.err, a.spin_limit, a.arrivals); };
  const int64_t wpb = blockDim.x >> 5;
  const int64_t pw = (int64_t)blockIdx.x * wpb + (threadIdx.x >> 5), PW = (int64_t)G * wpb;
  const int64_t tg = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, TG = (int64_t)G * blockDim.x;
  const int n_inst = a.n_inst;
  for (int64_t step = 0; step < a.max_global_steps; ++step) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.active_count = 0;
    if (!bar()) return;
    batch_active_body(a.g.n_chunks, a.g.chunk_inst, a.states, a.active, a.active_count, tg, TG);
    if (!bar()) return;
    batch_new_start_body<true>(a.g, a.V, a.spare, a.states, pw, PW);
    if (!bar()) return;
    for (int64_t i = tg; i < n_inst; i += TG) a.states[i].new_start = 0;
    if (blockIdx.x == 0)
      batch_schedule_body(a.g, a.states, n_inst, a.n_warps, a.w_slot, a.inst_cost, a.warp_begin, a.inst_w0,
                          a.inst_nseg, a.seg_base, a.next_run, a.inst_nwrite, total);
    if (!bar()) return;
    for (int j = 0; j < a.m_max; ++j) {
      for (int64_t vw = pw; vw < a.n_warps; vw += PW) {
        if (j > 0)
          batch_apply_warp<REAL, true, true>(a.g, a.sc, a.V, a.w, a.states, a.seg_partials, j, (int)vw);
        else
          batch_apply_warp<REAL, false, true>(a.g, a.sc, a.V, a.w, a.states, a.seg_partials, j, (int)vw);
      }
      if (!bar()) return;
      for (int64_t vw = pw; vw < a.n_warps; vw += PW)
        batch_update_warp<true>(a.g, a.sc, a.V, a.w, a.states, a.seg_partials, j, (int)vw);
      if (!bar()) return;
    }
    int pending, all_done, fatal;
    for (int mode = 0;; mode = 1) {
      for (int i = blockIdx.x; i < n_inst; i += G) krylov_step_body(a.states + i, mode, S);
      if (!bar()) return;
      batch_combine_body<true>(a.g, a.V, a.spare, a.sampled, a.states, 0, pw, PW);
      if (!bar()) return;
      for (int i = blockIdx.x * ngrp + grp; i < n_inst; i += G * ngrp)
        batch_obs_inst<true>(a.g, a.sampled, a.diag, a.n_obs, a.result_off, a.results, a.states, i, gtid,
                             TE_THREADS, gscratch, gsync);
      if (!bar()) return;
      batch_flags_all(a.states, n_inst, pending, all_done, fatal);
      if (!pending || fatal) break;
    }
    if (threadIdx.x == 0 && blockIdx.x == 0) *a.steps_done = step + 1;
    if (fatal || all_done) break;
  }
  for (int i = blockIdx.x * ngrp + grp; i < n_inst; i += G * ngrp)
    batch_norm_inst<true>(a.g, a.sampled, a.states, i, gtid, TE_THREADS, gscratch, gsync);
}

// ---------------------------------------------------------------- host side

static bool g_tables_uploaded = false;

int te_upload_quad_tables() {
  if (g_tables_uploaded) return TE_OK;
  TeQuadTables T;
  const double half_pi = 1.5707963267948966;
  int idx = 0;
  for (int k = 0; k <= TE_TS_KMAX; ++k) {
    T.ts_level_begin[k] = idx;
    auto add = [&](double tt) {
      double s = half_pi * std::sinh(tt);
      double cs = std::cosh(s);
      T.ts_t[idx] = tt;
      T.ts_u[idx] = std::tanh(s);
      T.ts_w[idx] = half_pi * std::cosh(tt) / (cs * cs);
      ++idx;
    };
    if (k == 0) {
      for (int i = 0; i <= 3; ++i) add((double)i);
    } else {
      double h = std::ldexp(1.0, -k);
      for (int i = 0;; ++i) {
        double tt = (2 * i + 1) * h;
        if (tt > 3.0) break;
        add(tt);
      }
    }
  }
  T.ts_level_begin[TE_TS_KMAX + 1] = idx;
  if (idx != TE_TS_NODES) {
    te_set_error("tanh-sinh table size mismatch (%d)", idx);
    return TE_ERR_UNSUPPORTED;
  }
  auto gauss = [](int n, double* x, double* w) {
    for (int i = 0; i < n; ++i) {
      double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
      for (int it = 0; it < 100; ++it) {
        double p0 = 1.0, p1 = z;
        for (int k = 2; k <= n; ++k) {
          double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
          p0 = p1;
          p1 = p2;
        }
        double pp = n * (z * p1 - p0) / (z * z - 1.0);
        double dz = p1 / pp;
        z -= dz;
        if (std::fabs(dz) < 1e-17) break;
      }
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      double pp = n * (z * p1 - p0) / (z * z - 1.0);
      x[i] = z;
      w[i] = 2.0 / ((1.0 - z * z) * pp * pp);
    }
  };
  gauss(15, T.g15_x, T.g15_w);
  gauss(7, T.g7_x, T.g7_w);
  TE_CUDA(cudaMemcpyToSymbol(c_quad, &T, sizeof(T)));
  TE_CUDA(cudaFuncSetAttribute(krylov_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(KSmem)));
  TE_CUDA(cudaFuncSetAttribute(krylov_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(KSmem)));
  g_tables_uploaded = true;
  return TE_OK;
}

void te_launch_krylov_step(TeDevState* ds, cudaStream_t st) {
  krylov_kernel<<<1, TE_THREADS, sizeof(KSmem), st>>>(ds, 0);
}

void te_launch_schedule_samples(TeDevState* ds, cudaStream_t st) {
  krylov_kernel<<<1, TE_THREADS, sizeof(KSmem), st>>>(ds, 1);
}

void te_launch_krylov_batch(TeDevState* states, int n_instances, int mode, cudaStream_t st) {
  krylov_batch_kernel<<<n_instances, TE_THREADS, sizeof(KSmem), st>>>(states, mode);
}

int te_batch_persistent_grid(bool is_real) {
  const void* k = is_real ? (const void*)batch_persistent_kernel<true> : (const void*)batch_persistent_kernel<false>;
  int dev = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return 0;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(KSmem)) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, TE_BATCH_PTHREADS, sizeof(KSmem)) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return per_sm >= 1 ? te_num_sms() : 0;  // one block per SM
}

int te_launch_batch_persistent(const TeBatchPersist& a, int grid, cudaStream_t st) {
  void* k = a.is_real ? (void*)batch_persistent_kernel<true> : (void*)batch_persistent_kernel<false>;
  TeBatchPersist arg = a;
  void* params[] = {&arg};
  return te_cuda_check(cudaLaunchCooperativeKernel(k, dim3(grid), dim3(TE_BATCH_PTHREADS), params, sizeof(KSmem), st),
                       "persistent batch launch");
}
