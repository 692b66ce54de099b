/*
 * te_quadrature.h -- the quadrature rules of the oracle (TEST INFRASTRUCTURE
 * ONLY), shared by te_oracle.cpp and the Boost.Math stand-in headers under
 * ref_shim/ that let the reference's own core/*.cpp compile here.
 *
 * The reference integrates its error bound with Boost.Math's
 * tanh_sinh<double> (Boost 1.83.0 in its CI) and gauss<double, 15/7>
 * (core/krylovTimeEvolver.cpp:584-618); neither library is on this machine.
 * The rules below follow the published methods, not Boost's source:
 *   - tanh-sinh (Takahasi-Mori double-exponential): nodes t in [-3, 3], level
 *     0 is t = 0, +-1, +-2, +-3 and level k >= 1 adds the odd multiples of
 *     2^-k; abscissa tanh(pi/2 sinh t), weight pi/2 cosh t / cosh^2(pi/2 sinh t);
 *     I_k = d 2^-k sum w f, error |I_k - I_{k-1}|, stop at the first level
 *     k >= 2 with error <= tol * L1_k, at most level kmax (8);
 *   - Gauss-Legendre with n nodes by Newton iteration on the three-term
 *     Legendre recurrence (Golub-Welsch gives the same nodes).
 * The GPU evaluates the same node tables.
 */
#pragma once

#include <cmath>
#include <cstddef>
#include <vector>

namespace te_quad {

const int TS_KMIN = 2;       // always evaluate levels 0..2 before testing convergence
const int TS_KMAX = 8;       // last refinement level
const double TS_TMAX = 3.0;  // nodes t in [-3, 3]

struct TanhSinhTable {
  // Nodes with t >= 0, grouped by level.  Level 0: t = 0,1,2,3; level k >= 1:
  // t = (2i+1) 2^-k <= 3.  u = tanh(pi/2 sinh t), w = pi/2 cosh t / cosh^2(pi/2 sinh t).
  std::vector<double> u, w, t;
  std::vector<int> level_begin;  // size TS_KMAX + 2
  TanhSinhTable() {
    const double half_pi = 1.5707963267948966;
    for (int k = 0; k <= TS_KMAX; ++k) {
      level_begin.push_back((int)u.size());
      if (k == 0) {
        for (int i = 0; i <= 3; ++i) add(i, half_pi);
      } else {
        double h = std::ldexp(1.0, -k);
        for (int i = 0;; ++i) {
          double tt = (2 * i + 1) * h;
          if (tt > TS_TMAX) break;
          add(tt, half_pi);
        }
      }
    }
    level_begin.push_back((int)u.size());
  }
  void add(double tt, double half_pi) {
    double s = half_pi * std::sinh(tt);
    double cs = std::cosh(s);
    t.push_back(tt);
    u.push_back(std::tanh(s));
    w.push_back(half_pi * std::cosh(tt) / (cs * cs));
  }
};

struct GaussTable {
  std::vector<double> x, w;  // full node set on [-1, 1]
  explicit GaussTable(int n) {
    // Newton iteration on P_n with the three-term Legendre recurrence,
    // starting from the Chebyshev-like guess cos(pi (i + 3/4) / (n + 1/2)).
    x.resize(n);
    w.resize(n);
    for (int i = 0; i < n; ++i) {
      double z = std::cos(3.14159265358979323846 * (i + 0.75) / (n + 0.5));
      double pp = 0;
      for (int it = 0; it < 100; ++it) {
        double p0 = 1.0, p1 = z;
        for (int k = 2; k <= n; ++k) {
          double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
          p0 = p1;
          p1 = p2;
        }
        pp = n * (z * p1 - p0) / (z * z - 1.0);
        double dz = p1 / pp;
        z -= dz;
        if (std::fabs(dz) < 1e-17) break;
      }
      // recompute derivative at the converged root
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      pp = n * (z * p1 - p0) / (z * z - 1.0);
      x[i] = z;
      w[i] = 2.0 / ((1.0 - z * z) * pp * pp);
    }
  }
};

inline const TanhSinhTable& ts_table() {
  static TanhSinhTable t;
  return t;
}
inline const GaussTable& gauss15() {
  static GaussTable g(15);
  return g;
}
inline const GaussTable& gauss7() {
  static GaussTable g(7);
  return g;
}

/* ------------------------------------------------------------ quadrature */

struct TSResult {
  double value, err, l1;
  int levels;
  bool nonfinite;
};

// Tanh-sinh on [a, b].  I_k = d h_k sum_{nodes of levels <= k} w f; the
// error estimate at level k is |I_k - I_{k-1}|; stop at the first k >= KMIN
// with err <= tol * L1_k, or at kmax.
template <class F>
TSResult tanh_sinh(F&& f, double a, double b, double tol, int kmax = TS_KMAX) {
  TSResult r = {0, 0, 0, 0, false};
  if (!(b > a)) return r;
  const TanhSinhTable& T = ts_table();
  double c = 0.5 * (a + b), d = 0.5 * (b - a);
  double sum = 0, sum_abs = 0, prev = 0;
  for (int k = 0; k <= kmax; ++k) {
    for (int j = T.level_begin[k]; j < T.level_begin[k + 1]; ++j) {
      double fv;
      if (T.t[j] == 0.0) {
        fv = f(c);
        sum += T.w[j] * fv;
        sum_abs += T.w[j] * std::fabs(fv);
      } else {
        double fp = f(c + d * T.u[j]);
        double fm = f(c - d * T.u[j]);
        fv = fp + fm;
        sum += T.w[j] * fv;
        sum_abs += T.w[j] * (std::fabs(fp) + std::fabs(fm));
      }
      if (!std::isfinite(fv)) r.nonfinite = true;
    }
    double hk = std::ldexp(1.0, -k);
    double I = d * hk * sum;
    double L1 = d * hk * sum_abs;
    r.levels = k;
    r.value = I;
    r.l1 = L1;
    if (k >= 1) {
      r.err = std::fabs(I - prev);
      if (k >= TS_KMIN && r.err <= tol * L1) break;
    }
    prev = I;
  }
  return r;
}

template <class F>
double gauss_rule(const GaussTable& g, F&& f, double a, double b) {
  double c = 0.5 * (a + b), d = 0.5 * (b - a);
  double s = 0;
  for (size_t i = 0; i < g.x.size(); ++i) s += g.w[i] * f(c + d * g.x[i]);
  return d * s;
}

}  // namespace te_quad
