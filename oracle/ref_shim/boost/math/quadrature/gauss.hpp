/*
 * Stand-in for Boost.Math's gauss<Real, N> (TEST INFRASTRUCTURE ONLY):
 * gauss<Real, N>::integrate(f, a, b) as the reference calls it
 * (core/krylovTimeEvolver.cpp:592-595), on the oracle's Gauss-Legendre nodes
 * (te_quadrature.h).
 */
#pragma once

#include "te_quadrature.h"

namespace boost {
namespace math {
namespace quadrature {

template <class Real, unsigned N>
class gauss {
 public:
  template <class F>
  static Real integrate(const F& f, Real a, Real b) {
    static const te_quad::GaussTable g((int)N);
    const Real c = 0.5 * (a + b), d = 0.5 * (b - a);
    Real s = 0;
    for (unsigned i = 0; i < N; ++i) s += g.w[i] * f(c + d * g.x[i]);
    return d * s;
  }
};

}  // namespace quadrature
}  // namespace math
}  // namespace boost
