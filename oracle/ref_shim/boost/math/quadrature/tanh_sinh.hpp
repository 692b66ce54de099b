/*
 * Stand-in for Boost.Math's tanh_sinh<Real> (TEST INFRASTRUCTURE ONLY), used to
 * compile the reference's core/krylovTimeEvolver.cpp here.  It offers the call
 * the reference makes, integrate(f, a, b, tolerance, &error, &L1)
 * (core/krylovTimeEvolver.cpp:596-606), on the oracle's own tanh-sinh rule
 * (te_quadrature.h).  A non-finite integrand throws, which takes the
 * reference's exception path (ret = 10 tol).  Like the real header it brings
 * in <atomic>, which core/krylovTimeEvolver.h uses without including it.
 */
#pragma once

#include <atomic>
#include <cstddef>
#include <stdexcept>

#include "te_quadrature.h"

namespace boost {
namespace math {
namespace quadrature {

template <class Real>
class tanh_sinh {
 public:
  template <class F>
  Real integrate(const F& f, Real a, Real b, Real tolerance, Real* error = nullptr, Real* L1 = nullptr,
                 std::size_t* levels = nullptr) const {
    const te_quad::TSResult r = te_quad::tanh_sinh(f, a, b, tolerance);
    if (r.nonfinite) throw std::domain_error("tanh_sinh: the integrand is not finite");
    if (error) *error = r.err;
    if (L1) *L1 = r.l1;
    if (levels) *levels = (std::size_t)r.levels;
    return r.value;
  }
};

}  // namespace quadrature
}  // namespace math
}  // namespace boost
