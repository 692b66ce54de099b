/* Stand-in for Boost.Log's core (TEST INFRASTRUCTURE ONLY): core::get() with
 * set_filter(severity >= level), see trivial.hpp. */
#pragma once

#include "trivial.hpp"

namespace boost {
namespace log {

class core {
 public:
  static core* get() {
    static core c;
    return &c;
  }
  void set_filter(trivial::level_filter f) { trivial::min_severity() = f.min_level; }
};

}  // namespace log
}  // namespace boost
