/*
 * Stand-in for Boost.Log's trivial logger (TEST INFRASTRUCTURE ONLY), enough
 * for the reference's core/krylovLogger.cpp: the severity levels, a global
 * minimum severity set through core::get()->set_filter(severity >= level),
 * and BOOST_LOG_TRIVIAL(level) << ... printing one line to std::clog when the
 * level passes.
 */
#pragma once

#include <iostream>
#include <sstream>
#include <string>

namespace boost {
namespace log {
namespace trivial {

enum severity_level { trace, debug, info, warning, error, fatal };

struct severity_keyword {};
inline constexpr severity_keyword severity{};

struct level_filter {
  severity_level min_level;
};
inline level_filter operator>=(severity_keyword, severity_level level) { return level_filter{level}; }

inline severity_level& min_severity() {
  static severity_level level = trace;
  return level;
}

class record {
 public:
  explicit record(severity_level level) : level_(level) {}
  ~record() {
    if (level_ >= min_severity()) std::clog << text_.str() << std::endl;
  }
  template <class T>
  record& operator<<(const T& x) {
    text_ << x;
    return *this;
  }

 private:
  severity_level level_;
  std::ostringstream text_;
};

}  // namespace trivial
}  // namespace log
}  // namespace boost

#define BOOST_LOG_TRIVIAL(level) ::boost::log::trivial::record(::boost::log::trivial::level)
