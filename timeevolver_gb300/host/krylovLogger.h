// krylovLogger.h -- severity-filtered logging of the GB300 TimeEvolver
// (same API as core/krylovLogger.h:11-27; messages go to std::clog).
#pragma once

#include <iomanip>
#include <sstream>
#include <string>

class krylovLogger {
 public:
  enum loggingLevel { DEBUG, INFO, WARNING, ERROR, FATAL };

  krylovLogger() = default;
  krylovLogger(loggingLevel level);
  void set_loggingLevel(loggingLevel level);
  void log_message(loggingLevel level, const std::string& msg);
  static std::string stringStreamWrapperd(double val);
};
