// krylovLogger.cpp -- one process-wide severity threshold, as the reference's
// global Boost.Log filter (core/krylovLogger.cpp:7-20).
#include "krylovLogger.h"

#include <atomic>
#include <iostream>

namespace {
std::atomic<int> g_threshold{krylovLogger::INFO};
const char* kNames[] = {"debug", "info", "warning", "error", "fatal"};
}  // namespace

krylovLogger::krylovLogger(loggingLevel level) { g_threshold = level; }

void krylovLogger::set_loggingLevel(loggingLevel level) { g_threshold = level; }

void krylovLogger::log_message(loggingLevel level, const std::string& msg) {
  if ((int)level < g_threshold.load()) return;
  std::clog << "[" << kNames[(int)level] << "] " << msg << std::endl;
}

std::string krylovLogger::stringStreamWrapperd(double val) {
  std::stringstream ss;
  ss << val;
  return ss.str();
}
