// Stand-in for glog: LOG(severity) streams to stderr (FATAL aborts);
// VLOG(n) prints only when GLOG_v >= n.
#pragma once
#include <cstdlib>
#include <iostream>
#include <sstream>
namespace google {
inline void InitGoogleLogging(const char *) {}
}  // namespace google
namespace shim_log {
inline int Verbosity() {
  static int v = [] { const char *e = std::getenv("GLOG_v"); return e ? std::atoi(e) : 0; }();
  return v;
}
class Line {
 public:
  Line(bool enabled, bool fatal) : enabled_(enabled), fatal_(fatal) {}
  ~Line() {
    if (enabled_) std::cerr << os_.str() << std::endl;
    if (fatal_) std::abort();
  }
  template <typename T>
  Line &operator<<(const T &v) { if (enabled_) os_ << v; return *this; }
 private:
  bool enabled_, fatal_;
  std::ostringstream os_;
};
}  // namespace shim_log
#define SHIM_LOG_INFO ::shim_log::Line(std::getenv("MUON_REF_LOG") != nullptr, false)
#define SHIM_LOG_WARNING ::shim_log::Line(std::getenv("MUON_REF_LOG") != nullptr, false)
#define SHIM_LOG_ERROR ::shim_log::Line(true, false)
#define SHIM_LOG_FATAL ::shim_log::Line(true, true)
#define LOG(sev) SHIM_LOG_##sev
#define VLOG(n) ::shim_log::Line(::shim_log::Verbosity() >= (n), false)
