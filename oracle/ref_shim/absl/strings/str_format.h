// Stand-in for abseil's StrFormat: printf-style formatting where every %d
// argument is widened to long long.
#pragma once
#include <cstdio>
#include <string>
#include "absl/strings/str_cat.h"
namespace absl {
template <typename... Args>
std::string StrFormat(const char *fmt, const Args &...args) {
  std::string f(fmt);
  std::string out;
  for (size_t i = 0; i < f.size(); ++i) {
    if (f[i] == '%' && i + 1 < f.size() && f[i + 1] == 'd') {
      out += "%lld";
      ++i;
    } else {
      out += f[i];
    }
  }
  char buf[1024];
  std::snprintf(buf, sizeof(buf), out.c_str(), static_cast<long long>(args)...);
  return buf;
}
}  // namespace absl
