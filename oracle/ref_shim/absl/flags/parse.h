#pragma once
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include "absl/flags/flag.h"
namespace absl {
inline std::vector<char *> ParseCommandLine(int argc, char **argv) {
  std::vector<char *> rest;
  rest.push_back(argv[0]);
  for (int i = 1; i < argc; ++i) {
    std::string a(argv[i]);
    if (a.rfind("--", 0) != 0) { rest.push_back(argv[i]); continue; }
    a = a.substr(2);
    std::string name = a, value;
    bool has_value = false;
    size_t eq = a.find('=');
    if (eq != std::string::npos) { name = a.substr(0, eq); value = a.substr(eq + 1); has_value = true; }
    auto &reg = shim_flags::Registry();
    auto it = reg.find(name);
    if (it == reg.end()) { std::fprintf(stderr, "unknown flag --%s\n", name.c_str()); std::exit(1); }
    if (!has_value && !it->second.is_bool) {
      if (i + 1 >= argc) { std::fprintf(stderr, "missing value for --%s\n", name.c_str()); std::exit(1); }
      value = argv[++i];
    }
    if (!it->second.parse(value)) { std::fprintf(stderr, "bad value for --%s\n", name.c_str()); std::exit(1); }
  }
  return rest;
}
}  // namespace absl
