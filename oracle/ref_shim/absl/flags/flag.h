// Stand-in for abseil flags: a registry of named flags parsed from
// "--name=value" / "--name value" / "--name" (bools).
#pragma once
#include <cstdint>
#include <functional>
#include <map>
#include <sstream>
#include <string>
#include <string_view>
#include <type_traits>
#include "absl/strings/str_cat.h"
#include "absl/strings/string_view.h"
namespace absl {
namespace shim_flags {
struct Entry {
  std::function<bool(const std::string &)> parse;
  bool is_bool = false;
};
inline std::map<std::string, Entry> &Registry() {
  static std::map<std::string, Entry> r;
  return r;
}
inline bool ParseValue(std::string_view s, std::string *out, std::string *) {
  *out = std::string(s);
  return true;
}
inline bool ParseValue(std::string_view s, bool *out, std::string *) {
  if (s == "true" || s == "1" || s.empty()) { *out = true; return true; }
  if (s == "false" || s == "0") { *out = false; return true; }
  return false;
}
template <typename T>
std::enable_if_t<std::is_arithmetic_v<T>, bool> ParseValue(std::string_view s, T *out, std::string *) {
  std::istringstream is{std::string(s)};
  is >> *out;
  return !is.fail();
}
// Custom flag types provide AbslParseFlag, found by argument-dependent lookup.
template <typename T>
std::enable_if_t<std::is_enum_v<T>, bool> ParseValue(std::string_view s, T *out, std::string *err) {
  return AbslParseFlag(s, out, err);
}
}  // namespace shim_flags
template <typename T>
class Flag {
 public:
  Flag(const char *name, T def) : value_(def) {
    shim_flags::Entry e;
    e.is_bool = std::is_same_v<T, bool>;
    e.parse = [this](const std::string &s) {
      std::string err;
      return shim_flags::ParseValue(s, &value_, &err);
    };
    shim_flags::Registry()[name] = e;
  }
  const T &Get() const { return value_; }
 private:
  T value_;
};
template <typename T>
const T &GetFlag(const Flag<T> &f) { return f.Get(); }
}  // namespace absl
#define ABSL_FLAG(Type, name, def, help) ::absl::Flag<Type> FLAGS_##name(#name, def)
