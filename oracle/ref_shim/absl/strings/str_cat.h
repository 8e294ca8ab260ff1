// Stand-in for abseil's StrCat; enums are printed as their integer value.
#pragma once
#include <sstream>
#include <string>
#include <type_traits>
namespace absl {
namespace shim_detail {
template <typename T>
void Put(std::ostringstream &os, const T &v) {
  if constexpr (std::is_enum_v<T>) {
    os << static_cast<long long>(v);
  } else {
    os << v;
  }
}
}  // namespace shim_detail
template <typename... Args>
std::string StrCat(const Args &...args) {
  std::ostringstream os;
  (shim_detail::Put(os, args), ...);
  return os.str();
}
}  // namespace absl
