#pragma once
#include <string_view>
namespace absl {
inline void SetProgramUsageMessage(std::string_view) {}
}  // namespace absl
