// Stand-in for abseil's optional: the C++17 standard type. Real abseil's
// optional.h pulls in absl/memory transitively, and reference headers rely on
// that (muon/acceleration.h:133 uses absl::make_unique), so it is included here.
#pragma once
#include <optional>
#include "absl/memory/memory.h"
namespace absl {
using std::optional;
using std::nullopt;
}  // namespace absl
