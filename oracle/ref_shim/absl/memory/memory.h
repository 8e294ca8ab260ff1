// Stand-in for abseil's make_unique.
#pragma once
#include <memory>
namespace absl {
using std::make_unique;
}  // namespace absl
