// Stand-in for assimp: no importer is available, so ReadFile always fails and
// the reference's `load` command logs a warning and loads nothing.
#pragma once
#include <string>
#include "assimp/scene.h"
namespace Assimp {
class Importer {
 public:
  template <typename P>
  const aiScene *ReadFile(const P &, unsigned int) { return nullptr; }
  const char *GetErrorString() const { return "mesh import unavailable in the oracle build"; }
};
}  // namespace Assimp
