// Triangle-mesh file reader for the `load` scene command.
//
// The reference imports meshes through assimp (muon/parser.cc:465-561): every
// triangle mesh in the file becomes vertices plus triangles under the current
// material and transform. assimp is not available here, so this reader covers
// the formats the reference's scenes use: PLY (ascii and binary, either byte
// order), STL (ascii and binary; identical positions are joined into one
// vertex, as assimp's JoinIdenticalVertices step does) and Wavefront OBJ
// (polygons fan-triangulated, as assimp's Triangulate step does).
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace muon_gpu {

struct MeshData {
  std::vector<std::array<float, 3>> positions;
  std::vector<std::array<int32_t, 3>> triangles;  // indices into positions
};

// Reads `path` (format from its extension, case-insensitive). Returns false
// with a message on an unreadable or malformed file; face indices are checked
// against the vertex count.
bool LoadMesh(const std::string &path, MeshData *out, std::string *error);

}  // namespace muon_gpu
