// Mesh readers for PLY, STL and OBJ (see mesh_io.h).
#include "mesh_io.h"

#include <algorithm>
#include <cctype>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>

namespace muon_gpu {

namespace {

std::string Lower(std::string s) {
  for (char &c : s) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
  return s;
}

bool ReadFile(const std::string &path, std::string *data, std::string *error) {
  std::ifstream f(path, std::ios::binary);
  if (!f) {
    *error = "cannot open mesh file " + path;
    return false;
  }
  std::ostringstream ss;
  ss << f.rdbuf();
  *data = ss.str();
  return true;
}

// Appends a polygon as a triangle fan (v0, vi, vi+1).
void AddPolygon(const std::vector<int32_t> &poly, MeshData *out) {
  for (size_t i = 1; i + 1 < poly.size(); ++i) out->triangles.push_back({poly[0], poly[i], poly[i + 1]});
}

bool CheckIndices(MeshData *out, std::string *error) {
  const int64_t n = static_cast<int64_t>(out->positions.size());
  for (const auto &t : out->triangles) {
    for (int32_t v : t) {
      if (v < 0 || v >= n) {
        *error = "mesh face refers to a missing vertex";
        return false;
      }
    }
  }
  return true;
}

// ---- PLY ----------------------------------------------------------------

enum class PlyType { kI8, kU8, kI16, kU16, kI32, kU32, kF32, kF64, kNone };

PlyType ParsePlyType(const std::string &t) {
  if (t == "char" || t == "int8") return PlyType::kI8;
  if (t == "uchar" || t == "uint8") return PlyType::kU8;
  if (t == "short" || t == "int16") return PlyType::kI16;
  if (t == "ushort" || t == "uint16") return PlyType::kU16;
  if (t == "int" || t == "int32") return PlyType::kI32;
  if (t == "uint" || t == "uint32") return PlyType::kU32;
  if (t == "float" || t == "float32") return PlyType::kF32;
  if (t == "double" || t == "float64") return PlyType::kF64;
  return PlyType::kNone;
}

int PlySize(PlyType t) {
  switch (t) {
    case PlyType::kI8:
    case PlyType::kU8: return 1;
    case PlyType::kI16:
    case PlyType::kU16: return 2;
    case PlyType::kI32:
    case PlyType::kU32:
    case PlyType::kF32: return 4;
    case PlyType::kF64: return 8;
    default: return 0;
  }
}

struct PlyProperty {
  std::string name;
  PlyType type = PlyType::kNone;
  bool list = false;
  PlyType count_type = PlyType::kNone;
};

struct PlyElement {
  std::string name;
  int64_t count = 0;
  std::vector<PlyProperty> props;
};

// Reads binary scalars of either byte order; `big` swaps bytes.
class BinReader {
 public:
  BinReader(const std::string &d, size_t pos, bool big) : d_(d), pos_(pos), big_(big) {}
  bool Read(PlyType t, double *v) {
    const int n = PlySize(t);
    if (n == 0 || pos_ + n > d_.size()) return false;
    unsigned char b[8];
    std::memcpy(b, d_.data() + pos_, n);
    pos_ += n;
    if (big_) std::reverse(b, b + n);
    switch (t) {
      case PlyType::kI8: { int8_t x; std::memcpy(&x, b, 1); *v = x; break; }
      case PlyType::kU8: { uint8_t x; std::memcpy(&x, b, 1); *v = x; break; }
      case PlyType::kI16: { int16_t x; std::memcpy(&x, b, 2); *v = x; break; }
      case PlyType::kU16: { uint16_t x; std::memcpy(&x, b, 2); *v = x; break; }
      case PlyType::kI32: { int32_t x; std::memcpy(&x, b, 4); *v = x; break; }
      case PlyType::kU32: { uint32_t x; std::memcpy(&x, b, 4); *v = x; break; }
      case PlyType::kF32: { float x; std::memcpy(&x, b, 4); *v = x; break; }
      case PlyType::kF64: { double x; std::memcpy(&x, b, 8); *v = x; break; }
      default: return false;
    }
    return true;
  }

 private:
  const std::string &d_;
  size_t pos_;
  bool big_;
};

class AsciiReader {
 public:
  AsciiReader(const std::string &d, size_t pos) : in_(d.substr(pos)) {}
  bool Read(PlyType, double *v) { return static_cast<bool>(in_ >> *v); }

 private:
  std::istringstream in_;
};

template <class Reader>
bool ReadPlyBody(Reader &r, const std::vector<PlyElement> &elems, MeshData *out, std::string *error) {
  for (const PlyElement &e : elems) {
    const bool is_vertex = e.name == "vertex", is_face = e.name == "face";
    int xi = -1, yi = -1, zi = -1;
    for (size_t k = 0; k < e.props.size(); ++k) {
      if (e.props[k].name == "x") xi = static_cast<int>(k);
      if (e.props[k].name == "y") yi = static_cast<int>(k);
      if (e.props[k].name == "z") zi = static_cast<int>(k);
    }
    if (is_vertex && (xi < 0 || yi < 0 || zi < 0)) {
      *error = "PLY vertex element without x, y, z";
      return false;
    }
    std::vector<int32_t> poly;
    for (int64_t i = 0; i < e.count; ++i) {
      std::array<float, 3> pos{0.0f, 0.0f, 0.0f};
      bool have_face = false;
      for (size_t k = 0; k < e.props.size(); ++k) {
        const PlyProperty &p = e.props[k];
        if (p.list) {
          double cnt;
          if (!r.Read(p.count_type, &cnt) || cnt < 0) {
            *error = "truncated PLY list";
            return false;
          }
          const bool take = is_face && !have_face && (p.name == "vertex_indices" || p.name == "vertex_index");
          if (take) poly.clear();
          for (int64_t j = 0; j < static_cast<int64_t>(cnt); ++j) {
            double v;
            if (!r.Read(p.type, &v)) {
              *error = "truncated PLY list";
              return false;
            }
            if (take) poly.push_back(static_cast<int32_t>(v));
          }
          if (take) {
            AddPolygon(poly, out);
            have_face = true;
          }
        } else {
          double v;
          if (!r.Read(p.type, &v)) {
            *error = "truncated PLY element " + e.name;
            return false;
          }
          if (is_vertex) {
            if (static_cast<int>(k) == xi) pos[0] = static_cast<float>(v);
            if (static_cast<int>(k) == yi) pos[1] = static_cast<float>(v);
            if (static_cast<int>(k) == zi) pos[2] = static_cast<float>(v);
          }
        }
      }
      if (is_vertex) out->positions.push_back(pos);
    }
  }
  return true;
}

bool LoadPly(const std::string &data, MeshData *out, std::string *error) {
  size_t end = data.find("end_header");
  if (data.compare(0, 3, "ply") != 0 || end == std::string::npos) {
    *error = "not a PLY file";
    return false;
  }
  size_t body = data.find('\n', end);
  if (body == std::string::npos) {
    *error = "PLY header without a body";
    return false;
  }
  ++body;
  std::istringstream hdr(data.substr(0, end));
  std::string line, format;
  std::vector<PlyElement> elems;
  while (std::getline(hdr, line)) {
    std::istringstream ls(line);
    std::string w;
    ls >> w;
    if (w == "format") {
      ls >> format;
    } else if (w == "element") {
      PlyElement e;
      ls >> e.name >> e.count;
      elems.push_back(e);
    } else if (w == "property" && !elems.empty()) {
      PlyProperty p;
      std::string t;
      ls >> t;
      if (t == "list") {
        std::string ct, it;
        ls >> ct >> it >> p.name;
        p.list = true;
        p.count_type = ParsePlyType(ct);
        p.type = ParsePlyType(it);
      } else {
        p.type = ParsePlyType(t);
        ls >> p.name;
      }
      if (p.type == PlyType::kNone || (p.list && p.count_type == PlyType::kNone)) {
        *error = "unsupported PLY property type";
        return false;
      }
      elems.back().props.push_back(p);
    }
  }
  if (format == "ascii") {
    AsciiReader r(data, body);
    return ReadPlyBody(r, elems, out, error);
  }
  if (format == "binary_little_endian" || format == "binary_big_endian") {
    BinReader r(data, body, format == "binary_big_endian");
    return ReadPlyBody(r, elems, out, error);
  }
  *error = "unsupported PLY format " + format;
  return false;
}

// ---- STL ----------------------------------------------------------------

// Joins identical positions into one vertex (first-seen order).
class VertexJoiner {
 public:
  explicit VertexJoiner(MeshData *out) : out_(out) {}
  int32_t Add(const std::array<float, 3> &p) {
    auto it = index_.find(p);
    if (it != index_.end()) return it->second;
    int32_t id = static_cast<int32_t>(out_->positions.size());
    out_->positions.push_back(p);
    index_.emplace(p, id);
    return id;
  }

 private:
  MeshData *out_;
  std::map<std::array<float, 3>, int32_t> index_;
};

bool LoadStl(const std::string &data, MeshData *out, std::string *error) {
  VertexJoiner join(out);
  // Binary STL: 80-byte header, uint32 count, 50 bytes per facet. An ascii
  // file starts with "solid" but some binary files do too, so the size decides.
  if (data.size() >= 84) {
    uint32_t n;
    std::memcpy(&n, data.data() + 80, 4);
    if (84 + 50 * static_cast<uint64_t>(n) == data.size()) {
      for (uint32_t i = 0; i < n; ++i) {
        const char *f = data.data() + 84 + 50 * static_cast<size_t>(i) + 12;
        std::array<int32_t, 3> t;
        for (int k = 0; k < 3; ++k) {
          std::array<float, 3> p;
          std::memcpy(p.data(), f + 12 * k, 12);
          t[k] = join.Add(p);
        }
        out->triangles.push_back(t);
      }
      return true;
    }
  }
  std::istringstream in(data);
  std::string w;
  std::vector<int32_t> poly;
  bool solid = false;
  while (in >> w) {
    if (w == "solid") solid = true;
    if (w == "outer") poly.clear();
    if (w == "vertex") {
      std::array<float, 3> p;
      if (!(in >> p[0] >> p[1] >> p[2])) {
        *error = "malformed STL vertex";
        return false;
      }
      poly.push_back(join.Add(p));
    }
    if (w == "endloop") AddPolygon(poly, out);
  }
  if (!solid) {
    *error = "not an STL file";
    return false;
  }
  return true;
}

// ---- OBJ ----------------------------------------------------------------

bool LoadObj(const std::string &data, MeshData *out, std::string *error) {
  std::istringstream in(data);
  std::string line;
  std::vector<int32_t> poly;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    std::string w;
    ls >> w;
    if (w == "v") {
      std::array<float, 3> p;
      if (!(ls >> p[0] >> p[1] >> p[2])) {
        *error = "malformed OBJ vertex";
        return false;
      }
      out->positions.push_back(p);
    } else if (w == "f") {
      poly.clear();
      std::string tok;
      while (ls >> tok) {
        // v, v/vt, v//vn or v/vt/vn; negative indices count from the end.
        long v = std::strtol(tok.c_str(), nullptr, 10);
        if (v == 0) {
          *error = "malformed OBJ face";
          return false;
        }
        poly.push_back(static_cast<int32_t>(v > 0 ? v - 1 : static_cast<long>(out->positions.size()) + v));
      }
      AddPolygon(poly, out);
    }
  }
  return true;
}

}  // namespace

bool LoadMesh(const std::string &path, MeshData *out, std::string *error) {
  out->positions.clear();
  out->triangles.clear();
  std::string data;
  if (!ReadFile(path, &data, error)) return false;
  const size_t dot = path.find_last_of('.');
  const std::string ext = dot == std::string::npos ? "" : Lower(path.substr(dot + 1));
  bool ok;
  if (ext == "ply") ok = LoadPly(data, out, error);
  else if (ext == "stl") ok = LoadStl(data, out, error);
  else if (ext == "obj") ok = LoadObj(data, out, error);
  else {
    *error = "unsupported mesh format: " + path;
    return false;
  }
  return ok && CheckIndices(out, error);
}

}  // namespace muon_gpu
