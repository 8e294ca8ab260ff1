// .muon scene parser with the reference parser's semantics
// (muon/parser.cc:230-880, Parser::Parse), producing flat arrays.
//
// Behaviours kept on purpose because they change what is rendered:
//  - `random_seed` falls through into `film_size` (muon/parser.cc:267-286): a
//    seed line that also carries two integers sets the film size.
//  - `brdf lambertian` instantiates the Phong BRDF (the switch in
//    CreateBRDF, muon/parser.cc:165-178, falls through).
//  - The camera keeps the film size in effect on its own line and pushes the
//    transform stack (muon/parser.cc:449-463).
//  - A quad light adds two emissive triangles (va,vc,vb) and (vb,vc,vd) with a
//    default-constructed material (ambient 0) and identity transforms
//    (muon/parser.cc:720-767).
//  - Vertex normals are accumulated per triangle while compute_vertex_normals
//    is on, and normalised at the end only if it is still on
//    (muon/parser.cc:630-637, 860-871).
//  - Unknown commands and malformed lines are skipped with a warning.
// Deviations (the reference has undefined behaviour here): out-of-range vertex
// indices and popping the last transform are rejected with a warning.
#include <cstdio>
#include <cstring>
#include <random>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "host_scene.h"
#include "mesh_io.h"

namespace muon_gpu {

namespace {

// The reference's default material (muon/defaults.h:58-70).
MuonMaterialDesc DefaultMaterial() {
  MuonMaterialDesc m{};
  for (int k = 0; k < 3; ++k) {
    m.ambient[k] = 0.2f;
    m.diffuse[k] = 0.0f;
    m.specular[k] = 0.0f;
    m.emission[k] = 0.0f;
  }
  m.shininess = 1.0f;
  m.roughness = 0.0f;
  m.brdf = MUON_BRDF_PHONG;
  return m;
}

void Trim(std::string &s) {
  size_t b = 0;
  while (b < s.size() && std::isspace(static_cast<unsigned char>(s[b]))) ++b;
  size_t e = s.size();
  while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) --e;
  s = s.substr(b, e - b);
}

struct Vertex {
  mm::v3 pos;
  mm::v3 normal;
};

class Parser {
 public:
  Parser(ParsedScene *out, const std::string &base_dir) : s_(out), base_dir_(base_dir) {
    std::random_device rd;
    seedgen_.seed(rd());
    material_ = DefaultMaterial();
    meshes_.emplace_back();
    xform_stack_.push_back(-1);
    s_->params.integrator = MUON_INTEGRATOR_RAYTRACER;
    s_->params.pixel_samples = 1;
    s_->params.light_samples = 1;
    s_->params.light_stratify = 0;
    s_->params.next_event_estimation = MUON_NEE_OFF;
    s_->params.russian_roulette = 0;
    s_->params.importance_sampling = MUON_IS_HEMISPHERE;
    s_->params.min_depth = 0;
    s_->params.max_depth = 5;
    s_->params.intersect_mode = MUON_ISECT_EXACT;
  }

  void Line(const std::string &raw);
  void Finish();

 private:
  void Warn(const std::string &line) {
    ++s_->warnings;
    if (std::getenv("MUON_PARSE_VERBOSE")) std::fprintf(stderr, "muon: malformed line: %s\n", line.c_str());
  }
  int CurrentMaterial() {
    if (material_index_ < 0) {
      material_index_ = static_cast<int>(s_->materials.size());
      s_->materials.push_back(material_);
    }
    return material_index_;
  }
  // Every material command copies the current material (GenMaterial,
  // muon/parser.cc:141-144), so primitives created earlier keep theirs.
  MuonMaterialDesc &EditMaterial() {
    material_index_ = -1;
    return material_;
  }
  void MultiplyTransform(const mm::m4 &m) {
    mm::m4 cur = xform_stack_.back() < 0 ? mm::identity4() : xforms_[xform_stack_.back()];
    mm::m4 next = mm::mul(cur, m);
    xform_stack_.back() = static_cast<int>(xforms_.size());
    xforms_.push_back(next);
    s_->transforms.push_back(MakeTransformDesc(next));
  }
  int32_t NextPrimId() { return prim_counter_++; }

  // Tri::Tri plus the vertex-normal accumulation of the `tri` command
  // (muon/parser.cc:619-639) for global vertex ids g.
  void AddTriangle(const int32_t g[3]) {
    MuonTriangleDesc t{};
    for (int k = 0; k < 3; ++k) {
      t.v[k][0] = vertices_[g[k]].pos.x;
      t.v[k][1] = vertices_[g[k]].pos.y;
      t.v[k][2] = vertices_[g[k]].pos.z;
      // Vertex ids are kept in the normal slots until Finish() resolves them.
      std::memcpy(&t.n[k][0], &g[k], sizeof(int32_t));
    }
    t.transform = xform_stack_.back();
    t.material = CurrentMaterial();
    t.light = -1;
    t.smooth = compute_vertex_normals_ ? 1 : 0;
    t.prim_id = NextPrimId();
    if (compute_vertex_normals_) {
      mm::v3 a = vertices_[g[0]].pos, b = vertices_[g[1]].pos, c = vertices_[g[2]].pos;
      mm::v3 face = mm::cross(b - a, c - a);
      for (int k = 0; k < 3; ++k) vertices_[g[k]].normal = vertices_[g[k]].normal + face;
    }
    s_->triangles.push_back(t);
  }

  ParsedScene *s_;
  std::string base_dir_;
  std::mt19937 seedgen_;
  bool seed_drawn_ = false;
  MuonMaterialDesc material_;
  int material_index_ = -1;
  std::vector<std::vector<int32_t>> meshes_;  // mesh -> global vertex ids
  int cur_mesh_ = 0;
  std::vector<Vertex> vertices_;
  std::vector<mm::m4> xforms_;
  std::vector<int> xform_stack_;
  mm::v3 attenuation_ = mm::make3(1.0f, 0.0f, 0.0f);
  bool compute_vertex_normals_ = false;
  int32_t prim_counter_ = 0;
  std::vector<int32_t> smooth_tris_;  // triangles whose normals are resolved at Finish()
};

template <typename T>
bool Read(std::istringstream &iss, T *v) {
  iss >> *v;
  return !iss.fail();
}

void Parser::Line(const std::string &raw) {
  std::string line = raw;
  Trim(line);
  if (line.empty() || line[0] == '#') return;
  std::istringstream iss(line);
  std::string cmd;
  iss >> cmd;
  MuonRenderParams &p = s_->params;

  auto on_off = [&](int32_t *dst) {
    std::string v;
    if (!Read(iss, &v)) return Warn(line);
    if (v == "on") *dst = 1;
    else if (v == "off") *dst = 0;
    else Warn(line);
  };
  auto read3 = [&](mm::v3 *v) { return Read(iss, &v->x) && Read(iss, &v->y) && Read(iss, &v->z); };

  if (cmd == "random_seed" || cmd == "film_size") {
    if (cmd == "random_seed") {
      unsigned int seed;
      if (!Read(iss, &seed)) return Warn(line);
      seedgen_.seed(seed);
      seed_drawn_ = false;
    }
    int w, h;
    iss >> w >> h;
    if (iss.fail()) return Warn(line);
    s_->width = w;
    s_->height = h;
  } else if (cmd == "min_depth") {
    int v;
    if (!Read(iss, &v)) return Warn(line);
    p.min_depth = v;
  } else if (cmd == "max_depth") {
    int v;
    if (!Read(iss, &v)) return Warn(line);
    p.max_depth = v;
  } else if (cmd == "output") {
    std::string v;
    if (!Read(iss, &v)) return Warn(line);
    s_->output = v;
    s_->has_output = true;
  } else if (cmd == "gamma") {
    float v;
    if (!Read(iss, &v)) return Warn(line);
    s_->gamma = v;
  } else if (cmd == "integrator") {
    std::string v;
    if (!Read(iss, &v)) return Warn(line);
    if (v == "normals") p.integrator = MUON_INTEGRATOR_NORMALS;
    else if (v == "albedo") p.integrator = MUON_INTEGRATOR_ALBEDO;
    else if (v == "depth") p.integrator = MUON_INTEGRATOR_DEPTH;
    else if (v == "raytracer") p.integrator = MUON_INTEGRATOR_RAYTRACER;
    else if (v == "analyticdirect") p.integrator = MUON_INTEGRATOR_ANALYTIC_DIRECT;
    else if (v == "pathtracer") {
      p.integrator = MUON_INTEGRATOR_PATHTRACER;
      // The path tracer's seed is drawn here (muon/parser.cc:347-349).
      p.seed = seedgen_();
      seed_drawn_ = true;
    } else {
      Warn(line);
    }
  } else if (cmd == "pixel_samples") {
    int v;
    if (!Read(iss, &v)) return Warn(line);
    p.pixel_samples = v;
  } else if (cmd == "light_samples") {
    int v;
    if (!Read(iss, &v)) return Warn(line);
    p.light_samples = v;
  } else if (cmd == "light_stratify") {
    on_off(&p.light_stratify);
  } else if (cmd == "next_event_estimation") {
    std::string v;
    if (!Read(iss, &v)) return Warn(line);
    if (v == "off") p.next_event_estimation = MUON_NEE_OFF;
    else if (v == "on") p.next_event_estimation = MUON_NEE_ON;
    else if (v == "mis") p.next_event_estimation = MUON_NEE_MIS;
    else Warn(line);
  } else if (cmd == "russian_roulette") {
    on_off(&p.russian_roulette);
  } else if (cmd == "importance_sampling") {
    std::string v;
    if (!Read(iss, &v)) return Warn(line);
    if (v == "hemisphere") p.importance_sampling = MUON_IS_HEMISPHERE;
    else if (v == "cosine") p.importance_sampling = MUON_IS_COSINE;
    else if (v == "brdf") p.importance_sampling = MUON_IS_BRDF;
    else Warn(line);
  } else if (cmd == "camera") {
    float f[10];
    for (int k = 0; k < 10; ++k) iss >> f[k];
    if (iss.fail()) return Warn(line);
    MuonCameraDesc &c = s_->camera;
    for (int k = 0; k < 3; ++k) {
      c.eye[k] = f[k];
      c.look_at[k] = f[3 + k];
      c.up[k] = f[6 + k];
    }
    c.fov_y_degrees = f[9];
    c.width = s_->width;
    c.height = s_->height;
    s_->has_camera = true;
    xform_stack_.push_back(xform_stack_.back());
  } else if (cmd == "load") {
    std::string v;
    if (!Read(iss, &v)) return Warn(line);
    // The reference imports through assimp relative to the scene file's
    // directory (muon/parser.cc:465-561): new vertices, and triangles under
    // the current material and transform. A file that cannot be read is
    // skipped with a warning, as there.
    std::string path = v;
    if (!base_dir_.empty() && !v.empty() && v[0] != '/') path = base_dir_ + "/" + v;
    MeshData mesh;
    std::string err;
    if (!LoadMesh(path, &mesh, &err)) {
      if (std::getenv("MUON_PARSE_VERBOSE")) std::fprintf(stderr, "muon: load: %s\n", err.c_str());
      return Warn(line);
    }
    const int32_t base = static_cast<int32_t>(vertices_.size());
    for (const auto &p : mesh.positions)
      vertices_.push_back(Vertex{mm::make3(p[0], p[1], p[2]), mm::splat3(0.0f)});
    for (const auto &t : mesh.triangles) {
      const int32_t g[3] = {base + t[0], base + t[1], base + t[2]};
      AddTriangle(g);
    }
  } else if (cmd == "compute_vertex_normals") {
    int32_t v = compute_vertex_normals_;
    std::string w;
    if (!Read(iss, &w)) return Warn(line);
    if (w == "on") v = 1;
    else if (w == "off") v = 0;
    else return Warn(line);
    compute_vertex_normals_ = v;
  } else if (cmd == "sphere") {
    float x, y, z, r;
    iss >> x >> y >> z >> r;
    if (iss.fail()) return Warn(line);
    MuonSphereDesc sp{};
    sp.center[0] = x;
    sp.center[1] = y;
    sp.center[2] = z;
    sp.radius = r;
    sp.transform = xform_stack_.back();
    sp.material = CurrentMaterial();
    sp.prim_id = NextPrimId();
    s_->spheres.push_back(sp);
  } else if (cmd == "start_mesh") {
    meshes_.emplace_back();
    cur_mesh_ = static_cast<int>(meshes_.size()) - 1;
  } else if (cmd == "end_mesh") {
    cur_mesh_ = 0;
  } else if (cmd == "vertex") {
    mm::v3 v;
    if (!read3(&v)) return Warn(line);
    meshes_[cur_mesh_].push_back(static_cast<int32_t>(vertices_.size()));
    vertices_.push_back(Vertex{v, mm::splat3(0.0f)});
  } else if (cmd == "vertex_normal" || cmd == "tri_normal") {
    // Accepted and ignored, as in the reference (muon/parser.cc:614-617, 641-644).
  } else if (cmd == "tri") {
    int i0, i1, i2;
    iss >> i0 >> i1 >> i2;
    if (iss.fail()) return Warn(line);
    const std::vector<int32_t> &mesh = meshes_[cur_mesh_];
    int n = static_cast<int>(mesh.size());
    if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= n || i1 >= n || i2 >= n) return Warn(line);
    const int32_t g[3] = {mesh[i0], mesh[i1], mesh[i2]};
    AddTriangle(g);
  } else if (cmd == "translate" || cmd == "scale") {
    mm::v3 v;
    if (!read3(&v)) return Warn(line);
    MultiplyTransform(cmd == "translate" ? mm::translate(v) : mm::scale(v));
  } else if (cmd == "rotate") {
    mm::v3 axis;
    float angle;
    if (!read3(&axis) || !Read(iss, &angle)) return Warn(line);
    MultiplyTransform(mm::rotate(mm::radians(angle), axis));
  } else if (cmd == "push_transform") {
    xform_stack_.push_back(xform_stack_.back());
  } else if (cmd == "pop_transform") {
    if (xform_stack_.size() <= 1) return Warn(line);
    xform_stack_.pop_back();
  } else if (cmd == "directional_light" || cmd == "point_light") {
    mm::v3 pos, color;
    if (!read3(&pos) || !read3(&color)) return Warn(line);
    MuonLightDesc l{};
    l.type = cmd == "point_light" ? MUON_LIGHT_POINT : MUON_LIGHT_DIRECTIONAL;
    l.color[0] = color.x, l.color[1] = color.y, l.color[2] = color.z;
    l.p0[0] = pos.x, l.p0[1] = pos.y, l.p0[2] = pos.z;
    l.p1[0] = attenuation_.x, l.p1[1] = attenuation_.y, l.p1[2] = attenuation_.z;
    s_->lights.push_back(l);
  } else if (cmd == "attenuation") {
    if (!read3(&attenuation_)) return Warn(line);
  } else if (cmd == "quad_light") {
    mm::v3 corner, e0, e1, color;
    if (!read3(&corner) || !read3(&e0) || !read3(&e1) || !read3(&color)) return Warn(line);
    int32_t light_id = static_cast<int32_t>(s_->lights.size());
    MuonLightDesc l{};
    l.type = MUON_LIGHT_QUAD;
    l.color[0] = color.x, l.color[1] = color.y, l.color[2] = color.z;
    l.p0[0] = corner.x, l.p0[1] = corner.y, l.p0[2] = corner.z;
    l.p1[0] = e0.x, l.p1[1] = e0.y, l.p1[2] = e0.z;
    l.p2[0] = e1.x, l.p2[1] = e1.y, l.p2[2] = e1.z;
    MuonMaterialDesc m{};
    m.brdf = MUON_BRDF_PHONG;
    m.emission[0] = color.x, m.emission[1] = color.y, m.emission[2] = color.z;
    int32_t mat = static_cast<int32_t>(s_->materials.size());
    s_->materials.push_back(m);
    mm::v3 va = corner, vb = corner + e0, vc = corner + e1, vd = corner + e0 + e1;
    const mm::v3 tris[2][3] = {{va, vc, vb}, {vb, vc, vd}};
    for (int t = 0; t < 2; ++t) {
      MuonTriangleDesc d{};
      for (int k = 0; k < 3; ++k) {
        d.v[k][0] = tris[t][k].x;
        d.v[k][1] = tris[t][k].y;
        d.v[k][2] = tris[t][k].z;
      }
      d.transform = -1;
      d.material = mat;
      d.light = light_id;
      d.smooth = 0;
      d.prim_id = NextPrimId();
      s_->triangles.push_back(d);
    }
    s_->lights.push_back(l);
  } else if (cmd == "brdf") {
    std::string v;
    if (!Read(iss, &v)) return Warn(line);
    int32_t type;
    if (v == "lambertian") type = MUON_BRDF_PHONG;  // switch fallthrough in the reference
    else if (v == "phong") type = MUON_BRDF_PHONG;
    else if (v == "ggx") type = MUON_BRDF_GGX;
    else return Warn(line);
    EditMaterial().brdf = type;
  } else if (cmd == "ambient" || cmd == "diffuse" || cmd == "specular" || cmd == "emission") {
    mm::v3 c;
    if (!read3(&c)) return Warn(line);
    MuonMaterialDesc &m = EditMaterial();
    float *dst = cmd == "ambient" ? m.ambient
                 : cmd == "diffuse" ? m.diffuse
                 : cmd == "specular" ? m.specular
                                     : m.emission;
    dst[0] = c.x, dst[1] = c.y, dst[2] = c.z;
  } else if (cmd == "shininess" || cmd == "roughness") {
    float v;
    if (!Read(iss, &v)) return Warn(line);
    if (cmd == "shininess") EditMaterial().shininess = v;
    else EditMaterial().roughness = v;
  } else {
    Warn(line);
  }
}

void Parser::Finish() {
  if (compute_vertex_normals_) {
    for (Vertex &v : vertices_) {
      float len2 = mm::dot(v.normal, v.normal);
      if (len2 > 0.0f) v.normal = mm::normalize(v.normal);
    }
  }
  for (MuonTriangleDesc &t : s_->triangles) {
    if (t.light >= 0) continue;
    for (int k = 0; k < 3; ++k) {
      int32_t g;
      std::memcpy(&g, &t.n[k][0], sizeof(int32_t));
      t.n[k][0] = vertices_[g].normal.x;
      t.n[k][1] = vertices_[g].normal.y;
      t.n[k][2] = vertices_[g].normal.z;
    }
  }
  if (!seed_drawn_) s_->params.seed = seedgen_();
}

}  // namespace

MuonTransformDesc MakeTransformDesc(const mm::m4 &m) {
  MuonTransformDesc d;
  mm::m4 inv = mm::inverse(m);
  mm::m4 inv_t = mm::transpose(inv);
  std::memcpy(d.object_to_world, &m, sizeof(float) * 16);
  std::memcpy(d.world_to_object, &inv, sizeof(float) * 16);
  std::memcpy(d.normal_to_world, &inv_t, sizeof(float) * 16);
  return d;
}

bool ParseScene(const std::string &text, const std::string &base_dir, ParsedScene *out,
                std::string *error) {
  Parser parser(out, base_dir);
  std::istringstream in(text);
  std::string line;
  while (std::getline(in, line)) parser.Line(line);
  parser.Finish();
  if (!out->has_camera) {
    *error = "scene has no camera";
    return false;
  }
  return true;
}

}  // namespace muon_gpu
