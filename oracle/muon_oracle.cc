// CPU oracle: a restatement of the reference renderer's hot path, used ONLY as
// the checker in tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// arm. It is never linked into or called by the product (muon_gb300/).
//
// It re-implements, in its own structure, what the reference computes:
//   scene parsing            muon/parser.cc:230-880 (quirks included)
//   camera                   muon/camera.cc:15-62
//   bounds / BVH / linear    muon/bounds.cc, muon/acceleration.cc:14-458
//   triangles / spheres      muon/objects.cc:9-274
//   lights                   muon/lighting.cc
//   BRDFs and sampling       muon/materials.cc, muon/hemisphere_sampling.cc,
//                            muon/transform.{h,cc}
//   integrators              muon/integration.cc:15-636 (all six)
//   tiling, sampler, film    muon/sampling.cc, muon/renderer.cc, muon/film.cc
//   RNG                      muon/random.{h,cc}: std::mt19937 feeding
//                            std::uniform_real_distribution<float>
// Every float expression keeps the reference's evaluation order (its vector
// library evaluates dot products as (x*x'+y*y')+z*z', normalize as
// v*(1/sqrt(dot)), matrix products column by column), so with T = float the
// results are bit-identical to the reference build; pinned against the
// reference's golden images by tests/test_oracle.py. With T = double the same
// code is the FP64 rebuild used for the 1e-5 relative value checks.
//
// Build: oracle/build.py (g++ -O2 -ffp-contract=off) -> oracle/lib/.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <optional>
#include <random>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace oracle {

// ---------------------------------------------------------------- vectors
template <class T>
struct V3 {
  T x = 0, y = 0, z = 0;
  V3() = default;
  V3(T a, T b, T c) : x(a), y(b), z(c) {}
  explicit V3(T s) : x(s), y(s), z(s) {}
  T &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> V3<T> &operator+=(V3<T> &a, V3<T> b) { return a = a + b; }
template <class T> V3<T> &operator-=(V3<T> &a, V3<T> b) { return a = a - b; }
template <class T> V3<T> &operator*=(V3<T> &a, T s) { return a = a * s; }
template <class T> V3<T> &operator/=(V3<T> &a, T s) { return a = a / s; }
template <class T> T Dot(V3<T> a, V3<T> b) { V3<T> t = a * b; return t.x + t.y + t.z; }
template <class T> V3<T> Cross(V3<T> a, V3<T> b) {
  return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <class T> T Len(V3<T> v) { return std::sqrt(Dot(v, v)); }
template <class T> V3<T> Norm(V3<T> v) { return v * (static_cast<T>(1) / std::sqrt(Dot(v, v))); }
template <class T> T Min(T a, T b) { return (b < a) ? b : a; }
template <class T> T Max(T a, T b) { return (a < b) ? b : a; }
template <class T> T Clamp(T x, T lo, T hi) { return Min(Max(x, lo), hi); }
template <class T> T CompAdd(V3<T> v) { T r(0); r += v.x; r += v.y; r += v.z; return r; }
template <class T> T CompMax(V3<T> v) { return Max(Max(v.x, v.y), v.z); }
template <class T> constexpr T Pi() { return static_cast<T>(3.14159265358979323846264338327950288); }
template <class T> constexpr T InvPi() { return static_cast<T>(0.318309886183790671537767526745028724); }
template <class T> constexpr T Eps() { return static_cast<T>(0.0001); }
template <class T> V3<T> Reflect(V3<T> d, V3<T> n) { return d - (2 * Dot(d, n) * n); }

template <class T>
struct V4 {
  T x = 0, y = 0, z = 0, w = 0;
};
template <class T> V4<T> operator+(V4<T> a, V4<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
template <class T> V4<T> operator-(V4<T> a, V4<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
template <class T> V4<T> operator*(V4<T> a, V4<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }
template <class T> V4<T> operator*(V4<T> a, T s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }

// Column-major 4x4.
template <class T>
struct M4 {
  V4<T> c[4];
  static M4 Identity() {
    M4 m;
    m.c[0] = {1, 0, 0, 0};
    m.c[1] = {0, 1, 0, 0};
    m.c[2] = {0, 0, 1, 0};
    m.c[3] = {0, 0, 0, 1};
    return m;
  }
  T e(int col, int row) const {
    const V4<T> &v = c[col];
    return row == 0 ? v.x : (row == 1 ? v.y : (row == 2 ? v.z : v.w));
  }
};
template <class T> V4<T> Mul(const M4<T> &m, V4<T> v) {
  V4<T> a = m.c[0] * v.x + m.c[1] * v.y;
  V4<T> b = m.c[2] * v.z + m.c[3] * v.w;
  return a + b;
}
template <class T> M4<T> Mul(const M4<T> &a, const M4<T> &b) {
  M4<T> r;
  for (int k = 0; k < 4; ++k) r.c[k] = a.c[0] * b.c[k].x + a.c[1] * b.c[k].y + a.c[2] * b.c[k].z + a.c[3] * b.c[k].w;
  return r;
}
template <class T> V3<T> XPoint(const M4<T> &m, V3<T> p) {
  V4<T> r = Mul(m, V4<T>{p.x, p.y, p.z, static_cast<T>(1)});
  return {r.x, r.y, r.z};
}
template <class T> V3<T> XDir(const M4<T> &m, V3<T> d) {
  V4<T> r = Mul(m, V4<T>{d.x, d.y, d.z, static_cast<T>(0)});
  return Norm(V3<T>{r.x, r.y, r.z});
}
template <class T> M4<T> Transpose(const M4<T> &m) {
  M4<T> r;
  for (int i = 0; i < 4; ++i) r.c[i] = {m.e(0, i), m.e(1, i), m.e(2, i), m.e(3, i)};
  return r;
}
// Cofactor inverse in the reference library's evaluation order.
template <class T> M4<T> Inverse(const M4<T> &m) {
  auto k = [&](int a, int b, int c, int d, int e, int f, int g, int h) {
    return m.e(a, b) * m.e(c, d) - m.e(e, f) * m.e(g, h);
  };
  T c00 = k(2, 2, 3, 3, 3, 2, 2, 3), c02 = k(1, 2, 3, 3, 3, 2, 1, 3), c03 = k(1, 2, 2, 3, 2, 2, 1, 3);
  T c04 = k(2, 1, 3, 3, 3, 1, 2, 3), c06 = k(1, 1, 3, 3, 3, 1, 1, 3), c07 = k(1, 1, 2, 3, 2, 1, 1, 3);
  T c08 = k(2, 1, 3, 2, 3, 1, 2, 2), c10 = k(1, 1, 3, 2, 3, 1, 1, 2), c11 = k(1, 1, 2, 2, 2, 1, 1, 2);
  T c12 = k(2, 0, 3, 3, 3, 0, 2, 3), c14 = k(1, 0, 3, 3, 3, 0, 1, 3), c15 = k(1, 0, 2, 3, 2, 0, 1, 3);
  T c16 = k(2, 0, 3, 2, 3, 0, 2, 2), c18 = k(1, 0, 3, 2, 3, 0, 1, 2), c19 = k(1, 0, 2, 2, 2, 0, 1, 2);
  T c20 = k(2, 0, 3, 1, 3, 0, 2, 1), c22 = k(1, 0, 3, 1, 3, 0, 1, 1), c23 = k(1, 0, 2, 1, 2, 0, 1, 1);
  V4<T> f0{c00, c00, c02, c03}, f1{c04, c04, c06, c07}, f2{c08, c08, c10, c11};
  V4<T> f3{c12, c12, c14, c15}, f4{c16, c16, c18, c19}, f5{c20, c20, c22, c23};
  V4<T> g0{m.e(1, 0), m.e(0, 0), m.e(0, 0), m.e(0, 0)}, g1{m.e(1, 1), m.e(0, 1), m.e(0, 1), m.e(0, 1)};
  V4<T> g2{m.e(1, 2), m.e(0, 2), m.e(0, 2), m.e(0, 2)}, g3{m.e(1, 3), m.e(0, 3), m.e(0, 3), m.e(0, 3)};
  V4<T> i0 = g1 * f0 - g2 * f1 + g3 * f2, i1 = g0 * f0 - g2 * f3 + g3 * f4;
  V4<T> i2 = g0 * f1 - g1 * f3 + g3 * f5, i3 = g0 * f2 - g1 * f4 + g2 * f5;
  V4<T> sa{1, -1, 1, -1}, sb{-1, 1, -1, 1};
  M4<T> r;
  r.c[0] = i0 * sa, r.c[1] = i1 * sb, r.c[2] = i2 * sa, r.c[3] = i3 * sb;
  V4<T> row0{r.c[0].x, r.c[1].x, r.c[2].x, r.c[3].x};
  V4<T> d0 = m.c[0] * row0;
  T det = (d0.x + d0.y) + (d0.z + d0.w);
  T inv = static_cast<T>(1) / det;
  for (int i = 0; i < 4; ++i) r.c[i] = r.c[i] * inv;
  return r;
}
template <class T> M4<T> Translate(V3<T> v) {
  M4<T> m = M4<T>::Identity(), r = m;
  r.c[3] = m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z + m.c[3];
  return r;
}
template <class T> M4<T> Scale(V3<T> v) {
  M4<T> m = M4<T>::Identity(), r;
  r.c[0] = m.c[0] * v.x, r.c[1] = m.c[1] * v.y, r.c[2] = m.c[2] * v.z, r.c[3] = m.c[3];
  return r;
}
template <class T> M4<T> Rotate(T angle, V3<T> v) {
  T c = std::cos(angle), s = std::sin(angle);
  V3<T> a = Norm(v);
  V3<T> t = (static_cast<T>(1) - c) * a;
  T r00 = c + t.x * a.x, r01 = t.x * a.y + s * a.z, r02 = t.x * a.z - s * a.y;
  T r10 = t.y * a.x - s * a.z, r11 = c + t.y * a.y, r12 = t.y * a.z + s * a.x;
  T r20 = t.z * a.x + s * a.y, r21 = t.z * a.y - s * a.x, r22 = c + t.z * a.z;
  M4<T> m = M4<T>::Identity(), r;
  r.c[0] = m.c[0] * r00 + m.c[1] * r01 + m.c[2] * r02;
  r.c[1] = m.c[0] * r10 + m.c[1] * r11 + m.c[2] * r12;
  r.c[2] = m.c[0] * r20 + m.c[1] * r21 + m.c[2] * r22;
  r.c[3] = m.c[3];
  return r;
}
template <class T> T Radians(T deg) { return deg * static_cast<T>(0.01745329251994329576923690768489); }
template <class T, class U> V3<T> Cv(V3<U> v) { return {static_cast<T>(v.x), static_cast<T>(v.y), static_cast<T>(v.z)}; }
template <class T, class U> M4<T> Cm(const M4<U> &m) {
  M4<T> r;
  for (int i = 0; i < 4; ++i) r.c[i] = {static_cast<T>(m.c[i].x), static_cast<T>(m.c[i].y), static_cast<T>(m.c[i].z), static_cast<T>(m.c[i].w)};
  return r;
}

// ---------------------------------------------------------------- RNG
struct UniformRandom {
  explicit UniformRandom(unsigned int seed) : gen(seed), dist(0.0f, 1.0f) {}
  float Next() { return dist(gen); }
  std::mt19937 gen;
  std::uniform_real_distribution<float> dist;
};

// ---------------------------------------------------------------- scene
struct Counters {
  uint64_t primary = 0, secondary = 0, obj_tests = 0, obj_hits = 0, bounds_tests = 0, bounds_hits = 0;
  void Add(const Counters &o) {
    primary += o.primary, secondary += o.secondary, obj_tests += o.obj_tests, obj_hits += o.obj_hits;
    bounds_tests += o.bounds_tests, bounds_hits += o.bounds_hits;
  }
};

enum class Brdf { kLambertian, kPhong, kGGX };
enum class Integ { kNormals, kAlbedo, kDepth, kRaytracer, kAnalytic, kPath };
enum class LightType { kDirectional, kPoint, kQuad };

template <class T>
struct Material {
  V3<T> ambient, diffuse, specular, emission;
  T shininess = 0, roughness = 0;
  Brdf brdf = Brdf::kPhong;
};

template <class T>
struct Light {
  LightType type;
  V3<T> color, a, b, c;  // quad: corner, edge0, edge1 | point: pos, atten | dir: direction
};

template <class T>
struct Vertex {
  V3<T> pos, normal;
};

template <class T>
struct Prim {
  bool sphere = false;
  // triangle: vertex ids into the scene's vertex store; sphere: centre/radius
  int32_t v[3] = {0, 0, 0};
  V3<T> normal;  // unnormalised object-space face normal
  T normal_len2 = 0;
  bool smooth = false;
  V3<T> centre;
  T radius = 0;
  int32_t xform = 0;  // index into the transform table (0 = identity)
  int32_t material = 0;
  int32_t light = -1;
};

template <class T>
struct Ray {
  V3<T> o, d;
  V3<T> At(T t) const { return o + d * t; }
};

template <class T>
struct Hit {
  T distance;
  V3<T> pos, normal;
  int32_t prim;
};

template <class T>
struct Bounds {
  V3<T> lo{std::numeric_limits<T>::infinity()}, hi{-std::numeric_limits<T>::infinity()};
  Bounds() = default;
  explicit Bounds(V3<T> p) : lo(p), hi(p) {}
  Bounds(V3<T> a, V3<T> b) : lo(Min(a.x, b.x), Min(a.y, b.y), Min(a.z, b.z)), hi(Max(a.x, b.x), Max(a.y, b.y), Max(a.z, b.z)) {}
  V3<T> Dim() const { return hi - lo; }
  int MaxAxis() const {
    V3<T> d = Dim();
    if (d.x > d.y && d.x > d.z) return 0;
    return d.y > d.z ? 1 : 2;
  }
  T Area() const {
    V3<T> d = Dim();
    return static_cast<T>(2) * (d.x * d.y + d.x * d.z + d.y * d.z);
  }
  static Bounds U(const Bounds &a, const Bounds &b) {
    Bounds r;
    r.lo = {Min(a.lo.x, b.lo.x), Min(a.lo.y, b.lo.y), Min(a.lo.z, b.lo.z)};
    r.hi = {Max(a.hi.x, b.hi.x), Max(a.hi.y, b.hi.y), Max(a.hi.z, b.hi.z)};
    return r;
  }
  static Bounds U(const Bounds &a, V3<T> p) {
    Bounds r;
    r.lo = {Min(a.lo.x, p.x), Min(a.lo.y, p.y), Min(a.lo.z, p.z)};
    r.hi = {Max(a.hi.x, p.x), Max(a.hi.y, p.y), Max(a.hi.z, p.z)};
    return r;
  }
  Bounds Xform(const M4<T> &m) const {
    Bounds b(XPoint(m, lo));
    b = U(b, XPoint(m, V3<T>(hi.x, lo.y, lo.z)));
    b = U(b, XPoint(m, V3<T>(lo.x, hi.y, lo.z)));
    b = U(b, XPoint(m, V3<T>(lo.x, lo.y, hi.z)));
    b = U(b, XPoint(m, V3<T>(lo.x, hi.y, hi.z)));
    b = U(b, XPoint(m, V3<T>(hi.x, lo.y, hi.z)));
    b = U(b, XPoint(m, V3<T>(hi.x, hi.y, lo.z)));
    return U(b, XPoint(m, hi));
  }
  bool Slab(const Ray<T> &r, T &tmin, T &tmax) const {
    tmin = 0;
    tmax = std::numeric_limits<T>::infinity();
    for (int i = 0; i < 3; ++i) {
      if (r.d[i] == static_cast<T>(0)) continue;
      T a = (lo[i] - r.o[i]) / r.d[i], b = (hi[i] - r.o[i]) / r.d[i];
      if (a > b) std::swap(a, b);
      tmin = Max(tmin, a);
      tmax = Min(tmax, b);
      if (tmin > tmax) return false;
    }
    return true;
  }
  bool HasIntersection(const Ray<T> &r, T maxd) const {
    T a, b;
    if (!Slab(r, a, b)) return false;
    return b > static_cast<T>(0) && a < maxd;
  }
};

template <class T>
struct Xf {
  M4<T> m, inv, inv_t;
};

struct BvhNode {
  size_t count = 0, start = 0;
  int axis = 0;
  int32_t kids[2] = {-1, -1};
};

template <class T>
struct Scene {
  int width = 150, height = 150, min_depth = 0, max_depth = 5;
  std::string output = "raytrace.png";
  float gamma = 1.0f;
  bool compute_vertex_normals = false;
  int pixel_samples = 1, light_samples = 1;
  bool light_stratify = false;
  int nee = 0;  // 0 off, 1 on, 2 mis
  bool rr = false;
  int is = 0;   // 0 hemisphere, 1 cosine, 2 brdf
  V3<T> attenuation{1, 0, 0};
  // camera
  bool has_camera = false;
  V3<T> eye, cu, cv, cw;
  T tan_x = 0, tan_y = 0;
  int cam_w = 0, cam_h = 0;
  // content
  std::vector<Xf<T>> xforms;
  std::vector<Material<T>> materials;
  std::vector<Light<T>> lights;
  std::vector<Vertex<T>> verts;
  std::vector<Prim<T>> prims;  // in AddPrimitive order
  Integ integ = Integ::kRaytracer;
  unsigned int path_seed = 0;
  std::mt19937 seedgen;
  // acceleration
  bool linear = false;
  std::vector<int32_t> order;  // BVH primitive order -> prim index
  std::vector<BvhNode> nodes;
  std::vector<Bounds<T>> node_bounds;
};

// Ray cast through screen position (x, y) (Camera::CastRay).
template <class T>
Ray<T> CastRay(const Scene<T> &s, T x, T y) {
  T hw = static_cast<T>(s.cam_w) / static_cast<T>(2), hh = static_cast<T>(s.cam_h) / static_cast<T>(2);
  T ox = (x - hw) / hw, oy = (hh - y) / hh;
  T alpha = s.tan_x * ox, beta = s.tan_y * oy;
  return {s.eye, Norm(alpha * s.cu + beta * s.cv - s.cw)};
}

// ---------------------------------------------------------------- primitives
template <class T>
std::optional<Hit<T>> IntersectObject(const Scene<T> &s, const Prim<T> &p, const Ray<T> &r, int32_t id) {
  if (p.sphere) {
    V3<T> dc = r.o - p.centre;
    T b = Dot(r.d, dc);
    T c = Dot(dc, dc) - p.radius * p.radius;
    T disc = b * b - c;
    if (disc < 0) return std::nullopt;
    T sq = std::sqrt(disc);
    T r0 = -b + sq, r1 = -b - sq;
    if (r0 < 0 && r1 < 0) return std::nullopt;
    T t = Min(r0, r1);
    if (t < 0) t = Max(r0, r1);
    V3<T> q = r.At(t);
    return Hit<T>{t, q, Norm(q - p.centre), id};
  }
  T dn = Dot(p.normal, r.d);
  if (dn > -Eps<T>() && dn < Eps<T>()) return std::nullopt;
  const V3<T> &a = s.verts[p.v[0]].pos, &b = s.verts[p.v[1]].pos, &c = s.verts[p.v[2]].pos;
  T t = (Dot(a, p.normal) - Dot(r.o, p.normal)) / dn;
  if (t < 0) return std::nullopt;
  V3<T> q = r.At(t);
  T v = Dot(p.normal, Cross(b - a, q - a));
  if (v < 0) return std::nullopt;
  T w = Dot(p.normal, Cross(c - b, q - b));
  if (w < 0) return std::nullopt;
  T u = Dot(p.normal, Cross(a - c, q - c));
  if (u < 0) return std::nullopt;
  u /= p.normal_len2;
  v /= p.normal_len2;
  w /= p.normal_len2;
  V3<T> n = p.smooth ? w * s.verts[p.v[0]].normal + u * s.verts[p.v[1]].normal + v * s.verts[p.v[2]].normal
                     : Norm(p.normal);
  return Hit<T>{t, q, n, id};
}

// Primitive::Intersect: object-space test, results carried back to world.
template <class T>
std::optional<Hit<T>> IntersectPrim(const Scene<T> &s, int32_t id, const Ray<T> &r) {
  const Prim<T> &p = s.prims[id];
  const Xf<T> &x = s.xforms[p.xform];
  Ray<T> tr{XPoint(x.inv, r.o), XDir(x.inv, r.d)};
  auto h = IntersectObject(s, p, tr, id);
  if (!h) return h;
  h->pos = XPoint(x.m, h->pos);
  h->normal = XDir(x.inv_t, h->normal);
  h->distance = Len(h->pos - r.o);
  return h;
}

template <class T>
Bounds<T> WorldBounds(const Scene<T> &s, const Prim<T> &p) {
  const M4<T> &m = s.xforms[p.xform].m;
  if (p.sphere) return Bounds<T>(p.centre - V3<T>(p.radius), p.centre + V3<T>(p.radius)).Xform(m);
  Bounds<T> b(XPoint(m, s.verts[p.v[0]].pos), XPoint(m, s.verts[p.v[1]].pos));
  return Bounds<T>::U(b, XPoint(m, s.verts[p.v[2]].pos));
}

// ---------------------------------------------------------------- BVH
template <class T>
struct PrimInfo {
  size_t index;
  Bounds<T> bounds;
  V3<T> centroid;
};

template <class T>
int32_t BuildBvh(Scene<T> &s, size_t start, size_t end, std::vector<PrimInfo<T>> &info) {
  size_t n = end - start;
  int32_t id = static_cast<int32_t>(s.nodes.size());
  s.nodes.emplace_back();
  s.node_bounds.emplace_back();
  if (n == 1) {
    s.nodes[id].count = 1;
    s.nodes[id].start = start;
    s.node_bounds[id] = info[start].bounds;
    return id;
  }
  Bounds<T> cb;
  for (size_t i = start; i < end; ++i) cb = Bounds<T>::U(cb, info[i].centroid);
  int axis = cb.MaxAxis();
  size_t split = static_cast<size_t>(-1);
  auto first = info.begin() + start, last = info.begin() + end;
  bool uniform = false;
  // 12-bucket surface area heuristic (muon/acceleration.cc:454-596).
  constexpr size_t kBuckets = 12;
  struct Bucket {
    size_t size = 0;
    Bounds<T> bounds;
  } buckets[kBuckets];
  V3<T> space = cb.Dim();
  auto bucket_of = [&](const PrimInfo<T> &pi) {
    T off = space[axis] == 0 ? static_cast<T>(0) : (pi.centroid[axis] - cb.lo[axis]) / space[axis];
    size_t b = static_cast<size_t>(off * kBuckets);
    if (b == kBuckets) b = kBuckets - 1;
    return b;
  };
  for (size_t i = start; i < end; ++i) {
    Bucket &b = buckets[bucket_of(info[i])];
    b.size++;
    b.bounds = Bounds<T>::U(b.bounds, info[i].bounds);
  }
  Bounds<T> all;
  for (size_t i = 0; i < kBuckets; ++i) all = Bounds<T>::U(all, buckets[i].bounds);
  T cost[kBuckets - 1];
  {
    size_t cs = 0;
    Bounds<T> acc;
    for (size_t i = 0; i < kBuckets - 1; ++i) {
      cs += buckets[i].size;
      if (cs == 0) continue;
      acc = Bounds<T>::U(acc, buckets[i].bounds);
      cost[i] = cs * acc.Area();
    }
  }
  {
    size_t cs = 0;
    Bounds<T> acc;
    for (int i = kBuckets - 2; i >= 0; --i) {
      cs += buckets[i + 1].size;
      if (cs == 0) continue;
      acc = Bounds<T>::U(acc, buckets[i + 1].bounds);
      cost[i] += cs * acc.Area();
    }
  }
  T total = all.Area();
  T min_cost = std::numeric_limits<T>::infinity();
  size_t split_bucket = 0;
  for (size_t i = 0; i < kBuckets - 1; ++i) {
    T c = static_cast<T>(0.125f) + cost[i] / total;
    if (c < min_cost) {
      min_cost = c;
      split_bucket = i;
    }
  }
  T leaf_cost = static_cast<T>(n);
  if (leaf_cost < min_cost) {
    s.nodes[id].count = n;
    s.nodes[id].start = start;
    s.node_bounds[id] = all;
    return id;
  }
  auto it = std::partition(first, last, [&](const PrimInfo<T> &pi) { return bucket_of(pi) <= split_bucket; });
  split = static_cast<size_t>(it - info.begin());
  if (split == start || split == end) uniform = true;
  if (uniform) {
    split = (start + end) / 2;
    std::nth_element(first, info.begin() + split, last,
                     [axis](const PrimInfo<T> &a, const PrimInfo<T> &b) { return a.centroid[axis] < b.centroid[axis]; });
  }
  int32_t l = BuildBvh(s, start, split, info);
  int32_t r = BuildBvh(s, split, end, info);
  s.nodes[id].kids[0] = l;
  s.nodes[id].kids[1] = r;
  s.nodes[id].axis = axis;
  s.node_bounds[id] = Bounds<T>::U(s.node_bounds[l], s.node_bounds[r]);
  return id;
}

template <class T>
void InitAccel(Scene<T> &s) {
  s.order.resize(s.prims.size());
  for (size_t i = 0; i < s.prims.size(); ++i) s.order[i] = static_cast<int32_t>(i);
  if (s.linear || s.prims.empty()) return;
  std::vector<PrimInfo<T>> info;
  info.reserve(s.prims.size());
  for (size_t i = 0; i < s.prims.size(); ++i) {
    Bounds<T> b = WorldBounds(s, s.prims[i]);
    V3<T> diag = b.hi - b.lo;
    info.push_back({i, b, b.lo + static_cast<T>(0.5f) * diag});
  }
  BuildBvh(s, 0, s.prims.size(), info);
  for (size_t i = 0; i < info.size(); ++i) s.order[i] = static_cast<int32_t>(info[i].index);
}

// Structure::Intersect / HasIntersection for the linear list and the BVH.
template <class T>
std::optional<Hit<T>> Intersect(const Scene<T> &s, const Ray<T> &r, Counters &st) {
  T min_dist = std::numeric_limits<T>::infinity();
  std::optional<Hit<T>> best;
  auto test = [&](int32_t id) {
    st.obj_tests++;
    auto h = IntersectPrim(s, id, r);
    if (!h) return;
    st.obj_hits++;
    if (h->distance > 0 && h->distance < min_dist) {
      min_dist = h->distance;
      best = h;
    }
  };
  if (s.linear || s.nodes.empty()) {
    for (size_t i = 0; i < s.prims.size(); ++i) test(static_cast<int32_t>(i));
    return best;
  }
  const size_t first[3] = {r.d.x < 0, r.d.y < 0, r.d.z < 0};
  std::vector<int32_t> stack;
  stack.reserve(64);
  int32_t node = 0;
  while (true) {
    st.bounds_tests++;
    if (!s.node_bounds[node].HasIntersection(r, min_dist)) {
      if (stack.empty()) break;
      node = stack.back();
      stack.pop_back();
      continue;
    }
    st.bounds_hits++;
    const BvhNode &nd = s.nodes[node];
    if (nd.count > 0) {
      for (size_t i = nd.start; i < nd.start + nd.count; ++i) test(s.order[i]);
      if (stack.empty()) break;
      node = stack.back();
      stack.pop_back();
      continue;
    }
    size_t c = first[nd.axis];
    stack.push_back(nd.kids[1 - c]);
    node = nd.kids[c];
  }
  return best;
}

template <class T>
bool Occluded(const Scene<T> &s, const Ray<T> &r, T maxd, Counters &st) {
  auto prim_hit = [&](int32_t id) {
    auto h = IntersectPrim(s, id, r);
    return h && h->distance > 0 && h->distance < maxd;
  };
  if (s.linear || s.nodes.empty()) {
    for (size_t i = 0; i < s.prims.size(); ++i)
      if (prim_hit(static_cast<int32_t>(i))) return true;
    return false;
  }
  const size_t first[3] = {r.d.x < 0, r.d.y < 0, r.d.z < 0};
  std::vector<int32_t> stack;
  stack.reserve(64);
  int32_t node = 0;
  while (true) {
    st.bounds_tests++;
    if (!s.node_bounds[node].HasIntersection(r, maxd)) {
      if (stack.empty()) break;
      node = stack.back();
      stack.pop_back();
      continue;
    }
    st.bounds_hits++;
    const BvhNode &nd = s.nodes[node];
    if (nd.count > 0) {
      for (size_t i = nd.start; i < nd.start + nd.count; ++i) {
        st.obj_tests++;
        if (prim_hit(s.order[i])) {
          st.obj_hits++;
          return true;
        }
      }
      if (stack.empty()) break;
      node = stack.back();
      stack.pop_back();
      continue;
    }
    size_t c = first[nd.axis];
    stack.push_back(nd.kids[1 - c]);
    node = nd.kids[c];
  }
  return false;
}

// ---------------------------------------------------------------- parser
template <class T>
bool Parse(const std::string &text, Scene<T> &s, std::string *err, int *warnings) {
  std::random_device rd;
  s.seedgen.seed(rd());
  Material<T> mat;
  mat.ambient = V3<T>(static_cast<T>(0.2f));
  mat.shininess = 1;
  mat.brdf = Brdf::kPhong;
  s.xforms.clear();
  s.xforms.push_back({M4<T>::Identity(), M4<T>::Identity(), M4<T>::Identity()});
  std::vector<int32_t> stack = {0};
  std::vector<std::vector<int32_t>> meshes(1);
  int cur_mesh = 0;
  std::map<int32_t, int> mat_ids;  // not shared; each material command makes a new one
  int cur_mat = -1;
  auto material_index = [&]() {
    if (cur_mat < 0) {
      cur_mat = static_cast<int>(s.materials.size());
      s.materials.push_back(mat);
    }
    return cur_mat;
  };
  auto edit = [&]() -> Material<T> & {
    cur_mat = -1;
    return mat;
  };
  auto multiply = [&](const M4<T> &m) {
    M4<T> next = Mul(s.xforms[stack.back()].m, m);
    M4<T> inv = Inverse(next);
    s.xforms.push_back({next, inv, Transpose(inv)});
    stack.back() = static_cast<int32_t>(s.xforms.size() - 1);
  };
  *warnings = 0;
  std::istringstream in(text);
  std::string line;
  while (std::getline(in, line)) {
    size_t b = 0, e = line.size();
    while (b < e && std::isspace(static_cast<unsigned char>(line[b]))) ++b;
    while (e > b && std::isspace(static_cast<unsigned char>(line[e - 1]))) --e;
    line = line.substr(b, e - b);
    if (line.empty() || line[0] == '#') continue;
    std::istringstream iss(line);
    std::string cmd;
    iss >> cmd;
    auto bad = [&]() { ++*warnings; };
    auto f3 = [&](V3<T> &v) {
      float x, y, z;
      iss >> x >> y >> z;
      v = V3<T>(x, y, z);
      return !iss.fail();
    };
    if (cmd == "random_seed" || cmd == "film_size") {
      if (cmd == "random_seed") {
        unsigned int seed;
        iss >> seed;
        if (iss.fail()) { bad(); continue; }
        s.seedgen.seed(seed);
      }
      int w, h;
      iss >> w >> h;
      if (iss.fail()) { bad(); continue; }
      s.width = w, s.height = h;
    } else if (cmd == "min_depth" || cmd == "max_depth" || cmd == "pixel_samples" || cmd == "light_samples") {
      int v;
      iss >> v;
      if (iss.fail()) { bad(); continue; }
      (cmd == "min_depth" ? s.min_depth : cmd == "max_depth" ? s.max_depth : cmd == "pixel_samples" ? s.pixel_samples : s.light_samples) = v;
    } else if (cmd == "output") {
      std::string v;
      iss >> v;
      if (iss.fail()) { bad(); continue; }
      s.output = v;
    } else if (cmd == "gamma") {
      float v;
      iss >> v;
      if (iss.fail()) { bad(); continue; }
      s.gamma = v;
    } else if (cmd == "integrator") {
      std::string v;
      iss >> v;
      if (iss.fail()) { bad(); continue; }
      if (v == "normals") s.integ = Integ::kNormals;
      else if (v == "albedo") s.integ = Integ::kAlbedo;
      else if (v == "depth") s.integ = Integ::kDepth;
      else if (v == "raytracer") s.integ = Integ::kRaytracer;
      else if (v == "analyticdirect") s.integ = Integ::kAnalytic;
      else if (v == "pathtracer") s.integ = Integ::kPath, s.path_seed = s.seedgen();
      else bad();
    } else if (cmd == "light_stratify" || cmd == "russian_roulette" || cmd == "compute_vertex_normals") {
      std::string v;
      iss >> v;
      if (iss.fail() || (v != "on" && v != "off")) { bad(); continue; }
      bool on = v == "on";
      (cmd == "light_stratify" ? s.light_stratify : cmd == "russian_roulette" ? s.rr : s.compute_vertex_normals) = on;
    } else if (cmd == "next_event_estimation") {
      std::string v;
      iss >> v;
      if (v == "off") s.nee = 0;
      else if (v == "on") s.nee = 1;
      else if (v == "mis") s.nee = 2;
      else bad();
    } else if (cmd == "importance_sampling") {
      std::string v;
      iss >> v;
      if (v == "hemisphere") s.is = 0;
      else if (v == "cosine") s.is = 1;
      else if (v == "brdf") s.is = 2;
      else bad();
    } else if (cmd == "camera") {
      float f[10];
      for (float &x : f) iss >> x;
      if (iss.fail()) { bad(); continue; }
      V3<T> eye(f[0], f[1], f[2]), look(f[3], f[4], f[5]), up(f[6], f[7], f[8]);
      T fov = f[9];
      s.cam_w = s.width, s.cam_h = s.height;
      s.tan_y = std::tan(Radians(fov) / static_cast<T>(2.0f));
      s.tan_x = s.tan_y * (static_cast<T>(static_cast<float>(s.width)) / static_cast<T>(s.height));
      s.eye = eye;
      s.cw = Norm(eye - look);
      s.cu = Norm(Cross(up, s.cw));
      s.cv = Cross(s.cw, s.cu);
      s.has_camera = true;
      stack.push_back(stack.back());
    } else if (cmd == "sphere") {
      float x, y, z, r;
      iss >> x >> y >> z >> r;
      if (iss.fail()) { bad(); continue; }
      Prim<T> p;
      p.sphere = true;
      p.centre = V3<T>(x, y, z);
      p.radius = r;
      p.xform = stack.back();
      p.material = material_index();
      s.prims.push_back(p);
    } else if (cmd == "start_mesh") {
      meshes.emplace_back();
      cur_mesh = static_cast<int>(meshes.size()) - 1;
    } else if (cmd == "end_mesh") {
      cur_mesh = 0;
    } else if (cmd == "vertex") {
      V3<T> v;
      if (!f3(v)) { bad(); continue; }
      meshes[cur_mesh].push_back(static_cast<int32_t>(s.verts.size()));
      s.verts.push_back({v, V3<T>(0)});
    } else if (cmd == "vertex_normal" || cmd == "tri_normal") {
    } else if (cmd == "tri") {
      int i0, i1, i2;
      iss >> i0 >> i1 >> i2;
      if (iss.fail()) { bad(); continue; }
      const auto &mesh = meshes[cur_mesh];
      int n = static_cast<int>(mesh.size());
      if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= n || i1 >= n || i2 >= n) { bad(); continue; }
      Prim<T> p;
      p.v[0] = mesh[i0], p.v[1] = mesh[i1], p.v[2] = mesh[i2];
      p.normal = Cross(s.verts[p.v[1]].pos - s.verts[p.v[0]].pos, s.verts[p.v[2]].pos - s.verts[p.v[0]].pos);
      p.normal_len2 = Dot(p.normal, p.normal);
      p.smooth = s.compute_vertex_normals;
      p.xform = stack.back();
      p.material = material_index();
      if (s.compute_vertex_normals)
        for (int k = 0; k < 3; ++k) s.verts[p.v[k]].normal += p.normal;
      s.prims.push_back(p);
    } else if (cmd == "translate" || cmd == "scale") {
      V3<T> v;
      if (!f3(v)) { bad(); continue; }
      multiply(cmd == "translate" ? Translate(v) : Scale(v));
    } else if (cmd == "rotate") {
      V3<T> v;
      float ang;
      if (!f3(v)) { bad(); continue; }
      iss >> ang;
      if (iss.fail()) { bad(); continue; }
      multiply(Rotate(Radians(static_cast<T>(ang)), v));
    } else if (cmd == "push_transform") {
      stack.push_back(stack.back());
    } else if (cmd == "pop_transform") {
      if (stack.size() <= 1) { bad(); continue; }
      stack.pop_back();
    } else if (cmd == "directional_light" || cmd == "point_light") {
      V3<T> p, c;
      if (!f3(p) || !f3(c)) { bad(); continue; }
      s.lights.push_back({cmd == "point_light" ? LightType::kPoint : LightType::kDirectional, c, p, s.attenuation, V3<T>()});
    } else if (cmd == "attenuation") {
      V3<T> a;
      if (!f3(a)) { bad(); continue; }
      s.attenuation = a;
    } else if (cmd == "quad_light") {
      V3<T> corner, e0, e1, color;
      if (!f3(corner) || !f3(e0) || !f3(e1) || !f3(color)) { bad(); continue; }
      int32_t light = static_cast<int32_t>(s.lights.size());
      int32_t base = static_cast<int32_t>(s.verts.size());
      s.verts.push_back({corner, V3<T>(0)});
      s.verts.push_back({corner + e0, V3<T>(0)});
      s.verts.push_back({corner + e1, V3<T>(0)});
      s.verts.push_back({corner + e0 + e1, V3<T>(0)});
      Material<T> m;
      m.brdf = Brdf::kPhong;
      m.emission = color;
      int32_t mi = static_cast<int32_t>(s.materials.size());
      s.materials.push_back(m);
      const int tris[2][3] = {{0, 2, 1}, {1, 2, 3}};
      for (auto &t : tris) {
        Prim<T> p;
        for (int k = 0; k < 3; ++k) p.v[k] = base + t[k];
        p.normal = Cross(s.verts[p.v[1]].pos - s.verts[p.v[0]].pos, s.verts[p.v[2]].pos - s.verts[p.v[0]].pos);
        p.normal_len2 = Dot(p.normal, p.normal);
        p.xform = 0;
        p.material = mi;
        p.light = light;
        s.prims.push_back(p);
      }
      s.lights.push_back({LightType::kQuad, color, corner, e0, e1});
    } else if (cmd == "brdf") {
      std::string v;
      iss >> v;
      if (v == "lambertian" || v == "phong") edit().brdf = Brdf::kPhong;
      else if (v == "ggx") edit().brdf = Brdf::kGGX;
      else bad();
    } else if (cmd == "ambient" || cmd == "diffuse" || cmd == "specular" || cmd == "emission") {
      V3<T> c;
      if (!f3(c)) { bad(); continue; }
      Material<T> &m = edit();
      (cmd == "ambient" ? m.ambient : cmd == "diffuse" ? m.diffuse : cmd == "specular" ? m.specular : m.emission) = c;
    } else if (cmd == "shininess" || cmd == "roughness") {
      float v;
      iss >> v;
      if (iss.fail()) { bad(); continue; }
      (cmd == "shininess" ? edit().shininess : edit().roughness) = v;
    } else if (cmd == "load") {
      bad();
    } else {
      bad();
    }
  }
  if (s.compute_vertex_normals) {
    for (int mesh = 0; mesh < static_cast<int>(meshes.size()); ++mesh)
      for (int32_t id : meshes[mesh]) {
        Vertex<T> &v = s.verts[id];
        if (Dot(v.normal, v.normal) > 0) v.normal = Norm(v.normal);
      }
  }
  if (!s.has_camera) {
    *err = "scene has no camera";
    return false;
  }
  return true;
}

// ---------------------------------------------------------------- shading
template <class T>
V3<T> RotateToFrame(V3<T> smp, V3<T> w) {
  V3<T> a = std::fabs(w.y) <= static_cast<T>(0.9f) ? V3<T>(0, 1, 0) : V3<T>(1, 0, 0);
  V3<T> u = Norm(Cross(a, w));
  V3<T> v = Norm(Cross(w, u));
  return smp.x * u + smp.y * v + smp.z * w;
}
template <class T>
V3<T> Polar(T theta, T phi) {
  return {std::cos(phi) * std::sin(theta), std::sin(phi) * std::sin(theta), std::cos(theta)};
}
template <class T>
V3<T> SampleHemisphere(V3<T> n, UniformRandom &r) {
  T r1 = r.Next(), r2 = r.Next();
  return RotateToFrame(Polar(std::acos(r1), static_cast<T>(2.0f) * Pi<T>() * r2), n);
}
template <class T>
V3<T> SampleCosine(V3<T> n, UniformRandom &r) {
  T r1 = r.Next(), r2 = r.Next();
  return RotateToFrame(Polar(std::acos(std::sqrt(r1)), static_cast<T>(2.0f) * Pi<T>() * r2), n);
}

template <class T>
T Reflectiveness(const Material<T> &m) {
  T spec = CompAdd(m.specular) / static_cast<T>(3.0f), diff = CompAdd(m.diffuse) / static_cast<T>(3.0f);
  T denom = diff + spec;
  if (m.brdf == Brdf::kGGX) return denom == 0 ? static_cast<T>(1) : Max(spec / denom, static_cast<T>(0.25f));
  return denom > 0 ? spec / denom : static_cast<T>(0);
}
template <class T>
T GgxD(V3<T> h, V3<T> n, T a) {
  T ang = std::acos(Clamp(Dot(h, n), static_cast<T>(0), static_cast<T>(1)));
  T a2 = a * a;
  T denom = Pi<T>() * std::pow(std::cos(ang), static_cast<T>(4.0f)) * std::pow(a2 + std::pow(std::tan(ang), static_cast<T>(2.0f)), static_cast<T>(2.0f));
  return denom > 0 ? a2 / denom : static_cast<T>(0);
}
template <class T>
T GgxG1(V3<T> v, V3<T> n, T a) {
  T dn = Dot(v, n);
  if (dn <= 0) return 0;
  T ang = std::acos(Clamp(dn, static_cast<T>(0), static_cast<T>(1)));
  T a2 = a * a;
  return static_cast<T>(2.0f) / (static_cast<T>(1.0f) + std::sqrt(static_cast<T>(1.0f) + a2 * std::pow(std::tan(ang), static_cast<T>(2.0f))));
}
template <class T>
V3<T> BrdfSample(const Material<T> &m, V3<T> rd, V3<T> n, UniformRandom &r) {
  if (m.brdf == Brdf::kLambertian) return SampleCosine(n, r);
  T r0 = r.Next();
  if (r0 > Reflectiveness(m)) return SampleCosine(n, r);
  T r1 = r.Next(), r2 = r.Next();
  T phi = static_cast<T>(2.0f) * Pi<T>() * r2;
  if (m.brdf == Brdf::kPhong) {
    T theta = std::acos(std::pow(r1, static_cast<T>(1.0f) / (m.shininess + static_cast<T>(1.0f))));
    return RotateToFrame(Polar(theta, phi), Reflect(rd, n));
  }
  T theta = std::atan(m.roughness * std::sqrt(r1) / std::sqrt(static_cast<T>(1.0f) - r1));
  return Reflect(rd, RotateToFrame(Polar(theta, phi), n));
}
template <class T>
T BrdfPdf(const Material<T> &m, V3<T> in, V3<T> rd, V3<T> n) {
  if (m.brdf == Brdf::kLambertian) return Max(Dot(n, in), static_cast<T>(0)) * InvPi<T>();
  T t = Reflectiveness(m);
  if (m.brdf == Brdf::kPhong) {
    return (static_cast<T>(1.0f) - t) * Max(Dot(n, in), static_cast<T>(0)) * InvPi<T>() +
           t * (m.shininess + 1) * static_cast<T>(0.5f) * InvPi<T>() * std::pow(Max(Dot(Reflect(rd, n), in), static_cast<T>(0)), m.shininess);
  }
  V3<T> h = Norm(in - rd);
  return (static_cast<T>(1.0f) - t) * Max(Dot(n, in), static_cast<T>(0)) * InvPi<T>() +
         t * GgxD(h, n, m.roughness) * Max(Dot(n, h), static_cast<T>(0)) / (static_cast<T>(4.0f) * Dot(h, in));
}
template <class T>
V3<T> BrdfEval(const Material<T> &m, V3<T> in, V3<T> rd, V3<T> n) {
  V3<T> diffuse = m.diffuse * InvPi<T>();
  if (m.brdf == Brdf::kLambertian) return diffuse;
  if (m.brdf == Brdf::kPhong) {
    V3<T> spec = m.specular * (m.shininess + static_cast<T>(2.0f)) * (static_cast<T>(0.5f) * InvPi<T>()) *
                 std::pow(Max(Dot(Reflect(rd, n), in), static_cast<T>(0)), m.shininess);
    return diffuse + spec;
  }
  V3<T> h = Norm(in - rd);
  V3<T> fres = m.specular + (V3<T>(1.0f) - m.specular) * std::pow(static_cast<T>(1.0f) - Dot(in, h), static_cast<T>(5.0f));
  T g = GgxG1(in, n, m.roughness) * GgxG1(-rd, n, m.roughness);
  T d = GgxD(h, n, m.roughness);
  V3<T> spec = (fres * g * d) / (static_cast<T>(4.0f) * Dot(in, n) * Dot(-rd, n));
  return diffuse + spec;
}

template <class T>
std::optional<Hit<T>> QuadIntersect(const Light<T> &l, const Ray<T> &r) {
  V3<T> n = Norm(Cross(l.c, l.b));
  T rdn = Dot(r.d, n);
  if (rdn == 0) return std::nullopt;
  T t = Dot(l.a - r.o, n) / rdn;
  if (t < 0) return std::nullopt;
  V3<T> p = r.At(t), pe = p - l.a;
  T l0 = Len(l.b), l1 = Len(l.c);
  T u = Dot(pe, l.b) / l0, v = Dot(pe, l.c) / l1;
  if (u > 0 && u < l0 && v > 0 && v < l1) return Hit<T>{t, p, n, -1};
  return std::nullopt;
}

template <class T>
struct ShadeInfo {
  V3<T> color, direction;
  T distance;
  const Light<T> *area;
};
template <class T>
ShadeInfo<T> ShadingInfoAt(const Light<T> &l, V3<T> pos) {
  if (l.type == LightType::kDirectional) return {l.color, l.a, std::numeric_limits<T>::infinity(), nullptr};
  if (l.type == LightType::kPoint) {
    V3<T> ptl = l.a - pos;
    V3<T> dir = Norm(ptl);
    T r = Len(ptl);
    T att = l.b.x + l.b.y * r + l.b.z * r * r;
    return {l.color / att, dir, r, nullptr};
  }
  return {l.color, V3<T>(0), 0, &l};
}

template <class T>
T PowerHeuristic(T a, T b) {
  T d = a * a + b * b;
  return d == 0 ? static_cast<T>(0) : (a * a) / d;
}

template <class T>
struct Tracer {
  const Scene<T> &s;
  UniformRandom rand;
  Counters st;
  Tracer(const Scene<T> &sc, unsigned int seed) : s(sc), rand(seed) {}

  V3<T> Trace(const Ray<T> &r, V3<T> tp, int depth) {
    if (s.max_depth != -1 && depth > (s.nee != 0 ? s.max_depth - 1 : s.max_depth)) return V3<T>(0);
    if (depth == 0) st.primary++;
    else st.secondary++;
    auto h = Intersect(s, r, st);
    if (!h) return V3<T>(0);
    return Shade(*h, r, tp, depth);
  }

  V3<T> Shade(const Hit<T> &h, const Ray<T> &r, V3<T> tp, int depth) {
    const Material<T> &m = s.materials[s.prims[h.prim].material];
    switch (s.integ) {
      case Integ::kNormals: return h.normal * static_cast<T>(0.5f) + V3<T>(0.5f);
      case Integ::kAlbedo: return m.diffuse + m.specular;
      case Integ::kDepth: return V3<T>(static_cast<T>(1.0f) / (static_cast<T>(1.0f) + h.distance));
      case Integ::kRaytracer: return ShadeRaytracer(h, r, tp, depth, m);
      case Integ::kAnalytic: return ShadeAnalytic(h, m);
      case Integ::kPath: return ShadePath(h, r, tp, depth, m);
    }
    return V3<T>(0);
  }

  V3<T> ShadeRaytracer(const Hit<T> &h, const Ray<T> &r, V3<T> tp, int depth, const Material<T> &m) {
    V3<T> color = m.ambient + m.emission;
    V3<T> shift = h.pos + Eps<T>() * h.normal;
    for (const Light<T> &l : s.lights) {
      ShadeInfo<T> info = ShadingInfoAt(l, h.pos);
      if (Occluded(s, Ray<T>{shift, info.direction}, info.distance, st)) continue;
      V3<T> dc = m.diffuse * Max(Dot(h.normal, info.direction), static_cast<T>(0));
      V3<T> half = Norm(info.direction - r.d);
      V3<T> sc = m.specular * std::pow(Max(Dot(h.normal, half), static_cast<T>(0)), m.shininess);
      color += info.color * (dc + sc);
    }
    if (m.specular.x > 0 || m.specular.y > 0 || m.specular.z > 0) {
      color += m.specular * Trace(Ray<T>{shift, Reflect(r.d, h.normal)}, tp, depth + 1);
    }
    return color;
  }

  V3<T> ShadeAnalytic(const Hit<T> &h, const Material<T> &m) {
    V3<T> color = m.emission;
    for (const Light<T> &l : s.lights) {
      ShadeInfo<T> info = ShadingInfoAt(l, h.pos);
      if (!info.area) continue;
      V3<T> vtx[4] = {l.a, l.a + l.b, l.a + l.b + l.c, l.a + l.c};
      V3<T> brdf = m.diffuse * InvPi<T>();
      V3<T> irr(0);
      for (int i = 0; i < 4; ++i) {
        V3<T> ui = Norm(vtx[i] - h.pos), un = Norm(vtx[(i + 1) % 4] - h.pos);
        T theta = std::acos(Dot(ui, un));
        irr += theta * Norm(Cross(ui, un));
      }
      irr *= static_cast<T>(0.5f);
      color += brdf * info.color * Dot(irr, h.normal);
    }
    return color;
  }

  bool SampleReflection(const Hit<T> &h, const Ray<T> &r, V3<T> tp, const Material<T> &m, V3<T> &dir, T &pdf, V3<T> &ntp) {
    if (s.is == 0) dir = SampleHemisphere(h.normal, rand);
    else if (s.is == 1) dir = SampleCosine(h.normal, rand);
    else dir = BrdfSample(m, r.d, h.normal, rand);
    if (Dot(dir, h.normal) <= 0) return false;
    V3<T> f = BrdfEval(m, dir, r.d, h.normal);
    pdf = IsPdf(dir, h, r, m);
    if (s.is == 0) ntp = tp * static_cast<T>(2.0f) * Pi<T>() * f * Max(Dot(h.normal, dir), static_cast<T>(0));
    else if (s.is == 1) ntp = tp * Pi<T>() * f;
    else ntp = tp * f / pdf * Max(Dot(h.normal, dir), static_cast<T>(0));
    return true;
  }

  T IsPdf(V3<T> dir, const Hit<T> &h, const Ray<T> &r, const Material<T> &m) {
    if (s.is == 0) return static_cast<T>(1.0f) / (static_cast<T>(2.0f) * Pi<T>());
    if (s.is == 1) return Max(Dot(h.normal, dir), static_cast<T>(0)) / Pi<T>();
    return BrdfPdf(m, dir, r.d, h.normal);
  }

  T NeePdf(const Ray<T> &r, V3<T> pos) {
    T pdf = 0;
    int affecting = 0;
    for (const Light<T> &l : s.lights) {
      ShadeInfo<T> info = ShadingInfoAt(l, pos);
      if (!info.area) continue;
      ++affecting;
      auto lh = QuadIntersect(l, r);
      if (!lh) continue;
      T area = Len(Cross(l.b, l.c));
      V3<T> rn = Norm(Cross(l.b, l.c));
      T denom = area * std::fabs(Dot(rn, r.d));
      if (denom == 0) continue;
      T d = Len(lh->pos - r.o);
      pdf += d * d / denom;
    }
    if (affecting == 0) return 0;
    return pdf / static_cast<T>(affecting);
  }

  V3<T> ShadePath(const Hit<T> &h, const Ray<T> &r, V3<T> tp, int depth, const Material<T> &m) {
    V3<T> shift = h.pos + Eps<T>() * h.normal;
    if (depth < s.min_depth) return Indirect(h, shift, r, tp, depth, m);
    V3<T> color;
    if ((s.nee != 0 && depth > 0) || Dot(h.normal, -r.d) < 0) color = V3<T>(0);
    else color = tp * m.emission;
    if (s.nee == 1) color += DirectNee(h, shift, r, tp, m, false);
    else if (s.nee == 2) color += DirectNee(h, shift, r, tp, m, true) + DirectIs(h, shift, r, tp, m);
    color += Indirect(h, shift, r, tp, depth, m);
    return color;
  }

  V3<T> Indirect(const Hit<T> &h, V3<T> shift, const Ray<T> &r, V3<T> tp, int depth, const Material<T> &m) {
    V3<T> dir, ntp;
    T pdf;
    if (!SampleReflection(h, r, tp, m, dir, pdf, ntp)) return V3<T>(0);
    if (s.rr) {
      T q = Min(CompMax(ntp), static_cast<T>(1.0f));
      if (q < rand.Next()) return V3<T>(0);
      ntp /= q;
    }
    return Trace(Ray<T>{shift, dir}, ntp, depth + 1);
  }

  V3<T> DirectNee(const Hit<T> &h, V3<T> shift, const Ray<T> &r, V3<T> tp, const Material<T> &m, bool mis) {
    V3<T> color(0);
    for (const Light<T> &l : s.lights) {
      ShadeInfo<T> info = ShadingInfoAt(l, h.pos);
      if (!info.area) {
        if (Occluded(s, Ray<T>{shift, info.direction}, info.distance, st)) continue;
        V3<T> irr = info.color;
        if (info.distance < std::numeric_limits<T>::infinity()) irr /= info.distance * info.distance;
        T ci = Max(Dot(h.normal, info.direction), static_cast<T>(0));
        color += irr * ci * BrdfEval(m, info.direction, r.d, h.normal);
        continue;
      }
      T area = Len(Cross(l.b, l.c));
      V3<T> rn = Norm(Cross(l.b, l.c));
      int strata = s.light_stratify ? static_cast<int>(std::sqrt(s.light_samples)) : 1;
      int per = s.light_stratify ? 1 : s.light_samples;
      V3<T> sum(0);
      for (int i = 0; i < strata; ++i)
        for (int j = 0; j < strata; ++j)
          for (int k = 0; k < per; ++k) {
            T u = rand.Next(), v = rand.Next();
            V3<T> lp = l.a + (i + u) / strata * l.b + (j + v) / strata * l.c;
            lp -= Eps<T>() * rn;
            V3<T> ptl = lp - shift;
            V3<T> ld = Norm(ptl);
            T dist = Len(ptl);
            Ray<T> sr{shift, ld};
            if (Occluded(s, sr, dist, st)) continue;
            T ci = Max(Dot(h.normal, ld), static_cast<T>(0));
            T cl = Max(Dot(rn, ld), static_cast<T>(0));
            T g = ci * cl / (dist * dist);
            V3<T> c = g * BrdfEval(m, ld, r.d, h.normal);
            if (mis) {
              T lpdf = NeePdf(sr, h.pos);
              T bpdf = IsPdf(ld, h, r, m);
              c *= PowerHeuristic(lpdf, bpdf);
            }
            sum += c;
          }
      sum *= area / s.light_samples;
      color += info.color * sum;
    }
    return tp * color;
  }

  V3<T> DirectIs(const Hit<T> &h, V3<T> shift, const Ray<T> &r, V3<T> tp, const Material<T> &m) {
    V3<T> dir, ntp;
    T bpdf;
    if (!SampleReflection(h, r, tp, m, dir, bpdf, ntp)) return V3<T>(0);
    Ray<T> sr{shift, dir};
    st.secondary++;
    auto nh = Intersect(s, sr, st);
    if (nh && s.prims[nh->prim].light >= 0) {
      const Light<T> &l = s.lights[s.prims[nh->prim].light];
      ShadeInfo<T> info = ShadingInfoAt(l, nh->pos);
      if (!info.area) return V3<T>(0);
      T w = PowerHeuristic(bpdf, NeePdf(sr, h.pos));
      return ntp * info.color * w;
    }
    return V3<T>(0);
  }
};

// ---------------------------------------------------------------- rendering
struct Tile {
  int x, y, w, h;
  unsigned int seed;
};

std::vector<Tile> MakeTiles(int w, int h, int spp, int parallelism, std::mt19937 &seedgen) {
  uint64_t total = static_cast<uint64_t>(w * h) * static_cast<uint64_t>(spp);
  int heuristic = static_cast<int>(total / (500 * 50 * 2));
  int num = std::min(std::max(heuristic, parallelism * 3), h);
  int th = h / num;
  int excess = h - th * num;
  std::vector<Tile> tiles;
  tiles.push_back({0, 0, w, th + excess, 0u});
  for (int i = 1; i < num; ++i) tiles.push_back({0, i * th + excess, w, th, static_cast<unsigned int>(seedgen())});
  return tiles;
}

template <class T>
struct RenderOut {
  std::vector<double> sum, sum_sq;
  std::vector<float> film32;  // the reference's FP32 accumulator, row-major
  Counters st;
};

template <class T>
void Render(Scene<T> &s, int parallelism, RenderOut<T> &out) {
  const int w = s.width, h = s.height, spp = s.pixel_samples;
  out.sum.assign(3 * static_cast<size_t>(w) * h, 0.0);
  out.sum_sq.assign(out.sum.size(), 0.0);
  out.film32.assign(out.sum.size(), 0.0f);
  std::vector<Tile> tiles = MakeTiles(w, h, spp, parallelism, s.seedgen);
  std::mutex mu;
  auto worker = [&]() {
    Tracer<T> tr(s, s.path_seed);
    while (true) {
      Tile t;
      {
        std::lock_guard<std::mutex> l(mu);
        if (tiles.empty()) break;
        t = tiles.back();
        tiles.pop_back();
      }
      UniformRandom srand(t.seed);
      for (int ty = 0; ty < t.h; ++ty)
        for (int tx = 0; tx < t.w; ++tx)
          for (int k = 0; k < spp; ++k) {
            float x, y;
            if (k == 0) {
              x = t.x + tx + 0.5f;
              y = t.y + ty + 0.5f;
            } else {
              float u = srand.Next(), v = srand.Next();
              x = t.x + tx + u;
              y = t.y + ty + v;
              if (x == (t.x + tx + 1.0f)) x = std::nextafter(x, -std::numeric_limits<float>::infinity());
              if (y == (t.y + ty + 1.0f)) y = std::nextafter(y, -std::numeric_limits<float>::infinity());
            }
            V3<T> c = tr.Trace(CastRay(s, static_cast<T>(x), static_cast<T>(y)), V3<T>(1.0f), 0);
            size_t p = static_cast<size_t>(static_cast<int>(y)) * w + static_cast<int>(x);
            for (int q = 0; q < 3; ++q) {
              double v = static_cast<double>(c[q]);
              out.sum[3 * p + q] += v;
              out.sum_sq[3 * p + q] += v * v;
              out.film32[3 * p + q] += static_cast<float>(c[q]);
            }
          }
    }
    std::lock_guard<std::mutex> l(mu);
    out.st.Add(tr.st);
  };
  if (parallelism <= 1) {
    worker();
  } else {
    std::vector<std::thread> th;
    for (int i = 0; i < parallelism; ++i) th.emplace_back(worker);
    for (auto &x : th) x.join();
  }
}

}  // namespace oracle

// ---------------------------------------------------------------- C entry points
namespace {
thread_local std::string g_err;

template <class T>
int LoadScene(const char *text, int linear, oracle::Scene<T> &s) {
  std::string err;
  int warnings = 0;
  if (!oracle::Parse<T>(text, s, &err, &warnings)) {
    g_err = err;
    return 5;
  }
  s.linear = linear != 0;
  oracle::InitAccel(s);
  return 0;
}
}  // namespace

extern "C" {

const char *oracle_last_error() { return g_err.c_str(); }

// Film size and settings of a scene text: out = {width, height, spp, integrator}.
int oracle_scene_info(const char *text, int32_t *out) {
  oracle::Scene<float> s;
  int rc = LoadScene(text, 1, s);
  if (rc) return rc;
  out[0] = s.width, out[1] = s.height, out[2] = s.pixel_samples, out[3] = static_cast<int32_t>(s.integ);
  return 0;
}

// Renders with the reference algorithm. spp > 0 overrides pixel_samples;
// seed >= 0 re-seeds the scene's seed generator (tiles and path tracer) as
// `random_seed <seed>` would. Outputs: sum, sum_sq (3*W*H doubles), film32
// (3*W*H floats, may be null), counters[8] (primary, secondary, object tests,
// object hits, bounds tests, bounds hits, build ns, render ns).
int oracle_render(const char *text, int precision_bits, int parallelism, int spp, long long seed, int linear,
                  double *sum, double *sum_sq, float *film32, uint64_t *counters) {
  auto run = [&](auto tag) -> int {
    using T = decltype(tag);
    oracle::Scene<T> s;
    // Build time (parse + acceleration structure) and render time are
    // measured apart, as the reference's Stats reports them
    // (muon/stats.cc:9-22, 41-55).
    const auto t0 = std::chrono::steady_clock::now();
    int rc = LoadScene(text, linear, s);
    if (rc) return rc;
    const auto t1 = std::chrono::steady_clock::now();
    if (seed >= 0) {
      s.seedgen.seed(static_cast<unsigned int>(seed));
      if (s.integ == oracle::Integ::kPath) s.path_seed = s.seedgen();
    }
    if (spp > 0) s.pixel_samples = spp;
    oracle::RenderOut<T> out;
    oracle::Render(s, parallelism, out);
    const auto t2 = std::chrono::steady_clock::now();
    std::memcpy(sum, out.sum.data(), out.sum.size() * sizeof(double));
    std::memcpy(sum_sq, out.sum_sq.data(), out.sum_sq.size() * sizeof(double));
    if (film32) std::memcpy(film32, out.film32.data(), out.film32.size() * sizeof(float));
    if (counters) {
      counters[0] = out.st.primary, counters[1] = out.st.secondary, counters[2] = out.st.obj_tests;
      counters[3] = out.st.obj_hits, counters[4] = out.st.bounds_tests, counters[5] = out.st.bounds_hits;
      counters[6] = static_cast<uint64_t>(std::chrono::duration_cast<std::chrono::nanoseconds>(t1 - t0).count());
      counters[7] = static_cast<uint64_t>(std::chrono::duration_cast<std::chrono::nanoseconds>(t2 - t1).count());
    }
    return 0;
  };
  return precision_bits == 64 ? run(double()) : run(float());
}

// A scene parsed and built once and rendered many times in float (for
// timing the reference algorithm on a large scene without re-parsing it per
// run). oracle_scene_render takes the same spp / seed overrides as
// oracle_render (seed < 0: the file's own seeds, restored every time) and
// fills sum, sum_sq (3*W*H doubles, may be null) and counters[8].
struct LoadedScene {
  oracle::Scene<float> s;
  std::mt19937 seedgen0;
  unsigned int path_seed0 = 0;
  int spp0 = 1;
};

void *oracle_scene_load(const char *text, int linear) {
  auto *h = new LoadedScene();
  if (LoadScene(text, linear, h->s)) {
    delete h;
    return nullptr;
  }
  h->seedgen0 = h->s.seedgen;
  h->path_seed0 = h->s.path_seed;
  h->spp0 = h->s.pixel_samples;
  return h;
}

int oracle_scene_render(void *handle, int parallelism, int spp, long long seed, double *sum, double *sum_sq,
                        uint64_t *counters) {
  auto *h = static_cast<LoadedScene *>(handle);
  if (!h) return 1;
  oracle::Scene<float> &s = h->s;
  s.seedgen = h->seedgen0;
  s.path_seed = h->path_seed0;
  if (seed >= 0) {
    s.seedgen.seed(static_cast<unsigned int>(seed));
    if (s.integ == oracle::Integ::kPath) s.path_seed = s.seedgen();
  }
  s.pixel_samples = spp > 0 ? spp : h->spp0;
  const auto t1 = std::chrono::steady_clock::now();
  oracle::RenderOut<float> out;
  oracle::Render(s, parallelism, out);
  const auto t2 = std::chrono::steady_clock::now();
  if (sum) std::memcpy(sum, out.sum.data(), out.sum.size() * sizeof(double));
  if (sum_sq) std::memcpy(sum_sq, out.sum_sq.data(), out.sum_sq.size() * sizeof(double));
  if (counters) {
    counters[0] = out.st.primary, counters[1] = out.st.secondary, counters[2] = out.st.obj_tests;
    counters[3] = out.st.obj_hits, counters[4] = out.st.bounds_tests, counters[5] = out.st.bounds_hits;
    counters[6] = 0;
    counters[7] = static_cast<uint64_t>(std::chrono::duration_cast<std::chrono::nanoseconds>(t2 - t1).count());
  }
  return 0;
}

void oracle_scene_free(void *handle) { delete static_cast<LoadedScene *>(handle); }

// Closest hits of caller-given rays (n x 6 floats) in float or double;
// out: n x 8 doubles (distance, prim id, position, normal), id -1 = miss.
int oracle_intersect(const char *text, int precision_bits, int linear, const float *rays, long long n,
                     double *out) {
  auto run = [&](auto tag) -> int {
    using T = decltype(tag);
    oracle::Scene<T> s;
    int rc = LoadScene(text, linear, s);
    if (rc) return rc;
    oracle::Counters st;
    for (long long i = 0; i < n; ++i) {
      const float *r = rays + 6 * i;
      oracle::Ray<T> ray{{r[0], r[1], r[2]}, {r[3], r[4], r[5]}};
      auto h = oracle::Intersect(s, ray, st);
      double *q = out + 8 * i;
      if (!h) {
        q[0] = std::numeric_limits<double>::infinity();
        q[1] = -1;
        for (int k = 2; k < 8; ++k) q[k] = 0;
        continue;
      }
      q[0] = h->distance;
      q[1] = h->prim;
      for (int k = 0; k < 3; ++k) q[2 + k] = h->pos[k], q[5 + k] = h->normal[k];
    }
    return 0;
  };
  return precision_bits == 64 ? run(double()) : run(float());
}

// The sample-0 camera rays of every pixel (row-major), n x 6 floats.
int oracle_camera_rays(const char *text, float *rays) {
  oracle::Scene<float> s;
  int rc = LoadScene(text, 1, s);
  if (rc) return rc;
  for (int y = 0; y < s.height; ++y)
    for (int x = 0; x < s.width; ++x) {
      oracle::Ray<float> r = oracle::CastRay(s, x + 0.5f, y + 0.5f);
      float *q = rays + 6 * (static_cast<size_t>(y) * s.width + x);
      q[0] = r.o.x, q[1] = r.o.y, q[2] = r.o.z, q[3] = r.d.x, q[4] = r.d.y, q[5] = r.d.z;
    }
  return 0;
}

}  // extern "C"

extern "C" {
// Film::WriteOutput's tone map (muon/film.cc:24-39) on an FP32 accumulator:
// mean over spp, powf(., 1/gamma), clamp to [0, 1], x255 truncated.
void oracle_tonemap(const float *film32, long long n, int spp, float gamma, uint8_t *out) {
  for (long long i = 0; i < n; ++i) {
    float v = film32[i] / static_cast<float>(spp);
    v = std::pow(v, 1.0f / gamma);
    v = oracle::Clamp(v, 0.0f, 1.0f);
    out[i] = static_cast<uint8_t>(v * 255);
  }
}
}
