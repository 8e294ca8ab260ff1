// Host walk of a scene's flattened BVH: the traversal work of a ray, counted
// the way the reference's TraceStats counts it (bounds tests and object
// tests, muon/stats.h:11-44, incremented in muon/acceleration.cc:65-202),
// on the arrays the GPU traverses and in the GPU kernels' visiting order
// (both child boxes of a node tested, nearer hit child first, farther one
// deferred on a stack; leaves tested record by record until the last). It is
// the independent measure of work behind a roofline's algorithmic bytes.
//
// Intersection follows the device code: the exact mode tests every
// primitive in its object space with the reference's operation order
// (muon/objects.cc:29-270, no contraction on the host either); the fast mode
// uses the world-space records. Box tests use fused multiply-adds as the
// device's contracted `lo * (1/d) - o/d` does.
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

#include "bvh_walk.h"

namespace muon_gpu {
namespace {

constexpr int kStack = 64;
constexpr float kEpsilon = 0.0001f;  // kEpsilon, muon/types.h:13

inline uint32_t Bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}
inline int32_t IntBits(float f) {
  int32_t i;
  std::memcpy(&i, &f, 4);
  return i;
}
inline float SafeInv(float x) {
  const float tiny = 1e-30f;
  return 1.0f / (std::fabs(x) > tiny ? x : std::copysign(tiny, x));
}
inline mm::v3 V(const F4 &v) { return mm::make3(v.x, v.y, v.z); }

// Rows 0..2 of M * (p, 1) and normalize(M * (d, 0)) for a packed affine
// matrix, in the reference library's column order.
mm::v3 XPoint(const float *m, mm::v3 p) {
  using namespace mm;
  return make3(add(add(mul(m[0], p.x), mul(m[3], p.y)), add(mul(m[6], p.z), m[9])),
               add(add(mul(m[1], p.x), mul(m[4], p.y)), add(mul(m[7], p.z), m[10])),
               add(add(mul(m[2], p.x), mul(m[5], p.y)), add(mul(m[8], p.z), m[11])));
}
mm::v3 XDir(const float *m, mm::v3 d) {
  using namespace mm;
  return normalize(make3(add(add(mul(m[0], d.x), mul(m[3], d.y)), mul(m[6], d.z)),
                         add(add(mul(m[1], d.x), mul(m[4], d.y)), mul(m[7], d.z)),
                         add(add(mul(m[2], d.x), mul(m[5], d.y)), mul(m[8], d.z))));
}

struct Ray {
  mm::v3 o, d, dn;  // dn: normalize(d), the exact mode's untransformed direction
  float idir[3], ood[3];
};

// Exact mode: object-space test; returns the world distance or -1.
float TestExact(const SceneImage &im, const Ray &r, const PrimRecord &p, uint32_t flags) {
  using namespace mm;
  const int xf = IntBits((flags & kPrimSphere) ? p.p1.y : p.p1.w);
  v3 o = r.o, d = r.dn;
  if (xf >= 0) {
    o = XPoint(im.transforms[xf].w2o, r.o);
    d = XDir(im.transforms[xf].w2o, r.d);
  }
  float t;
  if (flags & kPrimSphere) {
    v3 dc = o - V(p.p0);
    float b = dot(d, dc);
    float c = sub(dot(dc, dc), mul(p.p0.w, p.p0.w));
    float disc = sub(mul(b, b), c);
    if (disc < 0.0f) return -1.0f;
    float sq = fsqrt(disc);
    float r0 = add(-b, sq), r1 = sub(-b, sq);
    if (r0 < 0.0f && r1 < 0.0f) return -1.0f;
    t = fmin_ref(r0, r1);
    if (t < 0.0f) t = fmax_ref(r0, r1);
  } else {
    v3 n = V(p.p3);
    float dn = dot(n, d);
    if (dn > -kEpsilon && dn < kEpsilon) return -1.0f;
    v3 a = V(p.p0), b = V(p.p1), c = V(p.p2);
    t = div(sub(dot(a, n), dot(o, n)), dn);
    if (t < 0.0f) return -1.0f;
    v3 q = o + d * t;
    if (dot(n, cross(b - a, q - a)) < 0.0f) return -1.0f;
    if (dot(n, cross(c - b, q - b)) < 0.0f) return -1.0f;
    if (dot(n, cross(a - c, q - c)) < 0.0f) return -1.0f;
  }
  v3 q = o + d * t;
  v3 w = xf < 0 ? q : XPoint(im.transforms[xf].o2w, q);
  return length(w - r.o);
}

// Fast mode: world-space triangle (plane + edge functions) and sphere tests.
float TestFast(const SceneImage &im, const Ray &r, const PrimRecord &p, uint32_t flags) {
  using namespace mm;
  if (flags & kPrimSphere) {
    const int xf = IntBits(p.p1.y);
    v3 o = r.o, d = r.d;
    if (xf >= 0) {
      o = XPoint(im.transforms[xf].w2o, r.o);
      d = XDir(im.transforms[xf].w2o, r.d);
    }
    v3 oc = o - V(p.p0);
    float b = dot(d, oc);
    float cc = dot(oc, oc) - p.p0.w * p.p0.w;
    float disc = b * b - cc;
    if (disc < 0.0f) return -1.0f;
    float sq = std::sqrt(disc);
    float r0 = -b + sq, r1 = -b - sq;
    if (r0 < 0.0f && r1 < 0.0f) return -1.0f;
    float t = std::fmin(r0, r1);
    if (t < 0.0f) t = std::fmax(r0, r1);
    if (xf >= 0) t = length(XPoint(im.transforms[xf].o2w, o + d * t) - r.o);
    return t > 0.0f ? t : -1.0f;
  }
  v3 n = V(p.p3);
  float dn = dot(n, r.d);
  const float eps = p.p1.w;
  if (dn > -eps && dn < eps) return -1.0f;
  float t = (p.p0.w - dot(r.o, n)) / dn;
  if (!(t > 0.0f)) return -1.0f;
  v3 a = V(p.p0), b = V(p.p1), c = V(p.p2);
  v3 q = r.o + r.d * t;
  if (dot(n, cross(b - a, q - a)) < 0.0f) return -1.0f;
  if (dot(n, cross(c - b, q - b)) < 0.0f) return -1.0f;
  if (dot(n, cross(a - c, q - c)) < 0.0f) return -1.0f;
  return t;
}

}  // namespace

int WalkRay(const SceneImage &im, const float o[3], const float d[3], float tmax, int root, bool any_hit, int mode,
            MuonWalkCounts *cnt) {
  cnt->rays += 1;
  if (im.nodes.empty()) return -1;
  Ray r;
  r.o = mm::make3(o[0], o[1], o[2]);
  r.d = mm::make3(d[0], d[1], d[2]);
  r.dn = mm::normalize(r.d);
  for (int k = 0; k < 3; ++k) {
    r.idir[k] = SafeInv(d[k]);
    r.ood[k] = o[k] * r.idir[k];
  }
  const std::vector<PrimRecord> &recs = mode == MUON_ISECT_EXACT ? im.prims_obj : im.prims;
  int stack[kStack];
  int sp = 0, node = root, hit = -1;
  auto slab = [&](float lo, float hi, int k, float *tn, float *tf) {
    const float a = std::fmaf(lo, r.idir[k], -r.ood[k]), b = std::fmaf(hi, r.idir[k], -r.ood[k]);
    *tn = std::fmin(a, b);
    *tf = std::fmax(a, b);
  };
  while (true) {
    while (node >= 0) {
      const BvhNode &n = im.nodes[node];
      float x0n, x0f, y0n, y0f, z0n, z0f, x1n, x1f, y1n, y1f, z1n, z1f;
      slab(n.a.x, n.a.y, 0, &x0n, &x0f);
      slab(n.a.z, n.a.w, 1, &y0n, &y0f);
      slab(n.c.x, n.c.y, 2, &z0n, &z0f);
      slab(n.b.x, n.b.y, 0, &x1n, &x1f);
      slab(n.b.z, n.b.w, 1, &y1n, &y1f);
      slab(n.c.z, n.c.w, 2, &z1n, &z1f);
      const float c0min = std::fmax(std::fmax(x0n, y0n), std::fmax(z0n, 0.0f));
      const float c0max = std::fmin(std::fmin(x0f, y0f), std::fmin(z0f, tmax));
      const float c1min = std::fmax(std::fmax(x1n, y1n), std::fmax(z1n, 0.0f));
      const float c1max = std::fmin(std::fmin(x1f, y1f), std::fmin(z1f, tmax));
      const bool h0 = c0min <= c0max, h1 = c1min <= c1max;
      cnt->box_tests += 2;
      if (!h0 && !h1) {
        if (sp == 0) {
          node = kEmptyLink;
          break;
        }
        node = stack[--sp];
      } else {
        int near_child = h0 ? n.d.x : n.d.y;
        if (h0 && h1) {
          int far_child = n.d.y;
          if (c1min < c0min) {
            near_child = n.d.y;
            far_child = n.d.x;
          }
          if (sp < kStack) stack[sp++] = far_child;
        }
        node = near_child;
      }
    }
    if (node == kEmptyLink) break;
    for (int i = ~node;; ++i) {
      const PrimRecord &p = recs[i];
      const uint32_t flags = Bits(p.p3.w);
      const float t = mode == MUON_ISECT_EXACT ? TestExact(im, r, p, flags) : TestFast(im, r, p, flags);
      cnt->prim_tests += 1;
      if (t > 0.0f && t < tmax) {
        tmax = t;
        hit = i;
        if (any_hit) {
          cnt->hits += 1;
          return hit;
        }
      }
      if (flags & kPrimLast) break;
    }
    if (sp == 0) break;
    node = stack[--sp];
  }
  if (hit >= 0) cnt->hits += 1;
  return hit;
}

void WalkMany(const SceneImage &im, const WalkRayIn *rays, int64_t n, bool any_hit, int mode, int32_t *hit_slots,
              MuonWalkCounts *total) {
  const int threads = static_cast<int>(std::max<int64_t>(
      1, std::min<int64_t>(std::max(1u, std::thread::hardware_concurrency()), (n + 1023) / 1024)));
  std::vector<MuonWalkCounts> part(threads, MuonWalkCounts{0, 0, 0, 0});
  auto work = [&](int t) {
    for (int64_t i = t; i < n; i += threads) {
      const WalkRayIn &r = rays[i];
      const int h = WalkRay(im, r.o, r.d, r.tmax, r.root, any_hit, mode, &part[t]);
      if (hit_slots) hit_slots[i] = h;
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back(work, t);
  work(0);
  for (std::thread &th : pool) th.join();
  for (const MuonWalkCounts &c : part) {
    total->rays += c.rays;
    total->box_tests += c.box_tests;
    total->prim_tests += c.prim_tests;
    total->hits += c.hits;
  }
}

}  // namespace muon_gpu

using namespace muon_gpu;

extern "C" int muon_walk_rays(const MuonSceneDesc *desc, const MuonRay *rays, const float *tmax, int64_t n,
                              int32_t any_hit, int32_t intersect_mode, int32_t *hit_ids, MuonWalkCounts *out) {
  if (!desc || !out || n < 0 || (n > 0 && !rays)) return WalkFail(MUON_ERR_INVALID_ARG, "bad argument");
  if (intersect_mode != MUON_ISECT_EXACT && intersect_mode != MUON_ISECT_FAST)
    return WalkFail(MUON_ERR_INVALID_ARG, "the host walk supports the exact and fast intersection modes");
  *out = MuonWalkCounts{0, 0, 0, 0};
  try {
    SceneImage im;
    std::string err;
    if (!BuildSceneImage(*desc, &im, &err, false)) return WalkFail(MUON_ERR_INVALID_ARG, err);
    std::vector<WalkRayIn> in(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) {
      for (int k = 0; k < 3; ++k) in[i].o[k] = rays[i].origin[k], in[i].d[k] = rays[i].direction[k];
      in[i].tmax = tmax ? tmax[i] : std::numeric_limits<float>::infinity();
      in[i].root = 0;
    }
    std::vector<int32_t> slots(static_cast<size_t>(n), -1);
    WalkMany(im, in.data(), n, any_hit != 0, intersect_mode, slots.data(), out);
    if (hit_ids)
      for (int64_t i = 0; i < n; ++i) hit_ids[i] = slots[i] < 0 ? -1 : im.shade[slots[i]].s1.y;
  } catch (const std::bad_alloc &) {
    return WalkFail(MUON_ERR_OOM, "host allocation failed");
  }
  return MUON_OK;
}
