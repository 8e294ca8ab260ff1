// Ray/primitive tests and BVH traversal (closest hit and any hit).
//
// Replaces BVH::Intersect / BVH::HasIntersection (muon/acceleration.cc:65-202)
// and the primitive tests they call (muon/objects.cc:29-270). Acceptance
// follows the reference: a primitive hit counts when 0 < distance < limit
// (muon/acceleration.cc:120-124, muon/objects.cc:9-17).
#pragma once

#include "dev_common.cuh"

namespace muon_gpu {

constexpr int kStackSize = 64;

// Exact mode: keep the ray in the object space of the last transform a
// primitive test used, so that the primitives of one transformed mesh (which
// share their transform) do not each load the transform and re-transform the
// ray. The values are the ones the test would compute, so hits are unchanged.
// Off by default: within the 64 registers of four resident traversal blocks
// per SM its six registers spill, and the dense mesh ran 1.5% slower with it.
#ifndef MUON_XF_CACHE
#define MUON_XF_CACHE 0
#endif

struct RayPre {
  float3 o, d, idir, ood;
  // watertight-test shear
  int kx, ky, kz;
  float sx, sy, sz;
  // exact mode: the direction as the reference carries it into the object
  // space of an untransformed primitive, normalize(I * (d, 0))
  mm::v3 dn;
  // exact mode: transform index of the cached object-space ray (co, cd)
  int cxf;
  mm::v3 co, cd;
};

// Three-input min / max of the slab test as single instructions (same
// values: no operand is NaN, SafeInv keeps 1/d finite).
#ifndef MUON_MINMAX3
#define MUON_MINMAX3 1
#endif
__device__ __forceinline__ float Max3(float a, float b, float c) {
#if MUON_MINMAX3
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
#else
  return fmaxf(fmaxf(a, b), c);
#endif
}
__device__ __forceinline__ float Min3(float a, float b, float c) {
#if MUON_MINMAX3
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
#else
  return fminf(fminf(a, b), c);
#endif
}

// BVH nodes and primitive records (64 bytes, 64-byte aligned) read with two
// 256-bit loads instead of four 128-bit ones: half the load requests to L1.
#ifndef MUON_LD256
#define MUON_LD256 1
#endif
__device__ __forceinline__ void Load64B(const void *p, float4 &a, float4 &b, float4 &c, float4 &d) {
#if MUON_LD256
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(c.x), "=f"(c.y), "=f"(c.z), "=f"(c.w), "=f"(d.x), "=f"(d.y), "=f"(d.z), "=f"(d.w)
      : "l"(static_cast<const char *>(p) + 32));
#else
  const float4 *q = static_cast<const float4 *>(p);
  a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), d = __ldg(q + 3);
#endif
}

__device__ __forceinline__ float SafeInv(float x) {
  const float tiny = 1e-30f;
  return 1.0f / (fabsf(x) > tiny ? x : copysignf(tiny, x));
}

template <int kTriTest>
__device__ __forceinline__ RayPre Prepare(float3 o, float3 d) {
  RayPre r;
  r.o = o;
  r.d = d;
  r.idir = f3(SafeInv(d.x), SafeInv(d.y), SafeInv(d.z));
  r.ood = o * r.idir;
  if (kTriTest == MUON_ISECT_WATERTIGHT) {
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    r.kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    r.kx = r.kz == 2 ? 0 : r.kz + 1;
    r.ky = r.kx == 2 ? 0 : r.kx + 1;
    float dz = r.kz == 0 ? d.x : (r.kz == 1 ? d.y : d.z);
    if (dz < 0.0f) {
      int t = r.kx;
      r.kx = r.ky;
      r.ky = t;
    }
    float dx = r.kx == 0 ? d.x : (r.kx == 1 ? d.y : d.z);
    float dy = r.ky == 0 ? d.x : (r.ky == 1 ? d.y : d.z);
    r.sx = dx / dz;
    r.sy = dy / dz;
    r.sz = 1.0f / dz;
  }
  if (kTriTest == MUON_ISECT_EXACT) {
    r.dn = mm::normalize(mm::make3(d.x, d.y, d.z));
    r.cxf = -1;  // nothing cached (-1 is the identity, which needs no cache)
  }
  return r;
}

__device__ __forceinline__ float comp3(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// The reference's triangle test (muon/objects.cc:103-158) on world-space
// vertices: plane distance with the unnormalised normal, parallel rejection
// against the per-triangle threshold, then three edge functions >= 0.
__device__ __forceinline__ float TriReference(const RayPre &r, const PrimRecord &p) {
  float3 n = f3(p.p3);
  float dn = dot3(n, r.d);
  float eps = p.p1.w;
  if (dn > -eps && dn < eps) return -1.0f;
  float t = (p.p0.w - dot3(r.o, n)) / dn;
  if (!(t > 0.0f)) return -1.0f;
  float3 a = f3(p.p0), b = f3(p.p1), c = f3(p.p2);
  float3 q = r.o + r.d * t;
  if (dot3(n, cross3(b - a, q - a)) < 0.0f) return -1.0f;
  if (dot3(n, cross3(c - b, q - b)) < 0.0f) return -1.0f;
  if (dot3(n, cross3(a - c, q - c)) < 0.0f) return -1.0f;
  return t;
}

// Watertight ray/triangle test (Woop, Benthin, Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013); both faces count.
__device__ __forceinline__ float TriWatertight(const RayPre &r, const PrimRecord &p) {
  float3 A = f3(p.p0) - r.o, B = f3(p.p1) - r.o, C = f3(p.p2) - r.o;
  float az = comp3(A, r.kz), bz = comp3(B, r.kz), cz = comp3(C, r.kz);
  float ax = comp3(A, r.kx) - r.sx * az, ay = comp3(A, r.ky) - r.sy * az;
  float bx = comp3(B, r.kx) - r.sx * bz, by = comp3(B, r.ky) - r.sy * bz;
  float cx = comp3(C, r.kx) - r.sx * cz, cy = comp3(C, r.ky) - r.sy * cz;
  float U = cx * by - cy * bx;
  float V = ax * cy - ay * cx;
  float W = bx * ay - by * ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    double cxby = (double)cx * by, cybx = (double)cy * bx;
    U = (float)(cxby - cybx);
    double axcy = (double)ax * cy, aycx = (double)ay * cx;
    V = (float)(axcy - aycx);
    double bxay = (double)bx * ay, byax = (double)by * ax;
    W = (float)(bxay - byax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return -1.0f;
  float det = U + V + W;
  if (det == 0.0f) return -1.0f;
  float T = U * (r.sz * az) + V * (r.sz * bz) + W * (r.sz * cz);
  float t = T / det;
  return t > 0.0f ? t : -1.0f;
}

// Sphere test (muon/objects.cc:195-270). Identity-transform spheres are
// tested in world space; others in object space with the ray carried by the
// inverse transform and the direction re-normalised (muon/transform.h:13-18),
// the distance measured back in world space (muon/objects.cc:39-43).
__device__ __forceinline__ float SphereTest(const DevScene &s, const RayPre &r, const PrimRecord &p) {
  int xf = __float_as_int(p.p1.y);
  float3 c = f3(p.p0);
  float rad = p.p0.w;
  float3 o = r.o, d = r.d;
  if (xf >= 0) {
    const DevTransform &T = s.transforms[xf];
    o = xform_point3(T.w2o, r.o);
    d = normalize3(xform_vec3(T.w2o, r.d));
  }
  float3 oc = o - c;
  float b = dot3(d, oc);
  float cc = dot3(oc, oc) - rad * rad;
  float disc = b * b - cc;
  if (disc < 0.0f) return -1.0f;
  float sq = sqrtf(disc);
  float r0 = -b + sq, r1 = -b - sq;
  if (r0 < 0.0f && r1 < 0.0f) return -1.0f;
  float t = fminf(r0, r1);
  if (t < 0.0f) t = fmaxf(r0, r1);
  if (xf >= 0) {
    float3 pw = xform_point3(s.transforms[xf].o2w, o + d * t);
    t = length3(pw - r.o);
  }
  return t > 0.0f ? t : -1.0f;
}

// ---- exact mode: the reference's arithmetic, no contraction --------------
// Rows 0..2 of M * (p, 1) and of M * (d, 0) for a packed affine matrix, in
// the reference library's column order ((c0 x + c1 y) + (c2 z + c3 w)).
__device__ __forceinline__ mm::v3 XPointExact(const float *m, mm::v3 p) {
  using namespace mm;
  return make3(add(add(mul(m[0], p.x), mul(m[3], p.y)), add(mul(m[6], p.z), m[9])),
               add(add(mul(m[1], p.x), mul(m[4], p.y)), add(mul(m[7], p.z), m[10])),
               add(add(mul(m[2], p.x), mul(m[5], p.y)), add(mul(m[8], p.z), m[11])));
}
__device__ __forceinline__ mm::v3 XDirExact(const float *m, mm::v3 d) {
  using namespace mm;
  return normalize(make3(add(add(mul(m[0], d.x), mul(m[3], d.y)), mul(m[6], d.z)),
                         add(add(mul(m[1], d.x), mul(m[4], d.y)), mul(m[7], d.z)),
                         add(add(mul(m[2], d.x), mul(m[5], d.y)), mul(m[8], d.z))));
}
__device__ __forceinline__ mm::v3 V(const F4 &v) { return mm::make3(v.x, v.y, v.z); }
__device__ __forceinline__ mm::v3 V(float3 v) { return mm::make3(v.x, v.y, v.z); }

// The ray in a primitive's object space (Ray::Transform, muon/camera.cc:7-11).
__device__ __forceinline__ void ObjectRay(const DevScene &s, RayPre &r, int xf, mm::v3 *o, mm::v3 *d) {
  if (xf < 0) {
    *o = V(r.o);
    *d = r.dn;
  } else if (MUON_XF_CACHE == 1 && xf == r.cxf) {
    *o = r.co;
    *d = r.cd;
  } else if (MUON_XF_CACHE == 2 && xf == r.cxf) {
    // direction only (the normalisation is the costly part); the origin is
    // carried again
    *o = XPointExact(s.transforms[xf].w2o, V(r.o));
    *d = r.cd;
  } else {
    const DevTransform &T = s.transforms[xf];
    *o = XPointExact(T.w2o, V(r.o));
    *d = XDirExact(T.w2o, V(r.d));
    if (MUON_XF_CACHE) {
      r.cxf = xf;
      if (MUON_XF_CACHE == 1) r.co = *o;
      r.cd = *d;
    }
  }
}

// Object-space test with the reference's operations; returns the world
// distance |M p - o| (muon/objects.cc:38-43) or -1, and the object-space t.
__device__ __forceinline__ float PrimTestExact(const DevScene &s, RayPre &r, const PrimRecord &p, uint32_t flags,
                                               float *t_obj) {
  using namespace mm;
  const int xf = __float_as_int((flags & kPrimSphere) ? p.p1.y : p.p1.w);
  v3 o, d;
  ObjectRay(s, r, xf, &o, &d);
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
    if (dn > -kEps && dn < kEps) return -1.0f;
    v3 a = V(p.p0), b = V(p.p1), c = V(p.p2);
    t = div(sub(dot(a, n), dot(o, n)), dn);
    if (t < 0.0f) return -1.0f;
    v3 q = o + d * t;
    if (dot(n, cross(b - a, q - a)) < 0.0f) return -1.0f;
    if (dot(n, cross(c - b, q - b)) < 0.0f) return -1.0f;
    if (dot(n, cross(a - c, q - c)) < 0.0f) return -1.0f;
  }
  *t_obj = t;
  v3 q = o + d * t;
  v3 w = xf < 0 ? q : XPointExact(s.transforms[xf].o2w, q);
  return length(w - V(r.o));
}

template <int kTriTest>
__device__ __forceinline__ float PrimTest(const DevScene &s, RayPre &r, const PrimRecord &p, uint32_t flags,
                                          float *t_obj) {
  if (kTriTest == MUON_ISECT_EXACT) return PrimTestExact(s, r, p, flags, t_obj);
  if (flags & kPrimSphere) return SphereTest(s, r, p);
  return kTriTest == MUON_ISECT_WATERTIGHT ? TriWatertight(r, p) : TriReference(r, p);
}

__device__ __forceinline__ PrimRecord LoadPrim(const PrimRecord *prims, int i) {
  float4 a, b, c, d;
  Load64B(prims + i, a, b, c, d);
  PrimRecord p;
  p.p0 = F4{a.x, a.y, a.z, a.w};
  p.p1 = F4{b.x, b.y, b.z, b.w};
  p.p2 = F4{c.x, c.y, c.z, c.w};
  p.p3 = F4{d.x, d.y, d.z, d.w};
  return p;
}

struct TraceCounters {
  uint32_t box_tests = 0, box_hits = 0, prim_tests = 0, prim_hits = 0;
};

// Closest hit (kAnyHit = false) or first hit (kAnyHit = true) with
// 0 < t < tmax. Returns the leaf slot of the primitive hit, or -1; *t_hit
// receives its distance. A stack overflow sets *overflow.
template <bool kAnyHit, bool kStats, int kTriTest>
__device__ __forceinline__ int Trace(const DevScene &s, float3 o, float3 d, float tmax, float *t_hit,
                                     TraceCounters *cnt, bool *overflow, float *t_obj_hit = nullptr) {
  int hit = -1;
  if (s.num_nodes == 0) return -1;
  RayPre r = Prepare<kTriTest>(o, d);
  int stack[kStackSize];
  int sp = 0;
  int node = 0;
  while (true) {
    // Interior nodes: test both child boxes, descend into the nearer hit child
    // and defer the farther one.
    while (node >= 0) {
      float4 n0, n1, n2, n3f;
      Load64B(s.nodes + node, n0, n1, n2, n3f);
      const int4 n3 = make_int4(__float_as_int(n3f.x), __float_as_int(n3f.y), 0, 0);
      float c0lox = n0.x * r.idir.x - r.ood.x, c0hix = n0.y * r.idir.x - r.ood.x;
      float c0loy = n0.z * r.idir.y - r.ood.y, c0hiy = n0.w * r.idir.y - r.ood.y;
      float c0loz = n2.x * r.idir.z - r.ood.z, c0hiz = n2.y * r.idir.z - r.ood.z;
      float c1lox = n1.x * r.idir.x - r.ood.x, c1hix = n1.y * r.idir.x - r.ood.x;
      float c1loy = n1.z * r.idir.y - r.ood.y, c1hiy = n1.w * r.idir.y - r.ood.y;
      float c1loz = n2.z * r.idir.z - r.ood.z, c1hiz = n2.w * r.idir.z - r.ood.z;
      float c0min = Max3(fminf(c0lox, c0hix), fminf(c0loy, c0hiy), fmaxf(fminf(c0loz, c0hiz), 0.0f));
      float c0max = Min3(fmaxf(c0lox, c0hix), fmaxf(c0loy, c0hiy), fminf(fmaxf(c0loz, c0hiz), tmax));
      float c1min = Max3(fminf(c1lox, c1hix), fminf(c1loy, c1hiy), fmaxf(fminf(c1loz, c1hiz), 0.0f));
      float c1max = Min3(fmaxf(c1lox, c1hix), fmaxf(c1loy, c1hiy), fminf(fmaxf(c1loz, c1hiz), tmax));
      bool h0 = c0min <= c0max, h1 = c1min <= c1max;
      if (kStats) {
        cnt->box_tests += 2;
        cnt->box_hits += (int)h0 + (int)h1;
      }
      if (!h0 && !h1) {
        if (sp == 0) {
          node = kEmptyLink;
          break;
        }
        node = stack[--sp];
      } else {
        int near = h0 ? n3.x : n3.y;
        if (h0 && h1) {
          int far = n3.y;
          if (c1min < c0min) {
            near = n3.y;
            far = n3.x;
          }
          if (sp < kStackSize) {
            stack[sp++] = far;
          } else {
            *overflow = true;
          }
        }
        node = near;
      }
    }
    if (node == kEmptyLink) break;
    // Leaf: test its primitives until the record flagged as last.
    int i = ~node;
    const PrimRecord *recs = kTriTest == MUON_ISECT_EXACT ? s.prims_obj : s.prims;
    while (true) {
      PrimRecord p = LoadPrim(recs, i);
      uint32_t flags = __float_as_uint(p.p3.w);
      float t_obj = 0.0f;
      float t = PrimTest<kTriTest>(s, r, p, flags, &t_obj);
      if (kStats) cnt->prim_tests += 1;
      if (t > 0.0f && t < tmax) {
        if (kStats) cnt->prim_hits += 1;
        tmax = t;
        hit = i;
        if (kTriTest == MUON_ISECT_EXACT && t_obj_hit) *t_obj_hit = t_obj;
        if (kAnyHit) {
          *t_hit = t;
          return hit;
        }
      }
      if (flags & kPrimLast) break;
      ++i;
    }
    if (sp == 0) break;
    node = stack[--sp];
  }
  *t_hit = tmax;
  return hit;
}

// ---- resumable traversal for persistent kernels ---------------------------
// The top kShortStack entries of a traversal stack live in shared memory
// (a column of `stride` ints per thread, slot-major so a warp's accesses hit
// distinct banks), as a ring over the stack positions; deeper entries spill
// to local memory. 0 keeps the whole stack in local memory.
#ifndef MUON_SHORT_STACK
#define MUON_SHORT_STACK 8
#endif
constexpr int kShortStack = MUON_SHORT_STACK;
static_assert((kShortStack & (kShortStack - 1)) == 0, "short stack size must be a power of two");

// The state of one ray's traversal, kept across the refill points of a
// persistent kernel.
struct TravState {
  int node, sp, hit;
  float tmax, t_obj;
  int *sh;      // this thread's shared-memory column (short stack) or null
  int stride;   // ints between consecutive slots of the column
  int stack[kStackSize - kShortStack];
};

__device__ __forceinline__ void StackPush(TravState &t, int v) {
  if (kShortStack == 0) {
    t.stack[t.sp++] = v;
    return;
  }
  int *slot = t.sh + (t.sp & (kShortStack - 1)) * t.stride;
  if (t.sp >= kShortStack) t.stack[t.sp - kShortStack] = *slot;  // spill the entry the ring overwrites
  *slot = v;
  ++t.sp;
}

__device__ __forceinline__ int StackPop(TravState &t) {
  --t.sp;
  if (kShortStack == 0) return t.stack[t.sp];
  int *slot = t.sh + (t.sp & (kShortStack - 1)) * t.stride;
  const int v = *slot;
  if (t.sp >= kShortStack) *slot = t.stack[t.sp - kShortStack];  // refill the ring from the spill
  return v;
}

__device__ __forceinline__ void TravBegin(TravState &t, float tmax, int root) {
  t.node = root;
  t.sp = 0;
  t.hit = -1;
  t.tmax = tmax;
  t.t_obj = 0.0f;
}

// Advances a traversal (same visiting order and acceptance as Trace). Returns
// true when the ray is finished; returns false, with the state kept, when
// fewer than `min_active` lanes of the warp are still traversing, so that the
// finished lanes can take new rays.
template <bool kAnyHit, bool kStats, int kTriTest>
__device__ __forceinline__ bool TravRun(const DevScene &s, RayPre &r, TravState &t, TraceCounters *cnt,
                                        bool *overflow, int min_active) {
  if (s.num_nodes == 0) return true;
  while (true) {
    while (t.node >= 0) {
      float4 n0, n1, n2, n3f;
      Load64B(s.nodes + t.node, n0, n1, n2, n3f);
      const int4 n3 = make_int4(__float_as_int(n3f.x), __float_as_int(n3f.y), 0, 0);
      float c0lox = n0.x * r.idir.x - r.ood.x, c0hix = n0.y * r.idir.x - r.ood.x;
      float c0loy = n0.z * r.idir.y - r.ood.y, c0hiy = n0.w * r.idir.y - r.ood.y;
      float c0loz = n2.x * r.idir.z - r.ood.z, c0hiz = n2.y * r.idir.z - r.ood.z;
      float c1lox = n1.x * r.idir.x - r.ood.x, c1hix = n1.y * r.idir.x - r.ood.x;
      float c1loy = n1.z * r.idir.y - r.ood.y, c1hiy = n1.w * r.idir.y - r.ood.y;
      float c1loz = n2.z * r.idir.z - r.ood.z, c1hiz = n2.w * r.idir.z - r.ood.z;
      float c0min = Max3(fminf(c0lox, c0hix), fminf(c0loy, c0hiy), fmaxf(fminf(c0loz, c0hiz), 0.0f));
      float c0max = Min3(fmaxf(c0lox, c0hix), fmaxf(c0loy, c0hiy), fminf(fmaxf(c0loz, c0hiz), t.tmax));
      float c1min = Max3(fminf(c1lox, c1hix), fminf(c1loy, c1hiy), fmaxf(fminf(c1loz, c1hiz), 0.0f));
      float c1max = Min3(fmaxf(c1lox, c1hix), fmaxf(c1loy, c1hiy), fminf(fmaxf(c1loz, c1hiz), t.tmax));
      bool h0 = c0min <= c0max, h1 = c1min <= c1max;
      if (kStats) {
        cnt->box_tests += 2;
        cnt->box_hits += (int)h0 + (int)h1;
      }
      if (!h0 && !h1) {
        if (t.sp == 0) {
          t.node = kEmptyLink;
          break;
        }
        t.node = StackPop(t);
      } else {
        int near = h0 ? n3.x : n3.y;
        if (h0 && h1) {
          int far = n3.y;
          if (c1min < c0min) {
            near = n3.y;
            far = n3.x;
          }
          if (t.sp < kStackSize) StackPush(t, far);
          else *overflow = true;
        }
        t.node = near;
      }
    }
    if (t.node == kEmptyLink) return true;
    int i = ~t.node;
    const PrimRecord *recs = kTriTest == MUON_ISECT_EXACT ? s.prims_obj : s.prims;
    while (true) {
      PrimRecord p = LoadPrim(recs, i);
      uint32_t flags = __float_as_uint(p.p3.w);
      float t_obj = 0.0f;
      float d = PrimTest<kTriTest>(s, r, p, flags, &t_obj);
      if (kStats) cnt->prim_tests += 1;
      if (d > 0.0f && d < t.tmax) {
        if (kStats) cnt->prim_hits += 1;
        t.tmax = d;
        t.hit = i;
        t.t_obj = t_obj;
        if (kAnyHit) return true;
      }
      if (flags & kPrimLast) break;
      ++i;
    }
    if (t.sp == 0) return true;
    t.node = StackPop(t);
    if (__popc(__activemask()) < min_active) return false;
  }
}

// Speculative variant of TravRun (Aila and Laine, HPG 2009, "while-while"
// with postponed leaves): a lane that reaches a leaf keeps it aside and
// descends further from its stack until every lane still descending holds a
// leaf, so that the warp tests leaves together instead of serialising inner
// nodes of some lanes against leaves of others. Every leaf reached is tested;
// only the order changes (exact-distance ties may resolve differently).
#ifndef MUON_SPECULATIVE
#define MUON_SPECULATIVE 1
#endif
template <bool kAnyHit, bool kStats, int kTriTest>
__device__ __forceinline__ bool TravRunSpeculative(const DevScene &s, RayPre &r, TravState &t, TraceCounters *cnt,
                                                   bool *overflow, int min_active) {
  if (s.num_nodes == 0) return true;
  auto next = [&] { t.node = t.sp == 0 ? kEmptyLink : StackPop(t); };
  const PrimRecord *recs = kTriTest == MUON_ISECT_EXACT ? s.prims_obj : s.prims;
  while (true) {
    int leaf = 0;  // postponed leaf link (leaf links are negative; 0 = none)
    while (t.node >= 0) {
      float4 n0, n1, n2, n3f;
      Load64B(s.nodes + t.node, n0, n1, n2, n3f);
      const int4 n3 = make_int4(__float_as_int(n3f.x), __float_as_int(n3f.y), 0, 0);
      float c0lox = n0.x * r.idir.x - r.ood.x, c0hix = n0.y * r.idir.x - r.ood.x;
      float c0loy = n0.z * r.idir.y - r.ood.y, c0hiy = n0.w * r.idir.y - r.ood.y;
      float c0loz = n2.x * r.idir.z - r.ood.z, c0hiz = n2.y * r.idir.z - r.ood.z;
      float c1lox = n1.x * r.idir.x - r.ood.x, c1hix = n1.y * r.idir.x - r.ood.x;
      float c1loy = n1.z * r.idir.y - r.ood.y, c1hiy = n1.w * r.idir.y - r.ood.y;
      float c1loz = n2.z * r.idir.z - r.ood.z, c1hiz = n2.w * r.idir.z - r.ood.z;
      float c0min = Max3(fminf(c0lox, c0hix), fminf(c0loy, c0hiy), fmaxf(fminf(c0loz, c0hiz), 0.0f));
      float c0max = Min3(fmaxf(c0lox, c0hix), fmaxf(c0loy, c0hiy), fminf(fmaxf(c0loz, c0hiz), t.tmax));
      float c1min = Max3(fminf(c1lox, c1hix), fminf(c1loy, c1hiy), fmaxf(fminf(c1loz, c1hiz), 0.0f));
      float c1max = Min3(fmaxf(c1lox, c1hix), fmaxf(c1loy, c1hiy), fminf(fmaxf(c1loz, c1hiz), t.tmax));
      bool h0 = c0min <= c0max, h1 = c1min <= c1max;
      if (kStats) {
        cnt->box_tests += 2;
        cnt->box_hits += (int)h0 + (int)h1;
      }
      if (!h0 && !h1) {
        next();
      } else {
        int near = h0 ? n3.x : n3.y;
        if (h0 && h1) {
          int far = n3.y;
          if (c1min < c0min) {
            near = n3.y;
            far = n3.x;
          }
          if (t.sp < kStackSize) StackPush(t, far);
          else *overflow = true;
        }
        t.node = near;
      }
      if (t.node < 0 && t.node != kEmptyLink && leaf == 0) {
        leaf = t.node;  // postpone this leaf and keep descending
        next();
      }
      if (!__any_sync(__activemask(), leaf == 0)) break;
    }
    // the postponed leaf, then the current node for as long as it is a leaf
    if (leaf == 0 && t.node < 0 && t.node != kEmptyLink) {
      leaf = t.node;
      next();
    }
    while (leaf != 0) {
      for (int i = ~leaf;; ++i) {
        PrimRecord p = LoadPrim(recs, i);
        uint32_t flags = __float_as_uint(p.p3.w);
        float t_obj = 0.0f;
        float d = PrimTest<kTriTest>(s, r, p, flags, &t_obj);
        if (kStats) cnt->prim_tests += 1;
        if (d > 0.0f && d < t.tmax) {
          if (kStats) cnt->prim_hits += 1;
          t.tmax = d;
          t.hit = i;
          t.t_obj = t_obj;
          if (kAnyHit) return true;
        }
        if (flags & kPrimLast) break;
      }
      leaf = 0;
      if (t.node < 0 && t.node != kEmptyLink) {
        leaf = t.node;
        next();
      }
    }
    if (t.node == kEmptyLink) return true;
    if (__popc(__activemask()) < min_active) return false;
  }
}

}  // namespace muon_gpu
