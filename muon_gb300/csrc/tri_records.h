// The records of one triangle: world-space and object-space primitive
// records, shading record, pre-transformed vertex normals and world box.
// One function for the host scene builder and the device record kernel, so
// that both produce the same bits (mmath.h evaluates in the reference's
// order without fused multiply-adds on either side).
#pragma once

#include <string.h>

#include "../../include/muon_gpu.h"
#include "dev_layout.h"
#include "mmath.h"

namespace muon_gpu {

MM_HD mm::m4 LoadM4(const float *m) {
  mm::m4 r;
  for (int c = 0; c < 4; ++c) r.c[c] = mm::v4{m[4 * c], m[4 * c + 1], m[4 * c + 2], m[4 * c + 3]};
  return r;
}
MM_HD float FloatBits(int32_t v) {
  float f;
  memcpy(&f, &v, 4);
  return f;
}
MM_HD F4 Rec4(float x, float y, float z, float w) { return F4{x, y, z, w}; }
MM_HD mm::v3 Load3(const float *p) { return mm::make3(p[0], p[1], p[2]); }

struct TriangleOut {
  PrimRecord world, object;
  ShadeRecord shade;
  F4 normals[3], normals_obj[3];  // written when the triangle is smooth
  float lo[3], hi[3];
};

// |n| of the object-space face normal: a triangle with |n| < 1e-4 is never
// hit (|d.n| <= |n| for a unit direction), so it stays out of the BVH.
MM_HD bool TriangleCanBeHit(const MuonTriangleDesc &t) {
  const mm::v3 a = Load3(t.v[0]), b = Load3(t.v[1]), c = Load3(t.v[2]);
  return mm::length(mm::cross(b - a, c - a)) >= 1e-4f;
}

// Tri::Tri and Primitive's transforms (muon/objects.cc:58-175,
// muon/transform.h:13-18) flattened into the records the kernels read;
// `quad_index` maps a light index to its quad-light index (-1: not a quad),
// `materials` supplies the effective BRDF of the shading class. Returns
// TriangleCanBeHit(t).
MM_HD bool TriangleRecords(const MuonTriangleDesc &t, const MuonTransformDesc *transforms,
                           const DevMaterial *materials, const int32_t *quad_index, TriangleOut *o) {
  const mm::v3 ov[3] = {Load3(t.v[0]), Load3(t.v[1]), Load3(t.v[2])};
  mm::v3 wv[3];
  const mm::m4 m = t.transform >= 0 ? LoadM4(transforms[t.transform].object_to_world) : mm::identity4();
  for (int k = 0; k < 3; ++k) wv[k] = t.transform >= 0 ? mm::xform_point(m, ov[k]) : ov[k];
  const mm::v3 n_obj = mm::cross(ov[1] - ov[0], ov[2] - ov[0]);
  const mm::v3 n_w = mm::cross(wv[1] - wv[0], wv[2] - wv[0]);
  const float len_obj = mm::length(n_obj);
  float eps = 1e-4f;
  if (t.transform >= 0) eps = mm::mul(1e-4f, mm::div(mm::length(n_w), len_obj));
  PrimRecord &ro = o->object;
  ro.p0 = Rec4(ov[0].x, ov[0].y, ov[0].z, 0.0f);
  ro.p1 = Rec4(ov[1].x, ov[1].y, ov[1].z, FloatBits(t.transform));
  ro.p2 = Rec4(ov[2].x, ov[2].y, ov[2].z, mm::dot(n_obj, n_obj));
  PrimRecord &r = o->world;
  r.p0 = Rec4(wv[0].x, wv[0].y, wv[0].z, mm::dot(wv[0], n_w));
  r.p1 = Rec4(wv[1].x, wv[1].y, wv[1].z, eps);
  r.p2 = Rec4(wv[2].x, wv[2].y, wv[2].z, 0.0f);
  const uint32_t flags = t.smooth ? kPrimSmooth : 0u;
  // Shading normal as the reference forms it: the unit object-space normal
  // carried by the inverse transpose and normalised again (muon/objects.cc:
  // 40-41, 165-167); for a mirroring transform it points against n_w.
  const mm::m4 nt = t.transform >= 0 ? LoadM4(transforms[t.transform].normal_to_world) : mm::identity4();
  const mm::v3 un = mm::xform_dir(nt, mm::normalize(n_obj));
  ShadeRecord &s = o->shade;
  s.s0 = Rec4(un.x, un.y, un.z, FloatBits(t.material));
  int32_t brdf_eff;
  memcpy(&brdf_eff, &materials[t.material].emission.w, 4);
  const uint32_t shade_flags = flags | (static_cast<uint32_t>(brdf_eff) << kClassShift);
  s.s1 = I4{t.light >= 0 ? quad_index[t.light] : -1, t.prim_id, t.transform, static_cast<int32_t>(shade_flags)};
  // the primitive records carry the shading class too (read by the extend
  // kernel from the record it has just tested)
  float flag_bits;
  memcpy(&flag_bits, &shade_flags, 4);
  r.p3 = Rec4(n_w.x, n_w.y, n_w.z, flag_bits);
  ro.p3 = Rec4(n_obj.x, n_obj.y, n_obj.z, flag_bits);
  if (t.smooth) {
    // normalize(M^-T (w n0 + u n1 + v n2)) equals the normalised blend of
    // the pre-transformed vertex normals, by linearity.
    for (int k = 0; k < 3; ++k) {
      const mm::v3 vn = Load3(t.n[k]);
      const mm::v4 w4 = t.transform >= 0 ? mm::mul(nt, mm::v4{vn.x, vn.y, vn.z, 0.0f}) : mm::v4{vn.x, vn.y, vn.z, 0.0f};
      o->normals[k] = Rec4(w4.x, w4.y, w4.z, 0.0f);
      o->normals_obj[k] = Rec4(vn.x, vn.y, vn.z, 0.0f);
    }
  }
  for (int k = 0; k < 3; ++k) {
    o->lo[k] = mm::fmin_ref(mm::fmin_ref(mm::comp(wv[0], k), mm::comp(wv[1], k)), mm::comp(wv[2], k));
    o->hi[k] = mm::fmax_ref(mm::fmax_ref(mm::comp(wv[0], k), mm::comp(wv[1], k)), mm::comp(wv[2], k));
  }
  return len_obj >= 1e-4f;
}

}  // namespace muon_gpu
