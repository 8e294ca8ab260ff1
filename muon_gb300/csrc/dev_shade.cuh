// Camera rays, BRDFs, hemisphere sampling, light sampling and MIS weights.
//
// Restates the reference's estimator pieces: Camera::CastRay
// (muon/camera.cc:37-62), SampleHemisphere/SampleCosine
// (muon/hemisphere_sampling.cc:8-38), RotateToOrthonormalFrame
// (muon/transform.cc:5-19), the Lambertian/Phong/GGX BRDFs
// (muon/materials.cc:17-293), Quad::Intersect (muon/lighting.cc:7-36),
// PowerHeuristic, NEEPDF and ImportanceSamplingPDF
// (muon/integration.cc:332-338, 564-630). Where the reference goes through
// acos/tan/atan and back, the algebraically equal closed forms in cos(theta)
// are used (noted per function).
#pragma once

#include "dev_common.cuh"

namespace muon_gpu {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.318309886183790671538f;

// Camera ray through screen position (x, y), evaluated with the reference's
// operation order and no contraction, so primary rays match it bit for bit.
__device__ __forceinline__ void CastRay(const DevCamera &c, float x, float y, float3 *o, float3 *d) {
  float half_w = mm::div(static_cast<float>(c.width), 2.0f);
  float half_h = mm::div(static_cast<float>(c.height), 2.0f);
  float ox = mm::div(mm::sub(x, half_w), half_w);
  float oy = mm::div(mm::sub(half_h, y), half_h);
  float alpha = mm::mul(c.tan_fov_x, ox);
  float beta = mm::mul(c.tan_fov_y, oy);
  mm::v3 u = mm::make3(c.u[0], c.u[1], c.u[2]);
  mm::v3 v = mm::make3(c.v[0], c.v[1], c.v[2]);
  mm::v3 w = mm::make3(c.w[0], c.w[1], c.w[2]);
  mm::v3 dir = mm::normalize(alpha * u + beta * v - w);
  *o = f3(c.eye[0], c.eye[1], c.eye[2]);
  *d = f3(dir.x, dir.y, dir.z);
}

struct Mat {
  float3 kd, ks, ke;
  float shininess, roughness, reflect;
  int brdf;
};

__device__ __forceinline__ Mat LoadMat(const DevMaterial *mats, int i) {
  const float4 *q = reinterpret_cast<const float4 *>(mats + i);
  float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), d = __ldg(q + 3);
  Mat m;
  m.kd = f3(a.x, a.y, a.z);
  m.shininess = a.w;
  m.ks = f3(b.x, b.y, b.z);
  m.roughness = b.w;
  m.ke = f3(c.x, c.y, c.z);
  m.brdf = __float_as_int(c.w);
  m.reflect = d.w;
  return m;
}

// Rotates a z-up sample into the frame around w (muon/transform.cc:5-19).
__device__ __forceinline__ float3 RotateToFrame(float3 s, float3 w) {
  float3 a = fabsf(w.y) <= 0.9f ? f3(0.0f, 1.0f, 0.0f) : f3(1.0f, 0.0f, 0.0f);
  float3 u = normalize3(cross3(a, w));
  float3 v = normalize3(cross3(w, u));
  return s.x * u + s.y * v + s.z * w;
}

// Direction with polar angle cos = ct around w and azimuth 2 pi r2.
__device__ __forceinline__ float3 PolarDir(float ct, float r2, float3 w) {
  float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
  float sp, cp;
  sincospif(2.0f * r2, &sp, &cp);
  return RotateToFrame(f3(cp * st, sp * st, ct), w);
}

// theta = acos(r1): cos(theta) = r1.
__device__ __forceinline__ float3 SampleHemisphere(float3 n, Rng &rng) {
  float r1 = rng.Next(), r2 = rng.Next();
  return PolarDir(r1, r2, n);
}
// theta = acos(sqrt(r1)): cos(theta) = sqrt(r1).
__device__ __forceinline__ float3 SampleCosine(float3 n, Rng &rng) {
  float r1 = rng.Next(), r2 = rng.Next();
  return PolarDir(sqrtf(r1), r2, n);
}

// GGX microfacet distribution (muon/materials.cc:131-140):
// a^2 / (pi cos^4 (a^2 + tan^2)^2) = a^2 / (pi (c^2 (a^2 - 1) + 1)^2).
__device__ __forceinline__ float GgxD(float3 h, float3 n, float alpha) {
  float c = fminf(fmaxf(dot3(h, n), 0.0f), 1.0f);
  float a2 = alpha * alpha;
  float k = c * c * (a2 - 1.0f) + 1.0f;
  float denom = kPi * k * k;
  return denom > 0.0f ? a2 / denom : 0.0f;
}
// Smith G1 (muon/materials.cc:147-158) with tan^2 = (1 - c^2) / c^2.
__device__ __forceinline__ float GgxG1(float3 v, float3 n, float alpha) {
  float c = dot3(v, n);
  if (c <= 0.0f) return 0.0f;
  c = fminf(c, 1.0f);
  float tan2 = (1.0f - c * c) / (c * c);
  return 2.0f / (1.0f + sqrtf(1.0f + alpha * alpha * tan2));
}

__device__ __forceinline__ float3 BrdfSample(const Mat &m, float3 ray_dir, float3 n, Rng &rng) {
  if (m.brdf == MUON_BRDF_LAMBERTIAN) return SampleCosine(n, rng);
  float r0 = rng.Next();
  if (r0 > m.reflect) return SampleCosine(n, rng);
  float r1 = rng.Next(), r2 = rng.Next();
  if (m.brdf == MUON_BRDF_PHONG) {
    // theta = acos(r1^(1/(s+1))) about the mirror direction
    // (muon/materials.cc:62-73).
    float ct = powf(r1, 1.0f / (m.shininess + 1.0f));
    return PolarDir(ct, r2, reflect3(ray_dir, n));
  }
  // GGX half vector: theta = atan(a sqrt(r1) / sqrt(1 - r1)), so
  // cos^2(theta) = (1 - r1) / (1 - r1 + a^2 r1) (muon/materials.cc:193-207).
  float a2 = m.roughness * m.roughness;
  float ct = sqrtf((1.0f - r1) / ((1.0f - r1) + a2 * r1));
  float3 h = PolarDir(ct, r2, n);
  return reflect3(ray_dir, h);
}

__device__ __forceinline__ float BrdfPdf(const Mat &m, float3 in, float3 ray_dir, float3 n) {
  float cos_pdf = fmaxf(dot3(n, in), 0.0f) * kInvPi;
  if (m.brdf == MUON_BRDF_LAMBERTIAN) return cos_pdf;
  float t = m.reflect;
  if (m.brdf == MUON_BRDF_PHONG) {
    float rl = fmaxf(dot3(reflect3(ray_dir, n), in), 0.0f);
    return (1.0f - t) * cos_pdf + t * (m.shininess + 1.0f) * 0.5f * kInvPi * powf(rl, m.shininess);
  }
  float3 h = normalize3(in - ray_dir);
  return (1.0f - t) * cos_pdf + t * GgxD(h, n, m.roughness) * fmaxf(dot3(n, h), 0.0f) / (4.0f * dot3(h, in));
}

__device__ __forceinline__ float3 BrdfEval(const Mat &m, float3 in, float3 ray_dir, float3 n) {
  float3 diffuse = m.kd * kInvPi;
  if (m.brdf == MUON_BRDF_LAMBERTIAN) return diffuse;
  if (m.brdf == MUON_BRDF_PHONG) {
    float rl = fmaxf(dot3(reflect3(ray_dir, n), in), 0.0f);
    return diffuse + m.ks * ((m.shininess + 2.0f) * (0.5f * kInvPi) * powf(rl, m.shininess));
  }
  float3 h = normalize3(in - ray_dir);
  float x = 1.0f - dot3(in, h);
  float x5 = x * x * x * x * x;
  float3 fresnel = m.ks + (f3(1.0f, 1.0f, 1.0f) - m.ks) * x5;
  float g = GgxG1(in, n, m.roughness) * GgxG1(-ray_dir, n, m.roughness);
  float dist = GgxD(h, n, m.roughness);
  float denom = 4.0f * dot3(in, n) * dot3(-ray_dir, n);
  if (denom == 0.0f) return diffuse;
  return diffuse + fresnel * (g * dist / denom);
}

// Quad::Intersect (muon/lighting.cc:7-36): returns the hit distance or -1.
__device__ __forceinline__ float QuadHit(const DevLight &l, float3 o, float3 d, float3 *p_out) {
  float3 qn = f3(l.quad_normal);
  float rdn = dot3(d, qn);
  if (rdn == 0.0f) return -1.0f;
  float3 corner = f3(l.corner);
  float t = dot3(corner - o, qn) / rdn;
  if (t < 0.0f) return -1.0f;
  float3 p = o + d * t;
  float3 pe = p - corner;
  float l0 = l.edge0.w, l1 = l.edge1.w;
  float u = dot3(pe, f3(l.edge0)) / l0;
  float v = dot3(pe, f3(l.edge1)) / l1;
  if (u > 0.0f && u < l0 && v > 0.0f && v < l1) {
    *p_out = p;
    return t;
  }
  return -1.0f;
}

// NEEPDF (muon/integration.cc:564-608): the solid-angle density of light
// sampling, averaged over all area lights whether or not the ray meets them.
__device__ __forceinline__ float NeePdf(const DevScene &s, float3 o, float3 d) {
  if (s.num_lights == 0) return 0.0f;
  float sum = 0.0f;
  for (int i = 0; i < s.num_lights; ++i) {
    const DevLight &l = s.lights[i];
    float3 p;
    if (QuadHit(l, o, d, &p) < 0.0f) continue;
    float denom = l.color.w * fabsf(dot3(f3(l.rev_normal), d));
    if (denom == 0.0f) continue;
    float3 pl = p - o;
    sum += dot3(pl, pl) / denom;
  }
  return sum / static_cast<float>(s.num_lights);
}

__device__ __forceinline__ float PowerHeuristic(float a, float b) {
  float denom = a * a + b * b;
  return denom == 0.0f ? 0.0f : (a * a) / denom;
}

__device__ __forceinline__ float IsPdf(int mode, const Mat &m, float3 dir, float3 ray_dir, float3 n) {
  if (mode == MUON_IS_HEMISPHERE) return 1.0f / (2.0f * kPi);
  if (mode == MUON_IS_COSINE) return fmaxf(dot3(n, dir), 0.0f) * kInvPi;
  return BrdfPdf(m, dir, ray_dir, n);
}

// PathTracer::SampleReflection (muon/integration.cc:503-562). Returns false
// for a direction at or below the horizon. A sample whose density is zero is
// treated the same way (the reference divides by it).
__device__ __forceinline__ bool SampleReflection(int mode, const Mat &m, float3 n, float3 ray_dir, float3 tp,
                                                 Rng &rng, float3 *dir, float *pdf, float3 *next_tp) {
  float3 w;
  if (mode == MUON_IS_HEMISPHERE) w = SampleHemisphere(n, rng);
  else if (mode == MUON_IS_COSINE) w = SampleCosine(n, rng);
  else w = BrdfSample(m, ray_dir, n, rng);
  float cosn = dot3(w, n);
  if (cosn <= 0.0f) return false;
  float3 f = BrdfEval(m, w, ray_dir, n);
  float p = IsPdf(mode, m, w, ray_dir, n);
  if (mode == MUON_IS_HEMISPHERE) {
    *next_tp = tp * (2.0f * kPi) * f * cosn;
  } else if (mode == MUON_IS_COSINE) {
    *next_tp = tp * kPi * f;
  } else {
    if (!(p > 0.0f)) return false;
    *next_tp = tp * f * (cosn / p);
  }
  *dir = w;
  *pdf = p;
  return true;
}

}  // namespace muon_gpu
