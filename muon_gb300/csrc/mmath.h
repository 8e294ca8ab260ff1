// Single-precision vector/matrix arithmetic shared by the host scene builder
// and the device kernels.
//
// Every operation is evaluated in the order the reference renderer's vector
// library evaluates it (GLM 0.9.9.8 as vendored by the reference), so that
// hosts and kernels that use these helpers reproduce the reference's float
// results bit for bit:
//   dot(a,b)        = (a.x*b.x + a.y*b.y) + a.z*b.z
//   cross(x,y)      = (x.y*y.z - y.y*x.z, x.z*y.x - y.z*x.x, x.x*y.y - y.x*x.y)
//   normalize(v)    = v * (1 / sqrt(dot(v,v)))
//   mat4 * vec4     = (m0*v.x + m1*v.y) + (m2*v.z + m3*v.w)   (columns m0..m3)
//   mat4 * mat4     = column c: ((A0*B[c].x + A1*B[c].y) + A2*B[c].z) + A3*B[c].w
// Matrices are column-major: m.c[col].{x,y,z,w}.
//
// On the device, EXACT_* helpers use the round-to-nearest intrinsics so the
// compiler cannot contract a multiply and an add into one FMA; the host side is
// compiled with -ffp-contract=off for the same reason.
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define MM_HD __host__ __device__ __forceinline__
#else
#define MM_HD inline
#endif

namespace mm {

#if defined(__CUDA_ARCH__)
MM_HD float mul(float a, float b) { return __fmul_rn(a, b); }
MM_HD float add(float a, float b) { return __fadd_rn(a, b); }
MM_HD float sub(float a, float b) { return __fsub_rn(a, b); }
MM_HD float div(float a, float b) { return __fdiv_rn(a, b); }
MM_HD float fsqrt(float a) { return __fsqrt_rn(a); }
#else
MM_HD float mul(float a, float b) { return a * b; }
MM_HD float add(float a, float b) { return a + b; }
MM_HD float sub(float a, float b) { return a - b; }
MM_HD float div(float a, float b) { return a / b; }
MM_HD float fsqrt(float a) { return sqrtf(a); }
#endif

// The reference's min/max pick the second argument only when it compares
// strictly smaller/larger, which fixes their behaviour for NaN inputs.
MM_HD float fmin_ref(float a, float b) { return (b < a) ? b : a; }
MM_HD float fmax_ref(float a, float b) { return (a < b) ? b : a; }
MM_HD float clamp_ref(float x, float lo, float hi) { return fmin_ref(fmax_ref(x, lo), hi); }

struct v3 {
  float x, y, z;
};
struct v4 {
  float x, y, z, w;
};

MM_HD v3 make3(float x, float y, float z) { return v3{x, y, z}; }
MM_HD v3 splat3(float s) { return v3{s, s, s}; }
MM_HD v3 operator+(v3 a, v3 b) { return v3{add(a.x, b.x), add(a.y, b.y), add(a.z, b.z)}; }
MM_HD v3 operator-(v3 a, v3 b) { return v3{sub(a.x, b.x), sub(a.y, b.y), sub(a.z, b.z)}; }
MM_HD v3 operator-(v3 a) { return v3{-a.x, -a.y, -a.z}; }
MM_HD v3 operator*(v3 a, v3 b) { return v3{mul(a.x, b.x), mul(a.y, b.y), mul(a.z, b.z)}; }
MM_HD v3 operator*(v3 a, float s) { return v3{mul(a.x, s), mul(a.y, s), mul(a.z, s)}; }
MM_HD v3 operator*(float s, v3 a) { return v3{mul(s, a.x), mul(s, a.y), mul(s, a.z)}; }
MM_HD v3 operator/(v3 a, float s) { return v3{div(a.x, s), div(a.y, s), div(a.z, s)}; }
MM_HD float comp(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

MM_HD float dot(v3 a, v3 b) { return add(add(mul(a.x, b.x), mul(a.y, b.y)), mul(a.z, b.z)); }
MM_HD v3 cross(v3 x, v3 y) {
  return v3{sub(mul(x.y, y.z), mul(y.y, x.z)), sub(mul(x.z, y.x), mul(y.z, x.x)),
            sub(mul(x.x, y.y), mul(y.x, x.y))};
}
MM_HD float length(v3 v) { return fsqrt(dot(v, v)); }
MM_HD v3 normalize(v3 v) { return v * div(1.0f, fsqrt(dot(v, v))); }
// Mirror reflection of an incoming direction about a normal: d - 2 (d.n) n.
MM_HD v3 reflect(v3 d, v3 n) { return d - (mul(2.0f, dot(d, n)) * n); }

MM_HD v4 operator+(v4 a, v4 b) { return v4{add(a.x, b.x), add(a.y, b.y), add(a.z, b.z), add(a.w, b.w)}; }
MM_HD v4 operator-(v4 a, v4 b) { return v4{sub(a.x, b.x), sub(a.y, b.y), sub(a.z, b.z), sub(a.w, b.w)}; }
MM_HD v4 operator*(v4 a, float s) { return v4{mul(a.x, s), mul(a.y, s), mul(a.z, s), mul(a.w, s)}; }
MM_HD v4 operator*(v4 a, v4 b) { return v4{mul(a.x, b.x), mul(a.y, b.y), mul(a.z, b.z), mul(a.w, b.w)}; }

struct m4 {
  v4 c[4];
};

MM_HD m4 identity4() {
  m4 m;
  m.c[0] = v4{1, 0, 0, 0};
  m.c[1] = v4{0, 1, 0, 0};
  m.c[2] = v4{0, 0, 1, 0};
  m.c[3] = v4{0, 0, 0, 1};
  return m;
}

MM_HD v4 mul(const m4 &m, v4 v) {
  v4 a0 = m.c[0] * v.x + m.c[1] * v.y;
  v4 a1 = m.c[2] * v.z + m.c[3] * v.w;
  return a0 + a1;
}

MM_HD m4 mul(const m4 &a, const m4 &b) {
  m4 r;
  for (int c = 0; c < 4; ++c) {
    r.c[c] = a.c[0] * b.c[c].x + a.c[1] * b.c[c].y + a.c[2] * b.c[c].z + a.c[3] * b.c[c].w;
  }
  return r;
}

// Position transform: xyz of M * (p, 1).
MM_HD v3 xform_point(const m4 &m, v3 p) {
  v4 r = mul(m, v4{p.x, p.y, p.z, 1.0f});
  return v3{r.x, r.y, r.z};
}
// Direction transform, re-normalised: normalize(xyz of M * (d, 0)).
MM_HD v3 xform_dir(const m4 &m, v3 d) {
  v4 r = mul(m, v4{d.x, d.y, d.z, 0.0f});
  return normalize(v3{r.x, r.y, r.z});
}

MM_HD m4 transpose(const m4 &m) {
  m4 r;
  r.c[0] = v4{m.c[0].x, m.c[1].x, m.c[2].x, m.c[3].x};
  r.c[1] = v4{m.c[0].y, m.c[1].y, m.c[2].y, m.c[3].y};
  r.c[2] = v4{m.c[0].z, m.c[1].z, m.c[2].z, m.c[3].z};
  r.c[3] = v4{m.c[0].w, m.c[1].w, m.c[2].w, m.c[3].w};
  return r;
}

// Inverse by cofactor expansion along the first row, in the same evaluation
// order as the reference's matrix library: the 18 2x2 minors of the lower rows,
// then the signed cofactor columns, then the determinant as a pairwise sum of
// the first column times the first cofactor row, then a multiply by 1/det.
MM_HD m4 inverse(const m4 &m) {
  auto e = [&](int c, int r) -> float {
    const v4 &col = m.c[c];
    return r == 0 ? col.x : (r == 1 ? col.y : (r == 2 ? col.z : col.w));
  };
  auto minor2 = [&](int c0, int r0, int c1, int r1, int c2, int r2, int c3, int r3) {
    return sub(mul(e(c0, r0), e(c1, r1)), mul(e(c2, r2), e(c3, r3)));
  };
  float k00 = minor2(2, 2, 3, 3, 3, 2, 2, 3);
  float k02 = minor2(1, 2, 3, 3, 3, 2, 1, 3);
  float k03 = minor2(1, 2, 2, 3, 2, 2, 1, 3);
  float k04 = minor2(2, 1, 3, 3, 3, 1, 2, 3);
  float k06 = minor2(1, 1, 3, 3, 3, 1, 1, 3);
  float k07 = minor2(1, 1, 2, 3, 2, 1, 1, 3);
  float k08 = minor2(2, 1, 3, 2, 3, 1, 2, 2);
  float k10 = minor2(1, 1, 3, 2, 3, 1, 1, 2);
  float k11 = minor2(1, 1, 2, 2, 2, 1, 1, 2);
  float k12 = minor2(2, 0, 3, 3, 3, 0, 2, 3);
  float k14 = minor2(1, 0, 3, 3, 3, 0, 1, 3);
  float k15 = minor2(1, 0, 2, 3, 2, 0, 1, 3);
  float k16 = minor2(2, 0, 3, 2, 3, 0, 2, 2);
  float k18 = minor2(1, 0, 3, 2, 3, 0, 1, 2);
  float k19 = minor2(1, 0, 2, 2, 2, 0, 1, 2);
  float k20 = minor2(2, 0, 3, 1, 3, 0, 2, 1);
  float k22 = minor2(1, 0, 3, 1, 3, 0, 1, 1);
  float k23 = minor2(1, 0, 2, 1, 2, 0, 1, 1);
  v4 f0{k00, k00, k02, k03}, f1{k04, k04, k06, k07}, f2{k08, k08, k10, k11};
  v4 f3{k12, k12, k14, k15}, f4{k16, k16, k18, k19}, f5{k20, k20, k22, k23};
  v4 g0{e(1, 0), e(0, 0), e(0, 0), e(0, 0)};
  v4 g1{e(1, 1), e(0, 1), e(0, 1), e(0, 1)};
  v4 g2{e(1, 2), e(0, 2), e(0, 2), e(0, 2)};
  v4 g3{e(1, 3), e(0, 3), e(0, 3), e(0, 3)};
  v4 i0 = g1 * f0 - g2 * f1 + g3 * f2;
  v4 i1 = g0 * f0 - g2 * f3 + g3 * f4;
  v4 i2 = g0 * f1 - g1 * f3 + g3 * f5;
  v4 i3 = g0 * f2 - g1 * f4 + g2 * f5;
  v4 sa{1, -1, 1, -1}, sb{-1, 1, -1, 1};
  m4 inv;
  inv.c[0] = i0 * sa;
  inv.c[1] = i1 * sb;
  inv.c[2] = i2 * sa;
  inv.c[3] = i3 * sb;
  v4 row0{inv.c[0].x, inv.c[1].x, inv.c[2].x, inv.c[3].x};
  v4 d0 = m.c[0] * row0;
  float det = add(add(d0.x, d0.y), add(d0.z, d0.w));
  float one_over_det = div(1.0f, det);
  for (int c = 0; c < 4; ++c) inv.c[c] = inv.c[c] * one_over_det;
  return inv;
}

// Affine builders applied to the identity, as the scene parser uses them.
MM_HD m4 translate(v3 t) {
  m4 m = identity4();
  m.c[3] = m.c[0] * t.x + m.c[1] * t.y + m.c[2] * t.z + m.c[3];
  return m;
}
MM_HD m4 scale(v3 s) {
  m4 m = identity4();
  m4 r;
  r.c[0] = m.c[0] * s.x;
  r.c[1] = m.c[1] * s.y;
  r.c[2] = m.c[2] * s.z;
  r.c[3] = m.c[3];
  return r;
}
// Rotation by `angle` radians about `axis` (Rodrigues form); cos/sin are the
// single-precision libm functions on the host.
inline m4 rotate(float angle, v3 axis_in) {
  float c = cosf(angle);
  float s = sinf(angle);
  v3 axis = normalize(axis_in);
  v3 temp = sub(1.0f, c) * axis;
  float r00 = add(c, mul(temp.x, axis.x));
  float r01 = add(mul(temp.x, axis.y), mul(s, axis.z));
  float r02 = sub(mul(temp.x, axis.z), mul(s, axis.y));
  float r10 = sub(mul(temp.y, axis.x), mul(s, axis.z));
  float r11 = add(c, mul(temp.y, axis.y));
  float r12 = add(mul(temp.y, axis.z), mul(s, axis.x));
  float r20 = add(mul(temp.z, axis.x), mul(s, axis.y));
  float r21 = sub(mul(temp.z, axis.y), mul(s, axis.x));
  float r22 = add(c, mul(temp.z, axis.z));
  m4 m = identity4();
  m4 r;
  r.c[0] = m.c[0] * r00 + m.c[1] * r01 + m.c[2] * r02;
  r.c[1] = m.c[0] * r10 + m.c[1] * r11 + m.c[2] * r12;
  r.c[2] = m.c[0] * r20 + m.c[1] * r21 + m.c[2] * r22;
  r.c[3] = m.c[3];
  return r;
}
// Degrees to radians with the single-precision constant pi/180.
MM_HD float radians(float deg) { return mul(deg, 0.01745329251994329576923690768489f); }

}  // namespace mm
