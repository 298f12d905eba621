// geom.cuh — host/device vector, transform and bounds arithmetic for the
// ray pipeline. Every operation has a fixed evaluation order and the whole
// library is compiled without multiply-add contraction (nvcc -fmad=false,
// g++ -ffp-contract=off), so host and device produce identical bits.
//
// Conventions that follow the reference engine (WoodenPBREngine):
//   dot(a,b) = (ax*bx + ay*by) + az*bz, normalize(v) = v / |v|;
//   transforms are row-major 4x4 acting on column vectors; composition is
//   "left first" (compose(A, B) applies A then B), the order the reference
//   relies on in SCameraProjective::create (CSCameraProjective.h:35-47);
//   PI is the double literal 3.14 (pch.h:30) wherever the reference writes PI.
#pragma once

#include <float.h>
#include <stdint.h>

#include "wpbr_fmath.h"

namespace wpbr {

using namespace wpbr_fm;

constexpr double kPI = 3.14;                 // pch.h:30
constexpr float kMathPi = 0x1.921fb6p+1f;    // pi inside the math library
constexpr float kSlabScale = 0x1.000006p+0f; // 1 + 2*gamma(3) in float
constexpr uint32_t kNoHit = 0xFFFFFFFFu;

struct V3 {
  float x, y, z;
};
struct V2 {
  float x, y;
};

WPBR_HD V3 mk(float x, float y, float z) { return V3{x, y, z}; }
WPBR_HD V3 add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
WPBR_HD V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
WPBR_HD V3 neg(V3 a) { return V3{-a.x, -a.y, -a.z}; }
WPBR_HD V3 mul(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
WPBR_HD V3 mulv(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
WPBR_HD V3 divs(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
WPBR_HD float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
WPBR_HD V3 cross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
WPBR_HD float len2(V3 v) { return dot(v, v); }
WPBR_HD float len(V3 v) { return sqrt_(len2(v)); }
WPBR_HD V3 normalize(V3 v) { return divs(v, len(v)); }
WPBR_HD bool is_zero(V3 v) { return v.x == 0.0f && v.y == 0.0f && v.z == 0.0f; }
WPBR_HD float comp(V3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
WPBR_HD float fmin_(float a, float b) { return b < a ? b : a; }  // std::min
WPBR_HD float fmax_(float a, float b) { return a < b ? b : a; }  // std::max
WPBR_HD V3 vmin(V3 a, V3 b) { return V3{fmin_(a.x, b.x), fmin_(a.y, b.y), fmin_(a.z, b.z)}; }
WPBR_HD V3 vmax(V3 a, V3 b) { return V3{fmax_(a.x, b.x), fmax_(a.y, b.y), fmax_(a.z, b.z)}; }
WPBR_HD float clampf(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }

struct RGB3 {
  float r, g, b;
};
WPBR_HD RGB3 rgb1(float v) { return RGB3{v, v, v}; }
WPBR_HD RGB3 radd(RGB3 a, RGB3 b) { return RGB3{a.r + b.r, a.g + b.g, a.b + b.b}; }
WPBR_HD RGB3 rmul(RGB3 a, RGB3 b) { return RGB3{a.r * b.r, a.g * b.g, a.b * b.b}; }
WPBR_HD RGB3 rmuls(RGB3 a, float s) { return RGB3{a.r * s, a.g * s, a.b * s}; }
WPBR_HD bool rblack(RGB3 a) { return a.r == 0.0f && a.g == 0.0f && a.b == 0.0f; }

// ---- transforms ---------------------------------------------------------
struct Xf {
  float m[4][4];
};
WPBR_HD Xf xf_identity() {
  Xf r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) r.m[i][j] = (i == j) ? 1.0f : 0.0f;
  return r;
}
WPBR_HD V3 xpoint(const Xf& M, V3 p) {
  float x = ((M.m[0][0] * p.x + M.m[0][1] * p.y) + M.m[0][2] * p.z) + M.m[0][3];
  float y = ((M.m[1][0] * p.x + M.m[1][1] * p.y) + M.m[1][2] * p.z) + M.m[1][3];
  float z = ((M.m[2][0] * p.x + M.m[2][1] * p.y) + M.m[2][2] * p.z) + M.m[2][3];
  float w = ((M.m[3][0] * p.x + M.m[3][1] * p.y) + M.m[3][2] * p.z) + M.m[3][3];
  if (w == 1.0f) return V3{x, y, z};
  return V3{x / w, y / w, z / w};
}
WPBR_HD V3 xvector(const Xf& M, V3 v) {
  return V3{(M.m[0][0] * v.x + M.m[0][1] * v.y) + M.m[0][2] * v.z,
            (M.m[1][0] * v.x + M.m[1][1] * v.y) + M.m[1][2] * v.z,
            (M.m[2][0] * v.x + M.m[2][1] * v.y) + M.m[2][2] * v.z};
}
// normal transform with the inverse matrix (inverse transpose applied)
WPBR_HD V3 xnormal(const Xf& Minv, V3 n) {
  return V3{(Minv.m[0][0] * n.x + Minv.m[1][0] * n.y) + Minv.m[2][0] * n.z,
            (Minv.m[0][1] * n.x + Minv.m[1][1] * n.y) + Minv.m[2][1] * n.z,
            (Minv.m[0][2] * n.x + Minv.m[1][2] * n.y) + Minv.m[2][2] * n.z};
}
WPBR_HD Xf compose(const Xf& A, const Xf& B) {  // A then B
  Xf C;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      C.m[i][j] = ((B.m[i][0] * A.m[0][j] + B.m[i][1] * A.m[1][j]) + B.m[i][2] * A.m[2][j]) + B.m[i][3] * A.m[3][j];
  return C;
}

// ---- bounds -----------------------------------------------------------------
struct Bounds {
  V3 lo, hi;
};
WPBR_HD Bounds bempty() { return Bounds{V3{FLT_MAX, FLT_MAX, FLT_MAX}, V3{-FLT_MAX, -FLT_MAX, -FLT_MAX}}; }
WPBR_HD Bounds bunion(const Bounds& a, const Bounds& b) { return Bounds{vmin(a.lo, b.lo), vmax(a.hi, b.hi)}; }
WPBR_HD Bounds bunionp(const Bounds& a, V3 p) { return Bounds{vmin(a.lo, p), vmax(a.hi, p)}; }
WPBR_HD V3 bcentroid(const Bounds& b) { return add(mul(b.hi, 0.5f), mul(b.lo, 0.5f)); }  // CCentroid.h:11-13
WPBR_HD float barea(const Bounds& b) {
  V3 d = sub(b.hi, b.lo);
  return 2.0f * ((d.x * d.y + d.x * d.z) + d.y * d.z);
}
WPBR_HD int bmax_extent(const Bounds& b) {
  V3 d = sub(b.hi, b.lo);
  if (d.x > d.y && d.x > d.z) return 0;
  if (d.y > d.z) return 1;
  return 2;
}

}  // namespace wpbr
