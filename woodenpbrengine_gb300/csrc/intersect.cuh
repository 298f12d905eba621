// intersect.cuh — ray/box, ray/triangle and ray/sphere tests used by the
// traversal kernels and re-run by the shading kernels for the winning
// primitive (same arithmetic, same bits).
#pragma once

#include "geom.cuh"
#include "wpbr_scene.h"

namespace wpbr {

struct Ray {
  V3 o, d;
};

// Robust slab test of DBounds3f::intersect(ray, dirInv, dirIsNeg)
// (WoodenPBREngine/SLBVH.cpp:106), pbrt's Bounds3::IntersectP comparison
// order with tMax scaled by 1 + 2*gamma(3). lo/hi are the box corners; the
// entry distance is returned for closest-hit pruning.
WPBR_HD bool slab_test(V3 lo, V3 hi, V3 o, V3 inv, const int neg[3], float tmax_ray, float* tentry) {
  float tMin = ((neg[0] ? hi.x : lo.x) - o.x) * inv.x;
  float tMax = ((neg[0] ? lo.x : hi.x) - o.x) * inv.x;
  float tyMin = ((neg[1] ? hi.y : lo.y) - o.y) * inv.y;
  float tyMax = ((neg[1] ? lo.y : hi.y) - o.y) * inv.y;
  tMax = tMax * kSlabScale;
  tyMax = tyMax * kSlabScale;
  if (tMin > tyMax || tyMin > tMax) return false;
  if (tyMin > tMin) tMin = tyMin;
  if (tyMax < tMax) tMax = tyMax;
  float tzMin = ((neg[2] ? hi.z : lo.z) - o.z) * inv.z;
  float tzMax = ((neg[2] ? lo.z : hi.z) - o.z) * inv.z;
  tzMax = tzMax * kSlabScale;
  if (tMin > tzMax || tzMin > tMax) return false;
  if (tzMin > tMin) tMin = tzMin;
  if (tzMax < tMax) tMax = tzMax;
  *tentry = tMin;
  return (tMin < tmax_ray) && (tMax > 0.0f);
}

// slab_test without branches: all six plane distances, the same comparisons
// in the same order folded into selects and one boolean, so the result (and
// the entry distance when it is true) equals slab_test's for every input,
// NaN included; a warp never diverges inside it.
WPBR_HD bool slab_test_flat(V3 lo, V3 hi, V3 o, V3 inv, const int neg[3], float tmax_ray, float* tentry) {
  float tMin = ((neg[0] ? hi.x : lo.x) - o.x) * inv.x;
  float tMax = ((neg[0] ? lo.x : hi.x) - o.x) * inv.x;
  float tyMin = ((neg[1] ? hi.y : lo.y) - o.y) * inv.y;
  float tyMax = ((neg[1] ? lo.y : hi.y) - o.y) * inv.y;
  float tzMin = ((neg[2] ? hi.z : lo.z) - o.z) * inv.z;
  float tzMax = ((neg[2] ? lo.z : hi.z) - o.z) * inv.z;
  tMax = tMax * kSlabScale;
  tyMax = tyMax * kSlabScale;
  tzMax = tzMax * kSlabScale;
  bool ok = !(tMin > tyMax || tyMin > tMax);
  tMin = (tyMin > tMin) ? tyMin : tMin;
  tMax = (tyMax < tMax) ? tyMax : tMax;
  ok = ok && !(tMin > tzMax || tzMin > tMax);
  tMin = (tzMin > tMin) ? tzMin : tMin;
  tMax = (tzMax < tMax) ? tzMax : tMax;
  *tentry = tMin;
  return ok && (tMin < tmax_ray) && (tMax > 0.0f);
}

// JobProcessTriangleInteractionRequests (WoodenPBREngine/CSTriangle.cpp:9-108):
// watertight test in the reference's SIMD lane order. The edge functions come
// out as (e2, e0, e1), the determinant is (e2 + e0) + e1 and 1/det is
// rounded from double. Returns t, 0 on a miss.
WPBR_HD float tri_intersect(V3 p0, V3 p1, V3 p2, V3 ro, V3 rd, uint32_t quirks, float* b0, float* b1, float* b2) {
  float ax = fabs_(rd.x), ay = fabs_(rd.y), az = fabs_(rd.z);
  int kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
  int kx = (kz == 2) ? 0 : kz + 1;
  int ky = (kz == 2) ? 1 : kz + 2;
  if (ky == 3) {
    if (quirks & WPBR_Q_TRI_PERMUTATION_BUG) return 0.0f;
    ky = 0;
  }
  float dx = comp(rd, kx), dy = comp(rd, ky), dz = comp(rd, kz);
  float sx = -dx / dz, sy = -dy / dz, sz = 1.0f / dz;
  V3 q0 = sub(p0, ro), q1 = sub(p1, ro), q2 = sub(p2, ro);
  float x0 = comp(q0, kx), y0 = comp(q0, ky), z0 = comp(q0, kz);
  float x1 = comp(q1, kx), y1 = comp(q1, ky), z1 = comp(q1, kz);
  float x2 = comp(q2, kx), y2 = comp(q2, ky), z2 = comp(q2, kz);
  x0 = x0 + sx * z0;
  y0 = y0 + sy * z0;
  x1 = x1 + sx * z1;
  y1 = y1 + sy * z1;
  x2 = x2 + sx * z2;
  y2 = y2 + sy * z2;
  z0 = z0 + 0.0f * z0;
  z1 = z1 + 0.0f * z1;
  z2 = z2 + 0.0f * z2;
  float rx = x0 * y1 - x1 * y0;
  float ry = x1 * y2 - x2 * y1;
  float rz = x2 * y0 - x0 * y2;
  if ((rx < 0.0f || ry < 0.0f || rz < 0.0f) && (rx > 0.0f || ry > 0.0f || rz > 0.0f)) return 0.0f;
  float det = (rx + ry) + rz;
  if (det == 0.0f) return 0.0f;
  float e0 = ry, e1 = rz, e2 = rx;
  float ts = (e0 * (z0 * sz) + e1 * (z1 * sz)) + e2 * (z2 * sz);
  if (det < 0.0f && ts >= 0.0f) return 0.0f;
  if (det > 0.0f && ts <= 0.0f) return 0.0f;
  // float(1.0 / (double)det) as the reference writes it: a double quotient
  // rounded to float equals the correctly rounded float reciprocal (53 >=
  // 2*24 + 2 bits), which the device computes without double arithmetic.
#if defined(__CUDA_ARCH__)
  float inv_det = __frcp_rn(det);
#else
  float inv_det = (float)(1.0 / (double)det);
#endif
  *b0 = e0 * inv_det;
  *b1 = e1 * inv_det;
  *b2 = e2 * inv_det;
  return ts * inv_det;
}

// The per-ray part of tri_intersect (axis permutation, shear, permuted
// origin), evaluated once per ray: the same operations on the same operands,
// so tri_intersect_pre returns exactly what tri_intersect returns.
struct RayTri {
  int kx, ky, kz;
  float sx, sy, sz;
  float ox, oy, oz;
  bool miss_all;  // WPBR_Q_TRI_PERMUTATION_BUG with a y-dominant ray
};
WPBR_HD RayTri ray_tri_setup(V3 ro, V3 rd, uint32_t quirks) {
  RayTri R;
  float ax = fabs_(rd.x), ay = fabs_(rd.y), az = fabs_(rd.z);
  R.kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
  R.kx = (R.kz == 2) ? 0 : R.kz + 1;
  R.ky = (R.kz == 2) ? 1 : R.kz + 2;
  R.miss_all = false;
  if (R.ky == 3) {
    R.miss_all = (quirks & WPBR_Q_TRI_PERMUTATION_BUG) != 0;
    R.ky = 0;
  }
  float dx = comp(rd, R.kx), dy = comp(rd, R.ky), dz = comp(rd, R.kz);
  R.sx = -dx / dz;
  R.sy = -dy / dz;
  R.sz = 1.0f / dz;
  R.ox = comp(ro, R.kx);
  R.oy = comp(ro, R.ky);
  R.oz = comp(ro, R.kz);
  return R;
}
WPBR_HD float tri_intersect_pre(V3 p0, V3 p1, V3 p2, const RayTri& R, float* b0, float* b1, float* b2) {
  if (R.miss_all) return 0.0f;
  float x0 = comp(p0, R.kx) - R.ox, y0 = comp(p0, R.ky) - R.oy, z0 = comp(p0, R.kz) - R.oz;
  float x1 = comp(p1, R.kx) - R.ox, y1 = comp(p1, R.ky) - R.oy, z1 = comp(p1, R.kz) - R.oz;
  float x2 = comp(p2, R.kx) - R.ox, y2 = comp(p2, R.ky) - R.oy, z2 = comp(p2, R.kz) - R.oz;
  x0 = x0 + R.sx * z0;
  y0 = y0 + R.sy * z0;
  x1 = x1 + R.sx * z1;
  y1 = y1 + R.sy * z1;
  x2 = x2 + R.sx * z2;
  y2 = y2 + R.sy * z2;
  z0 = z0 + 0.0f * z0;
  z1 = z1 + 0.0f * z1;
  z2 = z2 + 0.0f * z2;
  float rx = x0 * y1 - x1 * y0;
  float ry = x1 * y2 - x2 * y1;
  float rz = x2 * y0 - x0 * y2;
  if ((rx < 0.0f || ry < 0.0f || rz < 0.0f) && (rx > 0.0f || ry > 0.0f || rz > 0.0f)) return 0.0f;
  float det = (rx + ry) + rz;
  if (det == 0.0f) return 0.0f;
  float e0 = ry, e1 = rz, e2 = rx;
  float ts = (e0 * (z0 * R.sz) + e1 * (z1 * R.sz)) + e2 * (z2 * R.sz);
  if (det < 0.0f && ts >= 0.0f) return 0.0f;
  if (det > 0.0f && ts <= 0.0f) return 0.0f;
#if defined(__CUDA_ARCH__)
  float inv_det = __frcp_rn(det);
#else
  float inv_det = (float)(1.0 / (double)det);
#endif
  *b0 = e0 * inv_det;
  *b1 = e1 * inv_det;
  *b2 = e2 * inv_det;
  return ts * inv_det;
}

// WoodenMath getRootsQuadraticEquation, restated as pbrt-v3's Quadratic
// (double-precision discriminant and roots, rounded to float).
WPBR_HD bool quadratic(float a, float b, float c, float* t0, float* t1) {
  double discrim = (double)b * (double)b - 4.0 * (double)a * (double)c;
  if (discrim < 0.0) return false;
  double root = sqrt_d(discrim);
  double q = (b < 0.0f) ? -0.5 * ((double)b - root) : -0.5 * ((double)b + root);
  float r0 = (float)(q / (double)a);
  float r1 = (float)((double)c / q);
  if (r0 > r1) {
    float t = r0;
    r0 = r1;
    r1 = t;
  }
  *t0 = r0;
  *t1 = r1;
  return true;
}

// SSphere::intersect (WoodenPBREngine/CSSphere.cpp:84-120). Returns t
// (0 = miss) and the object-space ray and hit point.
WPBR_HD float sphere_intersect(const Xf& w2o, float radius, V3 ro, V3 rd, V3* rlo, V3* rld, V3* phl) {
  V3 o = xpoint(w2o, ro);
  V3 d = xvector(w2o, rd);
  float a = len2(d);
  float b = 2.0f * dot(d, o);
  float c = len2(o) - radius * radius;
  float t0, t1;
  if (!quadratic(a, b, c, &t0, &t1)) return 0.0f;
  if (t1 <= 0.0f) return 0.0f;
  float t = t0;
  if (t <= 0.0f) t = t1;
  *rlo = o;
  *rld = d;
  *phl = add(o, mul(d, t));
  return t;
}

}  // namespace wpbr
