/*
 * oracle_math.hpp — TEST INFRASTRUCTURE. CPU restatement of WoodenPBREngine's
 * per-sample ray pipeline math, used only by tests/, the package smoke check
 * and bench.py's CPU-baseline leg as the checker. Nothing in the product links
 * or includes this file.
 *
 * Parity status: UNPINNED against the reference binary. The reference cannot be
 * compiled here (WoodenECS / WoodenMathLibrarry / WoodenAllocators are not
 * vendored, the code uses MSVC-only syntax) and ships no tests, golden images
 * or known-answer vectors. Every function below restates the reference source
 * at the cited file:line; functions the reference takes from the missing
 * WoodenMathLibrarry are restated from pbrt-v3's published algorithms (the
 * engine follows pbrt, README.md:40-42) and marked "[wml]".
 *
 * Arithmetic conventions (chosen once, shared with the GPU pipeline):
 *  - C++ promotion rules are kept literally: PI is the double literal 3.14
 *    (pch.h:30) and any expression touching it is evaluated in double and
 *    rounded to float on assignment; vector-by-scalar products convert the
 *    scalar to float first (SIMD vector classes take float scalars).
 *  - dot(a,b) = (ax*bx + ay*by) + az*bz; normalize(v) = v / |v|.
 *  - No fused multiply-add (built with -ffp-contract=off); IEEE division and
 *    square root; transcendental functions from include/wpbr_fmath.h.
 *  - [wml] internal constants use pi = 3.14159265f (float).
 */
#ifndef WPBR_ORACLE_MATH_HPP
#define WPBR_ORACLE_MATH_HPP

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "wpbr_fmath.h"
#include "wpbr_sampling.h"
#include "wpbr_scene.h"

namespace orc {

using namespace wpbr_fm;

static constexpr double PI_D = 3.14;                 /* pch.h:30 */
static constexpr float WML_PI = 0x1.921fb6p+1f;      /* [wml] */

struct V3 {
  float x, y, z;
};
struct V2 {
  float x, y;
};

inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float length2(V3 v) { return dot(v, v); }
inline float length(V3 v) { return sqrt_(length2(v)); }
inline V3 normalize(V3 v) { return v / length(v); }
inline bool is_zero(V3 v) { return v.x == 0.0f && v.y == 0.0f && v.z == 0.0f; }
inline float comp(V3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
inline V3 vmin(V3 a, V3 b) {
  return V3{b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y, b.z < a.z ? b.z : a.z};
}
inline V3 vmax(V3 a, V3 b) {
  return V3{a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y, a.z < b.z ? b.z : a.z};
}

/* RGB spectrum (the RGB3 instantiation of the reference's Spectrum). */
struct RGB {
  float r, g, b;
};
inline RGB rgb(float v) { return RGB{v, v, v}; }
inline RGB operator+(RGB a, RGB b) { return RGB{a.r + b.r, a.g + b.g, a.b + b.b}; }
inline RGB operator*(RGB a, RGB b) { return RGB{a.r * b.r, a.g * b.g, a.b * b.b}; }
inline RGB operator*(RGB a, float s) { return RGB{a.r * s, a.g * s, a.b * s}; }
inline bool is_black(RGB a) { return a.r == 0.0f && a.g == 0.0f && a.b == 0.0f; }

/* ---- transforms (row-major, column vectors) ------------------------------ */
struct M4 {
  float m[4][4];
};
inline M4 m4(const wpbr_mat4& a) {
  M4 r;
  memcpy(r.m, a.m, sizeof(r.m));
  return r;
}
inline M4 identity() {
  M4 r{};
  for (int i = 0; i < 4; ++i) r.m[i][i] = 1.0f;
  return r;
}
inline V3 xf_point(const M4& M, V3 p) {
  const float(*m)[4] = M.m;
  float x = ((m[0][0] * p.x + m[0][1] * p.y) + m[0][2] * p.z) + m[0][3];
  float y = ((m[1][0] * p.x + m[1][1] * p.y) + m[1][2] * p.z) + m[1][3];
  float z = ((m[2][0] * p.x + m[2][1] * p.y) + m[2][2] * p.z) + m[2][3];
  float w = ((m[3][0] * p.x + m[3][1] * p.y) + m[3][2] * p.z) + m[3][3];
  if (w == 1.0f) return V3{x, y, z};
  return V3{x / w, y / w, z / w};
}
inline V3 xf_vector(const M4& M, V3 v) {
  const float(*m)[4] = M.m;
  return V3{(m[0][0] * v.x + m[0][1] * v.y) + m[0][2] * v.z,
            (m[1][0] * v.x + m[1][1] * v.y) + m[1][2] * v.z,
            (m[2][0] * v.x + m[2][1] * v.y) + m[2][2] * v.z};
}
/* Normals transform by the inverse transpose; Minv is the inverse matrix. */
inline V3 xf_normal(const M4& Minv, V3 n) {
  const float(*m)[4] = Minv.m;
  return V3{(m[0][0] * n.x + m[1][0] * n.y) + m[2][0] * n.z,
            (m[0][1] * n.x + m[1][1] * n.y) + m[2][1] * n.z,
            (m[0][2] * n.x + m[1][2] * n.y) + m[2][2] * n.z};
}
/* "A then B" — the reference composes left-first (R/CSCameraProjective.h:35-47:
 * screenRaster = T * S1 * S2 maps screen to raster only if T applies first). */
inline M4 compose(const M4& A, const M4& B) {
  M4 C;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      C.m[i][j] = ((B.m[i][0] * A.m[0][j] + B.m[i][1] * A.m[1][j]) + B.m[i][2] * A.m[2][j]) +
                  B.m[i][3] * A.m[3][j];
  return C;
}
/* [wml] inverse: Gauss-Jordan with partial pivoting in double, rounded to float. */
inline M4 inverse(const M4& M) {
  double a[4][8];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 8; ++j) a[i][j] = j < 4 ? (double)M.m[i][j] : (j - 4 == i ? 1.0 : 0.0);
  for (int c = 0; c < 4; ++c) {
    int piv = c;
    for (int r = c + 1; r < 4; ++r)
      if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
    if (piv != c)
      for (int j = 0; j < 8; ++j) {
        double t = a[c][j];
        a[c][j] = a[piv][j];
        a[piv][j] = t;
      }
    double d = a[c][c];
    for (int j = 0; j < 8; ++j) a[c][j] /= d;
    for (int r = 0; r < 4; ++r)
      if (r != c) {
        double f = a[r][c];
        if (f != 0.0)
          for (int j = 0; j < 8; ++j) a[r][j] -= f * a[c][j];
      }
  }
  M4 R;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) R.m[i][j] = (float)a[i][j + 4];
  return R;
}
inline M4 translate(float x, float y, float z) {
  M4 r = identity();
  r.m[0][3] = x;
  r.m[1][3] = y;
  r.m[2][3] = z;
  return r;
}
inline M4 scale(float x, float y, float z) {
  M4 r = identity();
  r.m[0][0] = x;
  r.m[1][1] = y;
  r.m[2][2] = z;
  return r;
}
/* [wml] makePerspective (pbrt Perspective): Scale(invTan, invTan, 1) applied
 * after the projective divide matrix. */
inline M4 perspective(float fov_deg, float n, float f) {
  float rad = fov_deg * (WML_PI / 180.0f);
  float inv_tan = 1.0f / tanf_(rad / 2.0f);
  M4 r{};
  r.m[0][0] = inv_tan;
  r.m[1][1] = inv_tan;
  r.m[2][2] = f / (f - n);
  r.m[2][3] = -(f * n) / (f - n);
  r.m[3][2] = 1.0f;
  return r;
}

/* ---- rays and bounds --------------------------------------------------- */
struct Ray {
  V3 o, d;
};
inline V3 ray_at(const Ray& r, float t) { return r.o + r.d * t; }
inline Ray xf_ray(const M4& M, const Ray& r) { return Ray{xf_point(M, r.o), xf_vector(M, r.d)}; }

struct Bounds {
  V3 pmin{FLT_MAX, FLT_MAX, FLT_MAX};
  V3 pmax{-FLT_MAX, -FLT_MAX, -FLT_MAX};
};
inline Bounds bunion(const Bounds& a, const Bounds& b) { return Bounds{vmin(a.pmin, b.pmin), vmax(a.pmax, b.pmax)}; }
inline Bounds bunion(const Bounds& a, V3 p) { return Bounds{vmin(a.pmin, p), vmax(a.pmax, p)}; }
inline Bounds bpoint(V3 p) { return Bounds{p, p}; }
/* CCentroid(bounds) = pMax*0.5 + pMin*0.5 (R/CCentroid.h:11-13) */
inline V3 centroid(const Bounds& b) { return b.pmax * 0.5f + b.pmin * 0.5f; }
/* [wml] surface area and dominant axis (pbrt Bounds3::SurfaceArea/MaximumExtent) */
inline float area(const Bounds& b) {
  V3 d = b.pmax - b.pmin;
  return 2.0f * ((d.x * d.y + d.x * d.z) + d.y * d.z);
}
inline int max_extent(const Bounds& b) {
  V3 d = b.pmax - b.pmin;
  if (d.x > d.y && d.x > d.z) return 0;
  if (d.y > d.z) return 1;
  return 2;
}
/* pbrt's robust slab test scale 1 + 2*gamma(3) in float. */
static constexpr float kSlabScale = 0x1.000006p+0f;

/* [wml] DBounds3f::intersect(ray, dirInv, dirIsNeg) — R/SLBVH.cpp:106;
 * pbrt Bounds3::IntersectP with ray.tMax = tmax. Returns entry t via tmin_out. */
inline bool slab(const Bounds& b, const Ray& r, V3 inv, const int neg[3], float tmax_ray, float* tmin_out) {
  V3 lo = b.pmin, hi = b.pmax;
  float tMin = ((neg[0] ? hi.x : lo.x) - r.o.x) * inv.x;
  float tMax = ((neg[0] ? lo.x : hi.x) - r.o.x) * inv.x;
  float tyMin = ((neg[1] ? hi.y : lo.y) - r.o.y) * inv.y;
  float tyMax = ((neg[1] ? lo.y : hi.y) - r.o.y) * inv.y;
  tMax *= kSlabScale;
  tyMax *= kSlabScale;
  if (tMin > tyMax || tyMin > tMax) return false;
  if (tyMin > tMin) tMin = tyMin;
  if (tyMax < tMax) tMax = tyMax;
  float tzMin = ((neg[2] ? hi.z : lo.z) - r.o.z) * inv.z;
  float tzMax = ((neg[2] ? lo.z : hi.z) - r.o.z) * inv.z;
  tzMax *= kSlabScale;
  if (tMin > tzMax || tzMin > tMax) return false;
  if (tzMin > tMin) tMin = tzMin;
  if (tzMax < tMax) tMax = tzMax;
  *tmin_out = tMin;
  return (tMin < tmax_ray) && (tMax > 0.0f);
}

/* ---- primitive intersection -------------------------------------------- */
/* [wml] getRootsQuadraticEquation — pbrt-v3 Quadratic (double discriminant). */
inline bool quadratic(float a, float b, float c, float* t0, float* t1) {
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

/* SSphere::intersect (R/CSSphere.cpp:84-120). Returns t (0 = miss) and the
 * object-space ray / hit point the full interaction needs. */
inline float sphere_intersect(const M4& w2o, float radius, const Ray& rw, Ray* ray_l, V3* p_hit_l) {
  Ray rl = xf_ray(w2o, rw);
  float a = length2(rl.d);
  float b = 2.0f * dot(rl.d, rl.o);
  float c = length2(rl.o) - radius * radius;
  float t0, t1;
  if (!quadratic(a, b, c, &t0, &t1)) return 0.0f;
  if (t1 <= 0.0f) return 0.0f;
  float t = t0;
  if (t <= 0.0f) t = t1;
  if (ray_l) *ray_l = rl;
  if (p_hit_l) *p_hit_l = ray_at(rl, t);
  return t;
}

/* JobProcessTriangleInteractionRequests (R/CSTriangle.cpp:9-108): watertight
 * test with the reference's SIMD lane order. Returns t (0 = miss) and the
 * barycentric weights of v0, v1, v2. */
inline float triangle_intersect(V3 p0, V3 p1, V3 p2, const Ray& r, uint32_t quirks, float bary[3]) {
  V3 ad = V3{fabs_(r.d.x), fabs_(r.d.y), fabs_(r.d.z)};
  int kz = (ad.x > ad.y) ? ((ad.x > ad.z) ? 0 : 2) : ((ad.y > ad.z) ? 1 : 2); /* [wml] maxDimension */
  int kx = (kz == 2) ? 0 : kz + 1;
  int ky = (kz == 2) ? 1 : kz + 2; /* 3 when kz == 1 */
  bool lane3 = (ky == 3);
  if (lane3) {
    if (quirks & WPBR_Q_TRI_PERMUTATION_BUG) return 0.0f; /* lane 3 reads 0: det == 0 */
    ky = 0;
  }
  V3 d = V3{comp(r.d, kx), comp(r.d, ky), comp(r.d, kz)};
  float sx = -d.x / d.z, sy = -d.y / d.z, sz = 1.0f / d.z;
  V3 pt[3];
  V3 pv[3] = {p0, p1, p2};
  for (int i = 0; i < 3; ++i) {
    V3 p = pv[i] - r.o;
    p = V3{comp(p, kx), comp(p, ky), comp(p, kz)};
    p = V3{p.x + sx * p.z, p.y + sy * p.z, p.z + 0.0f * p.z};
    pt[i] = p;
  }
  /* res = X*rot(Y) - rot(X)*Y with rot = lanes (1,2,0): res = (e2, e0, e1) */
  float rx = pt[0].x * pt[1].y - pt[1].x * pt[0].y;
  float ry = pt[1].x * pt[2].y - pt[2].x * pt[1].y;
  float rz = pt[2].x * pt[0].y - pt[0].x * pt[2].y;
  if ((rx < 0 || ry < 0 || rz < 0) && (rx > 0 || ry > 0 || rz > 0)) return 0.0f;
  float det = (rx + ry) + rz;
  if (det == 0.0f) return 0.0f;
  float e0 = ry, e1 = rz, e2 = rx; /* res.permuteEach<1,2,0> */
  float z0 = pt[0].z * sz, z1 = pt[1].z * sz, z2 = pt[2].z * sz;
  float t_scaled = (e0 * z0 + e1 * z1) + e2 * z2;
  if (det < 0.0f && t_scaled >= 0.0f) return 0.0f;
  if (det > 0.0f && t_scaled <= 0.0f) return 0.0f;
  float inv_det = (float)(1.0 / (double)det);
  bary[0] = e0 * inv_det;
  bary[1] = e1 * inv_det;
  bary[2] = e2 * inv_det;
  return t_scaled * inv_det;
}

/* ---- surface interaction --------------------------------------------------- */
struct SI {
  V3 p, n, wo;
  V2 uv;
  V3 dpdu, dpdv, dndu, dndv;
  V3 sn, sdpdu, sdpdv, sdndu, sdndv; /* shading.* */
  float t;
  uint32_t prim;
};

/* SSphere::computeSurfInteraction (R/CSSphere.cpp:122-186) followed by
 * CTransform::operator()(CSurfaceInteraction) (R/CTransform.h:41-66), which
 * does not carry uv over. */
inline SI sphere_si(const M4& o2w, const M4& w2o, float radius, const Ray& rl, V3 ph, float t, uint32_t prim) {
  float phi = atan2f_(ph.y, ph.x);
  if (phi < 0.0f) phi = (float)((double)phi + 2.0 * PI_D);
  float u = (float)((double)phi / (2.0 * PI_D));
  float theta = acosf_(ph.z / radius);
  float v = (float)((double)theta / PI_D);
  float inv_zr = (float)(1.0 / (double)sqrt_(ph.x * ph.x + ph.y * ph.y));
  float phi_cos = ph.x * inv_zr;
  float phi_sin = ph.y * inv_zr;
  V3 dpdu = V3{-ph.y, ph.x, 0.0f} * (float)(2.0 * PI_D);
  V3 dpdv = V3{ph.z * phi_cos, ph.z * phi_sin, -radius * sinf_(theta)} * (float)PI_D;
  V3 d2uu = V3{ph.x, ph.y, 0.0f} * (float)(-2.0 * PI_D * 2.0 * PI_D);
  V3 d2uv = ((((V3{-phi_sin, phi_cos, 0.0f} * (float)PI_D) * ph.z) * 2.0f) * (float)PI_D);
  V3 d2vv = (V3{ph.x, ph.y, ph.z} * (float)(-PI_D)) * (float)PI_D;
  float E = dot(dpdu, dpdu), F = dot(dpdu, dpdv), G = dot(dpdv, dpdv);
  V3 N = normalize(cross(dpdu, dpdv));
  float e = dot(N, d2uu), f = dot(N, d2uv), g = dot(N, d2vv);
  float inv = 1.0f / (E * G - F * F);
  V3 dndu = dpdu * ((f * F - e * G) * inv) + dpdv * ((e * F - f * E) * inv);
  V3 dndv = dpdu * ((g * F - f * G) * inv) + dpdv * ((f * F - g * E) * inv);
  /* CSurfaceInteraction ctor (R/CSufraceInteraction.h:59-81) */
  V3 n = normalize(cross(dpdu, dpdv));
  SI s;
  s.p = xf_point(o2w, ph);
  s.n = normalize(xf_normal(w2o, n));
  s.wo = normalize(xf_vector(o2w, -rl.d));
  s.uv = V2{0.0f, 0.0f};
  (void)u;
  (void)v;
  s.dpdu = xf_vector(o2w, dpdu);
  s.dpdv = xf_vector(o2w, dpdv);
  s.dndu = xf_normal(w2o, dndu);
  s.dndv = xf_normal(w2o, dndv);
  s.sn = normalize(xf_normal(w2o, n));
  s.sdpdu = xf_vector(o2w, dpdu);
  s.sdpdv = xf_vector(o2w, dpdv);
  s.sdndu = xf_vector(o2w, dndu);
  s.sdndv = xf_vector(o2w, dndv);
  s.t = t;
  s.prim = prim;
  return s;
}

struct TriVerts {
  V3 p[3];
  V3 n[3], s[3];
  V2 uv[3];
  bool has_ns, has_uv;
};

/* JobProcessTriangleFullInteractionRequests (R/CSTriangle.cpp:149-319). */
inline SI triangle_si(const TriVerts& tv, const Ray& r, const float b[3], float t, uint32_t prim) {
  V2 uv[3];
  if (!tv.has_uv) {
    uv[0] = V2{0.0f, 0.0f};
    uv[1] = V2{1.0f, 0.0f};
    uv[2] = V2{1.0f, 1.0f};
  } else {
    uv[0] = tv.uv[0];
    uv[1] = tv.uv[1];
    uv[2] = tv.uv[2];
  }
  V3 dp02 = tv.p[0] - tv.p[2], dp12 = tv.p[1] - tv.p[2];
  V2 duv02{uv[0].x - uv[2].x, uv[0].y - uv[2].y};
  V2 duv12{uv[1].x - uv[2].x, uv[1].y - uv[2].y};
  float det = duv02.x * duv12.y - duv02.y * duv12.x;
  if (det == 0.0f) {
    const float s = (float)0.001;
    uv[0] = V2{0.0f * s, 0.0f * s};
    uv[1] = V2{1.0f * s, 0.0f * s};
    uv[2] = V2{1.0f * s, 1.0f * s};
    duv02 = V2{uv[0].x - uv[2].x, uv[0].y - uv[2].y};
    duv12 = V2{uv[1].x - uv[2].x, uv[1].y - uv[2].y};
    det = duv02.x * duv12.y - duv02.y * duv12.x;
  }
  float det_inv = 1.0f / det;
  V3 dpdu = (dp02 * duv12.y - dp12 * duv02.y) * det_inv;
  V3 dpdv = ((-dp02) * duv12.x + dp12 * duv02.x) * det_inv;
  V3 phit = (tv.p[0] * b[0] + tv.p[1] * b[1]) + tv.p[2] * b[2];
  V2 uvh{(uv[0].x * b[0] + uv[1].x * b[1]) + uv[2].x * b[2], (uv[0].y * b[0] + uv[1].y * b[1]) + uv[2].y * b[2]};
  SI s;
  s.p = phit;
  s.uv = uvh;
  s.wo = -r.d;
  s.dpdu = dpdu;
  s.dpdv = dpdv;
  s.dndu = V3{0, 0, 0};
  s.dndv = V3{0, 0, 0};
  s.sdpdu = dpdu;
  s.sdpdv = dpdv;
  s.sdndu = V3{0, 0, 0};
  s.sdndv = V3{0, 0, 0};
  s.t = t;
  s.prim = prim;
  s.n = normalize(cross(dp02, dp12));
  s.sn = s.n;
  if (tv.has_ns) {
    V3 ns = (tv.n[0] * b[0] + tv.n[1] * b[1]) + tv.n[2] * b[2];
    ns = !is_zero(ns) ? normalize(ns) : s.n;
    V3 ss = (tv.s[0] * b[0] + tv.s[1] * b[1]) + tv.s[2] * b[2];
    ss = !is_zero(ss) ? normalize(ss) : normalize(s.dpdu);
    V3 ts = cross(ss, ns);
    if (length2(ts) > 0.0f) {
      ts = normalize(ts);
      ss = cross(ts, ns);
    }
    V3 dn02 = tv.n[0] - tv.n[2], dn12 = tv.n[1] - tv.n[2];
    V3 dndu{0, 0, 0}, dndv{0, 0, 0};
    float det2 = duv02.x * duv12.y - duv02.y * duv12.x;
    if (det2 != 0.0f) {
      float inv2 = 1.0f / det2;
      dndu = (dn02 * duv12.y - dn12 * duv02.y) * inv2;
      dndv = ((-dn02) * duv12.x + dn12 * duv02.x) * inv2;
    }
    /* setShadingGeometry(ss, ts, dndu, dndv, true) (R/CSufraceInteraction.h:171-196) */
    s.sn = normalize(cross(ss, ts));
    s.sdpdu = ss;
    s.sdpdv = ts;
    s.sdndu = dndu;
    s.sdndv = dndv;
    if (dot(s.n, s.sn) < 0.0f) s.n = -s.n; /* [wml] faceForward */
  }
  return s;
}

/* ---- BSDF local frame (JobBSDFComputeTransform, R/CBSDF.cpp:12-24) ----------- */
struct Frame {
  V3 ss, ts, ns;
};
inline Frame bsdf_frame(const SI& s) {
  Frame f;
  f.ss = normalize(s.sdpdu);
  f.ns = s.sn;
  f.ts = cross(f.ns, f.ss);
  return f;
}
/* world(v): rows (ss, ts, ns) */
inline V3 to_local(const Frame& f, V3 v) { return V3{dot(f.ss, v), dot(f.ts, v), dot(f.ns, v)}; }
/* world(v, INV_TRANFORM): transpose */
inline V3 to_world(const Frame& f, V3 v) {
  return V3{(f.ss.x * v.x + f.ts.x * v.y) + f.ns.x * v.z, (f.ss.y * v.x + f.ts.y * v.y) + f.ns.y * v.z,
            (f.ss.z * v.x + f.ts.z * v.y) + f.ns.z * v.z};
}

/* ---- shading-space trigonometry [wml] ------------------------------------ */
inline float cos2t(V3 w) { return w.z * w.z; }
inline float abs_cos(V3 w) { return fabs_(w.z); }
inline float sin2t(V3 w) {
  float v = 1.0f - cos2t(w);
  return 0.0f < v ? v : 0.0f;
}
inline float sint(V3 w) { return sqrt_(sin2t(w)); }
inline float tan2t(V3 w) { return sin2t(w) / cos2t(w); }
inline float clampf(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }
inline float cosphi(V3 w) {
  float st = sint(w);
  return (st == 0.0f) ? 1.0f : clampf(w.x / st, -1.0f, 1.0f);
}
inline float sinphi(V3 w) {
  float st = sint(w);
  return (st == 0.0f) ? 0.0f : clampf(w.y / st, -1.0f, 1.0f);
}
inline bool same_hemi(V3 a, V3 b) { return a.z * b.z > 0.0f; }
inline V3 reflect(V3 wo, V3 n) { return (-wo) + n * (2.0f * dot(wo, n)); }
inline V3 spherical_dir(float st, float ct, float phi) { return V3{st * cosf_(phi), st * sinf_(phi), ct}; }
inline V3 spherical_dir(float st, float ct, float phi, V3 x, V3 y, V3 z) {
  return (x * (st * cosf_(phi)) + y * (st * sinf_(phi))) + z * ct;
}
inline float spherical_theta(V3 v) { return acosf_(clampf(v.z, -1.0f, 1.0f)); }
inline float spherical_phi(V3 v) {
  float p = atan2f_(v.y, v.x);
  return (p < 0.0f) ? p + 2.0f * WML_PI : p;
}
inline void make_basis(V3 v1, V3* v2, V3* v3) {
  if (fabs_(v1.x) > fabs_(v1.y))
    *v2 = V3{-v1.z, 0.0f, v1.x} / sqrt_(v1.x * v1.x + v1.z * v1.z);
  else
    *v2 = V3{0.0f, v1.z, -v1.y} / sqrt_(v1.y * v1.y + v1.z * v1.z);
  *v3 = cross(v1, *v2);
}
inline float cone_pdf(float cos_max) { return 1.0f / (2.0f * WML_PI * (1.0f - cos_max)); }

/* ---- Fresnel (R/CBXDF.h:23-62, 200-238) ---------------------------------- */
inline float fresnel_dielectric(float cos_i, float eta_i, float eta_t) {
  cos_i = clampf(cos_i, -1.0f, 1.0f);
  float ei = eta_i, et = eta_t;
  bool entering = cos_i > 0.0f;
  if (!entering) {
    float t = ei;
    ei = et;
    et = t;
    cos_i = fabs_(cos_i);
  }
  double a = 1.0 - (double)(cos_i * cos_i);
  float sin_i = (float)sqrt_d(0.0 > a ? 0.0 : a);
  float sin_t = ei / et * sin_i;
  if ((double)sin_t >= 1.0) return 1.0f;
  double b = 1.0 - (double)(sin_t * sin_t);
  float cos_t = (float)sqrt_d(0.0 > b ? 0.0 : b);
  float r_parl = ((et * cos_i) - (ei * cos_t)) / ((et * cos_i) + (ei * cos_t));
  float r_perp = ((ei * cos_i) - (et * cos_t)) / ((ei * cos_i) + (et * cos_t));
  return (r_parl * r_parl + r_perp * r_perp) / 2.0f;
}
inline float fresnel_conductor1(float cos_i, float eta_i, float eta_t, float kk) {
  cos_i = clampf(cos_i, -1.0f, 1.0f);
  float eta = eta_t / eta_i;
  float etak = kk / eta_i;
  float c2 = cos_i * cos_i;
  float s2 = (float)(1.0 - (double)c2);
  float eta2 = eta * eta;
  float etak2 = etak * etak;
  float t0 = (eta2 - etak2) - s2;
  float a2pb22 = t0 * t0 + (eta2 * etak2) * 4.0f;
  float a2pb2 = sqrt_(a2pb22);
  float t1 = a2pb2 + c2;
  float a = sqrt_((a2pb2 + t0) * 0.5f);
  float t2 = (a * cos_i) * 2.0f;
  float Rs = (t1 - t2) / (t1 + t2);
  float t3 = a2pb2 * c2 + s2 * s2;
  float t4 = t2 * s2;
  float Rp = (Rs * (t3 - t4)) / (t3 + t4);
  return (Rp + Rs) * 0.5f;
}

/* ---- Trowbridge-Reitz (R/MicrofaceDistr.h:12-88) --------------------------- */
inline float tr_d(float ax, float ay, V3 wh) {
  float t2 = tan2t(wh);
  if (std::isinf(t2)) return 0.0f;
  float c4 = cos2t(wh) * cos2t(wh);
  float cp = cosphi(wh), sp = sinphi(wh);
  float e = ((cp * cp) / (ax * ax) + (sp * sp) / (ay * ay)) * t2;
  double den = ((((PI_D * (double)ax) * (double)ay) * (double)c4) * (double)(1.0f + e)) * (double)(1.0f + e);
  return (float)(1.0 / den);
}
inline float tr_pdf(float d_wh, V3 wh) { return d_wh * abs_cos(wh); }
inline float roughness_to_alpha(float r) {
  r = r > 1e-3f ? r : 1e-3f;
  float x = logf_(r);
  return (((1.62142f + 0.819955f * x) + (0.1734f * x) * x) + ((0.0171201f * x) * x) * x) +
         (((0.000640711f * x) * x) * x) * x;
}
inline V3 tr_sample(float ax, float ay, V3 wo, float u0, float u1, float* d_out) {
  float cos_t = 0.0f;
  float phi = (float)((2.0 * PI_D) * (double)u1);
  if (ax == ay) {
    float tan2 = ((ax * ax) * u0) / (1.0f - u0);
    cos_t = 1.0f / sqrt_(1.0f + tan2);
  } else {
    phi = atanf_(ay / ax * tanf_((float)((2.0 * PI_D) * (double)u1 + 0.5 * PI_D)));
    if (u1 > 0.5f) phi = (float)((double)phi + PI_D);
    float sp = sinf_(phi), cp = cosf_(phi);
    float ax2 = ax * ax, ay2 = ay * ay;
    float alpha2 = 1.0f / ((cp * cp) / ax2 + (sp * sp) / ay2);
    float tan2 = (alpha2 * u0) / (1.0f - u0);
    cos_t = 1.0f / sqrt_(1.0f + tan2);
  }
  float v = 1.0f - cos_t * cos_t;
  float sin_t = sqrt_(0.0f > v ? 0.0f : v);
  V3 wh = spherical_dir(sin_t, cos_t, phi);
  if (!same_hemi(wo, wh)) wh = -wh;
  *d_out = tr_d(ax, ay, wh);
  return wh;
}

}  // namespace orc

#endif  // WPBR_ORACLE_MATH_HPP
