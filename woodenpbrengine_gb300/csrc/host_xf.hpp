// host_xf.hpp — host-only transform constructors for scene setup: inverse,
// translate/scale/rotate, perspective, look-at. Results are plain float
// matrices in the library's row-major, column-vector convention.
#pragma once

#include <cmath>

#include "geom.cuh"

namespace wpbr {

// Gauss-Jordan elimination with partial pivoting in double, rounded to float
// (WoodenMath's DTransform inverse is not available; this is the library's
// definition).
inline Xf xf_inverse(const Xf& M) {
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
  Xf R;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) R.m[i][j] = (float)a[i][j + 4];
  return R;
}

inline Xf xf_translate(float x, float y, float z) {
  Xf r = xf_identity();
  r.m[0][3] = x;
  r.m[1][3] = y;
  r.m[2][3] = z;
  return r;
}
inline Xf xf_scale(float x, float y, float z) {
  Xf r = xf_identity();
  r.m[0][0] = x;
  r.m[1][1] = y;
  r.m[2][2] = z;
  return r;
}
// makePerspective(fov, n, f): the projective divide matrix followed by
// Scale(1/tan(fov/2), 1/tan(fov/2), 1).
inline Xf xf_perspective(float fov_deg, float n, float f) {
  float rad = fov_deg * (kMathPi / 180.0f);
  float inv_tan = 1.0f / tanf_(rad / 2.0f);
  Xf r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) r.m[i][j] = 0.0f;
  r.m[0][0] = inv_tan;
  r.m[1][1] = inv_tan;
  r.m[2][2] = f / (f - n);
  r.m[2][3] = -(f * n) / (f - n);
  r.m[3][2] = 1.0f;
  return r;
}
// Camera-to-world frame looking from eye at target: columns (right, up,
// forward, eye); +z forward in camera space.
inline Xf xf_look_at(V3 eye, V3 target, V3 up) {
  V3 dir = normalize(sub(target, eye));
  V3 right = normalize(cross(normalize(up), dir));
  V3 nup = cross(dir, right);
  Xf r = xf_identity();
  r.m[0][0] = right.x; r.m[1][0] = right.y; r.m[2][0] = right.z;
  r.m[0][1] = nup.x;   r.m[1][1] = nup.y;   r.m[2][1] = nup.z;
  r.m[0][2] = dir.x;   r.m[1][2] = dir.y;   r.m[2][2] = dir.z;
  r.m[0][3] = eye.x;   r.m[1][3] = eye.y;   r.m[2][3] = eye.z;
  return r;
}

}  // namespace wpbr
