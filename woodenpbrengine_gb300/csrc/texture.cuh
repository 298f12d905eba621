// texture.cuh — textured metal (WPBR_MAT_METAL): ray differentials at the
// hit (CSurfaceInteraction::computeDifferentials,
// WoodenPBREngine/CSufraceInteraction.h:98-148), texture mapping
// (TextureMappingUV / TextureMappingSphere, CTextureMapping.h:39-94),
// MIP-mapped bilinear and anisotropic EWA lookups
// (STexture2DSampler::triangle, STexture2DSamplerAnisotropic::eval / ewa,
// CSTextureProcess.h:56-239) and the material built from them
// (JobGenerateBSDFMaterialMetal, CMaterialMetal.cpp:8-58).
#pragma once

#include "camera.cuh"
#include "geom.cuh"
#include "shade.cuh"

namespace wpbr {

constexpr int kGaussTable = 64;       // CFilterTableGaussing size (MEngine.cpp:92-94)
constexpr float kMaxAnisotropy = 32;  // CMaterialMetal.cpp:31

struct TexLevel {
  uint32_t offset, w, h, pad;  // texels of the level start at `offset` (row-major)
};
struct TexInfo {
  uint32_t first_level, n_levels;
};
struct TexView {
  const float4* texels;
  const TexLevel* levels;
  const TexInfo* tex;
  const float* gauss;  // kGaussTable weights
  uint32_t n_tex;
};

struct TexFootprint {
  V2 p, dstdx, dstdy;
};

WPBR_HD RGB3 tex_texel(const TexView& T, const TexLevel& L, int x, int y) {
  float4 v = T.texels[L.offset + (uint32_t)y * L.w + (uint32_t)x];
  return RGB3{v.x, v.y, v.z};
}

// Bilinear lookup; the lower clamp keeps the extrapolating weights, indices
// past the last texel are clamped (the reference reads past the row).
WPBR_HD RGB3 tex_triangle(const TexView& T, const TexInfo& ti, V2 st, uint32_t mip) {
  if (mip > ti.n_levels - 1) mip = ti.n_levels - 1;
  const TexLevel& L = T.levels[ti.first_level + mip];
  int W = (int)L.w, H = (int)L.h;
  float s = st.x * (float)W - 0.5f;
  float t = st.y * (float)H - 0.5f;
  int s0 = (int)floorf(s), t0 = (int)floorf(t);
  s0 = s0 > 0 ? s0 : 0;
  t0 = t0 > 0 ? t0 : 0;
  float ds = s - (float)s0, dt = t - (float)t0;
  int s0n = s0 + 1 < W - 1 ? s0 + 1 : W - 1;
  int t0n = t0 + 1 < H - 1 ? t0 + 1 : H - 1;
  s0n = s0n > 0 ? s0n : 0;
  t0n = t0n > 0 ? t0n : 0;
  s0 = s0 < W - 1 ? s0 : W - 1;
  t0 = t0 < H - 1 ? t0 : H - 1;
  RGB3 a = rmuls(rmuls(tex_texel(T, L, s0, t0), 1.0f - ds), 1.0f - dt);
  RGB3 b = rmuls(rmuls(tex_texel(T, L, s0, t0n), 1.0f - ds), dt);
  RGB3 c = rmuls(rmuls(tex_texel(T, L, s0n, t0), ds), 1.0f - dt);
  RGB3 d = rmuls(rmuls(tex_texel(T, L, s0n, t0n), ds), dt);
  return radd(radd(radd(a, b), c), d);
}

// Elliptically weighted average over one level with the Gaussian table.
WPBR_HD RGB3 tex_ewa(const TexView& T, const TexInfo& ti, const TexFootprint& fp, uint32_t mip) {
  const TexLevel& L = T.levels[ti.first_level + mip];
  float rx = (float)L.w, ry = (float)L.h;
  float sx = fp.p.x * rx - 0.5f, sy = fp.p.y * ry - 0.5f;
  float d0x = fp.dstdx.x * rx, d0y = fp.dstdx.y * ry;
  float d1x = fp.dstdy.x * rx, d1y = fp.dstdy.y * ry;
  float A = (d0y * d0y + d1y * d1y) + 1.0f;
  float B = -2.0f * (d0x * d0y + d1x * d1y);
  float C = (d0x * d0x + d1x * d1x) + 1.0f;
  float invF = 1.0f / (A * C - (B * B) * 0.25f);
  A = A * invF;
  B = B * invF;
  C = C * invF;
  float det = -B * B + (4.0f * A) * C;
  float invDet = 1.0f / det;
  float us = sqrt_(C * det) * (2.0f * invDet);
  float vs = sqrt_(A * det) * (2.0f * invDet);
  float s0f = clampf(sx - us, 0.0f, rx - 1.0f), t0f = clampf(sy - vs, 0.0f, ry - 1.0f);
  float s1f = clampf(sx + us, 0.0f, rx - 1.0f), t1f = clampf(sy + vs, 0.0f, ry - 1.0f);
  int is0 = (int)ceilf(s0f), it0 = (int)ceilf(t0f);
  int is1 = (int)floorf(s1f), it1 = (int)floorf(t1f);
  // a NaN footprint (from a NaN hit frame): no texel is visited, 0 / 0
  if (!(s0f == s0f && t0f == t0f && s1f == s1f && t1f == t1f)) {
    is0 = it0 = 1;
    is1 = it1 = 0;
  }
  RGB3 sum = rgb1(0.0f);
  float sw = 0.0f;
  for (int it = it0; it <= it1; ++it) {
    float tt = (float)it - sy;
    for (int is = is0; is <= is1; ++is) {
      float ss = (float)is - sx;
      float r2 = ((A * ss) * ss + (B * ss) * tt) + (C * tt) * tt;
      if (r2 < 1.0f) {
        int idx = (int)(r2 * (float)kGaussTable);
        if (idx > kGaussTable - 1) idx = kGaussTable - 1;
        float w = T.gauss[idx];
        sum = radd(sum, rmuls(tex_texel(T, L, is, it), w));
        sw = sw + w;
      }
    }
  }
  return RGB3{sum.r / sw, sum.g / sw, sum.b / sw};
}

WPBR_HD RGB3 rlerp(float t, RGB3 a, RGB3 b) {
  return RGB3{(1.0f - t) * a.r + t * b.r, (1.0f - t) * a.g + t * b.g, (1.0f - t) * a.b + t * b.b};
}

// STexture2DSamplerAnisotropic::eval. The reference compares dstdx with itself
// when picking the major axis (never swaps) and hands ewa the unclamped
// derivatives; the clamped minor axis only chooses the level.
WPBR_HD RGB3 tex_aniso(const TexView& T, uint32_t texid, const TexFootprint& fp) {
  const TexInfo& ti = T.tex[texid];
  V2 d1 = fp.dstdy;
  float major = sqrt_(fp.dstdx.x * fp.dstdx.x + fp.dstdx.y * fp.dstdx.y);
  float minor = sqrt_(d1.x * d1.x + d1.y * d1.y);
  if (minor * kMaxAnisotropy < major && minor > 0.0f) {
    float scale = major / (minor * kMaxAnisotropy);
    minor = minor * scale;
  }
  if (minor == 0.0f) return tex_triangle(T, ti, fp.p, 0);
  uint32_t n = ti.n_levels;
  float lod = (float)(n - 1) + log2f_(minor > 0.0f ? minor : 0.0f);
  lod = lod > 0.0f ? lod : 0.0f;
  int ilod = (int)floorf(lod);
  if (ilod >= (int)n - 1) return tex_ewa(T, ti, fp, n - 1);
  return rlerp(lod - (float)ilod, tex_ewa(T, ti, fp, (uint32_t)ilod), tex_ewa(T, ti, fp, (uint32_t)ilod + 1));
}

// STexture2DSamplerIsotropic::eval: the width is twice the largest signed
// derivative component (negative components never widen it); a width <= 0
// reads the finest level bilinearly, a level at or past the coarsest reads
// texel (0, 0) of the coarsest level, otherwise two bilinear levels are
// blended.
WPBR_HD RGB3 tex_iso(const TexView& T, uint32_t texid, const TexFootprint& fp) {
  const TexInfo& ti = T.tex[texid];
  float a = fp.dstdx.x < fp.dstdx.y ? fp.dstdx.y : fp.dstdx.x;
  float b = fp.dstdy.x < fp.dstdy.y ? fp.dstdy.y : fp.dstdy.x;
  float width = 2.0f * (a < b ? b : a);
  if (!(width > 0.0f)) return tex_triangle(T, ti, fp.p, 0);
  uint32_t n = ti.n_levels;
  float level = (float)(n - 1) + log2f_(width);
  if (level < 0.0f) return tex_triangle(T, ti, fp.p, 0);
  if (level >= (float)(n - 1)) return tex_texel(T, T.levels[ti.first_level + n - 1], 0, 0);
  int il = (int)floorf(level);
  return rlerp(level - (float)il, tex_triangle(T, ti, fp.p, (uint32_t)il), tex_triangle(T, ti, fp.p, (uint32_t)il + 1));
}

// pbrt's SolveLinearSystem2x2 (WoodenMath solveLinearSystem2x2).
WPBR_HD bool solve2x2(const float A[2][2], const float B[2], float* x0, float* x1) {
  float det = A[0][0] * A[1][1] - A[0][1] * A[1][0];
  if (fabs_(det) < 1e-10f) return false;
  *x0 = (A[1][1] * B[0] - A[0][1] * B[1]) / det;
  *x1 = (A[0][0] * B[1] - A[1][0] * B[0]) / det;
  if (*x0 != *x0 || *x1 != *x1) return false;
  return true;
}

struct SurfDiff {
  V3 dpdx, dpdy;
  float dudx, dvdx, dudy, dvdy;
};

WPBR_HD SurfDiff surf_differentials(const SurfInt& s, const RayD& r) {
  SurfDiff D;
  float d = dot(s.n, s.p);
  float tx = -(dot(s.n, r.dxo) - d) / dot(s.n, r.dxd);
  V3 px = add(r.dxo, mul(r.dxd, tx));
  float ty = -(dot(s.n, r.dyo) - d) / dot(s.n, r.dyd);
  V3 py = add(r.dyo, mul(r.dyd, ty));
  D.dpdx = sub(px, s.p);
  D.dpdy = sub(py, s.p);
  int d0, d1;
  float ax = fabs_(s.n.x), ay = fabs_(s.n.y), az = fabs_(s.n.z);
  if (ax > ay && ax > az) {
    d0 = 1;
    d1 = 2;
  } else if (ay > az) {
    d0 = 0;
    d1 = 2;
  } else {
    d0 = 0;
    d1 = 1;
  }
  const float A[2][2] = {{comp(s.dpdu, d0), comp(s.dpdv, d0)}, {comp(s.dpdu, d1), comp(s.dpdv, d1)}};
  const float Bx[2] = {comp(px, d0) - comp(s.p, d0), comp(px, d1) - comp(s.p, d1)};
  const float By[2] = {comp(py, d0) - comp(s.p, d0), comp(py, d1) - comp(s.p, d1)};
  if (!solve2x2(A, Bx, &D.dudx, &D.dvdx)) D.dudx = D.dvdx = 0.0f;
  if (!solve2x2(A, By, &D.dudy, &D.dvdy)) D.dudy = D.dvdy = 0.0f;
  return D;
}

// TextureMappingSphere::sphere: (theta / PI, phi / (2 PI)) of the object-space
// direction of the point.
WPBR_HD V2 sphere_st(const Xf& w2o, V3 p) {
  V3 v = normalize(xpoint(w2o, p));
  float theta = sph_theta(v), phi = sph_phi(v);
  return V2{(float)((double)theta * 1.0 / kPI), (float)((double)phi / (2.0 * kPI))};
}

WPBR_HD float sphere_wrap(float x) {
  if ((double)x > 0.5) return 1.0f - x;
  if (x < -0.5f) return -x + 1.0f;
  return x;
}

WPBR_HD TexFootprint sphere_footprint(const Xf& w2o, const SurfInt& s, const SurfDiff& D) {
  TexFootprint fp;
  V2 st = sphere_st(w2o, s.p);
  const float dt = 0.1f;
  V2 stdx = sphere_st(w2o, add(s.p, mul(D.dpdx, dt)));
  V2 stdy = sphere_st(w2o, add(s.p, mul(D.dpdy, dt)));
  fp.dstdx = V2{(stdx.x - st.x) / dt, (stdx.y - st.y) / dt};
  fp.dstdy = V2{(stdy.x - st.x) / dt, (stdy.y - st.y) / dt};
  fp.dstdx.y = sphere_wrap(fp.dstdx.y);
  fp.dstdy.y = sphere_wrap(fp.dstdy.y);
  fp.p = st;
  return fp;
}

// TextureMappingUV::map with scale (1, 1) and offset (0, 0).
WPBR_HD TexFootprint uv_footprint(const SurfInt& s, const SurfDiff& D) {
  TexFootprint fp;
  fp.dstdx = V2{1.0f * D.dudx + 0.0f, 1.0f * D.dvdx + 0.0f};
  fp.dstdy = V2{1.0f * D.dudy + 0.0f, 1.0f * D.dvdy + 0.0f};
  fp.p = V2{1.0f * s.uv.x + 0.0f, 1.0f * s.uv.y + 0.0f};
  return fp;
}

// roughnessToAlpha (MicrofaceDistr.h:18-24)
WPBR_HD float roughness_to_alpha(float r) {
  r = r > 1e-3f ? r : 1e-3f;
  float x = logf_(r);
  return (((1.62142f + 0.819955f * x) + (0.1734f * x) * x) + ((0.0171201f * x) * x) * x) +
         (((0.000640711f * x) * x) * x) * x;
}

// JobGenerateBSDFMaterialMetal: the conductor of one hit.
WPBR_HD wpbr_material metal_material(const TexView& T, const wpbr_material& m, const TexFootprint& fp) {
  bool iso = m.type == WPBR_MAT_METAL_ISOTROPIC;
  RGB3 metallic = iso ? tex_iso(T, m.tex[0], fp) : tex_aniso(T, m.tex[0], fp);
  RGB3 rough = iso ? tex_iso(T, m.tex[1], fp) : tex_aniso(T, m.tex[1], fp);
  float sv = clampf(rough.r * 90.0f, 0.0f, 90.0f);
  float alpha = roughness_to_alpha(sv);
  wpbr_material e;
  e.type = WPBR_MAT_CONDUCTOR;
  e.alpha_x = alpha;
  e.alpha_y = alpha;
  for (int c = 0; c < 3; ++c) {
    e.R[c] = 1.0f;
    e.eta_i[c] = 1.0f;
    e.eta_t[c] = 1.5f;
  }
  e.k[0] = metallic.r;
  e.k[1] = metallic.g;
  e.k[2] = metallic.b;
  e.tex[0] = e.tex[1] = 0;
  return e;
}

}  // namespace wpbr
