// shade.cuh — surface interactions, BSDFs, lights, MIS and the film filter
// of WoodenPBREngine's per-sample job list, as host/device functions.
// Each function cites the reference it restates; arithmetic follows the C++
// promotion rules of the reference source (PI = 3.14 as a double literal,
// vector-by-scalar products in float).
#pragma once

#include "geom.cuh"
#include "intersect.cuh"
#include "wpbr_scene.h"

namespace wpbr {

// ---- surface interaction ---------------------------------------------------
struct SurfInt {
  V3 p, n, wo;
  V3 dpdu, dpdv, dndu, dndv;
  V3 sn, sdpdu;
  V2 uv;  // triangles: interpolated uv; spheres: (0, 0), the world transform drops it
};

// SSphere::computeSurfInteraction (CSSphere.cpp:122-186) then
// CTransform::operator()(CSurfaceInteraction) (CTransform.h:41-66).
WPBR_HD SurfInt sphere_si(const Xf& o2w, const Xf& w2o, float radius, V3 rld, V3 ph) {
  float theta = acosf_(ph.z / radius);
  float inv_zr = (float)(1.0 / (double)sqrt_(ph.x * ph.x + ph.y * ph.y));
  float phi_cos = ph.x * inv_zr;
  float phi_sin = ph.y * inv_zr;
  V3 dpdu = mul(V3{-ph.y, ph.x, 0.0f}, (float)(2.0 * kPI));
  V3 dpdv = mul(V3{ph.z * phi_cos, ph.z * phi_sin, -radius * sinf_(theta)}, (float)kPI);
  V3 d2uu = mul(V3{ph.x, ph.y, 0.0f}, (float)(-2.0 * kPI * 2.0 * kPI));
  V3 d2uv = mul(mul(mul(mul(V3{-phi_sin, phi_cos, 0.0f}, (float)kPI), ph.z), 2.0f), (float)kPI);
  V3 d2vv = mul(mul(V3{ph.x, ph.y, ph.z}, (float)(-kPI)), (float)kPI);
  float E = dot(dpdu, dpdu), F = dot(dpdu, dpdv), G = dot(dpdv, dpdv);
  V3 N = normalize(cross(dpdu, dpdv));
  float e = dot(N, d2uu), f = dot(N, d2uv), g = dot(N, d2vv);
  float inv = 1.0f / (E * G - F * F);
  V3 dndu = add(mul(dpdu, (f * F - e * G) * inv), mul(dpdv, (e * F - f * E) * inv));
  V3 dndv = add(mul(dpdu, (g * F - f * G) * inv), mul(dpdv, (f * F - g * E) * inv));
  V3 n = normalize(cross(dpdu, dpdv));
  SurfInt s;
  s.uv = V2{0.0f, 0.0f};
  s.p = xpoint(o2w, ph);
  s.n = normalize(xnormal(w2o, n));
  s.wo = normalize(xvector(o2w, neg(rld)));
  s.dpdu = xvector(o2w, dpdu);
  s.dpdv = xvector(o2w, dpdv);
  s.dndu = xnormal(w2o, dndu);
  s.dndv = xnormal(w2o, dndv);
  s.sn = normalize(xnormal(w2o, n));
  s.sdpdu = xvector(o2w, dpdu);
  return s;
}

struct TriData {
  V3 p[3], n[3], s[3];
  V2 uv[3];
  bool has_ns, has_uv;
};

// JobProcessTriangleFullInteractionRequests (CSTriangle.cpp:149-319).
WPBR_HD SurfInt triangle_si(const TriData& tv, V3 rd, float b0, float b1, float b2) {
  V2 uv0, uv1, uv2;
  if (!tv.has_uv) {
    uv0 = V2{0.0f, 0.0f};
    uv1 = V2{1.0f, 0.0f};
    uv2 = V2{1.0f, 1.0f};
  } else {
    uv0 = tv.uv[0];
    uv1 = tv.uv[1];
    uv2 = tv.uv[2];
  }
  V3 dp02 = sub(tv.p[0], tv.p[2]), dp12 = sub(tv.p[1], tv.p[2]);
  V2 duv02{uv0.x - uv2.x, uv0.y - uv2.y};
  V2 duv12{uv1.x - uv2.x, uv1.y - uv2.y};
  float det = duv02.x * duv12.y - duv02.y * duv12.x;
  if (det == 0.0f) {
    const float s = (float)0.001;
    uv0 = V2{0.0f * s, 0.0f * s};
    uv1 = V2{1.0f * s, 0.0f * s};
    uv2 = V2{1.0f * s, 1.0f * s};
    duv02 = V2{uv0.x - uv2.x, uv0.y - uv2.y};
    duv12 = V2{uv1.x - uv2.x, uv1.y - uv2.y};
    det = duv02.x * duv12.y - duv02.y * duv12.x;
  }
  float det_inv = 1.0f / det;
  V3 dpdu = mul(sub(mul(dp02, duv12.y), mul(dp12, duv02.y)), det_inv);
  V3 dpdv = mul(add(mul(neg(dp02), duv12.x), mul(dp12, duv02.x)), det_inv);
  SurfInt s;
  s.p = add(add(mul(tv.p[0], b0), mul(tv.p[1], b1)), mul(tv.p[2], b2));
  s.uv = V2{(uv0.x * b0 + uv1.x * b1) + uv2.x * b2, (uv0.y * b0 + uv1.y * b1) + uv2.y * b2};
  s.wo = neg(rd);
  s.dpdu = dpdu;
  s.dpdv = dpdv;
  s.dndu = V3{0, 0, 0};
  s.dndv = V3{0, 0, 0};
  s.sdpdu = dpdu;
  s.n = normalize(cross(dp02, dp12));
  s.sn = s.n;
  if (tv.has_ns) {
    V3 ns = add(add(mul(tv.n[0], b0), mul(tv.n[1], b1)), mul(tv.n[2], b2));
    ns = !is_zero(ns) ? normalize(ns) : s.n;
    V3 ss = add(add(mul(tv.s[0], b0), mul(tv.s[1], b1)), mul(tv.s[2], b2));
    ss = !is_zero(ss) ? normalize(ss) : normalize(s.dpdu);
    V3 ts = cross(ss, ns);
    if (len2(ts) > 0.0f) {
      ts = normalize(ts);
      ss = cross(ts, ns);
    }
    // setShadingGeometry(ss, ts, dndu, dndv, true) (CSufraceInteraction.h:171-196)
    s.sn = normalize(cross(ss, ts));
    s.sdpdu = ss;
    if (dot(s.n, s.sn) < 0.0f) s.n = neg(s.n);  // faceForward
  }
  return s;
}

// ---- BSDF frame: JobBSDFComputeTransform (CBSDF.cpp:12-24) -------------------
struct Frame {
  V3 ss, ts, ns;
};
WPBR_HD Frame bsdf_frame(const SurfInt& s) {
  Frame f;
  f.ss = normalize(s.sdpdu);
  f.ns = s.sn;
  f.ts = cross(f.ns, f.ss);
  return f;
}
WPBR_HD V3 to_local(const Frame& f, V3 v) { return V3{dot(f.ss, v), dot(f.ts, v), dot(f.ns, v)}; }
WPBR_HD V3 to_world(const Frame& f, V3 v) {
  return V3{(f.ss.x * v.x + f.ts.x * v.y) + f.ns.x * v.z, (f.ss.y * v.x + f.ts.y * v.y) + f.ns.y * v.z,
            (f.ss.z * v.x + f.ts.z * v.y) + f.ns.z * v.z};
}

// ---- shading-space trigonometry (pbrt conventions) ---------------------------
WPBR_HD float cos2t(V3 w) { return w.z * w.z; }
WPBR_HD float abs_cos(V3 w) { return fabs_(w.z); }
WPBR_HD float sin2t(V3 w) {
  float v = 1.0f - cos2t(w);
  return 0.0f < v ? v : 0.0f;
}
WPBR_HD float sint(V3 w) { return sqrt_(sin2t(w)); }
WPBR_HD float tan2t(V3 w) { return sin2t(w) / cos2t(w); }
WPBR_HD float cosphi(V3 w) {
  float st = sint(w);
  return (st == 0.0f) ? 1.0f : clampf(w.x / st, -1.0f, 1.0f);
}
WPBR_HD float sinphi(V3 w) {
  float st = sint(w);
  return (st == 0.0f) ? 0.0f : clampf(w.y / st, -1.0f, 1.0f);
}
WPBR_HD bool same_hemi(V3 a, V3 b) { return a.z * b.z > 0.0f; }
WPBR_HD V3 reflect(V3 wo, V3 n) { return add(neg(wo), mul(n, 2.0f * dot(wo, n))); }
WPBR_HD V3 sph_dir(float st, float ct, float phi) { return V3{st * cosf_(phi), st * sinf_(phi), ct}; }
WPBR_HD V3 sph_dir(float st, float ct, float phi, V3 x, V3 y, V3 z) {
  return add(add(mul(x, st * cosf_(phi)), mul(y, st * sinf_(phi))), mul(z, ct));
}
WPBR_HD float sph_theta(V3 v) { return acosf_(clampf(v.z, -1.0f, 1.0f)); }
WPBR_HD float sph_phi(V3 v) {
  float p = atan2f_(v.y, v.x);
  return (p < 0.0f) ? p + 2.0f * kMathPi : p;
}
WPBR_HD void make_basis(V3 v1, V3* v2, V3* v3) {
  if (fabs_(v1.x) > fabs_(v1.y))
    *v2 = divs(V3{-v1.z, 0.0f, v1.x}, sqrt_(v1.x * v1.x + v1.z * v1.z));
  else
    *v2 = divs(V3{0.0f, v1.z, -v1.y}, sqrt_(v1.y * v1.y + v1.z * v1.z));
  *v3 = cross(v1, *v2);
}
WPBR_HD float cone_pdf(float cos_max) { return 1.0f / (2.0f * kMathPi * (1.0f - cos_max)); }

// ---- Fresnel (CBXDF.h:23-62, 200-238) -----------------------------------------
WPBR_HD float fresnel_dielectric(float cos_i, float eta_i, float eta_t) {
  cos_i = clampf(cos_i, -1.0f, 1.0f);
  float ei = eta_i, et = eta_t;
  if (!(cos_i > 0.0f)) {
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
WPBR_HD float fresnel_conductor(float cos_i, float eta_i, float eta_t, float kk) {
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

// ---- Trowbridge-Reitz (MicrofaceDistr.h:12-88) ------------------------------
WPBR_HD float tr_d(float ax, float ay, V3 wh) {
  float t2 = tan2t(wh);
  if (fabs_(t2) == inf_()) return 0.0f;
  float c4 = cos2t(wh) * cos2t(wh);
  float cp = cosphi(wh), sp = sinphi(wh);
  float e = ((cp * cp) / (ax * ax) + (sp * sp) / (ay * ay)) * t2;
  double den = ((((kPI * (double)ax) * (double)ay) * (double)c4) * (double)(1.0f + e)) * (double)(1.0f + e);
  return (float)(1.0 / den);
}
WPBR_HD V3 tr_sample(float ax, float ay, V3 wo, float u0, float u1, float* d_out) {
  float cos_t;
  float phi = (float)((2.0 * kPI) * (double)u1);
  if (ax == ay) {
    float tan2 = ((ax * ax) * u0) / (1.0f - u0);
    cos_t = 1.0f / sqrt_(1.0f + tan2);
  } else {
    phi = atanf_(ay / ax * tanf_((float)((2.0 * kPI) * (double)u1 + 0.5 * kPI)));
    if (u1 > 0.5f) phi = (float)((double)phi + kPI);
    float sp = sinf_(phi), cp = cosf_(phi);
    float alpha2 = 1.0f / ((cp * cp) / (ax * ax) + (sp * sp) / (ay * ay));
    float tan2 = (alpha2 * u0) / (1.0f - u0);
    cos_t = 1.0f / sqrt_(1.0f + tan2);
  }
  float v = 1.0f - cos_t * cos_t;
  float sin_t = sqrt_(0.0f > v ? 0.0f : v);
  V3 wh = sph_dir(sin_t, cos_t, phi);
  if (!same_hemi(wo, wh)) wh = neg(wh);
  *d_out = tr_d(ax, ay, wh);
  return wh;
}

// ---- BSDFs ---------------------------------------------------------------------
WPBR_HD RGB3 mf_f_impl(const wpbr_material& m, float d_wh, V3 wh, V3 wo, V3 wi) {
  float co = abs_cos(wo), ci = abs_cos(wi);
  if (ci == 0.0f || co == 0.0f) return rgb1(0.0f);
  if (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) return rgb1(0.0f);
  float c = dot(wi, wh);
  RGB3 R{m.R[0], m.R[1], m.R[2]};
  if (m.type == WPBR_MAT_CONDUCTOR) {
    RGB3 fr{fresnel_conductor(c, m.eta_i[0], m.eta_t[0], m.k[0]), fresnel_conductor(c, m.eta_i[1], m.eta_t[1], m.k[1]),
            fresnel_conductor(c, m.eta_i[2], m.eta_t[2], m.k[2])};
    return rmuls(rmul(fr, R), d_wh / ((4.0f * ci) * co));
  }
  float fr = fresnel_dielectric(c, m.eta_i[0], m.eta_t[0]);
  return rmuls(R, (fr * d_wh) / ((4.0f * ci) * co));
}
// JobBSDF{ConductorMicroface,DielectricMicroface,SpecularReflection}Compute
// (CBSDFConductorMicroface.cpp:44-58,84-97; CBSDFDielectricMicroface.cpp:44-58,
// 84-97; CBSDFSpecularReflectance.cpp:42-48,63-73): value already times |cos wi|.
WPBR_HD RGB3 bsdf_eval(const wpbr_material& m, V3 wo, V3 wi, float* pdf) {
  if (m.type == WPBR_MAT_SPECULAR) {
    *pdf = 0.0f;
    return rmuls(rgb1(0.0f), abs_cos(wi));
  }
  V3 wh = normalize(add(wo, wi));
  float d = tr_d(m.alpha_x, m.alpha_y, wh);
  *pdf = (d * abs_cos(wh)) / (4.0f * dot(wo, wh));
  return rmuls(mf_f_impl(m, d, wh, wo, wi), abs_cos(wi));
}
// JobBSDF*Sample (CBSDFConductorMicroface.cpp:61-82,99-115;
// CBSDFDielectricMicroface.cpp:61-82,99-115; CBSDFSpecularReflectance.cpp:51-61,
// 75-93). A microfacet sample in the opposite hemisphere is invalid (the
// reference leaves its pdf uninitialised) and contributes nothing.
WPBR_HD RGB3 bsdf_sample(const wpbr_material& m, V3 wo, float u0, float u1, V3* wi, float* pdf, bool* valid) {
  if (m.type == WPBR_MAT_SPECULAR) {
    *wi = V3{-wo.x, -wo.y, wo.z};
    *pdf = 1.0f;
    *valid = true;
    RGB3 f = rgb1(0.0f);
    if (abs_cos(*wi) != 0.0f) {
      float fr = fresnel_dielectric(wi->z, m.eta_i[0], m.eta_t[0]);
      f = rmuls(RGB3{m.R[0], m.R[1], m.R[2]}, fr / abs_cos(*wi));
    }
    return rmuls(f, abs_cos(*wi));
  }
  float d;
  V3 wh = tr_sample(m.alpha_x, m.alpha_y, wo, u0, u1, &d);
  *wi = reflect(wo, wh);
  if (!same_hemi(*wi, wo)) {
    *valid = false;
    *pdf = 0.0f;
    return rgb1(0.0f);
  }
  *valid = true;
  *pdf = (d * abs_cos(wh)) / (4.0f * dot(wo, wh));
  return rmuls(mf_f_impl(m, d, wh, wo, *wi), abs_cos(*wi));
}

// PowerHeuristic(1, f, 1, g) (SScattering.cpp:162-166, 249-253)
WPBR_HD float power_heuristic(float f, float g) {
  float a = 1.0f * f, b = 1.0f * g;
  return (a * a) / (a * a + b * b);
}

// ---- sphere light (CSSphere.cpp:221-281, CSSphere.h:187-267) ---------------
WPBR_HD void sphere_light_sample(const Xf& o2w, float r, V3 p, float u0, float u1, V3* wi, float* pdf) {
  V3 pc = xpoint(o2w, V3{0, 0, 0});
  V3 wc = normalize(sub(pc, p));
  V3 wcx, wcy;
  make_basis(wc, &wcx, &wcy);
  float s2 = (r * r) / len2(sub(p, pc));
  double a = 1.0 - (double)s2;
  float cos_max = (float)sqrt_d(0.0 > a ? 0.0 : a);
  float cos_t = (float)((double)u0 * (1.0 - (double)cos_max) + (double)cos_max);
  double b = 1.0 - (double)(cos_t * cos_t);
  float sin_t = (float)sqrt_d(0.0 > b ? 0.0 : b);
  float phi = (float)((double)(u1 * 2.0f) * kPI);
  float dc = len(sub(p, pc));
  float q = r * r - ((dc * dc) * sin_t) * sin_t;
  float ds = dc * cos_t - sqrt_(0.0f > q ? 0.0f : q);
  float cos_a = ((dc * dc + r * r) - ds * ds) / ((2.0f * dc) * r);
  float w = 1.0f - cos_a * cos_a;
  float sin_a = sqrt_(0.0f > w ? 0.0f : w);
  V3 nl = sph_dir(sin_a, cos_a, phi, neg(wcx), neg(wcy), neg(wc));
  V3 sp = xpoint(o2w, mul(nl, r));
  *pdf = cone_pdf(cos_max);
  *wi = normalize(sub(sp, p));
}
// SSphere::pdf: the comma operator in (inter.p, pCenteroidW).length2() makes
// the cone subtend from the world origin (CSSphere.cpp:228).
WPBR_HD float sphere_light_pdf(const Xf& o2w, float r, V3 p, uint32_t quirks) {
  V3 pc = xpoint(o2w, V3{0, 0, 0});
  V3 d = (quirks & WPBR_Q_SPHERE_PDF_FIX) ? sub(p, pc) : pc;
  float s2 = (r * r) / len2(d);
  float v = 1.0f - s2;
  float cos_max = sqrt_(0.0f > v ? 0.0f : v);
  return cone_pdf(cos_max);
}

// ---- environment light (CLightInfiniteArea.cpp, CSTextureProcess.h:58-82) ----
struct EnvView {
  int W, H;
  const float4* rgb;         // W*H texels
  const float* cond_func;    // H*W
  const float* cond_cdf;     // H*(W+1)
  const float* cond_int;     // H
  const float* marg_func;    // H
  const float* marg_cdf;     // H+1
  float marg_int;
  Xf l2w, w2l;
  RGB3 le;
};

WPBR_HD RGB3 env_texel(const EnvView& e, int x, int y) {
  float4 t = e.rgb[(size_t)y * e.W + x];
  return RGB3{t.x, t.y, t.z};
}
// STexture2DSampler::triangle on mip 0: lower indices clamp at 0 keeping the
// extrapolating weights; indices at or past the last texel are clamped.
WPBR_HD RGB3 env_bilerp(const EnvView& e, float si, float ti) {
  float s = si * (float)e.W - 0.5f;
  float t = ti * (float)e.H - 0.5f;
  float fs = floorf(s), ft = floorf(t);
  int s0 = (int)fs, t0 = (int)ft;
  s0 = s0 > 0 ? s0 : 0;
  t0 = t0 > 0 ? t0 : 0;
  float ds = s - (float)s0, dt = t - (float)t0;
  int s0n = s0 + 1 < e.W - 1 ? s0 + 1 : e.W - 1;
  int t0n = t0 + 1 < e.H - 1 ? t0 + 1 : e.H - 1;
  s0n = s0n > 0 ? s0n : 0;
  t0n = t0n > 0 ? t0n : 0;
  s0 = s0 < e.W - 1 ? s0 : e.W - 1;
  t0 = t0 < e.H - 1 ? t0 : e.H - 1;
  RGB3 a = rmuls(rmuls(env_texel(e, s0, t0), 1.0f - ds), 1.0f - dt);
  RGB3 b = rmuls(rmuls(env_texel(e, s0, t0n), 1.0f - ds), dt);
  RGB3 c = rmuls(rmuls(env_texel(e, s0n, t0), ds), 1.0f - dt);
  RGB3 d = rmuls(rmuls(env_texel(e, s0n, t0n), ds), dt);
  return radd(radd(radd(a, b), c), d);
}
// Distribution1D::SampleContinuous over cdf[0..n] (pbrt semantics).
WPBR_HD float dist_sample(const float* func, const float* cdf, float func_int, int n, float u, float* pdf, int* off) {
  int first = 0, len_ = n + 1;
  while (len_ > 0) {
    int half = len_ >> 1, middle = first + half;
    if (cdf[middle] <= u) {
      first = middle + 1;
      len_ -= half + 1;
    } else {
      len_ = half;
    }
  }
  int o = first - 1;
  o = o < 0 ? 0 : (o > n - 1 ? n - 1 : o);
  *off = o;
  float du = u - cdf[o];
  if ((cdf[o + 1] - cdf[o]) > 0.0f) du = du / (cdf[o + 1] - cdf[o]);
  *pdf = (func_int > 0.0f) ? func[o] / func_int : 0.0f;
  return ((float)o + du) / (float)n;
}
WPBR_HD void env_sample_uv(const EnvView& e, float u0, float u1, float* uv0, float* uv1, float* pdf) {
  float p1, p0;
  int v;
  *uv1 = dist_sample(e.marg_func, e.marg_cdf, e.marg_int, e.H, u1, &p1, &v);
  int o;
  *uv0 = dist_sample(e.cond_func + (size_t)v * e.W, e.cond_cdf + (size_t)v * (e.W + 1), e.cond_int[v], e.W, u0, &p0, &o);
  *pdf = p0 * p1;
}
WPBR_HD float env_pdf_uv(const EnvView& e, float u, float v) {
  int iu = (int)(u * (float)e.W), iv = (int)(v * (float)e.H);
  iu = iu < 0 ? 0 : (iu > e.W - 1 ? e.W - 1 : iu);
  iv = iv < 0 ? 0 : (iv > e.H - 1 ? e.H - 1 : iv);
  return e.cond_func[(size_t)iv * e.W + iu] / e.marg_int;
}
// JobLightInfiniteAreaLeCompute (CLightInfiniteArea.cpp:141-160)
WPBR_HD RGB3 env_le(const EnvView& e, V3 d) {
  V3 dl = xvector(e.w2l, d);
  float s = (float)((double)sph_phi(dl) / (2.0 * kPI));
  float t = (float)((double)sph_theta(dl) / kPI);
  return rmul(env_bilerp(e, s, t), e.le);
}
// JobLightInfiniteAreaLiSample (CLightInfiniteArea.cpp:163-204): the looked-up
// radiance is discarded unless WPBR_Q_ENV_LI_SAMPLE_FIX.
// uv_st (optional) receives the sampled map coordinates and sin(theta).
WPBR_HD void env_li_sample(const EnvView& e, uint32_t quirks, float u0, float u1, V3* wi, RGB3* li, float* pdf,
                           bool* ok, float* uv_st = nullptr) {
  float uv0, uv1, map_pdf;
  env_sample_uv(e, u0, u1, &uv0, &uv1, &map_pdf);
  *li = rgb1(0.0f);
  *ok = false;
  float st = 0.0f;
  if (map_pdf != 0.0f) {
    float theta = (float)((double)uv1 * kPI);
    float phi = (float)((double)(uv0 * 2.0f) * kPI);
    float ct = cosf_(theta);
    st = sinf_(theta);
    *wi = xvector(e.l2w, sph_dir(st, ct, phi));
    *pdf = (st != 0.0f) ? (float)((double)map_pdf / (((2.0 * kPI) * kPI) * (double)st)) : 0.0f;
    *ok = true;
  }
  if (quirks & WPBR_Q_ENV_LI_SAMPLE_FIX) *li = rmul(env_bilerp(e, uv0, uv1), e.le);
  if (uv_st) {
    uv_st[0] = uv0;
    uv_st[1] = uv1;
    uv_st[2] = st;
  }
}
// JobLightInfiniteAreaLiCompute (CLightInfiniteArea.cpp:206-237)
WPBR_HD void env_li_compute(const EnvView& e, V3 wi, RGB3* li, float* pdf) {
  V3 wl = xvector(e.w2l, wi);
  float theta = sph_theta(wl);
  float phi = sph_phi(wl);
  float u = (float)((double)phi / (2.0 * kPI));
  float v = (float)((double)theta / kPI);
  float st = sinf_(theta);
  *li = rgb1(0.0f);
  *pdf = 0.0f;
  if (st != 0.0f) {
    *pdf = (float)((double)env_pdf_uv(e, u, v) / (((2.0 * kPI) * kPI) * (double)st));
    *li = rmul(env_bilerp(e, u, v), e.le);
  }
}

// ---- film: MitchellFilter r=2, B=C=1/3 (CSFilm.h:20-44) -------------------------
WPBR_HD float mitchell1(float x) {
  const float B = (float)(1.0 / 3.0f), C = (float)(1.0 / 3.0f);
  x = fabs_(2.0f * x);
  if (x > 1.0f)
    return ((((((-B - 6.0f * C) * x) * x) * x + (((6.0f * B + 30.0f * C) * x) * x)) + ((-12.0f * B - 48.0f * C) * x)) +
            (8.0f * B + 24.0f * C)) *
           (1.0f / 6.0f);
  return (((((12.0f - 9.0f * B - 6.0f * C) * x) * x) * x + (((-18.0f + 12.0f * B + 6.0f * C) * x) * x)) +
          (6.0f - 2.0f * B)) *
         (1.0f / 6.0f);
}

}  // namespace wpbr
