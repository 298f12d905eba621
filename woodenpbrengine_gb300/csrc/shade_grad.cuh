// shade_grad.cuh — hand-written derivatives of the shading functions the
// differentiable estimator depends on: Trowbridge-Reitz D with respect to
// alpha, the conductor and dielectric Fresnel terms with respect to eta and k,
// the power heuristic, and the bilinear taps / piecewise-constant pdf of the
// environment light. Each function recomputes its forward value with the
// same operations as shade.cuh and returns the partial derivatives (reverse
// mode written out by hand).
#pragma once

#include "shade.cuh"

namespace wpbr {

// D(wh) of tr_d and dD/dalpha where alpha sets both alpha_x and alpha_y.
WPBR_HD float tr_d_grad(float ax, float ay, V3 wh, float* dD_dalpha) {
  *dD_dalpha = 0.0f;
  float t2 = tan2t(wh);
  if (fabs_(t2) == inf_()) return 0.0f;
  float c4 = cos2t(wh) * cos2t(wh);
  float cp = cosphi(wh), sp = sinphi(wh);
  float e = ((cp * cp) / (ax * ax) + (sp * sp) / (ay * ay)) * t2;
  double den = ((((kPI * (double)ax) * (double)ay) * (double)c4) * (double)(1.0f + e)) * (double)(1.0f + e);
  float D = (float)(1.0 / den);
  // ln D = -ln(pi ax ay c4) - 2 ln(1 + e)
  float de_dax = -2.0f * (cp * cp) * t2 / (ax * ax * ax);
  float de_day = -2.0f * (sp * sp) * t2 / (ay * ay * ay);
  float dlnD_dax = -1.0f / ax - 2.0f * de_dax / (1.0f + e);
  float dlnD_day = -1.0f / ay - 2.0f * de_day / (1.0f + e);
  *dD_dalpha = D * (dlnD_dax + dlnD_day);
  return D;
}

// fresnel_conductor and its partials with respect to eta_t and k.
WPBR_HD float fresnel_conductor_grad(float cos_i, float eta_i, float eta_t, float kk, float* dF_deta_t, float* dF_dk) {
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
  float Q = (t3 - t4) / (t3 + t4);
  float Rp = Rs * Q;
  // reverse sweep
  float gRp = 0.5f, gRs = 0.5f;
  gRs += gRp * Q;
  float gQ = gRp * Rs;
  float d34 = (t3 + t4) * (t3 + t4);
  float gt3 = gQ * 2.0f * t4 / d34;
  float gt4 = -gQ * 2.0f * t3 / d34;
  float gt2 = gt4 * s2;
  float ga2pb2 = gt3 * c2;
  float d12 = (t1 + t2) * (t1 + t2);
  float gt1 = gRs * 2.0f * t2 / d12;
  gt2 += -gRs * 2.0f * t1 / d12;
  float ga = gt2 * 2.0f * cos_i;
  float gt0 = 0.0f;
  if (a > 0.0f) {
    ga2pb2 += ga / (4.0f * a);
    gt0 += ga / (4.0f * a);
  }
  ga2pb2 += gt1;
  float ga2pb22 = (a2pb2 > 0.0f) ? ga2pb2 / (2.0f * a2pb2) : 0.0f;
  gt0 += ga2pb22 * 2.0f * t0;
  float geta2 = ga2pb22 * 4.0f * etak2 + gt0;
  float getak2 = ga2pb22 * 4.0f * eta2 - gt0;
  *dF_deta_t = geta2 * 2.0f * eta / eta_i;
  *dF_dk = getak2 * 2.0f * etak / eta_i;
  return (Rp + Rs) * 0.5f;
}

// fresnel_dielectric and its partial with respect to eta_t.
WPBR_HD float fresnel_dielectric_grad(float cos_i, float eta_i, float eta_t, float* dF_deta_t) {
  *dF_deta_t = 0.0f;
  cos_i = clampf(cos_i, -1.0f, 1.0f);
  float ei = eta_i, et = eta_t;
  bool swapped = false;
  if (!(cos_i > 0.0f)) {
    float t = ei;
    ei = et;
    et = t;
    cos_i = fabs_(cos_i);
    swapped = true;
  }
  double a = 1.0 - (double)(cos_i * cos_i);
  float sin_i = (float)sqrt_d(0.0 > a ? 0.0 : a);
  float sin_t = ei / et * sin_i;
  if ((double)sin_t >= 1.0) return 1.0f;
  double b = 1.0 - (double)(sin_t * sin_t);
  float cos_t = (float)sqrt_d(0.0 > b ? 0.0 : b);
  float A = et * cos_i, B = ei * cos_t;
  float C = ei * cos_i, E = et * cos_t;
  float r_parl = (A - B) / (A + B);
  float r_perp = (C - E) / (C + E);
  float F = (r_parl * r_parl + r_perp * r_perp) / 2.0f;
  float dAB = (A + B) * (A + B), dCE = (C + E) * (C + E);
  float gA = r_parl * 2.0f * B / dAB, gB = -r_parl * 2.0f * A / dAB;
  float gC = r_perp * 2.0f * E / dCE, gE = -r_perp * 2.0f * C / dCE;
  float get = gA * cos_i + gE * cos_t;
  float gei = gB * cos_t + gC * cos_i;
  float gct = gB * ei + gE * et;
  float gst = (cos_t > 0.0f) ? -gct * sin_t / cos_t : 0.0f;
  gei += gst * sin_i / et;
  get += -gst * ei * sin_i / (et * et);
  *dF_deta_t = swapped ? gei : get;
  return F;
}

// power_heuristic(a, b) = a^2 / (a^2 + b^2) and its partials.
WPBR_HD float power_heuristic_grad(float a, float b, float* dw_da, float* dw_db) {
  float a2 = a * a, b2 = b * b, s = a2 + b2;
  *dw_da = 2.0f * a * b2 / (s * s);
  *dw_db = -2.0f * b * a2 / (s * s);
  return a2 / s;
}

// The four texels env_bilerp blends at (si, ti) and their weights.
WPBR_HD void env_taps(const EnvView& e, float si, float ti, int idx[4], float w[4]) {
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
  idx[0] = t0 * e.W + s0;
  idx[1] = t0n * e.W + s0;
  idx[2] = t0 * e.W + s0n;
  idx[3] = t0n * e.W + s0n;
  w[0] = (1.0f - ds) * (1.0f - dt);
  w[1] = (1.0f - ds) * dt;
  w[2] = ds * (1.0f - dt);
  w[3] = ds * dt;
}

// Cell of the piecewise-constant map pdf at (u, v), as env_pdf_uv.
WPBR_HD int env_cell(const EnvView& e, float u, float v) {
  int iu = (int)(u * (float)e.W), iv = (int)(v * (float)e.H);
  iu = iu < 0 ? 0 : (iu > e.W - 1 ? e.W - 1 : iu);
  iv = iv < 0 ? 0 : (iv > e.H - 1 ? e.H - 1 : iv);
  return iv * e.W + iu;
}

// Solid-angle pdf of the environment light for map cell `cell` at sin(theta)
// st: func[cell] / Z / (2 pi^2 st), with Z the map's integral (e.marg_int).
WPBR_HD float env_pdf_cell(const EnvView& e, int cell, float st) {
  return (float)((double)(e.cond_func[cell] / e.marg_int) / (((2.0 * kPI) * kPI) * (double)st));
}

}  // namespace wpbr
