// spectral.cuh — the reference's 64-sample spectral representation
// (SampledSpectrum, WoodenPBREngine/CSpectrumSampled.h:14-289,
// CSpectrumSampled.cpp:27-44, CoefficientSpectrum.h:14-24) for the
// Sampled64 parity mode: 64 bins over 400-700 nm, RGB to spectrum through
// Smits' bases (reflectance or illuminant), spectrum to RGB through the CIE
// matching functions and the XYZ to RGB matrix. Host and device share these
// functions; the binned tables are computed once on the host.
#pragma once

#include "geom.cuh"
#include "wpbr_scene.h"
#include "wpbr_spectrum_data.h"

namespace wpbr {

constexpr int kSpecN = 64;

struct S64 {
  float v[kSpecN];
};

// Binned tables of SampledSpectrum::init (CSpectrumSampled.h:241-278).
struct SpecTables {
  float X[kSpecN], Y[kSpecN], Z[kSpecN];
  float refl[7][kSpecN];   // white, cyan, magenta, yellow, red, green, blue
  float illum[7][kSpecN];
};
enum { kSpWhite = 0, kSpCyan, kSpMagenta, kSpYellow, kSpRed, kSpGreen, kSpBlue };

WPBR_HD S64 s64_const(float v) {
  S64 s;
  for (int i = 0; i < kSpecN; ++i) s.v[i] = v;
  return s;
}
WPBR_HD bool s64_black(const S64& s) {
  for (int i = 0; i < kSpecN; ++i)
    if (s.v[i] != 0.0f) return false;
  return true;
}
// s += a * k
WPBR_HD void s64_axpy(S64& s, const float* a, float k) {
  for (int i = 0; i < kSpecN; ++i) s.v[i] = s.v[i] + a[i] * k;
}

// SampledSpectrum::fromRGB (CSpectrumSampled.h:101-203): white times the
// smallest channel plus the secondary and primary bases for the rest.
WPBR_HD S64 s64_from_rgb(const SpecTables& T, RGB3 c, bool illuminant) {
  const float(*B)[kSpecN] = illuminant ? T.illum : T.refl;
  float r = c.r, g = c.g, b = c.b;
  S64 s = s64_const(0.0f);
  bool red_min = r <= g && r <= b;
  bool green_min = g <= r && g <= b;
  if (red_min) {
    s64_axpy(s, B[kSpWhite], r);
    if (g <= b) {
      s64_axpy(s, B[kSpCyan], g - r);
      s64_axpy(s, B[kSpBlue], b - g);
    } else {
      s64_axpy(s, B[kSpCyan], b - r);
      s64_axpy(s, B[kSpGreen], g - b);
    }
  } else if (green_min) {
    s64_axpy(s, B[kSpWhite], g);
    if (r <= b) {
      s64_axpy(s, B[kSpMagenta], r - g);
      s64_axpy(s, B[kSpBlue], b - r);
    } else {
      s64_axpy(s, B[kSpMagenta], b - g);
      s64_axpy(s, B[kSpRed], r - b);
    }
  } else {
    s64_axpy(s, B[kSpWhite], b);
    if (r <= g) {
      s64_axpy(s, B[kSpYellow], r - b);
      s64_axpy(s, B[kSpGreen], g - r);
    } else {
      s64_axpy(s, B[kSpYellow], g - b);
      s64_axpy(s, B[kSpRed], r - g);
    }
  }
  return s;
}

// A scene RGB value as the reference builds its spectrum: a grey value is
// the constant Spectrum(v) (how the engine writes R = Spectrum(1.0),
// etaI = Spectrum(1.0f), LEmit = Spectrum(lemit)), any other colour goes
// through fromRGB (the implicit SampledSpectrum(RGBSpectrum) constructor,
// reflectance type unless stated otherwise).
WPBR_HD S64 s64_of_param(const SpecTables& T, RGB3 c, bool illuminant) {
  if (c.r == c.g && c.g == c.b) return s64_const(c.r);
  return s64_from_rgb(T, c, illuminant);
}

// toXYZ (CSpectrumSampled.cpp:27-37): dot products with the binned matching
// functions times the bin width — not divided by CIE_Y_integral — then
// xyzToRGB (CoefficientSpectrum.h:14-24) as a row vector times the stored
// matrix, whose third column has 0.041556 where the standard sRGB matrix has
// 0.055648 (WPBR_Q_XYZ_MATRIX_FIX restores it).
WPBR_HD RGB3 s64_to_rgb(const SpecTables& T, const float* s, uint32_t quirks) {
  float x = 0.0f, y = 0.0f, z = 0.0f;
  for (int i = 0; i < kSpecN; ++i) {
    x = x + s[i] * T.X[i];
    y = y + s[i] * T.Y[i];
    z = z + s[i] * T.Z[i];
  }
  float dl = (float)(wpbr_spec::kLambdaEnd - wpbr_spec::kLambdaStart) / (float)kSpecN;
  x = x * dl;
  y = y * dl;
  z = z * dl;
  float m20 = (quirks & WPBR_Q_XYZ_MATRIX_FIX) ? 0.055648f : 0.041556f;
  RGB3 c;
  c.r = (x * 3.240479f + y * -1.537150f) + z * -0.498535f;
  c.g = (x * -0.969256f + y * 1.875991f) + z * 0.041556f;
  c.b = (x * m20 + y * -0.204043f) + z * 1.057311f;
  return c;
}

}  // namespace wpbr
