/*
 * wpbr_sampling.h — deterministic per-sample random streams.
 *
 * The reference fills each pixel's CSamples1D / CSamples2D arrays with
 * std::random_device-seeded stratified values and shuffles them
 * (WoodenPBREngine/CSSamplerStratified.cpp:8-47,50-90), so no two runs see the
 * same numbers. This header replaces that source with a counter-based stream
 * that any implementation (GPU kernel, CPU restatement) can evaluate for any
 * (pixel, sample pass, dimension) without state:
 *
 *   bits  = Philox-4x32-10(counter = {pixel, pass, dim, 0}, key = {seed, stream})
 *           (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
 *           1, 2, 3", SC'11; the published round and key-schedule constants)
 *   xi    = (bits >> 8) * 2^-24            exactly representable, in [0, 1)
 *
 * Stratification over the S sample passes of a pixel (per dimension):
 *   offset = Philox({pixel, 0xFFFFFFFF, dim, 0}).x mod S    (random rotation)
 *   k      = (pass + offset) mod S
 *   1D:  u = min((k + xi0) / S, 1 - 2^-24)
 *   2D:  S = nx * ny (nx the largest divisor of S not above sqrt(S)),
 *        u = (min((k mod nx + xi0) / nx, 1-2^-24), min((k / nx + xi1) / ny, 1-2^-24))
 *
 * Dimensions are consumed in the reference's per-pass order:
 *   0 camera jitter (2D)      WoodenPBREngine/CSSampler.cpp:19
 *   1 light pick (1D)         WoodenPBREngine/SScattering.cpp:85
 *   2 light sample (2D)       WoodenPBREngine/CSSphere.h:218, CLightInfiniteArea.cpp:111
 *   3 BSDF sample (2D)        WoodenPBREngine/CBSDFConductorMicroface.cpp:107-108
 */
#ifndef WPBR_SAMPLING_H
#define WPBR_SAMPLING_H

#include <stdint.h>
#include "wpbr_fmath.h"

namespace wpbr_rng {

enum : uint32_t { DIM_CAMERA = 0, DIM_LIGHT_PICK = 1, DIM_LIGHT = 2, DIM_BSDF = 3 };

static constexpr float kOneMinusEps = 0x1.fffffep-1f;

WPBR_HD void mulhilo(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

/* Philox-4x32 with 10 rounds. */
WPBR_HD void philox4x32_10(const uint32_t in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo(0xD2511F53u, c0, &hi0, &lo0);
    mulhilo(0xCD9E8D57u, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n1 = lo1;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    uint32_t n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

WPBR_HD float bits_to_u01(uint32_t x) { return (float)(x >> 8) * 0x1p-24f; }

struct Stream {
  uint32_t seed;
  uint32_t stream;   /* scene id for batched rendering, 0 otherwise */
  uint32_t spp;      /* S, total passes per pixel */
};

WPBR_HD uint32_t stratum_offset(const Stream& s, uint32_t pixel, uint32_t dim) {
  uint32_t c[4] = {pixel, 0xFFFFFFFFu, dim, 0u};
  uint32_t k[2] = {s.seed, s.stream};
  uint32_t o[4];
  philox4x32_10(c, k, o);
  return o[0] % s.spp;
}

WPBR_HD void jitter(const Stream& s, uint32_t pixel, uint32_t pass, uint32_t dim, float* xi0, float* xi1) {
  uint32_t c[4] = {pixel, pass, dim, 0u};
  uint32_t k[2] = {s.seed, s.stream};
  uint32_t o[4];
  philox4x32_10(c, k, o);
  *xi0 = bits_to_u01(o[0]);
  *xi1 = bits_to_u01(o[1]);
}

WPBR_HD uint32_t grid_nx(uint32_t S) {
  uint32_t nx = 1;
  for (uint32_t d = 1; d * d <= S; ++d)
    if (S % d == 0) nx = d;
  return nx;
}

WPBR_HD float clamp_u(float u) { return u < kOneMinusEps ? u : kOneMinusEps; }

WPBR_HD float sample1d(const Stream& s, uint32_t pixel, uint32_t pass, uint32_t dim) {
  uint32_t k = (pass + stratum_offset(s, pixel, dim)) % s.spp;
  float xi0, xi1;
  jitter(s, pixel, pass, dim, &xi0, &xi1);
  return clamp_u(((float)k + xi0) / (float)s.spp);
}

WPBR_HD void sample2d(const Stream& s, uint32_t pixel, uint32_t pass, uint32_t dim, float* u0, float* u1) {
  uint32_t nx = grid_nx(s.spp);
  uint32_t ny = s.spp / nx;
  uint32_t k = (pass + stratum_offset(s, pixel, dim)) % s.spp;
  float xi0, xi1;
  jitter(s, pixel, pass, dim, &xi0, &xi1);
  *u0 = clamp_u(((float)(k % nx) + xi0) / (float)nx);
  *u1 = clamp_u(((float)(k / nx) + xi1) / (float)ny);
}

}  // namespace wpbr_rng

#endif  // WPBR_SAMPLING_H
