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
 *
 * Reference sample arrays (Stream::arrays != 0, quirk
 * WPBR_Q_REF_SAMPLER_ARRAYS). The reference gives every pixel one 1D array of
 * 16 + 64 = 80 values and one 2D array of 16 + 4*64 = 272 pairs
 * (CSFilm.cpp:22-23, NSAMPLERS_PER_PIXEL = 64), fills them once per tile
 * (CSSamplerStratified.cpp:8-47, 50-90) and reads them front to back with
 * next() / data[i++] over the tile's passes. Filled as written there:
 *   1D: element s = min((s + u_s) * float(1/80), 1)                      (:28-39)
 *   2D: element k = i*16 + j < 256 (n = int(sqrt(272)) = 16):
 *         ((i + dx_k) * float(1/272), (j + dy_k) * float(1/272))          (:68-84)
 *       (1/data.size() where 1/n was meant: every pair lies in [0, 1/17)^2),
 *       elements 256..271 stay (0, 0) (value-initialised, never written)
 * and each array is shuffled (:43, :87). Here the jitters are Philox draws
 * keyed by the element index, and the shuffle is a keyed bijection of the
 * positions (cycle walking over [0, 2^b) with an invertible integer mix).
 * A shuffled array is exchangeable, so which positions a pass reads does not
 * change the joint distribution: to keep passes independent of each other,
 * pass p reads 1D position p and 2D positions 3p (camera), 3p + 1 (light),
 * 3p + 2 (BSDF), every position modulo the array size (the reference reads
 * past its arrays after 64 passes).
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
  uint32_t arrays;   /* nonzero: the reference's shuffled per-pixel arrays */
};

enum : uint32_t { kRefArray1D = 80u, kRefArray2D = 272u, kRefGrid2D = 16u };

/* One invertible mixing step on b-bit integers (mask = 2^b - 1): xor with a
 * key, multiply by an odd key, xorshift, add a key, multiply, xorshift; each
 * step is a bijection modulo 2^b, so the composition is one. */
WPBR_HD uint32_t mix_bits(uint32_t x, const uint32_t k[4], uint32_t mask, uint32_t half) {
  x = (x ^ k[0]) & mask;
  x = (x * (k[1] | 1u)) & mask;
  x ^= x >> half;
  x = (x + k[2]) & mask;
  x = (x * (k[3] | 1u)) & mask;
  x ^= x >> (half + 1u);
  return x;
}

/* Keyed permutation of [0, n) (n <= 2^bits): cycle walking. x < n lies on a
 * cycle of the bijection on [0, 2^bits) that returns to x, so the walk meets
 * an element below n within 2^bits steps. */
WPBR_HD uint32_t shuffle_position(uint32_t x, uint32_t n, uint32_t bits, const uint32_t k[4]) {
  uint32_t mask = (1u << bits) - 1u, half = bits / 2u;
  for (uint32_t it = 0; it <= mask; ++it) {
    x = mix_bits(x, k, mask, half);
    if (x < n) break;
  }
  return x;
}

/* The element of a pixel's shuffled array at `pos`: its index before the
 * shuffle. kind 1: the 1D array, 2: the 2D array. */
WPBR_HD uint32_t ref_array_element(const Stream& s, uint32_t pixel, uint32_t kind, uint32_t pos) {
  uint32_t c[4] = {pixel, 0xFFFFFFFEu, kind, 0u};
  uint32_t key[2] = {s.seed, s.stream};
  uint32_t k[4];
  philox4x32_10(c, key, k);
  return kind == 1u ? shuffle_position(pos % kRefArray1D, kRefArray1D, 7u, k)
                    : shuffle_position(pos % kRefArray2D, kRefArray2D, 9u, k);
}

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

/* 1D element e of the reference array: min((e + u) * float(1/80), 1). */
WPBR_HD float ref_sample1d(const Stream& s, uint32_t pixel, uint32_t pass) {
  uint32_t e = ref_array_element(s, pixel, 1u, pass);
  float u0, u1;
  jitter(s, pixel, e, 0x100u | 1u, &u0, &u1);
  const float inv = (float)(1.0 / (double)kRefArray1D);
  float v = ((float)e + u0) * inv;
  return v < 1.0f ? v : 1.0f;
}

/* 2D element of the reference array for `slot` (0 camera, 1 light, 2 BSDF). */
WPBR_HD void ref_sample2d(const Stream& s, uint32_t pixel, uint32_t pass, uint32_t slot, float* u0, float* u1) {
  uint32_t e = ref_array_element(s, pixel, 2u, 3u * pass + slot);
  if (e >= kRefGrid2D * kRefGrid2D) {
    *u0 = 0.0f;
    *u1 = 0.0f;
    return;
  }
  float dx, dy;
  jitter(s, pixel, e, 0x100u | 2u, &dx, &dy);
  const float inv = (float)(1.0 / (double)kRefArray2D);
  float a = ((float)(e / kRefGrid2D) + dx) * inv, b = ((float)(e % kRefGrid2D) + dy) * inv;
  *u0 = a < 1.0f ? a : 1.0f;
  *u1 = b < 1.0f ? b : 1.0f;
}

WPBR_HD float sample1d(const Stream& s, uint32_t pixel, uint32_t pass, uint32_t dim) {
  if (s.arrays) return ref_sample1d(s, pixel, pass);
  uint32_t k = (pass + stratum_offset(s, pixel, dim)) % s.spp;
  float xi0, xi1;
  jitter(s, pixel, pass, dim, &xi0, &xi1);
  return clamp_u(((float)k + xi0) / (float)s.spp);
}

WPBR_HD void sample2d(const Stream& s, uint32_t pixel, uint32_t pass, uint32_t dim, float* u0, float* u1) {
  if (s.arrays) {
    ref_sample2d(s, pixel, pass, dim == DIM_CAMERA ? 0u : (dim == DIM_LIGHT ? 1u : 2u), u0, u1);
    return;
  }
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
