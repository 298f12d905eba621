// spectral.cu — the Sampled64 mode of the render pass: the same per-sample
// job list as the RGB path (MEngine::render, MEngine.cpp:393-442) with every
// radiance, reflectance and Fresnel value a 64-bin SampledSpectrum, as the
// reference computes it (Spectrum = SampledSpectrum, CSpectrum.h:8).
//
// Wavefront layout: the pass shares the RGB path's camera and shadow-ray
// persistent traversals (render.cu); k_sspawn (one thread per pixel) does
// the scalar part of shading and sampling and records, per pixel, the
// scalar factors every spectral term needs; k_sfinish gives each pixel a
// half-warp, 16 lanes x 4 bins, for the per-bin Fresnel terms and products;
// k_sfilm stages 8x8-pixel tiles of sample spectra in shared memory for the
// Mitchell film gather (4 threads x 16 bins per pixel); k_sresolve
// converts the film to RGB once per frame (or before a film read). Every per-bin value is
// computed with the same operations in the same order as the one-thread
// restatement, so the film is bit-identical to it; sums over bins (toXYZ)
// stay sequential in bin order.

#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "ctx.hpp"
#include "pass.cuh"
#include "spectral.cuh"

namespace wpbr {

namespace {

// The binned tables in global memory: the lanes of a pixel read different
// bins, which the constant cache would serialise.
__device__ __align__(16) SpecTables g_spec;

// Per material: R, eta_i, eta_t, k as spectra.
struct SpecMat {
  S64 R, eta_i, eta_t, k;
};

struct SpecCtx {
  const SpecMat* mats;
  const S64* light_le;  // per light: sphere Le, or the environment's LEmit
  float* L;             // per pixel, 64 floats
};

// Per-pixel record of k_sspawn (kSpecStateF4 float4):
//  [0] flags, light index (environment light on a miss), material id, w/lpdf
//  [1] light branch: cos(wi, wh), scalar BSDF factor, |cos wi|;  w/bpdf
//  [2] BSDF branch:  cos(wi, wh), scalar BSDF factor, |cos wi|;  -
//  [3] environment (s, t) of the light sample (or of the camera miss), of the BSDF sample
//  [4] textured metal: k (RGB)
constexpr int kSpecStateF4 = 5;
enum : uint32_t {
  SS_HIT = 1u,        // the camera ray hit and the scene has lights
  SS_MISS_ENV = 2u,   // the camera ray missed into the environment
  SS_LB = 4u,         // light branch: shadow ray traced, contribution if unoccluded and Li not black
  SS_BB = 8u,         // BSDF branch: likewise
  SS_COND = 16u,      // conductor Fresnel per bin (else the scalar dielectric form)
  SS_TEX = 32u,       // textured metal: eta 1 / 1.5, k from RGB
  SS_LZERO = 64u,     // light-branch f is 0 (grazing wi or wo, or wh = 0)
  SS_BZERO = 128u,    // BSDF-branch f is 0
  SS_LENV = 256u,     // light-branch Li is the environment lookup (WPBR_Q_ENV_LI_SAMPLE_FIX)
  SS_BENV = 512u      // BSDF-branch Li is the environment lookup
};
constexpr int kBinLanes = 16;  // lanes per pixel in the spectral kernels; 4 bins each

// averageSpectrumSamples (CSpectrumSampled.h:45-87): piecewise-linear average
// over [l0, l1], the trapezoid of each segment times 0.5 in double as the
// reference writes it.
float avg_samples(const float* lambda, const float* vals, int n, float l0, float l1) {
  if (l1 <= lambda[0]) return vals[0];
  if (l0 >= lambda[n - 1]) return vals[n - 1];
  if (n == 1) return vals[0];
  float sum = 0.0f;
  if (l0 < lambda[0]) sum += vals[0] * (lambda[0] - l0);
  if (l1 > lambda[n - 1]) sum += vals[n - 1] * (l1 - lambda[n - 1]);
  int j = 0;
  while (l0 > lambda[j + 1]) ++j;
  auto interp = [&](float w, int i) {
    float t = (w - lambda[i]) / (lambda[i + 1] - lambda[i]);
    return (1.0f - t) * vals[i] + t * vals[i + 1];
  };
  for (; j + 1 < n && l1 >= lambda[j]; ++j) {
    float s0 = std::max(l0, lambda[j]);
    float s1 = std::min(l1, lambda[j + 1]);
    sum = (float)((double)sum + (double)((interp(s0, j) + interp(s1, j)) * (s1 - s0)) * 0.5);
  }
  return sum / (l1 - l0);
}

void build_tables(SpecTables* T) {
  using namespace wpbr_spec;
  const float* refl[7] = {kReflWhite, kReflCyan, kReflMagenta, kReflYellow, kReflRed, kReflGreen, kReflBlue};
  const float* illum[7] = {kIllumWhite, kIllumCyan, kIllumMagenta, kIllumYellow, kIllumRed, kIllumGreen, kIllumBlue};
  const float a = (float)kLambdaStart, b = (float)kLambdaEnd;
  for (int i = 0; i < kSpecN; ++i) {
    float t0 = (float)i / (float)kSpecN, t1 = (float)(i + 1) / (float)kSpecN;
    float wl0 = (1.0f - t0) * a + t0 * b;
    float wl1 = (1.0f - t1) * a + t1 * b;
    T->X[i] = avg_samples(kCieLambda, kCieX, kCieSamples, wl0, wl1);
    T->Y[i] = avg_samples(kCieLambda, kCieY, kCieSamples, wl0, wl1);
    T->Z[i] = avg_samples(kCieLambda, kCieZ, kCieSamples, wl0, wl1);
    for (int k = 0; k < 7; ++k) {
      T->refl[k][i] = avg_samples(kRgbLambda, refl[k], kRgbSamples, wl0, wl1);
      T->illum[k][i] = avg_samples(kRgbLambda, illum[k], kRgbSamples, wl0, wl1);
    }
  }
}

// ---- scalar part (one thread per pixel) -----------------------------------

// Scalar factors of mf_f_impl for (wo, wi, wh, D): the per-bin value is
// ((F_conductor(c) * R) * kf) * fcos for a conductor and (R * kf) * fcos
// otherwise; zero when either cosine or wh is zero (then 0 * fcos).
struct FScalars {
  float c, kf, fcos;
  bool zero;
};
__device__ __forceinline__ FScalars f_scalars(const wpbr_material& m, float d_wh, V3 wh, V3 wo, V3 wi) {
  FScalars F;
  F.fcos = abs_cos(wi);
  F.c = 0.0f;
  F.kf = 0.0f;
  float co = abs_cos(wo), ci = abs_cos(wi);
  F.zero = ci == 0.0f || co == 0.0f || (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f);
  if (F.zero) return F;
  F.c = dot(wi, wh);
  if (m.type == WPBR_MAT_CONDUCTOR) {
    F.kf = d_wh / ((4.0f * ci) * co);
  } else {
    float fr = fresnel_dielectric(F.c, m.eta_i[0], m.eta_t[0]);
    F.kf = (fr * d_wh) / ((4.0f * ci) * co);
  }
  return F;
}

template <bool TEX>
__global__ void __launch_bounds__(kTB, TEX ? WPBR_SPAWN_TEX_MIN_BLOCKS : WPBR_SPAWN_MIN_BLOCKS) k_sspawn(PassCtx P, const uint32_t* pass_dev, const uint32_t* hit_prim,
                                                float4* state, ShadowQueue sq, float2* pf, const uint32_t* order) {
  uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= P.W * P.H) return;
  uint32_t pix = order ? order[slot] : slot;  // material-sorted (large films)
  if (pix >= P.W * P.H) return;
  uint32_t pass = *pass_dev;
  float fx, fy;
  camera_sample(P, pix, pass, &fx, &fy);
  pf[pix] = make_float2(fx, fy);
  RayD r = camera_ray(P.S.cam, fx, fy);
  uint32_t prim = hit_prim[pix];
  float4* st = state + (size_t)pix * kSpecStateF4;
  uint32_t nl = P.S.nlights;
  if (prim == kNoHit || nl == 0) {
    uint32_t flags = 0, env_light = 0;
    if (prim == kNoHit && P.S.has_env) {
      flags = SS_MISS_ENV;
      for (uint32_t i = 0; i < nl; ++i)
        if (P.S.lights[i].type == WPBR_LIGHT_ENV) env_light = i;
      V3 dl = xvector(P.S.env.w2l, r.d);
      float s = (float)((double)sph_phi(dl) / (2.0 * kPI));
      float t = (float)((double)sph_theta(dl) / kPI);
      st[3] = make_float4(s, t, 0.0f, 0.0f);
    }
    st[0] = make_float4(__uint_as_float(flags), __uint_as_float(env_light), 0.0f, 0.0f);
    return;
  }
  uint32_t flags = SS_HIT;
  SurfInt si = make_si(P.S, prim, r.o, r.d);
  Frame fr = bsdf_frame(si);
  uint32_t mid = prim_material(P.S, prim);
  const wpbr_material m = hit_material<TEX>(P.S, prim, mid, si, r);
  if (TEX && WPBR_MAT_TEXTURED(P.S.mats[mid].type)) {
    flags |= SS_TEX;
    st[4] = make_float4(m.k[0], m.k[1], m.k[2], 0.0f);
  }
  if (m.type == WPBR_MAT_CONDUCTOR) flags |= SS_COND;
  V3 wo_l = to_local(fr, si.wo);
  uint32_t li_idx = pick_light(P, pix, pass);
  const wpbr_light& lt = P.S.lights[li_idx];
  float4 s0 = make_float4(0.0f, __uint_as_float(li_idx), __uint_as_float(mid), 0.0f);
  float4 s1 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), s2 = s1, s3 = s1;
  // ---- light-sampling branch: Li is the sphere's LEmit, or (quirk fixed)
  // the environment lookup at the sampled (s, t); without the fix the
  // environment branch's Li is black and nothing is traced
  float u0, u1;
  wpbr_rng::sample2d(P.rs, pix, pass, wpbr_rng::DIM_LIGHT, &u0, &u1);
  V3 wi{0, 0, 0};
  float lpdf = 0.0f;
  bool ok = true, li_possible = true;
  if (lt.type == WPBR_LIGHT_SPHERE) {
    sphere_light_sample(P.S.sph_o2w[lt.sphere_index], P.S.sph_r[lt.sphere_index], si.p, u0, u1, &wi, &lpdf);
  } else {
    RGB3 li_rgb;
    float uv[3];
    env_li_sample(P.S.env, P.S.quirks, u0, u1, &wi, &li_rgb, &lpdf, &ok, uv);
    li_possible = (P.S.quirks & WPBR_Q_ENV_LI_SAMPLE_FIX) != 0;
    flags |= SS_LENV;
    s3.x = uv[0];
    s3.y = uv[1];
  }
  if (ok && li_possible && m.type != WPBR_MAT_SPECULAR) {
    // bsdf_eval: the specular lobe evaluates to pdf 0, which contributes nothing
    V3 wi_l = to_local(fr, wi);
    V3 wh = normalize(add(wo_l, wi_l));
    float d = tr_d(m.alpha_x, m.alpha_y, wh);
    float bpdf = (d * abs_cos(wh)) / (4.0f * dot(wo_l, wh));
    if (bpdf != 0.0f) {
      flags |= SS_LB;
      FScalars F = f_scalars(m, d, wh, wo_l, wi_l);
      if (F.zero) flags |= SS_LZERO;
      float w = power_heuristic(lpdf, bpdf);
      s0.w = w / lpdf;
      s1 = make_float4(F.c, F.kf, F.fcos, 0.0f);
      sq.push(true, 2 * pix, add(si.p, mul(wi, (float)0.1)), wi);
    }
  }
  // ---- BSDF-sampling branch
  wpbr_rng::sample2d(P.rs, pix, pass, wpbr_rng::DIM_BSDF, &u0, &u1);
  V3 wi_l;
  float bpdf = 0.0f;
  bool valid;
  FScalars F;
  if (m.type == WPBR_MAT_SPECULAR) {
    // SBXDFSpecularReflectance::sample_f: f = R * (Fr / |cos|) * |cos|
    wi_l = V3{-wo_l.x, -wo_l.y, wo_l.z};
    bpdf = 1.0f;
    valid = true;
    F.fcos = abs_cos(wi_l);
    F.c = 0.0f;
    F.zero = !(F.fcos != 0.0f);
    F.kf = F.zero ? 0.0f : fresnel_dielectric(wi_l.z, m.eta_i[0], m.eta_t[0]) / F.fcos;
  } else {
    float d;
    V3 wh = tr_sample(m.alpha_x, m.alpha_y, wo_l, u0, u1, &d);
    wi_l = reflect(wo_l, wh);
    valid = same_hemi(wi_l, wo_l);
    if (valid) {
      bpdf = (d * abs_cos(wh)) / (4.0f * dot(wo_l, wh));
      F = f_scalars(m, d, wh, wo_l, wi_l);
    }
  }
  if (valid) {
    V3 wi_w = to_world(fr, wi_l);
    bool contributes = true;
    float blpdf = 0.0f;
    if (lt.type == WPBR_LIGHT_SPHERE) {
      blpdf = sphere_light_pdf(P.S.sph_o2w[lt.sphere_index], P.S.sph_r[lt.sphere_index], si.p, P.S.quirks);
    } else {
      flags |= SS_BENV;
      V3 wl = xvector(P.S.env.w2l, wi_w);
      float theta = sph_theta(wl);
      float phi = sph_phi(wl);
      float uu = (float)((double)phi / (2.0 * kPI));
      float vv = (float)((double)theta / kPI);
      float stt = sinf_(theta);
      contributes = stt != 0.0f;  // else Li stays black
      if (contributes) blpdf = (float)((double)env_pdf_uv(P.S.env, uu, vv) / (((2.0 * kPI) * kPI) * (double)stt));
      s3.z = uu;
      s3.w = vv;
    }
    if (contributes) {
      flags |= SS_BB;
      if (F.zero) flags |= SS_BZERO;
      float w = (bpdf == 1.0f) ? 1.0f : power_heuristic(bpdf, blpdf);
      s1.w = w / bpdf;
      s2 = make_float4(F.c, F.kf, F.fcos, 0.0f);
      sq.push(true, 2 * pix + 1, add(si.p, mul(wi_w, (float)0.01)), wi_w);
    }
  }
  s0.x = __uint_as_float(flags);
  st[0] = s0;
  st[1] = s1;
  st[2] = s2;
  st[3] = s3;
}

// ---- per-bin part (a half-warp per pixel, 4 bins per lane) -----------------

struct Bins4 {
  float v[4];
};
__device__ __forceinline__ Bins4 ld_bins(const float* p) {
  float4 q = *reinterpret_cast<const float4*>(p);
  return Bins4{{q.x, q.y, q.z, q.w}};
}
__device__ __forceinline__ void st_bins(float* p, const Bins4& b) {
  *reinterpret_cast<float4*>(p) = make_float4(b.v[0], b.v[1], b.v[2], b.v[3]);
}
__device__ __forceinline__ Bins4 bins_const(float v) { return Bins4{{v, v, v, v}}; }
__device__ __forceinline__ bool bins_nonzero(const Bins4& b) {
  return b.v[0] != 0.0f || b.v[1] != 0.0f || b.v[2] != 0.0f || b.v[3] != 0.0f;
}
// s64_from_rgb at bins b0..b0+3: the same three accumulation steps per bin.
__device__ __forceinline__ Bins4 bins_from_rgb(RGB3 c, bool illuminant, int b0) {
  const float(*B)[kSpecN] = illuminant ? g_spec.illum : g_spec.refl;
  float r = c.r, g = c.g, b = c.b;
  int k0, k1, k2;
  float a0, a1, a2;
  if (r <= g && r <= b) {
    k0 = kSpWhite; a0 = r;
    if (g <= b) { k1 = kSpCyan; a1 = g - r; k2 = kSpBlue; a2 = b - g; }
    else { k1 = kSpCyan; a1 = b - r; k2 = kSpGreen; a2 = g - b; }
  } else if (g <= r && g <= b) {
    k0 = kSpWhite; a0 = g;
    if (r <= b) { k1 = kSpMagenta; a1 = r - g; k2 = kSpBlue; a2 = b - r; }
    else { k1 = kSpMagenta; a1 = b - g; k2 = kSpRed; a2 = r - b; }
  } else {
    k0 = kSpWhite; a0 = b;
    if (r <= g) { k1 = kSpYellow; a1 = r - b; k2 = kSpGreen; a2 = g - r; }
    else { k1 = kSpYellow; a1 = g - b; k2 = kSpRed; a2 = r - g; }
  }
  Bins4 s;
  for (int j = 0; j < 4; ++j) {
    float v = 0.0f + B[k0][b0 + j] * a0;
    v = v + B[k1][b0 + j] * a1;
    s.v[j] = v + B[k2][b0 + j] * a2;
  }
  return s;
}
// Spectrum(Spectrum(RGB texel lookup, Illuminant) * LEmit), bins b0..b0+3
__device__ __forceinline__ Bins4 bins_env(const EnvView& e, float s, float t, const float* lemit, int b0) {
  Bins4 r = bins_from_rgb(env_bilerp(e, s, t), true, b0);
  Bins4 le = ld_bins(lemit + b0);
  for (int j = 0; j < 4; ++j) r.v[j] = r.v[j] * le.v[j];
  return r;
}

struct MatBins {
  Bins4 R, eta_i, eta_t, k;
};

__device__ __forceinline__ Bins4 bins_f(bool cond, bool zero, float c, float kf, float fcos, const MatBins& M) {
  Bins4 f;
  for (int j = 0; j < 4; ++j) {
    float v;
    if (zero)
      v = 0.0f;
    else if (cond)
      v = (fresnel_conductor(c, M.eta_i.v[j], M.eta_t.v[j], M.k.v[j]) * M.R.v[j]) * kf;
    else
      v = M.R.v[j] * kf;
    f.v[j] = v * fcos;
  }
  return f;
}

// 12 resident blocks per SM (40 registers): 1080p Sampled64 669 -> 682
// Msamples/s against the unbounded 64 registers (16 blocks: 675).
__global__ void __launch_bounds__(128, 12) k_sfinish(PassCtx P, SpecCtx C, const float4* state,
                                                     const uint32_t* shadow, const uint32_t* order) {
  uint32_t slot = (blockIdx.x * blockDim.x + threadIdx.x) / kBinLanes;
  if (slot >= P.W * P.H) return;  // the whole half-warp leaves together
  uint32_t pix = order ? order[slot] : slot;  // material-sorted (large films)
  if (pix >= P.W * P.H) return;
  uint32_t lane = threadIdx.x & 31u;
  uint32_t hmask = 0xFFFFu << (lane & 16u);
  int b0 = 4 * (int)(lane & 15u);
  const float4* st = state + (size_t)pix * kSpecStateF4;
  float4 s0 = st[0];
  uint32_t flags = __float_as_uint(s0.x);
  uint32_t li_idx = __float_as_uint(s0.y);
  Bins4 L = bins_const(0.0f);
  if (flags & SS_MISS_ENV) {
    float4 s3 = st[3];
    Bins4 le = bins_env(P.S.env, s3.x, s3.y, C.light_le[li_idx].v, b0);
    for (int j = 0; j < 4; ++j) L.v[j] = L.v[j] + le.v[j];
  } else if (flags & (SS_LB | SS_BB)) {
    const wpbr_light& lt = P.S.lights[li_idx];
    uint32_t lp = light_prim(lt);
    const float* lemit = C.light_le[li_idx].v;
    MatBins M;
    if (flags & SS_TEX) {
      // R = Spectrum(1.0), etaI = Spectrum(1.0f), etaT = Spectrum(1.5f),
      // k = (Spectrum)metallic (CMaterialMetal.cpp:44-48)
      float4 kr = st[4];
      M.R = bins_const(1.0f);
      M.eta_i = bins_const(1.0f);
      M.eta_t = bins_const(1.5f);
      M.k = bins_from_rgb(RGB3{kr.x, kr.y, kr.z}, false, b0);
    } else {
      const SpecMat& sm = C.mats[__float_as_uint(s0.z)];
      M.R = ld_bins(sm.R.v + b0);
      M.eta_i = ld_bins(sm.eta_i.v + b0);
      M.eta_t = ld_bins(sm.eta_t.v + b0);
      M.k = ld_bins(sm.k.v + b0);
    }
    float4 s1 = st[1], s3 = st[3];
    bool cond = (flags & SS_COND) != 0;
    if (flags & SS_LB) {
      uint32_t hp = shadow[2 * pix];
      if (hp == kNoHit || hp == lp) {
        Bins4 li = (flags & SS_LENV) ? bins_env(P.S.env, s3.x, s3.y, lemit, b0) : ld_bins(lemit + b0);
        if (__ballot_sync(hmask, bins_nonzero(li)) & hmask) {
          Bins4 f = bins_f(cond, (flags & SS_LZERO) != 0, s1.x, s1.y, s1.z, M);
          for (int j = 0; j < 4; ++j) L.v[j] = L.v[j] + (li.v[j] * f.v[j]) * s0.w;
        }
      }
    }
    if (flags & SS_BB) {
      uint32_t hp = shadow[2 * pix + 1];
      if (hp == kNoHit || hp == lp) {
        Bins4 bli = (flags & SS_BENV) ? bins_env(P.S.env, s3.z, s3.w, lemit, b0) : ld_bins(lemit + b0);
        if (__ballot_sync(hmask, bins_nonzero(bli)) & hmask) {
          float4 s2 = st[2];
          Bins4 f = bins_f(cond, (flags & SS_BZERO) != 0, s2.x, s2.y, s2.z, M);
          for (int j = 0; j < 4; ++j) L.v[j] = L.v[j] + (bli.v[j] * f.v[j]) * s1.w;
        }
      }
    }
  }
  st_bins(C.L + (size_t)pix * kSpecN + b0, L);
}

// Tile-clipped Mitchell gather of k_film_tiles, 64 bins per sample. A block
// handles an 8x8 pixel tile (inside one 32x32 film tile): it stages the
// 12x12 halo of sample spectra (those inside the film tile's clipped window)
// in shared memory with asynchronous copies, computes the 64 x 25 neighbour
// weights and footprint tests meanwhile, flags black samples, then each
// pixel's 4 threads (16
// bins each) walk the 25 neighbours in row-major order — the reference's
// sample order within the clipped window — with invalid or black samples
// predicated off, so the threads of a warp never diverge.
constexpr int kFT = 8;                    // block tile side (pixels)
constexpr int kHalo = kFT + 4;            // staged samples per side
constexpr int kSStride = kSpecN + 4;      // floats per staged sample (float4-aligned, bank-skewed)
constexpr int kFilmThreads = kFT * kFT * 4;
constexpr int kFilmBins = kSpecN / 4;
// npass passes' samples (pass j's film positions at pf + j * W * H and
// spectra at L + j * W * H * 64) are added in pass order, each pass's
// neighbours in row-major order, to an accumulator held in registers: the
// same sums as npass one-pass gathers, with one read and one write of the
// 64-bin accumulator.
__global__ void __launch_bounds__(kFilmThreads, 4) k_sfilm(uint32_t W, uint32_t H, const float2* pf, const float* L,
                                                        uint32_t npass, float* acc, float4* accw) {
  __shared__ __align__(16) float S[kHalo * kHalo * kSStride];
  __shared__ float wt[kFT * kFT * 25];
  __shared__ uint32_t vmask[kFT * kFT];
  __shared__ uint8_t black[kHalo * kHalo];
  const int tid = (int)threadIdx.x;
  const int bx0 = (int)blockIdx.x * kFT, by0 = (int)blockIdx.y * kFT;
  const int tx0 = (bx0 / 32) * 32, ty0 = (by0 / 32) * 32;
  const int tx1 = min(tx0 + 31, (int)W - 1), ty1 = min(ty0 + 31, (int)H - 1);
  const int p = tid / 4, q = tid % 4;
  const int lx = p % kFT, ly = p / kFT;
  const int x = bx0 + lx, y = by0 + ly;
  const bool mine = x < (int)W && y < (int)H;  // this thread's pixel is on the film
  const size_t pix = mine ? (size_t)y * W + x : 0;
  float* ap = acc + pix * kSpecN + kFilmBins * q;
  float a[kFilmBins];
  float ws = 0.0f;
  if (mine) {
#pragma unroll
    for (int j = 0; j < kFilmBins / 4; ++j) {
      float4 t = *reinterpret_cast<const float4*>(ap + 4 * j);
      a[4 * j] = t.x; a[4 * j + 1] = t.y; a[4 * j + 2] = t.z; a[4 * j + 3] = t.w;
    }
    ws = accw[pix].w;
  }
  const size_t plane = (size_t)W * H;
  for (uint32_t ps = 0; ps < npass; ++ps) {
    const float2* pfp = pf + ps * plane;
    const float* Lp = L + ps * plane * kSpecN;
    // halo spectra: asynchronous 16-byte global-to-shared copies (cp.async),
    // zero-filled outside the film tile's clipped window; they land while
    // the weights are computed
    for (int i = tid; i < kHalo * kHalo * 16; i += kFilmThreads) {
      int h = i / 16, c = i % 16;
      int sy = by0 - 2 + h / kHalo, sx = bx0 - 2 + h % kHalo;
      bool in = sy >= ty0 && sy <= ty1 && sx >= tx0 && sx <= tx1;
      const float* src = in ? Lp + ((size_t)sy * W + sx) * kSpecN + 4 * c : Lp;
      uint32_t dst = (uint32_t)__cvta_generic_to_shared(S + h * kSStride + 4 * c);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(in ? 16 : 0) : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    if (tid < kFT * kFT) vmask[tid] = 0u;
    __syncthreads();
    // neighbour weights: entry p * 25 + k is neighbour k (row-major in the 5x5 window) of pixel p
    for (int e = tid; e < kFT * kFT * 25; e += kFilmThreads) {
      int pe = e / 25, k = e % 25;
      int xe = bx0 + pe % kFT, ye = by0 + pe / kFT;
      int sx = xe - 2 + k % 5, sy = ye - 2 + k / 5;
      float w = 0.0f;
      if (xe < (int)W && ye < (int)H && sx >= tx0 && sx <= tx1 && sy >= ty0 && sy <= ty1) {
        float2 f = pfp[(size_t)sy * W + sx];
        float dx0 = f.x - 0.5f, dy0 = f.y - 0.5f;
        int pminx = (int)ceilf(dx0 - 2.0f), pmaxx = (int)floorf(dx0 + 2.0f);
        int pminy = (int)ceilf(dy0 - 2.0f), pmaxy = (int)floorf(dy0 + 2.0f);
        pminx = max(pminx, tx0);
        pminy = max(pminy, ty0);
        pmaxx = min(pmaxx, tx1);
        pmaxy = min(pmaxy, ty1);
        if (!(xe < pminx || xe > pmaxx || ye < pminy || ye > pmaxy)) {
          w = mitchell1(((float)xe - f.x) / 2.0f) * mitchell1(((float)ye - f.y) / 2.0f);
          atomicOr(&vmask[pe], 1u << k);
        }
      }
      wt[e] = w;
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();
    // each sample's black flag, 16 threads (a half-warp) per sample
    for (int i = tid; i < kHalo * kHalo * 16; i += kFilmThreads) {
      int h = i / 16, c = i % 16;
      float4 v = *reinterpret_cast<const float4*>(S + h * kSStride + 4 * c);
      bool nz = v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || v.w != 0.0f;
      uint32_t bal = __ballot_sync(0xFFFFFFFFu, nz);
      if (c == 0) black[h] = ((bal >> (threadIdx.x & 16u)) & 0xFFFFu) == 0u;
    }
    __syncthreads();
    if (mine) {
      const uint32_t vm = vmask[p];
      const float* base = S + (ly * kHalo + lx) * kSStride + kFilmBins * q;
      const uint8_t* bl = black + ly * kHalo + lx;
      const float* wp = wt + p * 25;
#pragma unroll
      for (int k = 0; k < 25; ++k) {
        const int off = (k / 5) * kHalo + k % 5;
        const bool v = (vm >> k) & 1u;
        const float w = wp[k];
        const bool take = v && !bl[off];
        const float* sp = base + off * kSStride;
        if (take) {
#pragma unroll
          for (int j = 0; j < kFilmBins / 4; ++j) {
            float4 t = *reinterpret_cast<const float4*>(sp + 4 * j);
            a[4 * j] = a[4 * j] + t.x * w;
            a[4 * j + 1] = a[4 * j + 1] + t.y * w;
            a[4 * j + 2] = a[4 * j + 2] + t.z * w;
            a[4 * j + 3] = a[4 * j + 3] + t.w * w;
          }
        }
        ws = v ? ws + w : ws;
      }
    }
    __syncthreads();  // the next pass restages S, wt, vmask and black
  }
  if (!mine) return;
#pragma unroll
  for (int j = 0; j < kFilmBins / 4; ++j)
    *reinterpret_cast<float4*>(ap + 4 * j) = make_float4(a[4 * j], a[4 * j + 1], a[4 * j + 2], a[4 * j + 3]);
  if (q == 0) accw[pix].w = ws;
}

// toRGB of the accumulated spectra (s64_to_rgb: per bin products, the three
// sums taken sequentially in bin order, bin width, XYZ to RGB matrix). A
// warp stages 32 pixels' spectra in shared memory with coalesced loads, then
// each lane sums one pixel.
constexpr int kResolveRow = kSpecN + 1;  // padded row: lane l reads bank (l + i) mod 32
__global__ void __launch_bounds__(128) k_sresolve(uint32_t n, const float* acc, float4* accw, uint32_t quirks) {
  __shared__ float sh[4][32 * kResolveRow];
  uint32_t warp = threadIdx.x / 32, lane = threadIdx.x & 31u;
  uint64_t base = ((uint64_t)blockIdx.x * 4 + warp) * 32;
  if (base >= n) return;
  float* row = sh[warp];
  for (int i = 0; i < kSpecN; ++i) {
    uint32_t k = (uint32_t)i * 32 + lane;  // element k of the warp's 32 x 64 block
    uint64_t p = base + k / kSpecN;
    if (p < n) row[(k / kSpecN) * kResolveRow + k % kSpecN] = acc[p * kSpecN + k % kSpecN];
  }
  __syncwarp();
  uint64_t p = base + lane;
  if (p >= n) return;
  const float* s = row + lane * kResolveRow;
  float X = 0.0f, Y = 0.0f, Z = 0.0f;
  for (int i = 0; i < kSpecN; ++i) {
    float v = s[i];
    X = X + v * g_spec.X[i];
    Y = Y + v * g_spec.Y[i];
    Z = Z + v * g_spec.Z[i];
  }
  float dl = (float)(wpbr_spec::kLambdaEnd - wpbr_spec::kLambdaStart) / (float)kSpecN;
  X = X * dl;
  Y = Y * dl;
  Z = Z * dl;
  float m20 = (quirks & WPBR_Q_XYZ_MATRIX_FIX) ? 0.055648f : 0.041556f;
  float r = (X * 3.240479f + Y * -1.537150f) + Z * -0.498535f;
  float g = (X * -0.969256f + Y * 1.875991f) + Z * 0.041556f;
  float b = (X * m20 + Y * -0.204043f) + Z * 1.057311f;
  float4 a = accw[p];
  accw[p] = make_float4(r, g, b, a.w);
}

}  // namespace

wpbr_status spectral_setup(wpbr_ctx* ctx) {
  RenderState& R = ctx->rs;
  size_t n = (size_t)R.W * R.H;
  SpecTables T;
  build_tables(&T);
  WPBR_CUDA(cudaMemcpyToSymbolAsync(g_spec, &T, sizeof(T), 0, cudaMemcpyHostToDevice, ctx->stream));
  // material and light spectra from the scene's RGB parameters
  std::vector<wpbr_material> mats(ctx->nmat);
  WPBR_CUDA(cudaMemcpyAsync(mats.data(), ctx->mats.p, sizeof(wpbr_material) * ctx->nmat, cudaMemcpyDeviceToHost,
                            ctx->stream));
  WPBR_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<SpecMat> sm(ctx->nmat);
  for (uint32_t i = 0; i < ctx->nmat; ++i) {
    const wpbr_material& m = mats[i];
    sm[i].R = s64_of_param(T, RGB3{m.R[0], m.R[1], m.R[2]}, false);
    sm[i].eta_i = s64_of_param(T, RGB3{m.eta_i[0], m.eta_i[1], m.eta_i[2]}, false);
    sm[i].eta_t = s64_of_param(T, RGB3{m.eta_t[0], m.eta_t[1], m.eta_t[2]}, false);
    sm[i].k = s64_of_param(T, RGB3{m.k[0], m.k[1], m.k[2]}, false);
  }
  std::vector<S64> le(ctx->h_lights.size() ? ctx->h_lights.size() : 1);
  for (size_t i = 0; i < ctx->h_lights.size(); ++i) {
    const wpbr_light& l = ctx->h_lights[i];
    RGB3 c = l.type == WPBR_LIGHT_SPHERE ? RGB3{l.Le[0], l.Le[1], l.Le[2]} : ctx->env_le;
    le[i] = s64_of_param(T, c, false);
  }
  WPBR_CUDA(R.spec_mats.ensure(sizeof(SpecMat) * sm.size() / sizeof(float) + 1));
  WPBR_CUDA(R.spec_le.ensure(le.size() * kSpecN));
  WPBR_CUDA(cudaMemcpyAsync(R.spec_mats.p, sm.data(), sizeof(SpecMat) * sm.size(), cudaMemcpyHostToDevice,
                            ctx->stream));
  WPBR_CUDA(cudaMemcpyAsync(R.spec_le.p, le.data(), sizeof(S64) * le.size(), cudaMemcpyHostToDevice, ctx->stream));
  WPBR_CUDA(R.spec_L.ensure(n * kSpecN));
  WPBR_CUDA(R.spec_acc.ensure(n * kSpecN));
  WPBR_CUDA(cudaMemsetAsync(R.spec_acc.p, 0, sizeof(float) * n * kSpecN, ctx->stream));
  WPBR_CUDA(cudaStreamSynchronize(ctx->stream));
  return WPBR_OK;
}

static PassCtx spec_pass_ctx(wpbr_ctx* ctx) {
  PassCtx P;
  P.S = scene_view(ctx);
  P.Bv = render_traversal_view(ctx);
  P.rs = wpbr_rng::Stream{ctx->rs.seed, ctx->rs.stream, ctx->rs.spp, (ctx->quirks & WPBR_Q_REF_SAMPLER_ARRAYS) ? 1u : 0u};
  P.W = ctx->rs.W;
  P.H = ctx->rs.H;
  P.err = ctx->d_err.p;
  return P;
}

// Room for `slots` passes' film positions and sample spectra.
cudaError_t spectral_slots(wpbr_ctx* ctx, uint32_t slots) {
  RenderState& R = ctx->rs;
  const size_t n = (size_t)R.W * R.H;
  cudaError_t e = R.pfilm.ensure(slots * n);
  if (e == cudaSuccess) e = R.spec_L.ensure(slots * n * kSpecN);
  return e;
}

// The scalar spawn of the Sampled64 pass, between the camera traversal and
// the shadow-ray traversal (render_pass_launch); the pass's film positions go
// to sample slot `slot`.
cudaError_t spectral_spawn_launch(wpbr_ctx* ctx, const uint32_t* pass_ptr, const uint32_t* order, uint32_t slot) {
  RenderState& R = ctx->rs;
  uint32_t n = R.W * R.H;
  const ShadowQueue sq{R.shadow_rays.p, R.shadow_map.p, R.counters.p + kQueueCounter};
  (ctx->has_metal ? k_sspawn<true> : k_sspawn<false>)<<<div_up(n, kTB), kTB, 0, ctx->stream>>>(
      spec_pass_ctx(ctx), pass_ptr, R.hit_prim.p, R.pstate.p, sq, R.pfilm.p + (size_t)slot * n, order);
  return cudaGetLastError();
}

// The per-bin finish after the shadow-ray traversal (the pass's spectra to
// sample slot `slot`), then, when film_slots > 0, the film gather of slots
// 0 .. film_slots - 1 in slot order.
cudaError_t spectral_finish_launch(wpbr_ctx* ctx, const uint32_t* order, uint32_t slot, uint32_t film_slots) {
  RenderState& R = ctx->rs;
  uint32_t n = R.W * R.H;
  SpecCtx C{(const SpecMat*)R.spec_mats.p, (const S64*)R.spec_le.p, R.spec_L.p + (size_t)slot * n * kSpecN};
  k_sfinish<<<div_up((uint64_t)n * kBinLanes, 128), 128, 0, ctx->stream>>>(spec_pass_ctx(ctx), C, R.pstate.p,
                                                                            R.shadow_hit.p, order);
  if (film_slots) {
    dim3 fg(div_up(R.W, kFT), div_up(R.H, kFT));
    k_sfilm<<<fg, kFilmThreads, 0, ctx->stream>>>(R.W, R.H, R.pfilm.p, R.spec_L.p, film_slots, R.spec_acc.p,
                                                   (float4*)R.acc.p);
  }
  return cudaGetLastError();
}

// Converts the accumulated spectra to the RGB film (wpbr_film_read and
// wpbr_film_tonemap read it) when passes ran since the last conversion.
wpbr_status spectral_resolve(wpbr_ctx* ctx) {
  RenderState& R = ctx->rs;
  if (ctx->spectrum != WPBR_SPECTRUM_SAMPLED64 || !R.spec_dirty) return WPBR_OK;
  uint32_t n = R.W * R.H;
  k_sresolve<<<div_up(n, 128), 128, 0, ctx->stream>>>(n, R.spec_acc.p, (float4*)R.acc.p, ctx->quirks);
  WPBR_CUDA(cudaGetLastError());
  R.spec_dirty = false;
  return WPBR_OK;
}

}  // namespace wpbr
