// spectral.cu — the Sampled64 parity mode of the render pass: the same
// per-sample job list as the RGB path (MEngine::render, MEngine.cpp:393-442)
// with every radiance, reflectance and Fresnel value a 64-bin
// SampledSpectrum, as the reference computes it (Spectrum = SampledSpectrum,
// CSpectrum.h:8). One thread per pixel and sample (per-thread traversal);
// the film accumulates spectra and is resolved to RGB with toRGB after every
// pass, so wpbr_film_read and wpbr_film_tonemap read it as in RGB mode
// (JobOutputFilmTitles converts with toRGB, CSFilm.cpp:159).
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "ctx.hpp"
#include "pass.cuh"
#include "spectral.cuh"
#include "traverse.cuh"

namespace wpbr {

namespace {

__constant__ SpecTables c_spec;

// Per material: R, eta_i, eta_t, k as spectra.
struct SpecMat {
  S64 R, eta_i, eta_t, k;
};

struct SpecCtx {
  const SpecMat* mats;
  const S64* light_le;  // per light: sphere Le, or the environment's LEmit
  float* L;             // per pixel, 64 floats
};

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

__device__ __forceinline__ void s64_mul(S64& a, const S64& b) {
  for (int i = 0; i < kSpecN; ++i) a.v[i] = a.v[i] * b.v[i];
}

// Spectrum(Spectrum(RGB texel lookup, Illuminant) * LEmit)
__device__ S64 env_spectrum(const EnvView& e, float s, float t, const S64& lemit) {
  S64 r = s64_from_rgb(c_spec, env_bilerp(e, s, t), true);
  s64_mul(r, lemit);
  return r;
}

// mf_f_impl per bin: conductor Fresnel per bin from the eta/k spectra,
// dielectric Fresnel scalar (CFresnelDielectric keeps float etaI/etaT).
__device__ S64 mf_f_spec(const wpbr_material& m, const SpecMat& sm, float d_wh, V3 wh, V3 wo, V3 wi) {
  S64 f = s64_const(0.0f);
  float co = abs_cos(wo), ci = abs_cos(wi);
  if (ci == 0.0f || co == 0.0f) return f;
  if (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) return f;
  float c = dot(wi, wh);
  if (m.type == WPBR_MAT_CONDUCTOR) {
    float k = d_wh / ((4.0f * ci) * co);
    for (int i = 0; i < kSpecN; ++i)
      f.v[i] = (fresnel_conductor(c, sm.eta_i.v[i], sm.eta_t.v[i], sm.k.v[i]) * sm.R.v[i]) * k;
    return f;
  }
  float fr = fresnel_dielectric(c, m.eta_i[0], m.eta_t[0]);
  float k = (fr * d_wh) / ((4.0f * ci) * co);
  for (int i = 0; i < kSpecN; ++i) f.v[i] = sm.R.v[i] * k;
  return f;
}

__device__ S64 bsdf_eval_spec(const wpbr_material& m, const SpecMat& sm, V3 wo, V3 wi, float* pdf) {
  if (m.type == WPBR_MAT_SPECULAR) {
    *pdf = 0.0f;
    return s64_const(0.0f);
  }
  V3 wh = normalize(add(wo, wi));
  float d = tr_d(m.alpha_x, m.alpha_y, wh);
  *pdf = (d * abs_cos(wh)) / (4.0f * dot(wo, wh));
  S64 f = mf_f_spec(m, sm, d, wh, wo, wi);
  float c = abs_cos(wi);
  for (int i = 0; i < kSpecN; ++i) f.v[i] = f.v[i] * c;
  return f;
}

__device__ S64 bsdf_sample_spec(const wpbr_material& m, const SpecMat& sm, V3 wo, float u0, float u1, V3* wi,
                                float* pdf, bool* valid) {
  if (m.type == WPBR_MAT_SPECULAR) {
    *wi = V3{-wo.x, -wo.y, wo.z};
    *pdf = 1.0f;
    *valid = true;
    S64 f = s64_const(0.0f);
    float c = abs_cos(*wi);
    if (c != 0.0f) {
      float fr = fresnel_dielectric(wi->z, m.eta_i[0], m.eta_t[0]);
      for (int i = 0; i < kSpecN; ++i) f.v[i] = sm.R.v[i] * (fr / c);
    }
    for (int i = 0; i < kSpecN; ++i) f.v[i] = f.v[i] * c;
    return f;
  }
  float d;
  V3 wh = tr_sample(m.alpha_x, m.alpha_y, wo, u0, u1, &d);
  *wi = reflect(wo, wh);
  if (!same_hemi(*wi, wo)) {
    *valid = false;
    *pdf = 0.0f;
    return s64_const(0.0f);
  }
  *valid = true;
  *pdf = (d * abs_cos(wh)) / (4.0f * dot(wo, wh));
  S64 f = mf_f_spec(m, sm, d, wh, wo, *wi);
  float c = abs_cos(*wi);
  for (int i = 0; i < kSpecN; ++i) f.v[i] = f.v[i] * c;
  return f;
}

__device__ __forceinline__ uint32_t trace_closest_s(const PassCtx& P, V3 o, V3 d) {
  HitRec h = P.Bv.max_depth < 60 ? trace_ray<false, 64>(P.S, P.Bv, o, d, inf_(), nullptr, nullptr, P.err)
                                 : trace_ray<false, 256>(P.S, P.Bv, o, d, inf_(), nullptr, nullptr, P.err);
  return h.prim;
}

// L += a * b * k, per bin in the RGB path's order ((li * f) * k)
__device__ __forceinline__ void s64_acc(S64& L, const S64& a, const S64& b, float k) {
  for (int i = 0; i < kSpecN; ++i) L.v[i] = L.v[i] + (a.v[i] * b.v[i]) * k;
}

__global__ void k_spec_pass(PassCtx P, SpecCtx C, uint32_t pass, float2* pf) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H) return;
  float fx, fy;
  camera_sample(P, pix, pass, &fx, &fy);
  pf[pix] = make_float2(fx, fy);
  RayD r = camera_ray(P.S.cam, fx, fy);
  S64 L = s64_const(0.0f);
  uint32_t prim = trace_closest_s(P, r.o, r.d);
  uint32_t nl = P.S.nlights;
  if (prim == kNoHit) {
    if (P.S.has_env) {
      uint32_t env_light = 0;
      for (uint32_t i = 0; i < nl; ++i)
        if (P.S.lights[i].type == WPBR_LIGHT_ENV) env_light = i;
      V3 dl = xvector(P.S.env.w2l, r.d);
      float s = (float)((double)sph_phi(dl) / (2.0 * kPI));
      float t = (float)((double)sph_theta(dl) / kPI);
      S64 le = env_spectrum(P.S.env, s, t, C.light_le[env_light]);
      for (int i = 0; i < kSpecN; ++i) L.v[i] = L.v[i] + le.v[i];
    }
  } else if (nl > 0) {
    SurfInt si = make_si(P.S, prim, r.o, r.d);
    Frame fr = bsdf_frame(si);
    uint32_t mid = prim_material(P.S, prim);
    const wpbr_material m = hit_material(P.S, prim, mid, si, r);
    SpecMat tsm;
    if (WPBR_MAT_TEXTURED(P.S.mats[mid].type)) {
      // R = Spectrum(1.0), etaI = Spectrum(1.0f), etaT = Spectrum(1.5f),
      // k = (Spectrum)metallic (CMaterialMetal.cpp:44-48)
      tsm.R = s64_const(1.0f);
      tsm.eta_i = s64_const(1.0f);
      tsm.eta_t = s64_const(1.5f);
      tsm.k = s64_from_rgb(c_spec, RGB3{m.k[0], m.k[1], m.k[2]}, false);
    }
    const SpecMat& sm = (WPBR_MAT_TEXTURED(P.S.mats[mid].type)) ? tsm : C.mats[mid];
    V3 wo_l = to_local(fr, si.wo);
    uint32_t li_idx = pick_light(P, pix, pass);
    const wpbr_light& lt = P.S.lights[li_idx];
    uint32_t lp = light_prim(lt);
    const S64& lemit = C.light_le[li_idx];
    // ---- light-sampling branch
    float u0, u1;
    wpbr_rng::sample2d(P.rs, pix, pass, wpbr_rng::DIM_LIGHT, &u0, &u1);
    V3 wi{0, 0, 0};
    float lpdf = 0.0f;
    bool ok = true;
    S64 li = s64_const(0.0f);
    if (lt.type == WPBR_LIGHT_SPHERE) {
      sphere_light_sample(P.S.sph_o2w[lt.sphere_index], P.S.sph_r[lt.sphere_index], si.p, u0, u1, &wi, &lpdf);
      li = lemit;
    } else {
      RGB3 li_rgb;
      float uv[3];
      env_li_sample(P.S.env, P.S.quirks, u0, u1, &wi, &li_rgb, &lpdf, &ok, uv);
      if (P.S.quirks & WPBR_Q_ENV_LI_SAMPLE_FIX) li = env_spectrum(P.S.env, uv[0], uv[1], lemit);
    }
    if (ok && !s64_black(li)) {
      uint32_t hp = trace_closest_s(P, add(si.p, mul(wi, (float)0.1)), wi);
      if (hp == kNoHit || hp == lp) {
        float bpdf;
        S64 f = bsdf_eval_spec(m, sm, wo_l, to_local(fr, wi), &bpdf);
        if (bpdf != 0.0f) {
          float w = power_heuristic(lpdf, bpdf);
          s64_acc(L, li, f, w / lpdf);
        }
      }
    }
    // ---- BSDF-sampling branch
    wpbr_rng::sample2d(P.rs, pix, pass, wpbr_rng::DIM_BSDF, &u0, &u1);
    V3 wi_l;
    float bpdf;
    bool valid;
    S64 bf = bsdf_sample_spec(m, sm, wo_l, u0, u1, &wi_l, &bpdf, &valid);
    if (valid) {
      V3 wi_w = to_world(fr, wi_l);
      uint32_t hp = trace_closest_s(P, add(si.p, mul(wi_w, (float)0.01)), wi_w);
      if (hp == kNoHit || hp == lp) {
        S64 bli = s64_const(0.0f);
        float blpdf = 0.0f;
        if (lt.type == WPBR_LIGHT_SPHERE) {
          blpdf = sphere_light_pdf(P.S.sph_o2w[lt.sphere_index], P.S.sph_r[lt.sphere_index], si.p, P.S.quirks);
          bli = lemit;
        } else {
          V3 wl = xvector(P.S.env.w2l, wi_w);
          float theta = sph_theta(wl);
          float phi = sph_phi(wl);
          float uu = (float)((double)phi / (2.0 * kPI));
          float vv = (float)((double)theta / kPI);
          float st = sinf_(theta);
          if (st != 0.0f) {
            blpdf = (float)((double)env_pdf_uv(P.S.env, uu, vv) / (((2.0 * kPI) * kPI) * (double)st));
            bli = env_spectrum(P.S.env, uu, vv, lemit);
          }
        }
        if (!s64_black(bli)) {
          float w = (bpdf == 1.0f) ? 1.0f : power_heuristic(bpdf, blpdf);
          s64_acc(L, bli, bf, w / bpdf);
        }
      }
    }
  }
  float* out = C.L + (size_t)pix * kSpecN;
  for (int i = 0; i < kSpecN; ++i) out[i] = L.v[i];
}

// Tile-clipped Mitchell gather of film_gather, 64 bins per sample.
__global__ void k_spec_film(uint32_t W, uint32_t H, const float2* pf, const float* L, float* acc, float4* accw) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= W * H) return;
  uint32_t x = pix % W, y = pix / W;
  uint32_t tx0 = (x / 32) * 32, ty0 = (y / 32) * 32;
  uint32_t tx1 = min(tx0 + 31, W - 1), ty1 = min(ty0 + 31, H - 1);
  float* a = acc + (size_t)pix * kSpecN;
  float ws = accw[pix].w;
  int sy0 = max((int)ty0, (int)y - 2), sy1 = min((int)ty1, (int)y + 2);
  int sx0 = max((int)tx0, (int)x - 2), sx1 = min((int)tx1, (int)x + 2);
  for (int sy = sy0; sy <= sy1; ++sy)
    for (int sx = sx0; sx <= sx1; ++sx) {
      size_t sp = (size_t)sy * W + sx;
      float2 f = pf[sp];
      float dx0 = f.x - 0.5f, dy0 = f.y - 0.5f;
      int pminx = (int)ceilf(dx0 - 2.0f), pmaxx = (int)floorf(dx0 + 2.0f);
      int pminy = (int)ceilf(dy0 - 2.0f), pmaxy = (int)floorf(dy0 + 2.0f);
      pminx = max(pminx, (int)tx0);
      pminy = max(pminy, (int)ty0);
      pmaxx = min(pmaxx, (int)tx1);
      pmaxy = min(pmaxy, (int)ty1);
      if ((int)x < pminx || (int)x > pmaxx || (int)y < pminy || (int)y > pmaxy) continue;
      float w = mitchell1(((float)x - f.x) / 2.0f) * mitchell1(((float)y - f.y) / 2.0f);
      const float* s = L + sp * kSpecN;
      bool black = true;
      for (int i = 0; i < kSpecN; ++i) black = black && s[i] == 0.0f;
      if (!black)
        for (int i = 0; i < kSpecN; ++i) a[i] = a[i] + s[i] * w;
      ws = ws + w;
    }
  accw[pix].w = ws;
}

// toRGB of the accumulated spectra with the context's quirks (film output).
__global__ void k_spec_resolve(uint32_t n, const float* acc, float4* accw, uint32_t quirks) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= n) return;
  RGB3 c = s64_to_rgb(c_spec, acc + (size_t)pix * kSpecN, quirks);
  float4 a = accw[pix];
  accw[pix] = make_float4(c.r, c.g, c.b, a.w);
}

}  // namespace

wpbr_status spectral_setup(wpbr_ctx* ctx) {
  RenderState& R = ctx->rs;
  size_t n = (size_t)R.W * R.H;
  SpecTables T;
  build_tables(&T);
  WPBR_CUDA(cudaMemcpyToSymbolAsync(c_spec, &T, sizeof(T), 0, cudaMemcpyHostToDevice, ctx->stream));
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

wpbr_status spectral_pass(wpbr_ctx* ctx, uint32_t pass) {
  RenderState& R = ctx->rs;
  if (!R.ready) return set_err(ctx, WPBR_ERR_NOT_BUILT, "render_pass: render_setup not called");
  if (pass >= R.spp) return set_err(ctx, WPBR_ERR_INVALID_ARG, "render_pass: pass >= spp");
  PassCtx P;
  P.S = scene_view(ctx);
  P.Bv = ctx->bvh.view;
  P.rs = wpbr_rng::Stream{R.seed, R.stream, R.spp};
  P.W = R.W;
  P.H = R.H;
  P.err = ctx->d_err.p;
  uint32_t n = R.W * R.H;
  SpecCtx C{(const SpecMat*)R.spec_mats.p, (const S64*)R.spec_le.p, R.spec_L.p};
  cudaStream_t st = ctx->stream;
  k_spec_pass<<<div_up(n, 64), 64, 0, st>>>(P, C, pass, R.pfilm.p);
  k_spec_film<<<div_up(n, 128), 128, 0, st>>>(R.W, R.H, R.pfilm.p, R.spec_L.p, R.spec_acc.p, (float4*)R.acc.p);
  k_spec_resolve<<<div_up(n, 128), 128, 0, st>>>(n, R.spec_acc.p, (float4*)R.acc.p, ctx->quirks);
  WPBR_CUDA(cudaGetLastError());
  return WPBR_OK;
}

}  // namespace wpbr
