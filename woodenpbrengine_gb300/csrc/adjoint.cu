// adjoint.cu — the differentiable direct-lighting estimator: a forward /
// backward pair giving the gradient of an image L2 loss with respect to the
// per-material parameters (alpha, albedo R, eta, k) and the environment
// texels.
//
// The differentiated function is the frozen-direction estimator: every
// sample's directions (camera ray, light sample, BSDF sample), hit points and
// visibility come from the sampling parameters theta_s (set by
// wpbr_adjoint_freeze); the BSDF values, pdfs, MIS weights and emitted /
// incident radiance are evaluated at the current parameters theta. Its value
// at theta = theta_s is the render of MEngine::render's per-sample job list
// (WoodenPBREngine/MEngine.cpp:393-442), its derivative is the detached-
// sampling gradient, and central differences of it are well defined (no
// visibility or sampling-map discontinuities).
//
// Neither pass stores paths: the backward pass replays each sample pass
// (camera rays, primary traversal, light and BSDF sampling, shadow
// traversal) from the counter-based sample streams and runs the hand-written
// reverse sweep (shade_grad.cuh) per sample. Material gradients are summed in
// shared memory per block, then in double in global memory; texel gradients
// are atomics on a float array; the environment map's normalisation adds one
// global scalar that a final kernel spreads over every texel.
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "ctx.hpp"
#include "pass.cuh"
#include "shade_grad.cuh"
#include "traverse_persistent.cuh"

namespace wpbr {

namespace {

constexpr int kAdjF4 = 6;  // float4 of frozen state per pixel
enum : uint32_t { AF_HIT = 1u, AF_TRACE_L = 2u, AF_TRACE_B = 4u };
constexpr uint32_t kMaxAdjMaterials = 1024;  // shared-memory material accumulators

struct AdjView {
  const wpbr_material* mats_s;  // sampling parameters
  const wpbr_material* mats_e;  // evaluation parameters
  EnvView env_s;                // sampling texels + distribution
  EnvView env_e;                // evaluation texels, map function, integral
};

struct AdjGrad {
  const float4* gpix;  // dLoss/dI / film weight, per pixel
  double* g_mat;       // nmat * 10
  float* g_env;        // W * H * 3, per texel and channel
  float* g_func;       // W * H, per map cell
  double* g_Z;         // derivative with respect to the map integral
  uint32_t nmat;
};

struct MatGrad {
  float a;
  float R[3], eta[3], k[3];
};

__device__ __forceinline__ bool finite3(RGB3 c) { return isfinite(c.r) && isfinite(c.g) && isfinite(c.b); }

// ---- sample generation with the sampling parameters --------------------------
__global__ void __launch_bounds__(kTB, WPBR_ADJ_SPAWN_MIN_BLOCKS) k_adj_spawn(PassCtx P, AdjView A, const uint32_t* pass_dev,
                                                   const uint32_t* hit_prim, float4* state, ShadowQueue sq, float2* pf) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H) return;
  uint32_t pass = *pass_dev;
  float fx, fy;
  camera_sample(P, pix, pass, &fx, &fy);
  pf[pix] = make_float2(fx, fy);
  RayD r = camera_ray(P.S.cam, fx, fy);
  uint32_t prim = hit_prim[pix];
  float4* st = state + (size_t)pix * kAdjF4;
  if (prim == kNoHit || P.S.nlights == 0) {
    st[0] = make_float4(r.d.x, r.d.y, r.d.z, __uint_as_float(prim == kNoHit ? 0u : AF_HIT));
    st[1] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(0xFFFFFFFFu));  // no light: nothing to shade
    return;
  }
  uint32_t flags = AF_HIT;
  SurfInt s = make_si(P.S, prim, r.o, r.d);
  Frame fr = bsdf_frame(s);
  uint32_t mid = prim_material(P.S, prim);
  const wpbr_material& ms = A.mats_s[mid];
  V3 wo_l = to_local(fr, s.wo);
  uint32_t li_idx = pick_light(P, pix, pass);
  const wpbr_light& lt = P.S.lights[li_idx];
  float u0, u1;
  wpbr_rng::sample2d(P.rs, pix, pass, wpbr_rng::DIM_LIGHT, &u0, &u1);
  V3 wi{0, 0, 0};
  RGB3 li = rgb1(0.0f);
  float lpdf = 0.0f;
  bool ok = true;
  float uvs[3] = {0.0f, 0.0f, 0.0f};
  if (lt.type == WPBR_LIGHT_SPHERE) {
    sphere_light_sample(P.S.sph_o2w[lt.sphere_index], P.S.sph_r[lt.sphere_index], s.p, u0, u1, &wi, &lpdf);
    li = RGB3{lt.Le[0], lt.Le[1], lt.Le[2]};
  } else {
    env_li_sample(A.env_s, P.S.quirks, u0, u1, &wi, &li, &lpdf, &ok, uvs);
  }
  const bool trace_l = ok && !rblack(li);
  if (trace_l) flags |= AF_TRACE_L;
  sq.push(trace_l, 2 * pix, add(s.p, mul(wi, (float)0.1)), wi);
  wpbr_rng::sample2d(P.rs, pix, pass, wpbr_rng::DIM_BSDF, &u0, &u1);
  V3 bwi_l;
  float bpdf;
  bool valid;
  bsdf_sample(ms, wo_l, u0, u1, &bwi_l, &bpdf, &valid);
  V3 bwi = to_world(fr, bwi_l);
  if (valid) flags |= AF_TRACE_B;
  sq.push(valid, 2 * pix + 1, add(s.p, mul(bwi, (float)0.01)), bwi);
  V3 wi_l = to_local(fr, wi);
  st[0] = make_float4(wo_l.x, wo_l.y, wo_l.z, __uint_as_float(flags));
  st[1] = make_float4(wi_l.x, wi_l.y, wi_l.z, __uint_as_float(li_idx));
  st[2] = make_float4(bwi_l.x, bwi_l.y, bwi_l.z, __uint_as_float(mid));
  st[3] = make_float4(bwi.x, bwi.y, bwi.z, lpdf);
  st[4] = make_float4(s.p.x, s.p.y, s.p.z, uvs[0]);
  st[5] = make_float4(uvs[1], uvs[2], 0.0f, 0.0f);
}

// ---- evaluation at theta and its reverse sweep ---------------------------------
struct EvalCtx {
  const PassCtx* P;
  const AdjView* A;
  float* smem_mat;  // block accumulators (backward only)
  float* g_env;
  float* g_func;
  double gZ;        // this thread's share of dLoss/dZ
};

__device__ __forceinline__ void add_env_taps(EvalCtx& E, const EnvView& e, float s, float t, RGB3 g) {
  int idx[4];
  float w[4];
  env_taps(e, s, t, idx, w);
  for (int k = 0; k < 4; ++k) {
    if (w[k] == 0.0f) continue;
    float* d = E.g_env + 3 * (size_t)idx[k];
    atomicAdd(d, g.r * e.le.r * w[k]);
    atomicAdd(d + 1, g.g * e.le.g * w[k]);
    atomicAdd(d + 2, g.b * e.le.b * w[k]);
  }
}

// pdf = func[cell] / Z / K: local term to the cell, global term to Z
__device__ __forceinline__ void add_env_pdf(EvalCtx& E, const EnvView& e, int cell, float pdf, float g_pdf) {
  if (g_pdf == 0.0f) return;
  float f = e.cond_func[cell];
  if (f != 0.0f) atomicAdd(E.g_func + cell, g_pdf * pdf / f);
  E.gZ += (double)g_pdf * (-(double)pdf / (double)e.marg_int);
}

__device__ __forceinline__ void add_mat(EvalCtx& E, uint32_t mid, const MatGrad& g) {
  float* m = E.smem_mat + 10 * mid;
  if (g.a != 0.0f) atomicAdd(m, g.a);
  for (int c = 0; c < 3; ++c) {
    if (g.R[c] != 0.0f) atomicAdd(m + 1 + c, g.R[c]);
    if (g.eta[c] != 0.0f) atomicAdd(m + 4 + c, g.eta[c]);
    if (g.k[c] != 0.0f) atomicAdd(m + 7 + c, g.k[c]);
  }
}

// bsdf_eval at theta (value includes |cos wi|) and, given the upstream
// gradients of the value and the pdf, the material partials.
template <bool BACK>
__device__ RGB3 bsdf_eval_ad(const wpbr_material& m, V3 wo, V3 wi, float* pdf, RGB3 gf, float gpdf, MatGrad* g) {
  if (m.type == WPBR_MAT_SPECULAR) {
    *pdf = 0.0f;
    return rgb1(0.0f);
  }
  V3 wh = normalize(add(wo, wi));
  float dD;
  float D = tr_d_grad(m.alpha_x, m.alpha_y, wh, &dD);
  float cwh = abs_cos(wh), dow = dot(wo, wh);
  *pdf = (D * cwh) / (4.0f * dow);
  float co = abs_cos(wo), ci = abs_cos(wi);
  bool zero_f = (ci == 0.0f || co == 0.0f || (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f));
  float c = dot(wi, wh);
  float K = abs_cos(wi) / ((4.0f * ci) * co);
  RGB3 f = rgb1(0.0f);
  float gD = BACK ? gpdf * cwh / (4.0f * dow) : 0.0f;
  if (!zero_f) {
    if (m.type == WPBR_MAT_CONDUCTOR) {
      float Fc[3];
      for (int ch = 0; ch < 3; ++ch) {
        float de, dk;
        Fc[ch] = fresnel_conductor_grad(c, m.eta_i[ch], m.eta_t[ch], m.k[ch], &de, &dk);
        if (BACK) {
          float gfc = ch == 0 ? gf.r : (ch == 1 ? gf.g : gf.b);
          g->R[ch] += gfc * Fc[ch] * D * K;
          gD += gfc * Fc[ch] * m.R[ch] * K;
          float gF = gfc * m.R[ch] * D * K;
          g->eta[ch] += gF * de;
          g->k[ch] += gF * dk;
        }
      }
      f = RGB3{Fc[0] * m.R[0] * D * K, Fc[1] * m.R[1] * D * K, Fc[2] * m.R[2] * D * K};
    } else {
      float de;
      float Fd = fresnel_dielectric_grad(c, m.eta_i[0], m.eta_t[0], &de);
      if (BACK) {
        float gsum = 0.0f;
        for (int ch = 0; ch < 3; ++ch) {
          float gfc = ch == 0 ? gf.r : (ch == 1 ? gf.g : gf.b);
          g->R[ch] += gfc * Fd * D * K;
          gD += gfc * Fd * m.R[ch] * K;
          gsum += gfc * m.R[ch] * D * K;
        }
        g->eta[0] += gsum * de;
      }
      f = RGB3{m.R[0] * Fd * D * K, m.R[1] * Fd * D * K, m.R[2] * Fd * D * K};
    }
  }
  if (BACK) g->a += gD * dD;
  return f;
}

// value of a BSDF-sampled direction: the specular lobe's sample value, else
// the microfacet evaluation; pdf 1 marks the delta lobe.
template <bool BACK>
__device__ RGB3 bsdf_branch_f(const wpbr_material& m, V3 wo, V3 wi, float* pdf, RGB3 gf, float gpdf, MatGrad* g) {
  if (m.type != WPBR_MAT_SPECULAR) return bsdf_eval_ad<BACK>(m, wo, wi, pdf, gf, gpdf, g);
  *pdf = 1.0f;
  if (abs_cos(wi) == 0.0f) return rgb1(0.0f);
  float de;
  float fr = fresnel_dielectric_grad(wi.z, m.eta_i[0], m.eta_t[0], &de);
  if (BACK) {
    g->R[0] += gf.r * fr;
    g->R[1] += gf.g * fr;
    g->R[2] += gf.b * fr;
    g->eta[0] += (gf.r * m.R[0] + gf.g * m.R[1] + gf.b * m.R[2]) * de;
  }
  return RGB3{m.R[0] * fr, m.R[1] * fr, m.R[2] * fr};
}

// One sample at theta. With BACK, gL is dLoss/dL of this sample and the
// partials are accumulated; the return value is L either way.
template <bool BACK>
__device__ RGB3 eval_sample(EvalCtx& E, const float4* st, const uint32_t* shadow, uint32_t pix, RGB3 gL) {
  const PassCtx& P = *E.P;
  const AdjView& A = *E.A;
  float4 s0 = st[0];
  uint32_t flags = __float_as_uint(s0.w);
  RGB3 L = rgb1(0.0f);
  if (!(flags & AF_HIT)) {
    if (P.S.has_env) {
      V3 d{s0.x, s0.y, s0.z};
      V3 dl = xvector(A.env_e.w2l, d);
      float s = (float)((double)sph_phi(dl) / (2.0 * kPI));
      float t = (float)((double)sph_theta(dl) / kPI);
      L = rmul(env_bilerp(A.env_e, s, t), A.env_e.le);
      if (BACK) add_env_taps(E, A.env_e, s, t, gL);
    }
    return L;
  }
  float4 s1 = st[1];
  uint32_t li_idx = __float_as_uint(s1.w);
  if (li_idx == 0xFFFFFFFFu) return L;
  float4 s2 = st[2], s3 = st[3], s4 = st[4], s5 = st[5];
  uint32_t mid = __float_as_uint(s2.w);
  const wpbr_material& m = A.mats_e[mid];
  const wpbr_light& lt = P.S.lights[li_idx];
  uint32_t lp = light_prim(lt);
  V3 wo{s0.x, s0.y, s0.z};
  MatGrad g{};
  // ---- light-sampling branch: L += li f w / lpdf
  if ((flags & AF_TRACE_L) && (shadow[2 * pix] == kNoHit || shadow[2 * pix] == lp)) {
    V3 wi{s1.x, s1.y, s1.z};
    RGB3 li;
    float lpdf;
    int cell = -1;
    if (lt.type == WPBR_LIGHT_SPHERE) {
      li = RGB3{lt.Le[0], lt.Le[1], lt.Le[2]};
      lpdf = s3.w;
    } else {
      li = (P.S.quirks & WPBR_Q_ENV_LI_SAMPLE_FIX) ? rmul(env_bilerp(A.env_e, s4.w, s5.x), A.env_e.le) : rgb1(0.0f);
      cell = env_cell(A.env_e, s4.w, s5.x);
      lpdf = (s5.y != 0.0f) ? env_pdf_cell(A.env_e, cell, s5.y) : 0.0f;
    }
    float bpdf;
    RGB3 f = bsdf_eval_ad<false>(m, wo, wi, &bpdf, rgb1(0.0f), 0.0f, nullptr);
    if (bpdf != 0.0f) {
      float dw_da, dw_db;
      float w = power_heuristic_grad(lpdf, bpdf, &dw_da, &dw_db);
      float T = w / lpdf;
      L = radd(L, rmuls(rmul(li, f), T));
      if (BACK) {
        RGB3 gli{gL.r * f.r * T, gL.g * f.g * T, gL.b * f.b * T};
        RGB3 gf{gL.r * li.r * T, gL.g * li.g * T, gL.b * li.b * T};
        float gT = gL.r * li.r * f.r + gL.g * li.g * f.g + gL.b * li.b * f.b;
        float gw = gT / lpdf;
        float glpdf = -gT * w / (lpdf * lpdf) + gw * dw_da;
        float gbpdf = gw * dw_db;
        bsdf_eval_ad<true>(m, wo, wi, &bpdf, gf, gbpdf, &g);
        if (cell >= 0) {
          if (P.S.quirks & WPBR_Q_ENV_LI_SAMPLE_FIX) add_env_taps(E, A.env_e, s4.w, s5.x, gli);
          add_env_pdf(E, A.env_e, cell, lpdf, glpdf);
        }
      }
    }
  }
  // ---- BSDF-sampling branch: L += li f w / bpdf
  if ((flags & AF_TRACE_B) && (shadow[2 * pix + 1] == kNoHit || shadow[2 * pix + 1] == lp)) {
    V3 wi{s2.x, s2.y, s2.z};
    V3 wiw{s3.x, s3.y, s3.z};
    RGB3 li;
    float lpdf;
    int cell = -1;
    float eu = 0.0f, ev = 0.0f;
    if (lt.type == WPBR_LIGHT_SPHERE) {
      lpdf = sphere_light_pdf(P.S.sph_o2w[lt.sphere_index], P.S.sph_r[lt.sphere_index], V3{s4.x, s4.y, s4.z},
                              P.S.quirks);
      li = RGB3{lt.Le[0], lt.Le[1], lt.Le[2]};
    } else {
      V3 wl = xvector(A.env_e.w2l, wiw);
      float theta = sph_theta(wl);
      float phi = sph_phi(wl);
      eu = (float)((double)phi / (2.0 * kPI));
      ev = (float)((double)theta / kPI);
      float sth = sinf_(theta);
      li = rgb1(0.0f);
      lpdf = 0.0f;
      if (sth != 0.0f) {
        cell = env_cell(A.env_e, eu, ev);
        lpdf = env_pdf_cell(A.env_e, cell, sth);
        li = rmul(env_bilerp(A.env_e, eu, ev), A.env_e.le);
      }
    }
    if (!rblack(li)) {
      float bpdf;
      RGB3 f = bsdf_branch_f<false>(m, wo, wi, &bpdf, rgb1(0.0f), 0.0f, nullptr);
      if (bpdf != 0.0f) {
        float dw_da = 0.0f, dw_db = 0.0f;
        float w = (bpdf == 1.0f) ? 1.0f : power_heuristic_grad(bpdf, lpdf, &dw_da, &dw_db);
        float T = w / bpdf;
        L = radd(L, rmuls(rmul(li, f), T));
        if (BACK) {
          RGB3 gli{gL.r * f.r * T, gL.g * f.g * T, gL.b * f.b * T};
          RGB3 gf{gL.r * li.r * T, gL.g * li.g * T, gL.b * li.b * T};
          float gT = gL.r * li.r * f.r + gL.g * li.g * f.g + gL.b * li.b * f.b;
          float gw = gT / bpdf;
          float gbpdf = -gT * w / (bpdf * bpdf) + gw * dw_da;
          float glpdf = gw * dw_db;
          bsdf_branch_f<true>(m, wo, wi, &bpdf, gf, gbpdf, &g);
          if (cell >= 0) {
            add_env_taps(E, A.env_e, eu, ev, gli);
            add_env_pdf(E, A.env_e, cell, lpdf, glpdf);
          }
        }
      }
    }
  }
  if (BACK) add_mat(E, mid, g);
  return L;
}

// Forward: the sample's radiance (non-finite samples contribute nothing).
__global__ void __launch_bounds__(kTB) k_adj_eval(PassCtx P, AdjView A, const float4* state, const uint32_t* shadow,
                                                  float4* Lb) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H) return;
  EvalCtx E{&P, &A, nullptr, nullptr, nullptr, 0.0};
  RGB3 L = eval_sample<false>(E, state + (size_t)pix * kAdjF4, shadow, pix, rgb1(0.0f));
  if (!finite3(L)) L = rgb1(0.0f);
  Lb[pix] = make_float4(L.r, L.g, L.b, 0.0f);
}


// dLoss/dL of a sample: the transpose of the tile-clipped film gather.
__device__ RGB3 film_adjoint(uint32_t W, uint32_t H, uint32_t pix, float2 f, const float4* gpix) {
  uint32_t sx = pix % W, sy = pix / W;
  int tx0 = (int)((sx / 32) * 32), ty0 = (int)((sy / 32) * 32);
  int tx1 = min(tx0 + 31, (int)W - 1), ty1 = min(ty0 + 31, (int)H - 1);
  float dx0 = f.x - 0.5f, dy0 = f.y - 0.5f;
  int pminx = max((int)ceilf(dx0 - 2.0f), tx0), pmaxx = min((int)floorf(dx0 + 2.0f), tx1);
  int pminy = max((int)ceilf(dy0 - 2.0f), ty0), pmaxy = min((int)floorf(dy0 + 2.0f), ty1);
  RGB3 g = rgb1(0.0f);
  for (int y = pminy; y <= pmaxy; ++y)
    for (int x = pminx; x <= pmaxx; ++x) {
      float w = mitchell1(((float)x - f.x) / 2.0f) * mitchell1(((float)y - f.y) / 2.0f);
      float4 gp = gpix[(size_t)y * W + x];
      g = radd(g, RGB3{gp.x * w, gp.y * w, gp.z * w});
    }
  return g;
}

// Backward: replayed sample, film adjoint, reverse sweep.
__global__ void __launch_bounds__(kTB, WPBR_ADJ_BACK_MIN_BLOCKS) k_adj_back(PassCtx P, AdjView A, const float4* state, const uint32_t* shadow,
                                                  const float2* pf, AdjGrad G) {
  extern __shared__ float smem[];
  __shared__ double zsum[kTB / 32];
  uint32_t nm = G.nmat * 10;
  for (uint32_t j = threadIdx.x; j < nm; j += blockDim.x) smem[j] = 0.0f;
  __syncthreads();
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  EvalCtx E{&P, &A, smem, G.g_env, G.g_func, 0.0};
  if (pix < P.W * P.H) {
    const float4* st = state + (size_t)pix * kAdjF4;
    RGB3 L = eval_sample<false>(E, st, shadow, pix, rgb1(0.0f));
    if (finite3(L)) {
      RGB3 gL = film_adjoint(P.W, P.H, pix, pf[pix], G.gpix);
      if (!rblack(gL)) eval_sample<true>(E, st, shadow, pix, gL);
    }
  }
  double z = E.gZ;
  for (int o = 16; o > 0; o >>= 1) z += __shfl_down_sync(0xFFFFFFFFu, z, o);
  if ((threadIdx.x & 31) == 0) zsum[threadIdx.x >> 5] = z;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kTB / 32; ++w) t += zsum[w];
    if (t != 0.0) atomicAdd(G.g_Z, t);
  }
  for (uint32_t j = threadIdx.x; j < nm; j += blockDim.x)
    if (smem[j] != 0.0f) atomicAdd(G.g_mat + j, (double)smem[j]);
}

// Per pixel: I = acc.rgb / acc.w, loss += |I - T|^2, gpix = 2 (I - T) / (3 N acc.w).
__global__ void k_adj_loss(uint32_t n, const float4* acc, const float* target, float4* gpix, float* image,
                           double* loss) {
  __shared__ double part[256 / 32];
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (i < n) {
    float4 a = acc[i];
    float I[3] = {a.x / a.w, a.y / a.w, a.z / a.w};
    if (image) {
      image[3 * (size_t)i] = I[0];
      image[3 * (size_t)i + 1] = I[1];
      image[3 * (size_t)i + 2] = I[2];
    }
    if (target) {
      float g[3];
      float sc = 2.0f / (3.0f * (float)n * a.w);
      for (int c = 0; c < 3; ++c) {
        float d = I[c] - target[3 * (size_t)i + c];
        l += (double)d * (double)d;
        g[c] = d * sc;
      }
      gpix[i] = make_float4(g[0], g[1], g[2], 0.0f);
    }
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xFFFFFFFFu, l, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = l;
  __syncthreads();
  if (threadIdx.x == 0 && target) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) t += part[w];
    atomicAdd(loss, t);
  }
}

// Map function cells -> texel green channel, through k_env_lum's lookups:
// func[i] = green(bilerp(x/W, y/H)) * sin(theta_y); every cell also carries
// dLoss/dZ * dZ/dfunc = g_Z / (W H).
__global__ void k_adj_env_finish(EnvView e, uint32_t quirks, const float* g_func, const double* g_Z, float* g_env) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t W = e.W, H = e.H;
  if (i >= W * H) return;
  uint32_t x, y;
  if (quirks & WPBR_Q_ENV_DISTRIB_INDEX_BUG) {
    uint32_t yy = min(H - 1, i / H);
    uint32_t xx = i - yy * H;
    if (xx >= W) return;
    x = xx;
    y = yy;
  } else {
    x = i % W;
    y = i / W;
  }
  float g = g_func[i] + (float)(*g_Z / ((double)W * (double)H));
  if (g == 0.0f) return;
  float yN = (float)y / (float)H;
  float sin_t = (float)sin_d((kPI * (double)(float)((float)y + 0.5f)) / (double)(float)H);
  float xN = (float)x / (float)W;
  int idx[4];
  float w[4];
  env_taps(e, xN, yN, idx, w);
  for (int k = 0; k < 4; ++k)
    if (w[k] != 0.0f) atomicAdd(g_env + 3 * (size_t)idx[k] + 1, g * sin_t * w[k]);
}

__global__ void k_apply_mat_params(const float* prm, uint32_t nmat, wpbr_material* mats) {
  uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmat) return;
  const float* p = prm + 10 * (size_t)m;
  wpbr_material& d = mats[m];
  d.alpha_x = p[0];
  d.alpha_y = p[0];
  for (int c = 0; c < 3; ++c) {
    d.R[c] = p[1 + c];
    d.eta_t[c] = p[4 + c];
    d.k[c] = p[7 + c];
  }
}

__global__ void k_env_to_rgb4(const float* prm, uint32_t n, float4* rgb) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  rgb[i] = make_float4(prm[3 * (size_t)i], prm[3 * (size_t)i + 1], prm[3 * (size_t)i + 2], 0.0f);
}

__global__ void k_mat_grad_out(const double* g, uint32_t n, float* out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)g[i];
}

}  // namespace

// ---- host side ---------------------------------------------------------------------

namespace {

EnvView env_view_of(const wpbr_ctx* ctx, const float4* rgb, const float* func, const float* cdf, const float* cint,
                    const float* mfunc, const float* mcdf, float Z) {
  EnvView e = scene_view(ctx).env;
  e.rgb = rgb;
  e.cond_func = func;
  e.cond_cdf = cdf;
  e.cond_int = cint;
  e.marg_func = mfunc;
  e.marg_cdf = mcdf;
  e.marg_int = Z;
  return e;
}

AdjView adj_view(const wpbr_ctx* ctx) {
  const AdjState& J = ctx->adj;
  AdjView A;
  A.mats_s = J.mats_s.p;
  A.mats_e = J.mats_e.p;
  A.env_s = env_view_of(ctx, J.rgb_s.p, J.s_func.p, J.s_cdf.p, J.s_int.p, J.s_mfunc.p, J.s_mcdf.p, J.Z_s);
  A.env_e = env_view_of(ctx, J.rgb_e.p, J.e_func.p, J.e_cdf.p, J.e_int.p, J.e_mfunc.p, J.e_mcdf.p, J.Z_e);
  return A;
}

PassCtx adj_pass_ctx(wpbr_ctx* ctx) {
  PassCtx P;
  P.S = scene_view(ctx);
  P.Bv = render_traversal_view(ctx);
  P.rs = wpbr_rng::Stream{ctx->adj.seed, ctx->adj.stream, ctx->adj.spp, (ctx->quirks & WPBR_Q_REF_SAMPLER_ARRAYS) ? 1u : 0u};
  P.W = ctx->adj.W;
  P.H = ctx->adj.H;
  P.err = ctx->d_err.p;
  return P;
}

wpbr_status rebuild_eval_distribution(wpbr_ctx* ctx) {
  AdjState& J = ctx->adj;
  if (!ctx->has_env) return WPBR_OK;
  EnvDist d{J.e_func.p, J.e_cdf.p, J.e_int.p, J.e_mfunc.p, J.e_mcdf.p, J.e_mint.p};
  return env_distribution_build(ctx, J.rgb_e.p, d, &J.Z_e);
}

// camera + primary traversal + sampling + shadow traversal of one pass
wpbr_status replay_pass(wpbr_ctx* ctx, const PassCtx& P, const AdjView& A, uint32_t pass) {
  AdjState& J = ctx->adj;
  cudaStream_t st = ctx->stream;
  uint32_t n = J.W * J.H;
  WPBR_CUDA(cudaMemcpyAsync(J.pass_dev.p, &pass, 4, cudaMemcpyHostToDevice, st));
  WPBR_CUDA(cudaMemsetAsync(J.counters.p, 0, 3 * sizeof(uint32_t), st));
  launch_traversal<false>(P.S, P.Bv, CameraSrc{P, J.pass_dev.p}, PrimSink{J.hit_prim.p}, n, J.counters.p, P.err, st);
  // shadow rays: the spawn queues the ones it traces (counter word 2), the traversal walks the queue
  const ShadowQueue sq{J.rays.p, J.shadow_map.p, J.counters.p + 2};
  k_adj_spawn<<<div_up(n, kTB), kTB, 0, st>>>(P, A, J.pass_dev.p, J.hit_prim.p, J.state.p, sq, J.pf.p);
  launch_traversal<false>(P.S, P.Bv, QueueSrc{sq.rays, sq.count}, MapSink{J.shadow_hit.p, sq.map}, 2 * n,
                          J.counters.p + 1, P.err, st);
  WPBR_CUDA(cudaGetLastError());
  return WPBR_OK;
}

}  // namespace

wpbr_status adjoint_setup(wpbr_ctx* ctx, uint32_t spp, uint32_t seed, uint32_t stream) {
  if (!ctx->has_scene) return set_err(ctx, WPBR_ERR_NOT_BUILT, "adjoint_setup: no scene");
  if (!ctx->bvh.built) return set_err(ctx, WPBR_ERR_NOT_BUILT, "adjoint_setup: BVH not built");
  if (spp == 0) return set_err(ctx, WPBR_ERR_INVALID_ARG, "adjoint_setup: spp must be > 0");
  if (ctx->spectrum != WPBR_SPECTRUM_RGB)
    return set_err(ctx, WPBR_ERR_INVALID_ARG, "adjoint_setup: the differentiable estimator runs in RGB mode only");
  if (ctx->has_metal)
    return set_err(ctx, WPBR_ERR_INVALID_ARG, "adjoint_setup: textured metal materials have no material parameters");
  if (ctx->nmat > kMaxAdjMaterials)
    return set_err(ctx, WPBR_ERR_INVALID_ARG, "adjoint_setup: more than 1024 materials");
  AdjState& J = ctx->adj;
  cudaStream_t st = ctx->stream;
  J.ready = false;  // until every buffer below exists
  J.spp = spp;
  J.seed = seed;
  J.stream = stream;
  J.W = ctx->cam.W;
  J.H = ctx->cam.H;
  J.nmat = ctx->nmat;
  size_t n = (size_t)J.W * J.H;
  WPBR_CUDA(J.mats_s.ensure(J.nmat));
  WPBR_CUDA(J.mats_e.ensure(J.nmat));
  WPBR_CUDA(cudaMemcpyAsync(J.mats_s.p, ctx->mats.p, sizeof(wpbr_material) * J.nmat, cudaMemcpyDeviceToDevice, st));
  WPBR_CUDA(cudaMemcpyAsync(J.mats_e.p, ctx->mats.p, sizeof(wpbr_material) * J.nmat, cudaMemcpyDeviceToDevice, st));
  J.h_mats.resize(J.nmat);
  WPBR_CUDA(cudaMemcpyAsync(J.h_mats.data(), ctx->mats.p, sizeof(wpbr_material) * J.nmat, cudaMemcpyDeviceToHost, st));
  size_t nt = ctx->has_env ? (size_t)ctx->envW * ctx->envH : 0;
  J.n_texels = nt;
  if (ctx->has_env) {
    uint32_t EW = ctx->envW, EH = ctx->envH;
    for (DevBuf<float4>* b : {&J.rgb_s, &J.rgb_e}) WPBR_CUDA(b->ensure(nt));
    for (DevBuf<float>* b : {&J.s_func, &J.e_func}) WPBR_CUDA(b->ensure(nt));
    for (DevBuf<float>* b : {&J.s_cdf, &J.e_cdf}) WPBR_CUDA(b->ensure((size_t)EH * (EW + 1)));
    for (DevBuf<float>* b : {&J.s_int, &J.e_int, &J.s_mfunc, &J.e_mfunc}) WPBR_CUDA(b->ensure(EH));
    for (DevBuf<float>* b : {&J.s_mcdf, &J.e_mcdf}) WPBR_CUDA(b->ensure(EH + 1));
    for (DevBuf<float>* b : {&J.s_mint, &J.e_mint}) WPBR_CUDA(b->ensure(1));
    WPBR_CUDA(J.g_env.ensure(nt * 3));
    WPBR_CUDA(J.g_func.ensure(nt));
    WPBR_CUDA(J.env_prm.ensure(nt * 3));
    WPBR_CUDA(cudaMemcpyAsync(J.rgb_e.p, ctx->env_rgb.p, sizeof(float4) * nt, cudaMemcpyDeviceToDevice, st));
    WPBR_CUDA(cudaMemcpyAsync(J.rgb_s.p, ctx->env_rgb.p, sizeof(float4) * nt, cudaMemcpyDeviceToDevice, st));
    wpbr_status s = rebuild_eval_distribution(ctx);
    if (s != WPBR_OK) return s;
    EnvDist d{J.s_func.p, J.s_cdf.p, J.s_int.p, J.s_mfunc.p, J.s_mcdf.p, J.s_mint.p};
    s = env_distribution_build(ctx, J.rgb_s.p, d, &J.Z_s);
    if (s != WPBR_OK) return s;
  } else {
    WPBR_CUDA(J.g_env.ensure(1));
    WPBR_CUDA(J.g_func.ensure(1));
  }
  WPBR_CUDA(J.mat_prm.ensure((size_t)J.nmat * 10));
  WPBR_CUDA(J.g_mat.ensure((size_t)J.nmat * 10));
  WPBR_CUDA(J.g_scalar.ensure(2));
  WPBR_CUDA(J.state.ensure(n * kAdjF4));
  WPBR_CUDA(J.rays.ensure(n * 4));
  WPBR_CUDA(J.pf.ensure(n));
  WPBR_CUDA(J.Lb.ensure(n));
  WPBR_CUDA(J.acc.ensure(n));
  WPBR_CUDA(J.gpix.ensure(n));
  WPBR_CUDA(J.target.ensure(n * 3));
  WPBR_CUDA(J.image.ensure(n * 3));
  WPBR_CUDA(J.hit_prim.ensure(n));
  WPBR_CUDA(J.shadow_hit.ensure(2 * n));
  WPBR_CUDA(J.shadow_map.ensure(2 * n));
  WPBR_CUDA(J.pass_dev.ensure(1));
  WPBR_CUDA(J.counters.ensure(3));
  WPBR_CUDA(cudaStreamSynchronize(st));
  J.ready = true;
  J.param_gen += 1;
  J.fwd_gen = 0;
  return WPBR_OK;
}

wpbr_status adjoint_get_params(wpbr_ctx* ctx, float* mat, float* env) {
  AdjState& J = ctx->adj;
  if (!J.ready) return set_err(ctx, WPBR_ERR_NOT_BUILT, "adjoint: adjoint_setup not called");
  cudaStream_t st = ctx->stream;
  if (mat) {
    std::vector<wpbr_material> m(J.nmat);
    WPBR_CUDA(cudaMemcpyAsync(m.data(), J.mats_e.p, sizeof(wpbr_material) * J.nmat, cudaMemcpyDeviceToHost, st));
    WPBR_CUDA(cudaStreamSynchronize(st));
    for (uint32_t i = 0; i < J.nmat; ++i) {
      float* p = mat + 10 * (size_t)i;
      p[0] = m[i].alpha_x;
      for (int c = 0; c < 3; ++c) {
        p[1 + c] = m[i].R[c];
        p[4 + c] = m[i].eta_t[c];
        p[7 + c] = m[i].k[c];
      }
    }
  }
  if (env && J.n_texels) {
    std::vector<float4> t(J.n_texels);
    WPBR_CUDA(cudaMemcpyAsync(t.data(), J.rgb_e.p, sizeof(float4) * J.n_texels, cudaMemcpyDeviceToHost, st));
    WPBR_CUDA(cudaStreamSynchronize(st));
    for (size_t i = 0; i < J.n_texels; ++i) {
      env[3 * i] = t[i].x;
      env[3 * i + 1] = t[i].y;
      env[3 * i + 2] = t[i].z;
    }
  }
  return WPBR_OK;
}

wpbr_status adjoint_set_params(wpbr_ctx* ctx, const float* mat, const float* env, bool device) {
  AdjState& J = ctx->adj;
  if (!J.ready) return set_err(ctx, WPBR_ERR_NOT_BUILT, "adjoint: adjoint_setup not called");
  cudaStream_t st = ctx->stream;
  if (mat) {
    const float* src = mat;
    if (!device) {
      WPBR_CUDA(cudaMemcpyAsync(J.mat_prm.p, mat, sizeof(float) * 10 * J.nmat, cudaMemcpyHostToDevice, st));
      src = J.mat_prm.p;
    }
    k_apply_mat_params<<<div_up(J.nmat, 128), 128, 0, st>>>(src, J.nmat, J.mats_e.p);
    WPBR_CUDA(cudaGetLastError());
  }
  if (env && J.n_texels) {
    const float* src = env;
    if (!device) {
      WPBR_CUDA(cudaMemcpyAsync(J.env_prm.p, env, sizeof(float) * 3 * J.n_texels, cudaMemcpyHostToDevice, st));
      src = J.env_prm.p;
    }
    k_env_to_rgb4<<<div_up(J.n_texels, 256), 256, 0, st>>>(src, (uint32_t)J.n_texels, J.rgb_e.p);
    WPBR_CUDA(cudaGetLastError());
    wpbr_status s = rebuild_eval_distribution(ctx);
    if (s != WPBR_OK) return s;
  }
  J.param_gen += 1;
  return WPBR_OK;
}

wpbr_status adjoint_freeze(wpbr_ctx* ctx) {
  AdjState& J = ctx->adj;
  if (!J.ready) return set_err(ctx, WPBR_ERR_NOT_BUILT, "adjoint: adjoint_setup not called");
  cudaStream_t st = ctx->stream;
  WPBR_CUDA(cudaMemcpyAsync(J.mats_s.p, J.mats_e.p, sizeof(wpbr_material) * J.nmat, cudaMemcpyDeviceToDevice, st));
  if (J.n_texels) {
    uint32_t EW = ctx->envW, EH = ctx->envH;
    size_t nt = J.n_texels;
    auto cp = [&](float* d, const float* s, size_t cnt) {
      return cudaMemcpyAsync(d, s, sizeof(float) * cnt, cudaMemcpyDeviceToDevice, st);
    };
    WPBR_CUDA(cudaMemcpyAsync(J.rgb_s.p, J.rgb_e.p, sizeof(float4) * nt, cudaMemcpyDeviceToDevice, st));
    WPBR_CUDA(cp(J.s_func.p, J.e_func.p, nt));
    WPBR_CUDA(cp(J.s_cdf.p, J.e_cdf.p, (size_t)EH * (EW + 1)));
    WPBR_CUDA(cp(J.s_int.p, J.e_int.p, EH));
    WPBR_CUDA(cp(J.s_mfunc.p, J.e_mfunc.p, EH));
    WPBR_CUDA(cp(J.s_mcdf.p, J.e_mcdf.p, EH + 1));
    WPBR_CUDA(cp(J.s_mint.p, J.e_mint.p, 1));
    J.Z_s = J.Z_e;
  }
  J.param_gen += 1;
  return WPBR_OK;
}

wpbr_status adjoint_forward(wpbr_ctx* ctx, const float* target, float* image, double* loss, bool device) {
  AdjState& J = ctx->adj;
  if (!J.ready) return set_err(ctx, WPBR_ERR_NOT_BUILT, "adjoint: adjoint_setup not called");
  cudaStream_t st = ctx->stream;
  uint32_t n = J.W * J.H;
  PassCtx P = adj_pass_ctx(ctx);
  AdjView A = adj_view(ctx);
  WPBR_CUDA(cudaMemsetAsync(J.acc.p, 0, sizeof(float4) * n, st));
  for (uint32_t p = 0; p < J.spp; ++p) {
    wpbr_status s = replay_pass(ctx, P, A, p);
    if (s != WPBR_OK) return s;
    k_adj_eval<<<div_up(n, kTB), kTB, 0, st>>>(P, A, J.state.p, J.shadow_hit.p, J.Lb.p);
    k_film_tiles<<<dim3(div_up(J.W, kFilmTile), div_up(J.H, kFilmTile)), kFilmThreadsRGB, 0, st>>>(
        J.W, J.H, J.pf.p, J.Lb.p, J.acc.p);
  }
  const float* d_target = nullptr;
  if (target) {
    d_target = target;
    if (!device) {
      WPBR_CUDA(cudaMemcpyAsync(J.target.p, target, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
      d_target = J.target.p;
    }
  }
  float* d_image = image ? (device ? image : J.image.p) : nullptr;
  WPBR_CUDA(cudaMemsetAsync(J.g_scalar.p, 0, sizeof(double) * 2, st));
  k_adj_loss<<<div_up(n, 256), 256, 0, st>>>(n, J.acc.p, d_target, J.gpix.p, d_image, J.g_scalar.p);
  WPBR_CUDA(cudaGetLastError());
  if (image && !device)
    WPBR_CUDA(cudaMemcpyAsync(image, J.image.p, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, st));
  double l = 0.0;
  WPBR_CUDA(cudaMemcpyAsync(&l, J.g_scalar.p, sizeof(double), cudaMemcpyDeviceToHost, st));
  WPBR_CUDA(cudaStreamSynchronize(st));
  if (loss) *loss = target ? l / (3.0 * (double)n) : 0.0;
  J.fwd_gen = target ? J.param_gen : 0;
  return WPBR_OK;
}

wpbr_status adjoint_backward(wpbr_ctx* ctx, float* grad_mat, float* grad_env, bool device) {
  AdjState& J = ctx->adj;
  if (!J.ready) return set_err(ctx, WPBR_ERR_NOT_BUILT, "adjoint: adjoint_setup not called");
  if (J.fwd_gen != J.param_gen)
    return set_err(ctx, WPBR_ERR_NOT_BUILT, "adjoint_backward: no forward pass with a target at these parameters");
  cudaStream_t st = ctx->stream;
  uint32_t n = J.W * J.H;
  PassCtx P = adj_pass_ctx(ctx);
  AdjView A = adj_view(ctx);
  WPBR_CUDA(cudaMemsetAsync(J.g_mat.p, 0, sizeof(double) * 10 * J.nmat, st));
  WPBR_CUDA(cudaMemsetAsync(J.g_scalar.p + 1, 0, sizeof(double), st));
  if (J.n_texels) {
    WPBR_CUDA(cudaMemsetAsync(J.g_env.p, 0, sizeof(float) * 3 * J.n_texels, st));
    WPBR_CUDA(cudaMemsetAsync(J.g_func.p, 0, sizeof(float) * J.n_texels, st));
  }
  AdjGrad G{J.gpix.p, J.g_mat.p, J.g_env.p, J.g_func.p, J.g_scalar.p + 1, J.nmat};
  size_t smem = sizeof(float) * 10 * J.nmat;
  for (uint32_t p = 0; p < J.spp; ++p) {
    wpbr_status s = replay_pass(ctx, P, A, p);
    if (s != WPBR_OK) return s;
    k_adj_back<<<div_up(n, kTB), kTB, smem, st>>>(P, A, J.state.p, J.shadow_hit.p, J.pf.p, G);
  }
  if (J.n_texels)
    k_adj_env_finish<<<div_up(J.n_texels, 256), 256, 0, st>>>(A.env_e, ctx->quirks, J.g_func.p, J.g_scalar.p + 1,
                                                              J.g_env.p);
  WPBR_CUDA(cudaGetLastError());
  float* d_gm = grad_mat ? (device ? grad_mat : J.mat_prm.p) : nullptr;
  if (d_gm) k_mat_grad_out<<<div_up(10 * J.nmat, 256), 256, 0, st>>>(J.g_mat.p, 10 * J.nmat, d_gm);
  if (grad_mat && !device)
    WPBR_CUDA(cudaMemcpyAsync(grad_mat, J.mat_prm.p, sizeof(float) * 10 * J.nmat, cudaMemcpyDeviceToHost, st));
  if (grad_env && J.n_texels) {
    WPBR_CUDA(cudaMemcpyAsync(grad_env, J.g_env.p, sizeof(float) * 3 * J.n_texels,
                              device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
  }
  WPBR_CUDA(cudaGetLastError());
  WPBR_CUDA(cudaStreamSynchronize(st));
  return WPBR_OK;
}

}  // namespace wpbr

using namespace wpbr;

extern "C" {

WPBR_API wpbr_status wpbr_adjoint_setup(wpbr_ctx* ctx, uint32_t spp, uint32_t seed, uint32_t stream) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  return adjoint_setup(ctx, spp, seed, stream);
}

WPBR_API wpbr_status wpbr_adjoint_param_counts(wpbr_ctx* ctx, uint32_t* n_mat_params, uint32_t* n_env_params) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  if (!ctx->adj.ready) return set_err(ctx, WPBR_ERR_NOT_BUILT, "adjoint: adjoint_setup not called");
  if (n_mat_params) *n_mat_params = 10 * ctx->adj.nmat;
  if (n_env_params) *n_env_params = (uint32_t)(3 * ctx->adj.n_texels);
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_adjoint_get_params(wpbr_ctx* ctx, float* mat_params, float* env_params) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  return adjoint_get_params(ctx, mat_params, env_params);
}

WPBR_API wpbr_status wpbr_adjoint_set_params(wpbr_ctx* ctx, const float* mat_params, const float* env_params) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  return adjoint_set_params(ctx, mat_params, env_params, false);
}

WPBR_API wpbr_status wpbr_adjoint_set_params_device(wpbr_ctx* ctx, const float* d_mat_params,
                                                    const float* d_env_params) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  return adjoint_set_params(ctx, d_mat_params, d_env_params, true);
}

WPBR_API wpbr_status wpbr_adjoint_freeze(wpbr_ctx* ctx) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  return adjoint_freeze(ctx);
}

WPBR_API wpbr_status wpbr_adjoint_forward(wpbr_ctx* ctx, const float* target, float* image, double* loss) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  return adjoint_forward(ctx, target, image, loss, false);
}

WPBR_API wpbr_status wpbr_adjoint_forward_device(wpbr_ctx* ctx, const float* d_target, float* d_image, double* loss) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  return adjoint_forward(ctx, d_target, d_image, loss, true);
}

WPBR_API wpbr_status wpbr_adjoint_backward(wpbr_ctx* ctx, float* grad_mat, float* grad_env) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  return adjoint_backward(ctx, grad_mat, grad_env, false);
}

WPBR_API wpbr_status wpbr_adjoint_backward_device(wpbr_ctx* ctx, float* d_grad_mat, float* d_grad_env) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  return adjoint_backward(ctx, d_grad_mat, d_grad_env, true);
}

}  // extern "C"
