// render.cu — the per-sample job list of MEngine::render
// (WoodenPBREngine/MEngine.cpp:380-448) as wavefront kernels.
//
// Two forms share the same device functions:
//  * the staged path (wpbr_job_run): one kernel per reference job group over
//    per-pixel state buffers, each recordable for stage-by-stage parity;
//  * the fused path (wpbr_render_pass): camera+primary traversal, shading +
//    sample generation (spawn), one traversal launch for both shadow rays,
//    MIS finish, film gather — five kernels per sample pass, captured once as
//    a CUDA graph that reads the pass index from device memory.
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "ctx.hpp"
#include "pass.cuh"
#include "traverse.cuh"
#include "traverse_persistent.cuh"

namespace wpbr {

namespace {

// Staged-path field slots (float and uint buffers in RenderState).
enum FF {
  F_PFILM, F_RAY_O, F_RAY_D, F_RAY_DX, F_RAY_DY, F_HIT_T, F_SI_P, F_SI_N, F_SI_WO, F_SI_SN, F_SI_SDPDU, F_SI_DPDU,
  F_SI_DPDV, F_SI_DNDU, F_SI_DNDV, F_FRAME, F_LE, F_L_WI, F_L_LI, F_L_PDF, F_L_F, F_L_FPDF, F_B_WI, F_B_F, F_B_PDF,
  F_B_LI, F_B_LPDF, F_L, F_MAT, F_COUNT
};
constexpr int kFW_h[F_COUNT] = {2, 3, 3, 3, 3, 1, 3, 3, 3, 3, 3, 3, 3, 3, 3, 9, 3, 3, 3, 1, 3, 1, 3, 3, 1, 3, 1, 3, 4};
__constant__ int kFW_d[F_COUNT] = {2, 3, 3, 3, 3, 1, 3, 3, 3, 3, 3, 3, 3, 3, 3, 9, 3, 3, 3, 1, 3, 1, 3, 3, 1, 3, 1, 3, 4};
#ifdef __CUDA_ARCH__
#define kFW kFW_d
#else
#define kFW kFW_h
#endif
enum UF { U_HIT_PRIM, U_LIGHT_IDX, U_L_FLAGS, U_B_FLAGS, U_LOK, U_COUNT };

struct Staged {
  float* f[F_COUNT];
  uint32_t* u[U_COUNT];
};

__device__ __forceinline__ uint32_t trace_closest(const PassCtx& P, V3 o, V3 d) {
  HitRec h = P.Bv.max_depth < 60 ? trace_ray<false, 64>(P.S, P.Bv, o, d, inf_(), nullptr, nullptr, P.err)
                                 : trace_ray<false, 256>(P.S, P.Bv, o, d, inf_(), nullptr, nullptr, P.err);
  return h.prim;
}

// ============================== staged jobs =================================
#define kNaN __int_as_float(0x7fc00000)

__global__ void kj_camera(PassCtx P, uint32_t pass, Staged G) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H) return;
  for (int f = 0; f < F_COUNT; ++f)
    for (int c = 0; c < kFW[f]; ++c) G.f[f][(size_t)pix * kFW[f] + c] = kNaN;
  for (int u = 0; u < U_COUNT; ++u) G.u[u][pix] = 0xFFFFFFFFu;
  float fx, fy;
  camera_sample(P, pix, pass, &fx, &fy);
  RayD r = camera_ray(P.S.cam, fx, fy);
  G.f[F_PFILM][2 * pix] = fx;
  G.f[F_PFILM][2 * pix + 1] = fy;
  st3(G.f[F_RAY_O], pix, r.o);
  st3(G.f[F_RAY_D], pix, r.d);
  st3(G.f[F_RAY_DX], pix, r.dxd);
  st3(G.f[F_RAY_DY], pix, r.dyd);
  stc(G.f[F_L], pix, rgb1(0.0f));
}

__global__ void kj_collide(PassCtx P, Staged G) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H) return;
  V3 o = ld3(G.f[F_RAY_O], pix), d = ld3(G.f[F_RAY_D], pix);
  HitRec h = P.Bv.max_depth < 60 ? trace_ray<false, 64>(P.S, P.Bv, o, d, inf_(), nullptr, nullptr, P.err)
                                 : trace_ray<false, 256>(P.S, P.Bv, o, d, inf_(), nullptr, nullptr, P.err);
  G.u[U_HIT_PRIM][pix] = h.prim;
  G.f[F_HIT_T][pix] = h.t;
  if (h.prim == kNoHit) return;
  SurfInt s = make_si(P.S, h.prim, o, d);
  st3(G.f[F_SI_P], pix, s.p);
  st3(G.f[F_SI_N], pix, s.n);
  st3(G.f[F_SI_WO], pix, s.wo);
  st3(G.f[F_SI_SN], pix, s.sn);
  st3(G.f[F_SI_SDPDU], pix, s.sdpdu);
  st3(G.f[F_SI_DPDU], pix, s.dpdu);
  st3(G.f[F_SI_DPDV], pix, s.dpdv);
  st3(G.f[F_SI_DNDU], pix, s.dndu);
  st3(G.f[F_SI_DNDV], pix, s.dndv);
}

__global__ void kj_emitted(PassCtx P, Staged G) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H) return;
  if (G.u[U_HIT_PRIM][pix] != kNoHit || !P.S.has_env) return;
  RGB3 le = env_le(P.S.env, ld3(G.f[F_RAY_D], pix));
  stc(G.f[F_LE], pix, le);
  stc(G.f[F_L], pix, radd(ldc(G.f[F_L], pix), le));
}

__device__ __forceinline__ Frame load_frame(const float* f, uint32_t pix) {
  const float* q = f + 9 * (size_t)pix;
  return Frame{V3{q[0], q[1], q[2]}, V3{q[3], q[4], q[5]}, V3{q[6], q[7], q[8]}};
}

__global__ void kj_bsdf_setup(PassCtx P, Staged G) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H || G.u[U_HIT_PRIM][pix] == kNoHit) return;
  uint32_t prim = G.u[U_HIT_PRIM][pix];
  uint32_t mid = prim_material(P.S, prim);
  if (WPBR_MAT_TEXTURED(P.S.mats[mid].type)) {
    // JobComputeDifferentialsForSurfInter + the uv mapping jobs +
    // JobGenerateBSDFMaterialMetal (MEngine.cpp:399-403)
    RayD r = camera_ray(P.S.cam, G.f[F_PFILM][2 * pix], G.f[F_PFILM][2 * pix + 1]);
    SurfInt hs = make_si(P.S, prim, r.o, r.d);
    float4 v = metal_pack(hit_material(P.S, prim, mid, hs, r));
    float* q = G.f[F_MAT] + 4 * (size_t)pix;
    q[0] = v.x; q[1] = v.y; q[2] = v.z; q[3] = v.w;
  }
  SurfInt s;
  s.sdpdu = ld3(G.f[F_SI_SDPDU], pix);
  s.sn = ld3(G.f[F_SI_SN], pix);
  Frame fr = bsdf_frame(s);
  float* q = G.f[F_FRAME] + 9 * (size_t)pix;
  q[0] = fr.ss.x; q[1] = fr.ss.y; q[2] = fr.ss.z;
  q[3] = fr.ts.x; q[4] = fr.ts.y; q[5] = fr.ts.z;
  q[6] = fr.ns.x; q[7] = fr.ns.y; q[8] = fr.ns.z;
}

__global__ void kj_sample_light(PassCtx P, uint32_t pass, Staged G) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H || G.u[U_HIT_PRIM][pix] == kNoHit || P.S.nlights == 0) return;
  uint32_t li = pick_light(P, pix, pass);
  G.u[U_LIGHT_IDX][pix] = li;
  LightSample ls = sample_light(P, P.S.lights[li], ld3(G.f[F_SI_P], pix), pix, pass);
  st3(G.f[F_L_WI], pix, ls.wi);
  stc(G.f[F_L_LI], pix, ls.li);
  G.f[F_L_PDF][pix] = ls.pdf;
  G.u[U_LOK][pix] = ls.ok ? 1u : 0u;
  G.u[U_L_FLAGS][pix] = 0u;
}

__global__ void kj_shadow_light(PassCtx P, Staged G) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H || G.u[U_HIT_PRIM][pix] == kNoHit || P.S.nlights == 0) return;
  if (!G.u[U_LOK][pix] || rblack(ldc(G.f[F_L_LI], pix))) return;
  V3 wi = ld3(G.f[F_L_WI], pix);
  V3 o = add(ld3(G.f[F_SI_P], pix), mul(wi, (float)0.1));
  uint32_t hp = trace_closest(P, o, wi);
  uint32_t lp = light_prim(P.S.lights[G.u[U_LIGHT_IDX][pix]]);
  G.u[U_L_FLAGS][pix] = 1u | ((hp == kNoHit || hp == lp) ? 2u : 0u);
}

__device__ __forceinline__ wpbr_material staged_material(const PassCtx& P, const Staged& G, uint32_t pix) {
  const wpbr_material& m = P.S.mats[prim_material(P.S, G.u[U_HIT_PRIM][pix])];
  if (!WPBR_MAT_TEXTURED(m.type)) return m;
  const float* q = G.f[F_MAT] + 4 * (size_t)pix;
  return metal_unpack(make_float4(q[0], q[1], q[2], q[3]));
}

__global__ void kj_bsdf_compute(PassCtx P, Staged G) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H || G.u[U_HIT_PRIM][pix] == kNoHit || P.S.nlights == 0) return;
  if (!(G.u[U_L_FLAGS][pix] & 2u)) return;
  Frame fr = load_frame(G.f[F_FRAME], pix);
  wpbr_material m = staged_material(P, G, pix);
  float pdf;
  RGB3 f = bsdf_eval(m, to_local(fr, ld3(G.f[F_SI_WO], pix)), to_local(fr, ld3(G.f[F_L_WI], pix)), &pdf);
  stc(G.f[F_L_F], pix, f);
  G.f[F_L_FPDF][pix] = pdf;
}

__global__ void kj_integrate_light(PassCtx P, Staged G) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H || G.u[U_HIT_PRIM][pix] == kNoHit || P.S.nlights == 0) return;
  if (!(G.u[U_L_FLAGS][pix] & 2u)) return;
  float bpdf = G.f[F_L_FPDF][pix];
  if (bpdf == 0.0f) return;
  float lpdf = G.f[F_L_PDF][pix];
  float w = power_heuristic(lpdf, bpdf);
  RGB3 c = rmuls(rmul(ldc(G.f[F_L_LI], pix), ldc(G.f[F_L_F], pix)), w / lpdf);
  stc(G.f[F_L], pix, radd(ldc(G.f[F_L], pix), c));
}

__global__ void kj_sample_bsdf(PassCtx P, uint32_t pass, Staged G) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H || G.u[U_HIT_PRIM][pix] == kNoHit || P.S.nlights == 0) return;
  Frame fr = load_frame(G.f[F_FRAME], pix);
  wpbr_material m = staged_material(P, G, pix);
  float u0, u1;
  wpbr_rng::sample2d(P.rs, pix, pass, wpbr_rng::DIM_BSDF, &u0, &u1);
  V3 wi_l;
  float pdf;
  bool valid;
  RGB3 f = bsdf_sample(m, to_local(fr, ld3(G.f[F_SI_WO], pix)), u0, u1, &wi_l, &pdf, &valid);
  st3(G.f[F_B_WI], pix, to_world(fr, wi_l));
  stc(G.f[F_B_F], pix, f);
  G.f[F_B_PDF][pix] = pdf;
  G.u[U_B_FLAGS][pix] = valid ? 1u : 0u;
}

__global__ void kj_shadow_bsdf(PassCtx P, Staged G) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H || G.u[U_HIT_PRIM][pix] == kNoHit || P.S.nlights == 0) return;
  uint32_t fl = G.u[U_B_FLAGS][pix];
  if (!(fl & 1u)) return;
  V3 wi = ld3(G.f[F_B_WI], pix);
  V3 o = add(ld3(G.f[F_SI_P], pix), mul(wi, (float)0.01));
  uint32_t hp = trace_closest(P, o, wi);
  uint32_t lp = light_prim(P.S.lights[G.u[U_LIGHT_IDX][pix]]);
  G.u[U_B_FLAGS][pix] = fl | 2u | ((hp == kNoHit || hp == lp) ? 4u : 0u);
}

__global__ void kj_light_compute(PassCtx P, Staged G) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H || G.u[U_HIT_PRIM][pix] == kNoHit || P.S.nlights == 0) return;
  if (!(G.u[U_B_FLAGS][pix] & 4u)) return;
  RGB3 li;
  float pdf;
  light_compute(P, P.S.lights[G.u[U_LIGHT_IDX][pix]], ld3(G.f[F_SI_P], pix), ld3(G.f[F_B_WI], pix), &li, &pdf);
  stc(G.f[F_B_LI], pix, li);
  G.f[F_B_LPDF][pix] = pdf;
}

__global__ void kj_integrate_bsdf(PassCtx P, Staged G) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H || G.u[U_HIT_PRIM][pix] == kNoHit || P.S.nlights == 0) return;
  if (!(G.u[U_B_FLAGS][pix] & 4u)) return;
  RGB3 li = ldc(G.f[F_B_LI], pix);
  if (rblack(li)) return;
  float bpdf = G.f[F_B_PDF][pix];
  float w = (bpdf == 1.0f) ? 1.0f : power_heuristic(bpdf, G.f[F_B_LPDF][pix]);
  RGB3 c = rmuls(rmul(li, ldc(G.f[F_B_F], pix)), w / bpdf);
  stc(G.f[F_L], pix, radd(ldc(G.f[F_L], pix), c));
}

__global__ void kj_film_pack(PassCtx P, Staged G, float2* pf, float4* Lb) {
  uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.W * P.H) return;
  pf[pix] = make_float2(G.f[F_PFILM][2 * pix], G.f[F_PFILM][2 * pix + 1]);
  RGB3 L = ldc(G.f[F_L], pix);
  Lb[pix] = make_float4(L.r, L.g, L.b, 0.0f);
}


// ============================== fused pass ==================================
// Compact per-pixel state written by k_spawn and read by k_finish.
constexpr int kStateF4 = kPassStateF4;
enum : uint32_t { SF_VALID = 1u, SF_TRACE_L = 2u, SF_TRACE_B = 4u, SF_HIT = 8u, SF_METAL = 16u };

template <bool TEX>
__global__ void __launch_bounds__(kTB, TEX ? WPBR_SPAWN_TEX_MIN_BLOCKS : WPBR_SPAWN_MIN_BLOCKS) k_spawn(PassCtx P, const uint32_t* pass_dev, const uint32_t* hit_prim,
                                               float4* state, ShadowQueue sq, float4* Lb, float2* pf,
                                               const uint32_t* order) {
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
  float4* st = state + (size_t)pix * kStateF4;
  RGB3 L = rgb1(0.0f);
  uint32_t flags = 0;
  if (prim == kNoHit || P.S.nlights == 0) {
    if (prim == kNoHit && P.S.has_env) L = radd(L, env_le(P.S.env, r.d));
    st[4] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(flags));
    Lb[pix] = make_float4(L.r, L.g, L.b, 0.0f);
    return;
  }
  flags |= SF_HIT;
  SurfInt s = make_si(P.S, prim, r.o, r.d);
  Frame fr = bsdf_frame(s);
  uint32_t mid = prim_material(P.S, prim);
  const wpbr_material m = hit_material<TEX>(P.S, prim, mid, s, r);
  if (TEX && WPBR_MAT_TEXTURED(P.S.mats[mid].type)) {
    flags |= SF_METAL;
    st[6] = metal_pack(m);
  }
  V3 wo_l = to_local(fr, s.wo);
  uint32_t li_idx = pick_light(P, pix, pass);
  const wpbr_light& lt = P.S.lights[li_idx];
  LightSample ls = sample_light(P, lt, s.p, pix, pass);
  const bool trace_l = ls.ok && !rblack(ls.li);
  if (trace_l) flags |= SF_TRACE_L;
  sq.push(trace_l, 2 * pix, add(s.p, mul(ls.wi, (float)0.1)), ls.wi);
  float u0, u1;
  wpbr_rng::sample2d(P.rs, pix, pass, wpbr_rng::DIM_BSDF, &u0, &u1);
  V3 bwi_l;
  float bpdf;
  bool valid;
  RGB3 bf = bsdf_sample(m, wo_l, u0, u1, &bwi_l, &bpdf, &valid);
  V3 bwi = to_world(fr, bwi_l);
  if (valid) flags |= SF_VALID | SF_TRACE_B;
  sq.push(valid, 2 * pix + 1, add(s.p, mul(bwi, (float)0.01)), bwi);
  V3 wi_l = to_local(fr, ls.wi);
  st[0] = make_float4(ls.li.r, ls.li.g, ls.li.b, ls.pdf);
  st[1] = make_float4(wi_l.x, wi_l.y, wi_l.z, __uint_as_float(li_idx));
  st[2] = make_float4(wo_l.x, wo_l.y, wo_l.z, __uint_as_float(mid));
  st[3] = make_float4(bf.r, bf.g, bf.b, bpdf);
  st[4] = make_float4(bwi.x, bwi.y, bwi.z, __uint_as_float(flags));
  st[5] = make_float4(s.p.x, s.p.y, s.p.z, 0.0f);
  Lb[pix] = make_float4(L.r, L.g, L.b, 0.0f);
}

__global__ void __launch_bounds__(kTB) k_finish(PassCtx P, const float4* state, const uint32_t* shadow, float4* Lb,
                                                const uint32_t* order) {
  uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= P.W * P.H) return;
  uint32_t pix = order ? order[slot] : slot;  // material-sorted (large films)
  if (pix >= P.W * P.H) return;
  const float4* st = state + (size_t)pix * kStateF4;
  float4 s4 = st[4];
  uint32_t flags = __float_as_uint(s4.w);
  if (!(flags & SF_HIT)) return;
  float4 s0 = st[0], s1 = st[1], s2 = st[2], s3 = st[3], s5 = st[5];
  uint32_t li_idx = __float_as_uint(s1.w);
  const wpbr_light& lt = P.S.lights[li_idx];
  uint32_t lp = light_prim(lt);
  const wpbr_material m = (flags & SF_METAL) ? metal_unpack(st[6]) : P.S.mats[__float_as_uint(s2.w)];
  float4 l4 = Lb[pix];
  RGB3 L{l4.x, l4.y, l4.z};
  if (flags & SF_TRACE_L) {
    uint32_t hp = shadow[2 * pix];
    if (hp == kNoHit || hp == lp) {
      float bpdf;
      RGB3 f = bsdf_eval(m, V3{s2.x, s2.y, s2.z}, V3{s1.x, s1.y, s1.z}, &bpdf);
      if (bpdf != 0.0f) {
        float lpdf = s0.w;
        float w = power_heuristic(lpdf, bpdf);
        L = radd(L, rmuls(rmul(RGB3{s0.x, s0.y, s0.z}, f), w / lpdf));
      }
    }
  }
  if (flags & SF_TRACE_B) {
    uint32_t hp = shadow[2 * pix + 1];
    if (hp == kNoHit || hp == lp) {
      RGB3 li;
      float lpdf;
      light_compute(P, lt, V3{s5.x, s5.y, s5.z}, V3{s4.x, s4.y, s4.z}, &li, &lpdf);
      if (!rblack(li)) {
        float bpdf = s3.w;
        float w = (bpdf == 1.0f) ? 1.0f : power_heuristic(bpdf, lpdf);
        L = radd(L, rmuls(rmul(li, RGB3{s3.x, s3.y, s3.z}), w / bpdf));
      }
    }
  }
  Lb[pix] = make_float4(L.r, L.g, L.b, 0.0f);
}

// ============================== environment =================================
// JobLightInfiniteAreaPreprocessSampling (CLightInfiniteArea.cpp:113-139)
__global__ void k_env_lum(EnvView e, float* data, uint32_t quirks) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t W = e.W, H = e.H;
  if (i >= W * H) return;
  uint32_t x, y;
  if (quirks & WPBR_Q_ENV_DISTRIB_INDEX_BUG) {
    // data[x + y*resY] written in row order: the last writer of index i is
    // the one with the largest row.
    uint32_t yy = min(H - 1, i / H);
    uint32_t xx = i - yy * H;
    if (xx >= W) {
      data[i] = 0.0f;
      return;
    }
    x = xx;
    y = yy;
  } else {
    x = i % W;
    y = i / W;
  }
  float yN = (float)y / (float)H;
  float sin_t = (float)sin_d((kPI * (double)(float)((float)y + 0.5f)) / (double)(float)H);
  float xN = (float)x / (float)W;
  float v = env_bilerp(e, xN, yN).g;
  data[i] = v * sin_t;
}
// Distribution1D rows: sequential prefix sums (same rounding as the
// reference's serial loop), one thread per row.
__global__ void k_distrib_rows(const float* func, uint32_t n, uint32_t rows, float* cdf, float* fint) {
  uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const float* f = func + (size_t)r * n;
  float* c = cdf + (size_t)r * (n + 1);
  c[0] = 0.0f;
  for (uint32_t i = 1; i < n + 1; ++i) c[i] = c[i - 1] + f[i - 1] / (float)n;
  float fi = c[n];
  fint[r] = fi;
  if (fi == 0.0f) {
    for (uint32_t i = 1; i < n + 1; ++i) c[i] = (float)i / (float)n;
  } else {
    for (uint32_t i = 1; i < n + 1; ++i) c[i] = c[i] / fi;
  }
}

// JobOutputFilmTitles (CSFilm.cpp:129-170): /(w*800000), clamp, sRGB-like
// curve with the reference's 12.98 linear slope, x255, truncated to bytes.
__device__ float gamma_correct(float v) {
  if (v <= 0.0031308f) return 12.98f * v;
  return 1.055f * expf_(logf_(v) * (float)(1.0f / 2.4f)) - 0.055f;
}
__global__ void k_tonemap(uint32_t n, const float4* acc, uint8_t* out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 a = acc[i];
  if (a.x == 0.0f && a.y == 0.0f && a.z == 0.0f) {
    out[3 * i] = out[3 * i + 1] = out[3 * i + 2] = 0;
    return;
  }
  float d = a.w * 800000.f;
  float c[3] = {a.x / d, a.y / d, a.z / d};
  for (int k = 0; k < 3; ++k) {
    float v = clampf(c[k], 0.0f, 1.0f);
    v = gamma_correct(v) * 255.0f;
    out[3 * i + k] = (uint8_t)(int)v;
  }
}

PassCtx make_pass_ctx(wpbr_ctx* ctx) {
  PassCtx P;
  P.S = scene_view(ctx);
  P.Bv = render_traversal_view(ctx);
  P.rs = wpbr_rng::Stream{ctx->rs.seed, ctx->rs.stream, ctx->rs.spp, (ctx->quirks & WPBR_Q_REF_SAMPLER_ARRAYS) ? 1u : 0u};
  P.W = ctx->rs.W;
  P.H = ctx->rs.H;
  P.err = ctx->d_err.p;
  return P;
}

Staged staged_view(wpbr_ctx* ctx) {
  Staged G;
  for (int i = 0; i < F_COUNT; ++i) G.f[i] = ctx->rs.f[i].p;
  for (int i = 0; i < U_COUNT; ++i) G.u[i] = ctx->rs.u[i].p;
  return G;
}

wpbr_status ensure_staged(wpbr_ctx* ctx) {
  size_t n = (size_t)ctx->rs.W * ctx->rs.H;
  for (int i = 0; i < F_COUNT; ++i) WPBR_CUDA(ctx->rs.f[i].ensure(n * kFW[i]));
  for (int i = 0; i < U_COUNT; ++i) WPBR_CUDA(ctx->rs.u[i].ensure(n));
  return WPBR_OK;
}

}  // namespace

wpbr_status env_distribution_build(wpbr_ctx* ctx, const float4* rgb, const EnvDist& out, float* marg_int_host) {
  SceneView S = scene_view(ctx);
  S.env.rgb = rgb;
  uint32_t W = ctx->envW, H = ctx->envH;
  cudaStream_t st = ctx->stream;
  k_env_lum<<<div_up((uint64_t)W * H, 256), 256, 0, st>>>(S.env, out.cond_func, ctx->quirks);
  k_distrib_rows<<<div_up(H, 64), 64, 0, st>>>(out.cond_func, W, H, out.cond_cdf, out.cond_int);
  WPBR_CUDA(cudaMemcpyAsync(out.marg_func, out.cond_int, sizeof(float) * H, cudaMemcpyDeviceToDevice, st));
  k_distrib_rows<<<1, 32, 0, st>>>(out.marg_func, H, 1, out.marg_cdf, out.marg_int);
  WPBR_CUDA(cudaGetLastError());
  float mi = 0.0f;
  WPBR_CUDA(cudaMemcpyAsync(&mi, out.marg_int, 4, cudaMemcpyDeviceToHost, st));
  WPBR_CUDA(cudaStreamSynchronize(st));
  *marg_int_host = mi;
  return WPBR_OK;
}

wpbr_status env_preprocess(wpbr_ctx* ctx) {
  if (!ctx->has_env) return WPBR_OK;
  EnvDist d{ctx->cond_func.p, ctx->cond_cdf.p, ctx->cond_int.p, ctx->marg_func.p, ctx->marg_cdf.p, ctx->marg_int.p};
  return env_distribution_build(ctx, ctx->env_rgb.p, d, &ctx->env_marg_int);
}

static_assert(kQueueCounter == 2 + 2 * kPixCats, "pass counters: fetches, categories, then the queue");

wpbr_status render_setup(wpbr_ctx* ctx, uint32_t spp, uint32_t seed, uint32_t stream) {
  if (!ctx->has_scene) return set_err(ctx, WPBR_ERR_NOT_BUILT, "render_setup: no scene");
  if (!ctx->bvh.built) return set_err(ctx, WPBR_ERR_NOT_BUILT, "render_setup: BVH not built");
  if (spp == 0) return set_err(ctx, WPBR_ERR_INVALID_ARG, "render_setup: spp must be > 0");
  RenderState& R = ctx->rs;
  // not ready until every buffer below exists: a failed allocation here must
  // not leave an earlier setup's graph (or its freed buffers) usable
  R.ready = false;
  R.spp = spp;
  R.seed = seed;
  R.stream = stream;
  R.W = ctx->cam.W;
  R.H = ctx->cam.H;
  size_t n = (size_t)R.W * R.H;
  WPBR_CUDA(R.acc.ensure(n * 4));
  WPBR_CUDA(R.hit_prim.ensure(n));
  WPBR_CUDA(R.shadow_rays.ensure(n * 4));
  WPBR_CUDA(R.shadow_map.ensure(n * 2));
  WPBR_CUDA(R.shadow_hit.ensure(n * 2));
  WPBR_CUDA(R.pstate.ensure(n * kStateF4));
  WPBR_CUDA(R.Lbuf.ensure(n));
  WPBR_CUDA(R.pfilm.ensure(n));
  WPBR_CUDA(R.pass_dev.ensure(1));
  WPBR_CUDA(R.counters.ensure(kPassCounters));  // allocated before any graph capture
  WPBR_CUDA(R.order.ensure(n));
  WPBR_CUDA(cudaMemsetAsync(R.acc.p, 0, n * 4 * sizeof(float), ctx->stream));
  if (ctx->spectrum == WPBR_SPECTRUM_SAMPLED64) {
    wpbr_status sst = spectral_setup(ctx);
    if (sst != WPBR_OK) return sst;
  }
  R.ready = true;  // a captured pass graph stays valid while pass_graph_key is unchanged
  return WPBR_OK;
}


namespace {
// The kernels of one sample pass on stream `st` over state slice g of a pass
// group (per-pixel arrays offset by g films, counters by g sets), reading the
// pass index at pass_ptr; with_film appends the film gather. Sampled64
// passes write sample slot spec_slot and, when spec_film > 0, gather slots
// 0 .. spec_film - 1 into the film.
wpbr_status pass_kernels(wpbr_ctx* ctx, uint32_t g, const uint32_t* pass_ptr, cudaStream_t st, uint32_t grid,
                         bool with_film, uint32_t spec_slot = 0, uint32_t spec_film = 1) {
  RenderState& R = ctx->rs;
  PassCtx P = make_pass_ctx(ctx);
  const uint32_t n = R.W * R.H;
  const size_t o = (size_t)g * n;
  uint32_t* counters = R.counters.p + (size_t)g * kPassCounters;
  uint32_t* hit_prim = R.hit_prim.p + o;
  float4* pstate = R.pstate.p + o * kStateF4;
  float4* Lbuf = R.Lbuf.p + o;
  float2* pfilm = R.pfilm.p + o;
  uint32_t* shadow_hit = R.shadow_hit.p + 2 * o;
  uint32_t* order_buf = R.order.p + o;
  WPBR_CUDA(cudaMemsetAsync(counters, 0, kPassCounters * sizeof(uint32_t), st));
  const ShadowQueue sq{R.shadow_rays.p + 4 * o, R.shadow_map.p + 2 * o, counters + kQueueCounter};
  bool spectral = ctx->spectrum == WPBR_SPECTRUM_SAMPLED64;
  launch_traversal<false>(P.S, P.Bv, CameraSrc{P, pass_ptr}, PrimSink{hit_prim}, n, counters, P.err, st, grid);
  // the pixels in material-sorted order for the spawn and finish kernels
  const uint32_t* order = nullptr;
  if (n >= kSortMinPixels) {
    uint32_t* cat_counts = counters + 2;
    k_cat_count<<<div_up(n, kCatBlock), kCatBlock, 0, st>>>(P.S, n, hit_prim, cat_counts);
    k_cat_scatter<<<div_up(n, kCatBlock), kCatBlock, 0, st>>>(P.S, n, hit_prim, cat_counts, cat_counts + kPixCats,
                                                              order_buf, P.err);
    order = order_buf;
  }
  if (spectral)
    WPBR_CUDA(spectral_spawn_launch(ctx, pass_ptr, order, spec_slot));
  else
    (ctx->has_metal ? k_spawn<true> : k_spawn<false>)<<<div_up(n, kTB), kTB, 0, st>>>(P, pass_ptr, hit_prim, pstate,
                                                                                      sq, Lbuf, pfilm, order);
  // shadow rays: unoccluded iff no hit or the closest hit is the sampled
  // light's primitive; with environment lights only that is "no hit", which
  // the any-hit traversal decides with the same primitive tests, stopping at
  // the first hit (the stored id is then some hit, never a light's)
  // (the spawn queued only the rays it traces; the traversal walks the queue)
  const QueueSrc qsrc{sq.rays, sq.count};
  const MapSink qsink{shadow_hit, sq.map};
  if (ctx->env_lights_only)
    launch_traversal<true>(P.S, P.Bv, qsrc, qsink, 2 * n, counters + 1, P.err, st, grid);
  else
    launch_traversal<false>(P.S, P.Bv, qsrc, qsink, 2 * n, counters + 1, P.err, st, grid);
  if (spectral) {
    WPBR_CUDA(spectral_finish_launch(ctx, order, spec_slot, spec_film));
  } else {
    k_finish<<<div_up(n, kTB), kTB, 0, st>>>(P, pstate, shadow_hit, Lbuf, order);
    if (with_film)
      k_film_tiles<<<dim3(div_up(R.W, kFilmTile), div_up(R.H, kFilmTile)), kFilmThreadsRGB, 0, st>>>(
          R.W, R.H, pfilm, Lbuf, (float4*)R.acc.p);
  }
  WPBR_CUDA(cudaGetLastError());
  return WPBR_OK;
}
}  // namespace

// Launches the five kernels of one sample pass on the context's stream. The
// pass index is read from device memory (R.pass_ptr, shared across the scenes
// of a batch, else R.pass_dev); R.trace_grid caps the persistent traversal
// grids (0: one full wave of resident blocks).
wpbr_status render_pass_launch(wpbr_ctx* ctx) {
  RenderState& R = ctx->rs;
  const uint32_t n = R.W * R.H;
  WPBR_CUDA(R.counters.ensure(kPassCounters));
  WPBR_CUDA(R.shadow_map.ensure((size_t)2 * n));
  WPBR_CUDA(R.order.ensure(n));
  return pass_kernels(ctx, 0, R.pass_ptr ? R.pass_ptr : R.pass_dev.p, ctx->stream, R.trace_grid, true);
}

uint32_t persistent_full_grid() {
  return persistent_grid((const void*)k_trace_persistent<false, 64, CameraSrc, PrimSink>);
}

// Everything the captured pass graph bakes into its kernel arguments: the
// scene/BVH epoch, the sample-stream parameters, the film size and every
// device pointer the five kernels receive.
static uint64_t pass_graph_key(const wpbr_ctx* ctx) {
  const RenderState& R = ctx->rs;
  uint64_t h = 0xCBF29CE484222325ull;
  auto mix = [&h](uint64_t v) {
    for (int i = 0; i < 8; ++i) {
      h ^= (v >> (8 * i)) & 0xFFu;
      h *= 0x100000001B3ull;
    }
  };
  mix(ctx->epoch);
  mix(R.spp);
  mix(R.seed);
  mix(R.stream);
  mix(((uint64_t)R.W << 32) | R.H);
  mix((uint64_t)R.trace_grid);
  mix((uint64_t)ctx->spectrum | ((uint64_t)ctx->quirks << 8));
  const void* ptrs[] = {R.acc.p,    R.hit_prim.p, R.shadow_rays.p,     R.shadow_hit.p,      R.shadow_map.p, R.pstate.p,
                        R.Lbuf.p,   R.pfilm.p,    R.pass_dev.p,        R.counters.p,        R.pass_ptr, R.order.p,
                        ctx->d_err.p, ctx->bvh.view.nodes,
                        ctx->bvh.view.prims, R.spec_mats.p, R.spec_le.p, R.spec_L.p, R.spec_acc.p};
  for (const void* q : ptrs) mix((uint64_t)(uintptr_t)q);
  return h;
}

wpbr_status render_pass_fused(wpbr_ctx* ctx, uint32_t pass) {
  RenderState& R = ctx->rs;
  if (!R.ready) return set_err(ctx, WPBR_ERR_NOT_BUILT, "render_pass: render_setup not called");
  if (pass >= R.spp) return set_err(ctx, WPBR_ERR_INVALID_ARG, "render_pass: pass >= spp");
  cudaStream_t st = ctx->stream;
  WPBR_CUDA(cudaMemcpyAsync(R.pass_dev.p, &pass, 4, cudaMemcpyHostToDevice, st));
  if (ctx->spectrum == WPBR_SPECTRUM_SAMPLED64) R.spec_dirty = true;
  uint64_t key = pass_graph_key(ctx);
  if (R.graph && R.graph_key != key) {
    cudaGraphExecDestroy(R.graph);
    R.graph = nullptr;
    R.graph_ok = false;
  }
  if (!R.graph_ok) {
    R.graph_key = key;
    // capture the five kernels once; later passes replay the graph
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      wpbr_status s = render_pass_launch(ctx);
      cudaError_t e = cudaStreamEndCapture(st, &g);
      if (s == WPBR_OK && e == cudaSuccess && g) {
        if (cudaGraphInstantiate(&R.graph, g, 0) == cudaSuccess) R.graph_ok = true;
      }
      if (g) cudaGraphDestroy(g);
    }
    // capture is not possible on the legacy default stream: clear the error
    // and launch the kernels directly
    cudaGetLastError();
    if (!R.graph_ok) return render_pass_launch(ctx);
  }
  WPBR_CUDA(cudaGraphLaunch(R.graph, st));
  return WPBR_OK;
}

// Passes per group for a frame: small films leave most of the GPU idle in one
// pass (its traversals hold a few tens of thousands of rays), so the passes
// of a group run as concurrent branches until a group holds about 2^18 rays;
// the size divides spp, so every group is whole.
uint32_t group_size(uint32_t n, uint32_t spp) {
  uint32_t k = (uint32_t)std::min<uint64_t>(RenderState::kMaxGroup, ((1ull << 18) + n - 1) / n);
  k = std::min(k, spp);
  while (k > 1 && spp % k) --k;
  return std::max(k, 1u);
}

// A Sampled64 frame in groups of J sequential passes: one graph runs the J
// passes, each writing its film positions and spectra to its own sample
// slot, then one film gather adds the J slots in pass order (each pass's
// neighbours in row-major order), so the film is identical to J one-pass
// gathers while the 64-bin accumulator is read and written once per group.
static wpbr_status spectral_frame(wpbr_ctx* ctx, uint32_t J) {
  RenderState& R = ctx->rs;
  cudaStream_t st = ctx->stream;
  const uint32_t n = R.W * R.H;
  WPBR_CUDA(spectral_slots(ctx, J));
  WPBR_CUDA(R.pass_dev.ensure(J));
  WPBR_CUDA(R.counters.ensure(kPassCounters));
  WPBR_CUDA(R.shadow_map.ensure((size_t)2 * n));
  WPBR_CUDA(R.order.ensure(n));
  const uint64_t key = pass_graph_key(ctx) * 0x100000001B3ull + 0x5300u + J;
  if (R.sgraph && (R.sgraph_key != key || R.sgroup != J)) {
    cudaGraphExecDestroy(R.sgraph);
    R.sgraph = nullptr;
  }
  if (!R.sgraph) {
    cudaGraph_t gr = nullptr;
    WPBR_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    wpbr_status s = WPBR_OK;
    for (uint32_t j = 0; j < J && s == WPBR_OK; ++j)
      s = pass_kernels(ctx, 0, R.pass_dev.p + j, st, R.trace_grid, false, j, j + 1 == J ? J : 0);
    cudaError_t e2 = cudaStreamEndCapture(st, &gr);
    cudaError_t e = cudaSuccess;
    if (s == WPBR_OK && e2 == cudaSuccess && gr) e = cudaGraphInstantiate(&R.sgraph, gr, 0);
    if (gr) cudaGraphDestroy(gr);
    if (s != WPBR_OK) {
      cudaGetLastError();
      return s;
    }
    if (e != cudaSuccess || e2 != cudaSuccess || !R.sgraph) {
      cudaGetLastError();
      R.sgraph = nullptr;
      return set_err(ctx, WPBR_ERR_CUDA, "render: Sampled64 pass-group graph capture failed");
    }
    R.sgraph_key = key;
    R.sgroup = J;
  }
  R.spec_dirty = true;
  uint32_t passes[4];
  for (uint32_t base = 0; base < R.spp; base += J) {
    for (uint32_t j = 0; j < J; ++j) passes[j] = base + j;
    WPBR_CUDA(cudaMemcpyAsync(R.pass_dev.p, passes, sizeof(uint32_t) * J, cudaMemcpyHostToDevice, st));
    WPBR_CUDA(cudaGraphLaunch(R.sgraph, st));
  }
  return WPBR_OK;
}

// A whole frame (every pass of render_setup's spp) through the fused pass.
// Films of RGB frames that fit a group of several passes render a group at a
// time: one fork/join graph whose K branches run the pass kernels of passes
// base .. base + K - 1 on their own streams, state slices and pass index
// words (each traversal capped at a K-th of the resident grid), then the K
// film gathers in pass order on the context's stream. Every pass computes
// what it computes alone, and the film adds the passes in the same order, so
// the film is identical to spp calls of render_pass_fused.
wpbr_status render_frame(wpbr_ctx* ctx) {
  RenderState& R = ctx->rs;
  if (!R.ready) return set_err(ctx, WPBR_ERR_NOT_BUILT, "render: render_setup not called");
  const uint32_t n = R.W * R.H;
  if (ctx->spectrum == WPBR_SPECTRUM_SAMPLED64 && !R.pass_ptr) {
    const uint32_t J = R.spp % 4 == 0 ? 4u : (R.spp % 2 == 0 ? 2u : 1u);
    if (J > 1) return spectral_frame(ctx, J);
  }
  const uint32_t K = (ctx->spectrum == WPBR_SPECTRUM_RGB && !R.pass_ptr) ? group_size(n, R.spp) : 1u;
  if (K <= 1) {
    for (uint32_t p = 0; p < R.spp; ++p) {
      wpbr_status s = render_pass_fused(ctx, p);
      if (s != WPBR_OK) return s;
    }
    return WPBR_OK;
  }
  cudaStream_t st = ctx->stream;
  const size_t kn = (size_t)K * n;
  WPBR_CUDA(R.hit_prim.ensure(kn));
  WPBR_CUDA(R.pstate.ensure(kn * kStateF4));
  WPBR_CUDA(R.Lbuf.ensure(kn));
  WPBR_CUDA(R.pfilm.ensure(kn));
  WPBR_CUDA(R.shadow_rays.ensure(4 * kn));
  WPBR_CUDA(R.shadow_map.ensure(2 * kn));
  WPBR_CUDA(R.shadow_hit.ensure(2 * kn));
  WPBR_CUDA(R.order.ensure(kn));
  WPBR_CUDA(R.counters.ensure((size_t)K * kPassCounters));
  WPBR_CUDA(R.pass_dev.ensure(K));
  for (uint32_t g = 0; g < K; ++g)
    if (!R.gstream[g]) WPBR_CUDA(cudaStreamCreateWithFlags(&R.gstream[g], cudaStreamNonBlocking));
  if (!R.gfork) WPBR_CUDA(cudaEventCreateWithFlags(&R.gfork, cudaEventDisableTiming));
  for (uint32_t g = 0; g < K; ++g)
    if (!R.gjoin[g]) WPBR_CUDA(cudaEventCreateWithFlags(&R.gjoin[g], cudaEventDisableTiming));
  const uint64_t key = pass_graph_key(ctx) * 0x100000001B3ull + K;
  if (R.ggraph && (R.ggraph_key != key || R.group != K)) {
    cudaGraphExecDestroy(R.ggraph);
    R.ggraph = nullptr;
  }
  if (!R.ggraph) {
    const uint32_t full = persistent_full_grid();
    const uint32_t grid = std::max(1u, full / K);
    cudaGraph_t gr = nullptr;
    WPBR_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    wpbr_status s = WPBR_OK;
    cudaError_t e = cudaEventRecord(R.gfork, st);
    for (uint32_t g = 0; g < K && e == cudaSuccess && s == WPBR_OK; ++g) {
      e = cudaStreamWaitEvent(R.gstream[g], R.gfork, 0);
      if (e != cudaSuccess) break;
      s = pass_kernels(ctx, g, R.pass_dev.p + g, R.gstream[g], grid, false);
      if (s != WPBR_OK) break;
      e = cudaEventRecord(R.gjoin[g], R.gstream[g]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st, R.gjoin[g], 0);
    }
    for (uint32_t g = 0; g < K && e == cudaSuccess && s == WPBR_OK; ++g)
      k_film_tiles<<<dim3(div_up(R.W, kFilmTile), div_up(R.H, kFilmTile)), kFilmThreadsRGB, 0, st>>>(
          R.W, R.H, R.pfilm.p + (size_t)g * n, R.Lbuf.p + (size_t)g * n, (float4*)R.acc.p);
    cudaError_t e2 = cudaStreamEndCapture(st, &gr);
    if (s == WPBR_OK && e == cudaSuccess && e2 == cudaSuccess && gr) e = cudaGraphInstantiate(&R.ggraph, gr, 0);
    if (gr) cudaGraphDestroy(gr);
    if (s != WPBR_OK) {
      cudaGetLastError();
      return s;
    }
    if (e != cudaSuccess || e2 != cudaSuccess || !R.ggraph) {
      cudaGetLastError();
      R.ggraph = nullptr;
      return set_err(ctx, WPBR_ERR_CUDA, "render: pass-group graph capture failed");
    }
    R.ggraph_key = key;
    R.group = K;
  }
  uint32_t passes[RenderState::kMaxGroup];
  for (uint32_t base = 0; base < R.spp; base += K) {
    for (uint32_t g = 0; g < K; ++g) passes[g] = base + g;
    WPBR_CUDA(cudaMemcpyAsync(R.pass_dev.p, passes, sizeof(uint32_t) * K, cudaMemcpyHostToDevice, st));
    WPBR_CUDA(cudaGraphLaunch(R.ggraph, st));
  }
  return WPBR_OK;
}

wpbr_status job_run(wpbr_ctx* ctx, uint32_t job, uint32_t pass) {
  RenderState& R = ctx->rs;
  if (ctx->spectrum != WPBR_SPECTRUM_RGB)
    return set_err(ctx, WPBR_ERR_INVALID_ARG, "job_run: the staged jobs run in RGB mode only");
  if (!R.ready) return set_err(ctx, WPBR_ERR_NOT_BUILT, "job_run: render_setup not called");
  if (job >= WPBR_JOB_COUNT) return set_err(ctx, WPBR_ERR_INVALID_ARG, "job_run: unknown job id");
  if (pass >= R.spp) return set_err(ctx, WPBR_ERR_INVALID_ARG, "job_run: pass >= spp");
  wpbr_status s = ensure_staged(ctx);
  if (s != WPBR_OK) return s;
  PassCtx P = make_pass_ctx(ctx);
  Staged G = staged_view(ctx);
  uint32_t n = R.W * R.H;
  unsigned g = div_up(n, kTB);
  cudaStream_t st = ctx->stream;
  switch (job) {
    case WPBR_JOB_CAMERA_RAYS: kj_camera<<<g, kTB, 0, st>>>(P, pass, G); break;
    case WPBR_JOB_COLLIDE_PRIMARY: kj_collide<<<g, kTB, 0, st>>>(P, G); break;
    case WPBR_JOB_EMITTED_LIGHT: kj_emitted<<<g, kTB, 0, st>>>(P, G); break;
    case WPBR_JOB_BSDF_SETUP: kj_bsdf_setup<<<g, kTB, 0, st>>>(P, G); break;
    case WPBR_JOB_SAMPLE_LIGHT: kj_sample_light<<<g, kTB, 0, st>>>(P, pass, G); break;
    case WPBR_JOB_SHADOW_LIGHT: kj_shadow_light<<<g, kTB, 0, st>>>(P, G); break;
    case WPBR_JOB_BSDF_COMPUTE: kj_bsdf_compute<<<g, kTB, 0, st>>>(P, G); break;
    case WPBR_JOB_INTEGRATE_LIGHT: kj_integrate_light<<<g, kTB, 0, st>>>(P, G); break;
    case WPBR_JOB_SAMPLE_BSDF: kj_sample_bsdf<<<g, kTB, 0, st>>>(P, pass, G); break;
    case WPBR_JOB_SHADOW_BSDF: kj_shadow_bsdf<<<g, kTB, 0, st>>>(P, G); break;
    case WPBR_JOB_LIGHT_COMPUTE: kj_light_compute<<<g, kTB, 0, st>>>(P, G); break;
    case WPBR_JOB_INTEGRATE_BSDF: kj_integrate_bsdf<<<g, kTB, 0, st>>>(P, G); break;
    case WPBR_JOB_FILM_ACCUMULATE:
      kj_film_pack<<<g, kTB, 0, st>>>(P, G, R.pfilm.p, R.Lbuf.p);
      k_film_tiles<<<dim3(div_up(R.W, kFilmTile), div_up(R.H, kFilmTile)), kFilmThreadsRGB, 0, st>>>(
          R.W, R.H, R.pfilm.p, R.Lbuf.p, (float4*)R.acc.p);
      break;
  }
  WPBR_CUDA(cudaGetLastError());
  return WPBR_OK;
}

wpbr_status job_record(wpbr_ctx* ctx, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1, wpbr_pass_record* rec) {
  RenderState& R = ctx->rs;
  if (!R.ready || !R.f[0].p) return set_err(ctx, WPBR_ERR_NOT_BUILT, "job_record: no staged pass");
  if (x1 > R.W || y1 > R.H || x0 >= x1 || y0 >= y1 || !rec)
    return set_err(ctx, WPBR_ERR_INVALID_ARG, "job_record: bad rectangle");
  float* fptr[F_COUNT] = {rec->pfilm, rec->ray_o, rec->ray_d, rec->ray_dx_d, rec->ray_dy_d, rec->hit_t,
                          rec->si_p, rec->si_n, rec->si_wo, rec->si_sn, rec->si_sdpdu, rec->si_dpdu,
                          rec->si_dpdv, rec->si_dndu, rec->si_dndv, rec->frame, rec->le, rec->l_wi,
                          rec->l_li, rec->l_pdf, rec->l_f, rec->l_fpdf, rec->b_wi, rec->b_f,
                          rec->b_pdf, rec->b_li, rec->b_lpdf, rec->L, nullptr};
  uint32_t* uptr[4] = {rec->hit_prim, rec->light_idx, rec->l_flags, rec->b_flags};
  cudaStream_t st = ctx->stream;
  uint32_t w = x1 - x0;
  for (uint32_t y = y0; y < y1; ++y) {
    size_t src = (size_t)y * R.W + x0;
    size_t dst = (size_t)(y - y0) * w;
    for (int f = 0; f < F_COUNT; ++f)
      if (fptr[f])
        WPBR_CUDA(cudaMemcpyAsync(fptr[f] + dst * kFW[f], R.f[f].p + src * kFW[f], sizeof(float) * w * kFW[f],
                                  cudaMemcpyDeviceToHost, st));
    for (int u = 0; u < 4; ++u)
      if (uptr[u])
        WPBR_CUDA(cudaMemcpyAsync(uptr[u] + dst, R.u[u].p + src, sizeof(uint32_t) * w, cudaMemcpyDeviceToHost, st));
  }
  WPBR_CUDA(cudaStreamSynchronize(st));
  return WPBR_OK;
}

wpbr_status film_tonemap(wpbr_ctx* ctx, uint8_t* out) {
  RenderState& R = ctx->rs;
  if (!R.ready) return set_err(ctx, WPBR_ERR_NOT_BUILT, "tonemap: render_setup not called");
  wpbr_status rs = spectral_resolve(ctx);
  if (rs != WPBR_OK) return rs;
  uint32_t n = R.W * R.H;
  DevBuf<uint8_t> tmp;
  WPBR_CUDA(tmp.ensure((size_t)n * 3));
  k_tonemap<<<div_up(n, 256), 256, 0, ctx->stream>>>(n, (const float4*)R.acc.p, tmp.p);
  cudaError_t e = cudaMemcpyAsync(out, tmp.p, (size_t)n * 3, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  tmp.release();
  if (e != cudaSuccess) return cuda_err(ctx, e, "tonemap");
  return WPBR_OK;
}

}  // namespace wpbr
