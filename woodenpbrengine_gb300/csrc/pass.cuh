// pass.cuh — device pieces of one sample pass shared by the render kernels
// (render.cu) and the differentiable estimator (adjoint.cu): camera samples and
// rays, surface interactions of a hit, light pick and light sampling, the
// light evaluation for BSDF-sampled directions and the film gather.
#pragma once

#include "camera.cuh"
#include "common.cuh"
#include "shade.cuh"
#include "views.cuh"
#include "wpbr_sampling.h"

namespace wpbr {

namespace {

constexpr int kTB = 128;
// Resident blocks per SM of the spawn kernels (surface interaction and
// sampling, 127 registers unbounded): the light and environment sampling is
// a chain of dependent loads (CDF searches), so occupancy pays even with
// spills. 1080p full frame, RGB / Sampled64 Msamples/s: unbounded 1093 /
// 621, 8 blocks 1188 / 649, 12 blocks (40 registers) 1229 / 667, 14 blocks
// 1246 / 677 but the 256x256 frame 4% slower.
#ifndef WPBR_SPAWN_MIN_BLOCKS
#define WPBR_SPAWN_MIN_BLOCKS 12
#endif
// The same kernels compiled with the texture path (scenes with textured
// metal): the EWA loops need registers, and bounding them lost (textured
// scene at 1080p: 1535 Msamples/s unbounded, 1487 at 8 blocks, 1439 at 12).
#ifndef WPBR_SPAWN_TEX_MIN_BLOCKS
#define WPBR_SPAWN_TEX_MIN_BLOCKS 1
#endif
// The differentiable estimator's spawn: forward 4.06 -> 3.84 ms at 12 blocks
// (512x512 x 16 spp).
#ifndef WPBR_ADJ_SPAWN_MIN_BLOCKS
#define WPBR_ADJ_SPAWN_MIN_BLOCKS 12
#endif
// ... and its reverse sweep: backward 5.63 -> 5.19 ms at 12 blocks (8: 5.43).
#ifndef WPBR_ADJ_BACK_MIN_BLOCKS
#define WPBR_ADJ_BACK_MIN_BLOCKS 12
#endif

struct PassCtx {
  SceneView S;
  BvhView Bv;
  wpbr_rng::Stream rs;
  uint32_t W, H;
  uint32_t* err;
};

__device__ __forceinline__ V3 ld3(const float* f, uint32_t i) { return V3{f[3 * i], f[3 * i + 1], f[3 * i + 2]}; }
__device__ __forceinline__ void st3(float* f, uint32_t i, V3 v) {
  f[3 * i] = v.x;
  f[3 * i + 1] = v.y;
  f[3 * i + 2] = v.z;
}
__device__ __forceinline__ RGB3 ldc(const float* f, uint32_t i) { return RGB3{f[3 * i], f[3 * i + 1], f[3 * i + 2]}; }
__device__ __forceinline__ void stc(float* f, uint32_t i, RGB3 c) {
  f[3 * i] = c.r;
  f[3 * i + 1] = c.g;
  f[3 * i + 2] = c.b;
}

__device__ __forceinline__ uint32_t prim_material(const SceneView& S, uint32_t prim) {
  return prim < S.ns ? S.sph_mat[prim] : S.tri_mat[prim - S.ns];
}

// ---- material-sorted pixel order ----------------------------------------------
// The reference shades each kind of surface in a job of its own over that
// kind's component group: one BSDF job per material kind
// (CBSDFConductorMicroface.cpp:84-115, CBSDFDielectricMicroface.cpp:84-115,
// CBSDFSpecularReflectance.cpp:63-93) after the sphere or the triangle
// surface-interaction job (CSSphere.cpp:122-186, CSTriangle.cpp:149-319).
// The wavefront shades the pixels of a pass in that grouping: after the
// camera traversal the pixels are ordered by category = primitive kind x
// material type (2 x 5), camera misses (and scenes without lights) last, so
// the spawn and finish kernels' warps mostly run one code path. Within a
// category pixels keep their film order in runs of a block (one atomic per
// block and category claims a run).
constexpr uint32_t kMatTypes = 5;                  // WPBR_MAT_CONDUCTOR .. WPBR_MAT_METAL_ISOTROPIC
constexpr uint32_t kPixCats = 2 * kMatTypes + 1;   // last: misses
constexpr uint32_t kCatBlock = 256;
// Films of fewer pixels are shaded in film order: the two ordering launches
// cost more than they save there (256x256 x 4 spp: 647 Msamples/s in film
// order, 614 sorted; 1920x1080 x 64 spp: 1,276 in film order, 1,364 sorted).
constexpr uint32_t kSortMinPixels = 1u << 17;

__device__ __forceinline__ uint32_t pixel_category(const SceneView& S, uint32_t prim) {
  if (prim == kNoHit || S.nlights == 0) return kPixCats - 1;
  uint32_t t = S.mats[prim_material(S, prim)].type;
  return (prim < S.ns ? 0u : kMatTypes) + (t < kMatTypes ? t : kMatTypes - 1);
}

// counts[0..kPixCats): pixels per category (zeroed before the pass)
__global__ void __launch_bounds__(kCatBlock) k_cat_count(SceneView S, uint32_t n, const uint32_t* hit_prim,
                                                         uint32_t* counts) {
  __shared__ uint32_t s_cnt[kPixCats];
  if (threadIdx.x < kPixCats) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  uint32_t i = blockIdx.x * kCatBlock + threadIdx.x;
  if (i < n) atomicAdd(&s_cnt[pixel_category(S, hit_prim[i])], 1u);
  __syncthreads();
  if (threadIdx.x < kPixCats && s_cnt[threadIdx.x]) atomicAdd(&counts[threadIdx.x], s_cnt[threadIdx.x]);
}

// order[]: the pixels grouped by category (category c starts at the sum of
// the counts before it); cursor[0..kPixCats) zeroed before the pass.
__global__ void __launch_bounds__(kCatBlock) k_cat_scatter(SceneView S, uint32_t n, const uint32_t* hit_prim,
                                                           const uint32_t* counts, uint32_t* cursor,
                                                           uint32_t* order, uint32_t* err) {
  __shared__ uint32_t s_cnt[kPixCats], s_base[kPixCats];
  if (threadIdx.x < kPixCats) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t i = blockIdx.x * kCatBlock + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t c = i < n ? pixel_category(S, hit_prim[i]) : kPixCats;  // kPixCats: no pixel
  uint32_t peers = __match_any_sync(0xFFFFFFFFu, c);
  uint32_t leader = __ffs(peers) - 1u;
  uint32_t wbase = 0;
  if (lane == leader && c < kPixCats) wbase = atomicAdd(&s_cnt[c], (uint32_t)__popc(peers));
  wbase = __shfl_sync(0xFFFFFFFFu, wbase, leader);
  uint32_t rank = wbase + __popc(peers & ((1u << lane) - 1u));
  __syncthreads();
  if (threadIdx.x < kPixCats) {
    uint32_t start = 0;
    for (uint32_t k = 0; k < threadIdx.x; ++k) start += counts[k];
    s_base[threadIdx.x] = s_cnt[threadIdx.x] ? start + atomicAdd(&cursor[threadIdx.x], s_cnt[threadIdx.x]) : 0u;
  }
  __syncthreads();
  if (c < kPixCats) {
    uint32_t pos = s_base[c] + rank;  // < n when the counts are this pass's
    if (pos < n)
      order[pos] = i;
    else
      atomicOr(err, kErrBuild);
  }
}

// Full interaction for the winning primitive: re-runs its intersection test
// (identical bits) and builds the surface interaction.
__device__ SurfInt make_si(const SceneView& S, uint32_t prim, V3 o, V3 d) {
  if (prim < S.ns) {
    V3 rlo, rld, ph;
    sphere_intersect(S.sph_w2o[prim], S.sph_r[prim], o, d, &rlo, &rld, &ph);
    return sphere_si(S.sph_o2w[prim], S.sph_w2o[prim], S.sph_r[prim], rld, ph);
  }
  uint32_t t = prim - S.ns;
  const uint32_t* ix = S.idx + 3 * (size_t)t;
  TriData td;
  uint32_t fl = S.tri_flags[t];
  td.has_ns = (fl & WPBR_MESH_NORMALS_TANGENTS) != 0;
  td.has_uv = (fl & WPBR_MESH_UVS) != 0;
  for (int k = 0; k < 3; ++k) {
    uint32_t v = ix[k];
    td.p[k] = V3{S.pos[3 * v], S.pos[3 * v + 1], S.pos[3 * v + 2]};
    td.n[k] = td.has_ns ? V3{S.nrm[3 * v], S.nrm[3 * v + 1], S.nrm[3 * v + 2]} : V3{0, 0, 0};
    td.s[k] = td.has_ns ? V3{S.tan[3 * v], S.tan[3 * v + 1], S.tan[3 * v + 2]} : V3{0, 0, 0};
    td.uv[k] = td.has_uv ? V2{S.uv[2 * v], S.uv[2 * v + 1]} : V2{0, 0};
  }
  float b0, b1, b2;
  tri_intersect(td.p[0], td.p[1], td.p[2], o, d, S.quirks, &b0, &b1, &b2);
  return triangle_si(td, d, b0, b1, b2);
}

// The material of a hit: the scene's, or for textured metal the conductor
// built from its textures at the hit's footprint (camera-ray differentials,
// sphere or uv mapping).
// TEX = false compiles the texture path out, for scenes without textured
// materials (the context knows: has_metal).
template <bool TEX = true>
__device__ wpbr_material hit_material(const SceneView& S, uint32_t prim, uint32_t mid, const SurfInt& s,
                                      const RayD& r) {
  wpbr_material m = S.mats[mid];
  if (!TEX || !WPBR_MAT_TEXTURED(m.type)) return m;
  SurfDiff D = surf_differentials(s, r);
  TexFootprint fp = prim < S.ns ? sphere_footprint(S.sph_w2o[prim], s, D) : uv_footprint(s, D);
  return metal_material(S.tex, m, fp);
}
// The part of a textured-metal material that varies per hit, packed in a
// float4 (alpha, k.rgb), and its inverse.
__device__ __forceinline__ float4 metal_pack(const wpbr_material& m) {
  return make_float4(m.alpha_x, m.k[0], m.k[1], m.k[2]);
}
__device__ __forceinline__ wpbr_material metal_unpack(float4 v) {
  wpbr_material e;
  e.type = WPBR_MAT_CONDUCTOR;
  e.alpha_x = v.x;
  e.alpha_y = v.x;
  for (int c = 0; c < 3; ++c) {
    e.R[c] = 1.0f;
    e.eta_i[c] = 1.0f;
    e.eta_t[c] = 1.5f;
  }
  e.k[0] = v.y;
  e.k[1] = v.z;
  e.k[2] = v.w;
  e.tex[0] = e.tex[1] = 0;
  return e;
}

__device__ __forceinline__ void pixel_xy(uint32_t pix, uint32_t W, uint32_t* x, uint32_t* y) {
  *x = pix % W;
  *y = pix / W;
}

// JobSamplerUpdateCameraSamples (CSSampler.cpp:7-23): pFilm = pixel + u2
__device__ __forceinline__ void camera_sample(const PassCtx& P, uint32_t pix, uint32_t pass, float* fx, float* fy) {
  uint32_t x, y;
  pixel_xy(pix, P.W, &x, &y);
  float u0, u1;
  wpbr_rng::sample2d(P.rs, pix, pass, wpbr_rng::DIM_CAMERA, &u0, &u1);
  *fx = (float)x + u0;
  *fy = (float)y + u1;
}

// JobScatteringSampleLight (SScattering.cpp:82-88), index clamped
__device__ __forceinline__ uint32_t pick_light(const PassCtx& P, uint32_t pix, uint32_t pass) {
  uint32_t nl = P.S.nlights;
  float ul = wpbr_rng::sample1d(P.rs, pix, pass, wpbr_rng::DIM_LIGHT_PICK);
  float fl = (ul + 0.5f) * (float)(nl - 1);
  uint32_t li = (uint32_t)fl;
  return li > nl - 1 ? nl - 1 : li;
}

struct LightSample {
  V3 wi;
  RGB3 li;
  float pdf;
  bool ok;
};
__device__ LightSample sample_light(const PassCtx& P, const wpbr_light& lt, V3 p, uint32_t pix, uint32_t pass) {
  float u0, u1;
  wpbr_rng::sample2d(P.rs, pix, pass, wpbr_rng::DIM_LIGHT, &u0, &u1);
  LightSample s;
  s.wi = V3{0, 0, 0};
  s.li = rgb1(0.0f);
  s.pdf = 0.0f;
  s.ok = true;
  if (lt.type == WPBR_LIGHT_SPHERE) {
    sphere_light_sample(P.S.sph_o2w[lt.sphere_index], P.S.sph_r[lt.sphere_index], p, u0, u1, &s.wi, &s.pdf);
    s.li = RGB3{lt.Le[0], lt.Le[1], lt.Le[2]};
  } else {
    env_li_sample(P.S.env, P.S.quirks, u0, u1, &s.wi, &s.li, &s.pdf, &s.ok);
  }
  return s;
}

__device__ void light_compute(const PassCtx& P, const wpbr_light& lt, V3 p, V3 wi, RGB3* li, float* pdf) {
  if (lt.type == WPBR_LIGHT_SPHERE) {
    *pdf = sphere_light_pdf(P.S.sph_o2w[lt.sphere_index], P.S.sph_r[lt.sphere_index], p, P.S.quirks);
    *li = RGB3{lt.Le[0], lt.Le[1], lt.Le[2]};
  } else {
    env_li_compute(P.S.env, wi, li, pdf);
  }
}

__device__ __forceinline__ uint32_t light_prim(const wpbr_light& lt) {
  return lt.type == WPBR_LIGHT_SPHERE ? lt.sphere_index : 0xFFFFFFFEu;
}

// JobAccumalateLIFromSamples (CSFilm.cpp:70-122) as a gather: each pixel
// sums, in the reference's row-major sample order, the Mitchell-weighted
// samples of its 32x32 tile whose splat footprint covers it. A block takes
// kFilmTile x kFilmTile pixels and first stages the samples of its halo in
// shared memory, once each: the sample's value, its splat footprint clipped
// to its own 32x32 tile (bit masks over the five pixel columns and rows it
// can reach: a pixel of another tile is never inside it, so the clip by the
// pixel's tile and the clip by the sample's agree), and the Mitchell factors
// of those columns and rows. A pixel's weight is then the product of the same
// two factors, in the same order, as one computed per (pixel, sample) pair,
// so the film is bit-identical to that gather.
constexpr int kFilmTile = 16;
constexpr int kFilmHalo = kFilmTile + 4;
constexpr int kFilmThreadsRGB = kFilmTile * kFilmTile;
__global__ void __launch_bounds__(kFilmThreadsRGB) k_film_tiles(uint32_t W, uint32_t H, const float2* pf,
                                                                 const float4* Lb, float4* acc) {
  __shared__ float4 s_L[kFilmHalo * kFilmHalo];
  __shared__ float s_mx[kFilmHalo * kFilmHalo][5], s_my[kFilmHalo * kFilmHalo][5];
  __shared__ uint32_t s_mask[kFilmHalo * kFilmHalo];  // bits 0-4: columns sx-2..sx+2; 5-9: rows; 10: black
  const int bx0 = (int)blockIdx.x * kFilmTile, by0 = (int)blockIdx.y * kFilmTile;
  for (int h = (int)threadIdx.x; h < kFilmHalo * kFilmHalo; h += kFilmThreadsRGB) {
    const int sx = bx0 - 2 + h % kFilmHalo, sy = by0 - 2 + h / kFilmHalo;
    uint32_t m = 0;
    if (sx >= 0 && sy >= 0 && sx < (int)W && sy < (int)H) {
      const int tx0 = (sx / 32) * 32, ty0 = (sy / 32) * 32;
      const int tx1 = min(tx0 + 31, (int)W - 1), ty1 = min(ty0 + 31, (int)H - 1);
      const size_t sp = (size_t)sy * W + sx;
      const float2 f = pf[sp];
      const float dx0 = f.x - 0.5f, dy0 = f.y - 0.5f;
      int pminx = (int)ceilf(dx0 - 2.0f), pmaxx = (int)floorf(dx0 + 2.0f);
      int pminy = (int)ceilf(dy0 - 2.0f), pmaxy = (int)floorf(dy0 + 2.0f);
      pminx = max(pminx, tx0);
      pminy = max(pminy, ty0);
      pmaxx = min(pmaxx, tx1);
      pmaxy = min(pmaxy, ty1);
#pragma unroll
      for (int d = 0; d < 5; ++d) {
        const int x = sx - 2 + d, y = sy - 2 + d;
        if (x >= pminx && x <= pmaxx) {
          m |= 1u << d;
          s_mx[h][d] = mitchell1(((float)x - f.x) / 2.0f);
        }
        if (y >= pminy && y <= pmaxy) {
          m |= 1u << (5 + d);
          s_my[h][d] = mitchell1(((float)y - f.y) / 2.0f);
        }
      }
      const float4 c = Lb[sp];
      s_L[h] = c;
      if (rblack(RGB3{c.x, c.y, c.z})) m |= 1u << 10;
    }
    s_mask[h] = m;
  }
  __syncthreads();
  const int lx = (int)threadIdx.x % kFilmTile, ly = (int)threadIdx.x / kFilmTile;
  const uint32_t x = (uint32_t)(bx0 + lx), y = (uint32_t)(by0 + ly);
  if (x >= W || y >= H) return;
  float4 a = acc[(size_t)y * W + x];
  RGB3 L{a.x, a.y, a.z};
  float ws = a.w;
  // the neighbours sy = y-2..y+2 (outer), sx = x-2..x+2 (inner); this pixel
  // is column 4 - dx and row 4 - dy of a neighbour's reach
  for (int dy = 0; dy < 5; ++dy)
    for (int dx = 0; dx < 5; ++dx) {
      const int h = (ly + dy) * kFilmHalo + (lx + dx);
      const uint32_t m = s_mask[h];
      if (!((m >> (4 - dx)) & 1u) || !((m >> (9 - dy)) & 1u)) continue;
      const float w = s_mx[h][4 - dx] * s_my[h][4 - dy];
      if (!(m & (1u << 10))) {
        const float4 c = s_L[h];
        L = radd(L, rmuls(RGB3{c.x, c.y, c.z}, w));
      }
      ws = ws + w;
    }
  acc[(size_t)y * W + x] = make_float4(L.r, L.g, L.b, ws);
}

// Shadow rays of a pass, queued densely: a kernel that decides per pixel
// whether to trace a ray pushes only the rays it traces (one atomic per warp
// and call) with the slot of their result (2 * pixel + branch), and the
// traversal walks just the queue, so its warps do not refill lanes with
// empty slots. All lanes that reach a push call it, each with its own
// `want`.
struct ShadowQueue {
  float4* rays;     // 2 float4 per queued ray
  uint32_t* map;    // result slot of each queued ray
  uint32_t* count;  // rays queued in this pass (zeroed before the pass)
  __device__ __forceinline__ void push(bool want, uint32_t slot, V3 o, V3 d) const {
    const uint32_t act = __activemask();
    const uint32_t m = __ballot_sync(act, want);
    if (!m) return;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t leader = __ffs(m) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(act, base, leader);
    if (!want) return;
    const uint32_t q = base + __popc(m & ((1u << lane) - 1u));
    rays[2 * (size_t)q] = make_float4(o.x, o.y, o.z, 0.0f);
    rays[2 * (size_t)q + 1] = make_float4(d.x, d.y, d.z, inf_());
    map[q] = slot;
  }
};

// Camera rays generated inside the persistent traversal's ray source.
struct CameraSrc {
  PassCtx P;
  const uint32_t* pass_dev;
  __device__ __forceinline__ uint32_t limit(uint32_t n) const { return n; }
  __device__ __forceinline__ void load(uint32_t pix, float4* o, float4* d) const {
    float fx, fy;
    camera_sample(P, pix, *pass_dev, &fx, &fy);
    RayD r = camera_ray(P.S.cam, fx, fy);
    *o = make_float4(r.o.x, r.o.y, r.o.z, 0.0f);
    *d = make_float4(r.d.x, r.d.y, r.d.z, inf_());
  }
};

}  // namespace

}  // namespace wpbr
