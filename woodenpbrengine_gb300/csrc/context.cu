// context.cu — the C ABI (include/wpbr_gpu.h): context lifetime, scene
// upload, BVH build/export, collision, rendering entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "camera.cuh"
#include "common.cuh"
#include "ctx.hpp"
#include "wpbr_gpu.h"

namespace wpbr {

wpbr_status set_err(wpbr_ctx* ctx, wpbr_status st, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return st;
}
wpbr_status cuda_err(wpbr_ctx* ctx, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  if (e == cudaErrorMemoryAllocation) return set_err(ctx, WPBR_ERR_OOM, m);
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return set_err(ctx, WPBR_ERR_NO_DEVICE, m);
  return set_err(ctx, WPBR_ERR_CUDA, m);
}

SceneView scene_view(const wpbr_ctx* ctx) {
  SceneView S{};
  S.ns = ctx->ns;
  S.nt = ctx->nt;
  S.N = ctx->N;
  S.sph_o2w = ctx->sph_o2w.p;
  S.sph_w2o = ctx->sph_w2o.p;
  S.sph_r = ctx->sph_r.p;
  S.sph_mat = ctx->sph_mat.p;
  S.pos = ctx->pos.p;
  S.idx = ctx->idx.p;
  S.nrm = ctx->has_nrm ? ctx->nrm.p : nullptr;
  S.tan = ctx->has_nrm ? ctx->tan.p : nullptr;
  S.uv = ctx->has_uv ? ctx->uv.p : nullptr;
  S.tri_mat = ctx->tri_mat.p;
  S.tri_flags = ctx->tri_flags.p;
  S.mats = ctx->mats.p;
  S.lights = ctx->lights.p;
  S.nlights = (uint32_t)ctx->h_lights.size();
  S.has_env = ctx->has_env ? 1 : 0;
  EnvView& e = S.env;
  e.W = ctx->envW;
  e.H = ctx->envH;
  e.rgb = ctx->env_rgb.p;
  e.cond_func = ctx->cond_func.p;
  e.cond_cdf = ctx->cond_cdf.p;
  e.cond_int = ctx->cond_int.p;
  e.marg_func = ctx->marg_func.p;
  e.marg_cdf = ctx->marg_cdf.p;
  e.marg_int = ctx->env_marg_int;
  e.l2w = ctx->env_l2w;
  e.w2l = ctx->env_w2l;
  e.le = ctx->env_le;
  S.cam = ctx->cam;
  S.quirks = ctx->quirks;
  S.tex = TexView{ctx->tex_texels.p, ctx->tex_levels.p, ctx->tex_info.p, ctx->tex_gauss.p, ctx->ntex};
  return S;
}

}  // namespace wpbr

using namespace wpbr;

namespace {

// SLoadTexture::generateMIPS (CSTextureProcess.h:352-400): floor(log2(max
// side)) - 1 levels, each the 2x2 box average of the previous one; the last
// column and row average the previous level's last column / row only, the
// corner copies its last texel.
void build_mips(const wpbr_texture& t, std::vector<float4>& tx, std::vector<TexLevel>& lv, std::vector<TexInfo>& ti) {
  uint32_t n = (uint32_t)(uint16_t)(std::log2((double)std::max(t.width, t.height)) - 1.0);
  if (n < 1) n = 1;
  TexInfo info{(uint32_t)lv.size(), n};
  uint32_t W = t.width, H = t.height;
  uint32_t base = (uint32_t)tx.size();
  lv.push_back(TexLevel{base, W, H, 0});
  for (size_t i = 0; i < (size_t)W * H; ++i) tx.push_back(make_float4(t.rgb[3 * i], t.rgb[3 * i + 1], t.rgb[3 * i + 2], 0.0f));
  for (uint32_t l = 1; l < n; ++l) {
    TexLevel pv = lv.back();
    uint32_t w = std::max(1u, pv.w / 2), h = std::max(1u, pv.h / 2);
    uint32_t off = (uint32_t)tx.size();
    tx.resize(tx.size() + (size_t)w * h);
    auto P = [&](uint32_t x, uint32_t y) { return tx[pv.offset + (size_t)y * pv.w + x]; };
    auto avg4 = [](float4 a, float4 b, float4 c, float4 d) {
      return make_float4((((a.x + b.x) + c.x) + d.x) * 0.25f, (((a.y + b.y) + c.y) + d.y) * 0.25f,
                         (((a.z + b.z) + c.z) + d.z) * 0.25f, 0.0f);
    };
    auto avg2 = [](float4 a, float4 b) {
      return make_float4((a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f, 0.0f);
    };
    for (uint32_t y = 0; y + 1 < h; ++y) {
      for (uint32_t x = 0; x + 1 < w; ++x)
        tx[off + (size_t)y * w + x] = avg4(P(2 * x, 2 * y), P(2 * x + 1, 2 * y), P(2 * x, 2 * y + 1), P(2 * x + 1, 2 * y + 1));
      tx[off + (size_t)y * w + (w - 1)] = avg2(P(pv.w - 1, 2 * y), P(pv.w - 1, 2 * y + 1));
    }
    for (uint32_t x = 0; x + 1 < w; ++x) tx[off + (size_t)(h - 1) * w + x] = avg2(P(2 * x, pv.h - 1), P(2 * x + 1, pv.h - 1));
    tx[off + (size_t)(h - 1) * w + (w - 1)] = P(pv.w - 1, pv.h - 1);
    lv.push_back(TexLevel{off, w, h, 0});
  }
  ti.push_back(info);
}

// JobFilterTableGaussing (CSTextureProcess.cpp:16-32): exp(-2 r2) - exp(-2)
void gauss_table(float* w) {
  for (int i = 0; i < kGaussTable; ++i) {
    float r2 = (float)i / (float)(kGaussTable - 1);
    w[i] = wpbr_fm::expf_(-2.0f * r2) - wpbr_fm::expf_(-2.0f);
  }
}

template <typename T>
cudaError_t upload(DevBuf<T>& d, const T* h, size_t n, cudaStream_t s) {
  cudaError_t e = d.ensure(n);
  if (e != cudaSuccess || n == 0) return e;
  return cudaMemcpyAsync(d.p, h, n * sizeof(T), cudaMemcpyHostToDevice, s);
}

}  // namespace

namespace wpbr {
// Frees the build scratch of the BVH; with keep_traversal the traversal
// layout (Node2 array, primitive records) stays, else it goes too.
void bvh_release(wpbr_ctx* ctx, bool keep_traversal) {
  BvhState& B = ctx->bvh;
  B.pb_lo.release(); B.pb_hi.release(); B.centroid.release(); B.codes.release(); B.cb_enc.release();
  B.k0.release(); B.k1.release(); B.v0.release(); B.v1.release(); B.hist.release(); B.scan_tmp.release();
  B.tid.release(); B.tstart.release(); B.troot.release();
  B.rng_lo.release(); B.rng_hi.release(); B.child0.release(); B.child1.release(); B.parent.release();
  B.visits.release(); B.size.release(); B.nb_lo.release(); B.nb_hi.release();
  B.cur.release(); B.nxt.release(); B.seg_of.release(); B.posF.release(); B.posT.release(); B.rnk.release();
  B.pos_lo.release(); B.pos_hi.release(); B.bucket.release(); B.ftl.release();
  B.seg_start.release(); B.seg_end.release(); B.seg_node.release(); B.seg_acc.release(); B.seg_bk.release();
  B.seg_best.release(); B.seg_dec.release(); B.seg_pre.release(); B.chunk_tot.release(); B.lvl.release();
  B.bar.release(); B.small_start.release(); B.small_end.release();
  B.small_node.release(); B.med_start.release(); B.med_end.release(); B.med_node.release(); B.sah_rng.release(); B.tpos.release(); B.sah_ld.release(); B.t_ld.release(); B.tinv.release(); B.seg_ld.release();
  B.med_ld.release(); B.small_ld.release(); B.role.release(); B.counters.release(); B.dinfo.release(); B.sah_axis.release(); B.lin_node.release();
  B.lin_bounds.release(); B.is_int.release(); B.int_index.release(); B.depth_max.release();
  B.int_kids.release(); B.int_slot.release();
  B.split_off.release();
  if (!keep_traversal) {
    B.nodes2.release();
    B.nodes_split.release();
    B.prims.release();
  }
}

std::atomic<long long> g_alloc_budget{-1};

}  // namespace wpbr

extern "C" {

WPBR_API const char* wpbr_version(void) { return "wpbr-gb300 1.0 (sm_103a)"; }

WPBR_API wpbr_status wpbr_set_traversal_limits(wpbr_ctx* ctx, uint32_t max_stack_entries, uint32_t max_loop_steps) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  if (max_stack_entries > 256)
    return set_err(ctx, WPBR_ERR_INVALID_ARG, "set_traversal_limits: at most 256 stack entries");
  ctx->lim_stack = max_stack_entries;
  ctx->lim_steps = max_loop_steps;
  ++ctx->epoch;  // the pass graphs bake the bounds into their kernel arguments
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_debug_ray_order(wpbr_ctx* ctx, const float* rays, uint64_t n, uint32_t* keys,
                                          uint32_t* perm) {
  if (!ctx || (n && (!rays || !keys || !perm))) return WPBR_ERR_INVALID_ARG;
  return ray_order_debug(ctx, rays, n, keys, perm);
}
WPBR_API void wpbr_debug_fail_allocations(int64_t n) { g_alloc_budget.store(n < 0 ? -1 : (long long)n); }

WPBR_API wpbr_status wpbr_create(int device, wpbr_ctx** out) {
  if (!out) return WPBR_ERR_INVALID_ARG;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return WPBR_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return WPBR_ERR_INVALID_ARG;
  wpbr_ctx* ctx = new (std::nothrow) wpbr_ctx();
  if (!ctx) return WPBR_ERR_OOM;
  ctx->device = device;
  e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = ctx->d_err.ensure(1);
  if (e == cudaSuccess) e = cudaMemset(ctx->d_err.p, 0, 4);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ctx->d_err.release();
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return e == cudaErrorMemoryAllocation ? WPBR_ERR_OOM : WPBR_ERR_CUDA;
  }
  ctx->own_stream = true;
  *out = ctx;
  return WPBR_OK;
}

WPBR_API void wpbr_destroy(wpbr_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->rs.graph) cudaGraphExecDestroy(ctx->rs.graph);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  // DevBuf members free their memory through cudaFree in release(); collect them
  ctx->d_err.release();
  ctx->sph_o2w.release(); ctx->sph_w2o.release(); ctx->sph_r.release(); ctx->pos.release();
  ctx->nrm.release(); ctx->tan.release(); ctx->uv.release(); ctx->sph_mat.release(); ctx->idx.release();
  ctx->tri_mat.release(); ctx->tri_flags.release(); ctx->mats.release(); ctx->lights.release();
  ctx->env_rgb.release(); ctx->cond_func.release(); ctx->cond_cdf.release(); ctx->cond_int.release();
  ctx->marg_func.release(); ctx->marg_cdf.release(); ctx->marg_int.release(); ctx->env_lum.release();
  ctx->tex_texels.release(); ctx->tex_levels.release(); ctx->tex_info.release(); ctx->tex_gauss.release();
  bvh_release(ctx, false);
  if (ctx->bvh.h_info) cudaFreeHost(ctx->bvh.h_info);
  RenderState& R = ctx->rs;
  if (R.ggraph) cudaGraphExecDestroy(R.ggraph);
  if (R.sgraph) cudaGraphExecDestroy(R.sgraph);
  for (uint32_t g = 0; g < RenderState::kMaxGroup; ++g) {
    if (R.gstream[g]) cudaStreamDestroy(R.gstream[g]);
    if (R.gjoin[g]) cudaEventDestroy(R.gjoin[g]);
  }
  if (R.gfork) cudaEventDestroy(R.gfork);
  R.acc.release(); R.hit_prim.release(); R.shadow_rays.release(); R.shadow_hit.release(); R.shadow_map.release();
  R.pstate.release();
  R.Lbuf.release(); R.pfilm.release(); R.pass_dev.release(); R.counters.release();
  R.spec_mats.release(); R.spec_le.release(); R.spec_L.release(); R.spec_acc.release();
  ctx->io_rays.release(); ctx->io_hits.release(); ctx->io_stats.release();
  ctx->tscr[0].release(); ctx->tscr[1].release();
  for (cudaEvent_t& ev : ctx->io_ev)
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t& ev : ctx->tev)
    if (ev) cudaEventDestroy(ev);
  if (ctx->io_h2d) cudaStreamDestroy(ctx->io_h2d);
  if (ctx->io_comp) cudaStreamDestroy(ctx->io_comp);
  if (ctx->io_d2h) cudaStreamDestroy(ctx->io_d2h);
  for (auto& f : R.f) f.release();
  for (auto& u : R.u) u.release();
  ctx->adj.release();
  delete ctx;
}

WPBR_API const char* wpbr_last_error(const wpbr_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

WPBR_API wpbr_status wpbr_set_stream(wpbr_ctx* ctx, void* stream) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  if (ctx->own_stream && ctx->stream) {
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
  }
  ctx->stream = (cudaStream_t)stream;
  ctx->own_stream = false;
  if (ctx->rs.graph) {
    cudaGraphExecDestroy(ctx->rs.graph);
    ctx->rs.graph = nullptr;
  }
  ctx->rs.graph_ok = false;
  return WPBR_OK;
}

WPBR_API void* wpbr_get_stream(const wpbr_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

WPBR_API wpbr_status wpbr_set_quirks(wpbr_ctx* ctx, uint32_t quirks) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  if (quirks & ~WPBR_QUIRK_MASK) return set_err(ctx, WPBR_ERR_INVALID_ARG, "set_quirks: unknown bits");
  uint32_t changed = ctx->quirks ^ quirks;
  ctx->quirks = quirks;
  ++ctx->epoch;
  // the sort order changes the tree; the index bug changes the env distribution
  if (changed & WPBR_Q_FULL_MORTON_SORT) ctx->bvh.built = false;
  if ((changed & WPBR_Q_ENV_DISTRIB_INDEX_BUG) && ctx->has_scene && ctx->has_env) {
    wpbr_status s = env_preprocess(ctx);
    if (s != WPBR_OK) return s;
  }
  ctx->rs.graph_ok = false;
  if (ctx->rs.graph) {
    cudaGraphExecDestroy(ctx->rs.graph);
    ctx->rs.graph = nullptr;
  }
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_set_traversal(wpbr_ctx* ctx, uint32_t mode) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  if (mode != WPBR_TRAVERSAL_BINARY && mode != WPBR_TRAVERSAL_BINARY_FULL_LEAVES)
    return set_err(ctx, WPBR_ERR_INVALID_ARG, "set_traversal: unknown mode");
  ctx->traversal = mode;
  ++ctx->epoch;
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_set_ray_sort(wpbr_ctx* ctx, uint32_t bits_per_axis) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  if (bits_per_axis > 10) return set_err(ctx, WPBR_ERR_INVALID_ARG, "set_ray_sort: at most 10 bits per axis");
  ctx->ray_sort = bits_per_axis;
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_set_spectrum(wpbr_ctx* ctx, uint32_t mode) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  if (mode > WPBR_SPECTRUM_SAMPLED64) return set_err(ctx, WPBR_ERR_INVALID_ARG, "set_spectrum: unknown mode");
  ctx->spectrum = mode;
  ctx->rs.ready = false;  // render_setup allocates the mode's buffers
  ++ctx->epoch;
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_synchronize(wpbr_ctx* ctx) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_err(ctx, e, "synchronize");
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_check_device_errors(wpbr_ctx* ctx) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  uint32_t v = 0;
  WPBR_CUDA(cudaMemcpyAsync(&v, ctx->d_err.p, 4, cudaMemcpyDeviceToHost, ctx->stream));
  WPBR_CUDA(cudaStreamSynchronize(ctx->stream));
  if (v) {
    WPBR_CUDA(cudaMemsetAsync(ctx->d_err.p, 0, 4, ctx->stream));
    WPBR_CUDA(cudaStreamSynchronize(ctx->stream));
    char buf[96];
    snprintf(buf, sizeof(buf), "device error word 0x%x (1 stack overflow, 2 loop limit, 4 build)", v);
    return set_err(ctx, WPBR_ERR_TRAVERSAL_LIMIT, buf);
  }
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_scene_upload(wpbr_ctx* ctx, const wpbr_scene_desc* d) {
  if (!ctx || !d) return WPBR_ERR_INVALID_ARG;
  // validation (the reference asserts or crashes on these)
  if (d->n_triangles && (!d->indices || !d->positions))
    return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: triangles without indices/positions");
  if (d->n_spheres && !d->spheres) return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: spheres pointer is null");
  for (uint64_t i = 0; i < 3ull * d->n_triangles; ++i)
    if (d->indices[i] >= d->n_vertices) return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: vertex index out of range");
  for (uint32_t i = 0; i < d->n_spheres; ++i)
    if (d->spheres[i].material >= d->n_materials || !(d->spheres[i].radius > 0.0f) ||
        !std::isfinite(d->spheres[i].radius))
      return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: sphere material or radius invalid");
  // non-finite geometry would give NaN bounds and Morton codes (the
  // reference's float-to-integer conversion of them is undefined)
  for (uint32_t i = 0; i < d->n_spheres; ++i)
    for (int k = 0; k < 16; ++k)
      if (!std::isfinite(d->spheres[i].object_to_world.m[k]) || !std::isfinite(d->spheres[i].world_to_object.m[k]))
        return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: non-finite sphere transform");
  if (d->n_triangles)
    for (uint64_t i = 0; i < 3ull * d->n_vertices; ++i)
      if (!std::isfinite(d->positions[i])) return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: non-finite vertex position");
  std::vector<uint32_t> tmat(d->n_triangles, 0xFFFFFFFFu), tfl(d->n_triangles, 0);
  for (uint32_t m = 0; m < d->n_meshes; ++m) {
    const wpbr_mesh& ms = d->meshes[m];
    if ((uint64_t)ms.tri_begin + ms.tri_count > d->n_triangles || ms.material >= d->n_materials)
      return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: mesh range or material invalid");
    uint32_t fl = ms.flags;
    if (!d->normals || !d->tangents) fl &= ~(uint32_t)WPBR_MESH_NORMALS_TANGENTS;
    if (!d->uvs) fl &= ~(uint32_t)WPBR_MESH_UVS;
    for (uint32_t t = ms.tri_begin; t < ms.tri_begin + ms.tri_count; ++t) {
      tmat[t] = ms.material;
      tfl[t] = fl;
    }
  }
  for (uint32_t t = 0; t < d->n_triangles; ++t)
    if (tmat[t] == 0xFFFFFFFFu) return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: triangle not covered by a mesh");
  int n_env = 0;
  for (uint32_t i = 0; i < d->n_lights; ++i) {
    if (d->lights[i].type == WPBR_LIGHT_SPHERE && d->lights[i].sphere_index >= d->n_spheres)
      return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: sphere light index out of range");
    if (d->lights[i].type == WPBR_LIGHT_ENV) ++n_env;
    if (d->lights[i].type > WPBR_LIGHT_ENV) return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: unknown light type");
  }
  if (n_env > 0 && !d->envmap) return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: env light without envmap");
  if (d->envmap && (d->envmap->width < 2 || d->envmap->height < 2 || !d->envmap->rgb))
    return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: envmap must be at least 2x2");
  if (d->camera.res_x == 0 || d->camera.res_y == 0)
    return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: camera resolution is zero");
  if (d->n_spheres + (uint64_t)d->n_triangles >= (1ull << 29))
    return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: more than 2^29 primitives");
  if (d->n_textures && !d->textures) return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: textures pointer is null");
  uint64_t texels = 0;
  for (uint32_t i = 0; i < d->n_textures; ++i) {
    if (d->textures[i].width < 4 || d->textures[i].height < 4 || !d->textures[i].rgb)
      return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: textures must be at least 4x4");
    texels += 2 * (uint64_t)d->textures[i].width * d->textures[i].height;  // bound on the pyramid
  }
  if (texels >= (1ull << 31))
    return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: more than 2^30 texels of textures");
  bool has_metal = false;
  for (uint32_t m = 0; m < d->n_materials; ++m) {
    const wpbr_material& mt = d->materials[m];
    if (mt.type > WPBR_MAT_METAL_ISOTROPIC) return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: unknown material type");
    if (WPBR_MAT_TEXTURED(mt.type)) {
      if (mt.tex[0] >= d->n_textures || mt.tex[1] >= d->n_textures)
        return set_err(ctx, WPBR_ERR_INVALID_ARG, "scene: metal material texture index out of range");
      has_metal = true;
    }
  }

  cudaStream_t st = ctx->stream;
  ctx->has_scene = false;
  ++ctx->epoch;
  ctx->bvh.built = false;
  ctx->rs.ready = false;
  ctx->ns = d->n_spheres;
  ctx->nt = d->n_triangles;
  ctx->nv = d->n_vertices;
  ctx->N = ctx->ns + ctx->nt;
  std::vector<Xf> o2w(ctx->ns), w2o(ctx->ns);
  std::vector<float> rad(ctx->ns);
  std::vector<uint32_t> smat(ctx->ns);
  for (uint32_t i = 0; i < ctx->ns; ++i) {
    o2w[i] = xf_from(d->spheres[i].object_to_world);
    w2o[i] = xf_from(d->spheres[i].world_to_object);
    rad[i] = d->spheres[i].radius;
    smat[i] = d->spheres[i].material;
  }
  WPBR_CUDA(upload(ctx->sph_o2w, o2w.data(), ctx->ns, st));
  WPBR_CUDA(upload(ctx->sph_w2o, w2o.data(), ctx->ns, st));
  WPBR_CUDA(upload(ctx->sph_r, rad.data(), ctx->ns, st));
  WPBR_CUDA(upload(ctx->sph_mat, smat.data(), ctx->ns, st));
  WPBR_CUDA(upload(ctx->pos, d->positions, 3ull * ctx->nv, st));
  ctx->has_nrm = d->normals && d->tangents;
  ctx->has_uv = d->uvs != nullptr;
  if (ctx->has_nrm) {
    WPBR_CUDA(upload(ctx->nrm, d->normals, 3ull * ctx->nv, st));
    WPBR_CUDA(upload(ctx->tan, d->tangents, 3ull * ctx->nv, st));
  }
  if (ctx->has_uv) WPBR_CUDA(upload(ctx->uv, d->uvs, 2ull * ctx->nv, st));
  WPBR_CUDA(upload(ctx->idx, d->indices, 3ull * ctx->nt, st));
  WPBR_CUDA(upload(ctx->tri_mat, tmat.data(), ctx->nt, st));
  WPBR_CUDA(upload(ctx->tri_flags, tfl.data(), ctx->nt, st));
  WPBR_CUDA(upload(ctx->mats, d->materials, d->n_materials, st));
  ctx->nmat = d->n_materials;
  ctx->h_lights.assign(d->lights, d->lights + d->n_lights);
  WPBR_CUDA(upload(ctx->lights, d->lights, d->n_lights, st));
  ctx->has_env = d->envmap != nullptr;
  ctx->env_lights_only = d->n_lights > 0;
  for (uint32_t i = 0; i < d->n_lights; ++i)
    if (d->lights[i].type != WPBR_LIGHT_ENV) ctx->env_lights_only = false;
  if (ctx->has_env) {
    const wpbr_envmap& e = *d->envmap;
    ctx->envW = (int)e.width;
    ctx->envH = (int)e.height;
    size_t n = (size_t)e.width * e.height;
    std::vector<float4> rgb(n);
    for (size_t i = 0; i < n; ++i) rgb[i] = make_float4(e.rgb[3 * i], e.rgb[3 * i + 1], e.rgb[3 * i + 2], 0.0f);
    WPBR_CUDA(upload(ctx->env_rgb, rgb.data(), n, st));
    WPBR_CUDA(ctx->cond_func.ensure(n));
    WPBR_CUDA(ctx->cond_cdf.ensure((size_t)e.height * (e.width + 1)));
    WPBR_CUDA(ctx->cond_int.ensure(e.height));
    WPBR_CUDA(ctx->marg_func.ensure(e.height));
    WPBR_CUDA(ctx->marg_cdf.ensure(e.height + 1));
    WPBR_CUDA(ctx->marg_int.ensure(1));
    ctx->env_l2w = xf_from(e.light_to_world);
    ctx->env_w2l = xf_from(e.world_to_light);
    ctx->env_le = RGB3{1.0f, 1.0f, 1.0f};
    for (uint32_t i = 0; i < d->n_lights; ++i)
      if (d->lights[i].type == WPBR_LIGHT_ENV) ctx->env_le = RGB3{d->lights[i].Le[0], d->lights[i].Le[1], d->lights[i].Le[2]};
  }
  // textures: MIP pyramids on the host (SLoadTexture::generateMIPS), one
  // float4 array for every level of every texture, and the EWA filter table
  std::vector<float4> tx;
  std::vector<TexLevel> lv;
  std::vector<TexInfo> ti;
  for (uint32_t i = 0; i < d->n_textures; ++i) build_mips(d->textures[i], tx, lv, ti);
  ctx->ntex = d->n_textures;
  ctx->has_metal = has_metal;
  WPBR_CUDA(upload(ctx->tex_texels, tx.empty() ? nullptr : tx.data(), tx.size(), st));
  WPBR_CUDA(upload(ctx->tex_levels, lv.empty() ? nullptr : lv.data(), lv.size(), st));
  WPBR_CUDA(upload(ctx->tex_info, ti.empty() ? nullptr : ti.data(), ti.size(), st));
  float gauss[kGaussTable];
  gauss_table(gauss);
  WPBR_CUDA(upload(ctx->tex_gauss, gauss, kGaussTable, st));
  ctx->cam = camera_setup(d->camera);
  WPBR_CUDA(cudaStreamSynchronize(st));
  ctx->has_scene = true;
  wpbr_status s = env_preprocess(ctx);
  if (s != WPBR_OK) return s;
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_camera_info(wpbr_ctx* ctx, float* raster_camera, float* dx, float* dy) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  if (!ctx->has_scene) return set_err(ctx, WPBR_ERR_NOT_BUILT, "camera_info: no scene");
  if (raster_camera)
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) raster_camera[4 * i + j] = ctx->cam.raster_camera.m[i][j];
  if (dx) { dx[0] = ctx->cam.dx.x; dx[1] = ctx->cam.dx.y; dx[2] = ctx->cam.dx.z; }
  if (dy) { dy[0] = ctx->cam.dy.x; dy[1] = ctx->cam.dy.y; dy[2] = ctx->cam.dy.z; }
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_camera_setup(const wpbr_camera* camera, float* raster_camera, float* dx, float* dy) {
  if (!camera || !raster_camera || !dx || !dy) return WPBR_ERR_INVALID_ARG;
  CameraParams c = camera_setup(*camera);
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) raster_camera[4 * i + j] = c.raster_camera.m[i][j];
  dx[0] = c.dx.x; dx[1] = c.dx.y; dx[2] = c.dx.z;
  dy[0] = c.dy.x; dy[1] = c.dy.y; dy[2] = c.dy.z;
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_env_distribution(wpbr_ctx* ctx, float* cond_cdf, float* cond_int, float* marg_cdf,
                                           float* marg_int) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  if (!ctx->has_env) return set_err(ctx, WPBR_ERR_NOT_BUILT, "env_distribution: no environment light");
  cudaStream_t st = ctx->stream;
  size_t W = ctx->envW, H = ctx->envH;
  if (cond_cdf) WPBR_CUDA(cudaMemcpyAsync(cond_cdf, ctx->cond_cdf.p, sizeof(float) * H * (W + 1), cudaMemcpyDeviceToHost, st));
  if (cond_int) WPBR_CUDA(cudaMemcpyAsync(cond_int, ctx->cond_int.p, sizeof(float) * H, cudaMemcpyDeviceToHost, st));
  if (marg_cdf) WPBR_CUDA(cudaMemcpyAsync(marg_cdf, ctx->marg_cdf.p, sizeof(float) * (H + 1), cudaMemcpyDeviceToHost, st));
  if (marg_int) WPBR_CUDA(cudaMemcpyAsync(marg_int, ctx->marg_int.p, sizeof(float), cudaMemcpyDeviceToHost, st));
  WPBR_CUDA(cudaStreamSynchronize(st));
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_bvh_build(wpbr_ctx* ctx) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  return bvh_build(ctx);
}

WPBR_API wpbr_status wpbr_bvh_info(wpbr_ctx* ctx, uint32_t* out4) {
  if (!ctx || !out4) return WPBR_ERR_INVALID_ARG;
  if (!ctx->bvh.built) return set_err(ctx, WPBR_ERR_NOT_BUILT, "bvh_info: BVH not built");
  out4[0] = ctx->bvh.N;
  out4[1] = ctx->bvh.M;
  out4[2] = ctx->bvh.T;
  out4[3] = ctx->bvh.max_depth;
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_bvh_export(wpbr_ctx* ctx, float* prim_bounds, float* centroids, float* cbounds,
                                     uint32_t* codes, uint32_t* sorted_codes, uint32_t* sorted_prims,
                                     uint32_t* treelet_start, uint32_t* nodes, float* node_bounds, uint32_t* shapes) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  BvhState& B = ctx->bvh;
  if (!B.built) return set_err(ctx, WPBR_ERR_NOT_BUILT, "bvh_export: BVH not built");
  cudaStream_t st = ctx->stream;
  size_t N = B.N;
  if (N == 0) return WPBR_OK;
  std::vector<float4> lo, hi, ce;
  if (prim_bounds) {
    lo.resize(N);
    hi.resize(N);
    WPBR_CUDA(cudaMemcpyAsync(lo.data(), B.pb_lo.p, 16 * N, cudaMemcpyDeviceToHost, st));
    WPBR_CUDA(cudaMemcpyAsync(hi.data(), B.pb_hi.p, 16 * N, cudaMemcpyDeviceToHost, st));
  }
  if (centroids) {
    ce.resize(N);
    WPBR_CUDA(cudaMemcpyAsync(ce.data(), B.centroid.p, 16 * N, cudaMemcpyDeviceToHost, st));
  }
  uint32_t cb[6];
  if (cbounds) WPBR_CUDA(cudaMemcpyAsync(cb, B.cb_enc.p, 24, cudaMemcpyDeviceToHost, st));
  if (codes) WPBR_CUDA(cudaMemcpyAsync(codes, B.codes.p, 4 * N, cudaMemcpyDeviceToHost, st));
  if (sorted_codes) WPBR_CUDA(cudaMemcpyAsync(sorted_codes, B.skey, 4 * N, cudaMemcpyDeviceToHost, st));
  if (sorted_prims) WPBR_CUDA(cudaMemcpyAsync(sorted_prims, B.sprim, 4 * N, cudaMemcpyDeviceToHost, st));
  if (shapes) WPBR_CUDA(cudaMemcpyAsync(shapes, B.sprim, 4 * N, cudaMemcpyDeviceToHost, st));
  if (treelet_start) WPBR_CUDA(cudaMemcpyAsync(treelet_start, B.tstart.p, 4 * (size_t)B.T, cudaMemcpyDeviceToHost, st));
  if (nodes) WPBR_CUDA(cudaMemcpyAsync(nodes, B.lin_node.p, 12 * (size_t)B.M, cudaMemcpyDeviceToHost, st));
  if (node_bounds) WPBR_CUDA(cudaMemcpyAsync(node_bounds, B.lin_bounds.p, 24 * (size_t)B.M, cudaMemcpyDeviceToHost, st));
  WPBR_CUDA(cudaStreamSynchronize(st));
  for (size_t i = 0; prim_bounds && i < N; ++i) {
    float v[6] = {lo[i].x, lo[i].y, lo[i].z, hi[i].x, hi[i].y, hi[i].z};
    memcpy(prim_bounds + 6 * i, v, sizeof(v));
  }
  for (size_t i = 0; centroids && i < N; ++i) {
    centroids[3 * i] = ce[i].x;
    centroids[3 * i + 1] = ce[i].y;
    centroids[3 * i + 2] = ce[i].z;
  }
  if (cbounds)
    for (int k = 0; k < 6; ++k) {
      uint32_t u = cb[k];
      uint32_t bits = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
      memcpy(&cbounds[k], &bits, 4);
    }
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_collide_device(wpbr_ctx* ctx, const void* d_rays, uint64_t n, void* d_hits, uint32_t mode) {
  if (!ctx || (n && (!d_rays || !d_hits)) || mode > WPBR_TRACE_ANY) return WPBR_ERR_INVALID_ARG;
  return trace_rays(ctx, (const float4*)d_rays, n, (float4*)d_hits, mode, nullptr);
}

// Batches of at least kPipeMin rays are collided in four chunks (1/8, 3/8,
// 3/8, 1/8 of the batch): rays go up on one copy stream, hits come down on
// another, and the chunks are traced alternately on the context's stream
// and a second traversal stream (each with its own scratch), so one chunk's
// copies overlap its neighbours' traversal, the tail of one traversal
// overlaps the start of the next, and the two copies nothing overlaps (the
// first up, the last down) are short. Measured on 8.4M rays with 210 / 190
// GB/s host copies: 7.35 ms serial; equal quarters 6.72 ms on one traversal
// stream, 6.06 ms on two; 1/8-3/8-3/8-1/8 5.76 ms (eight equal chunks 6.29
// ms, five uneven ones 5.82 ms: every chunk also pays its own ray-order
// sort).
constexpr uint64_t kPipeMin = 1ull << 22;
// Edge chunks of 1/E of the batch; 8.4M rays through pinned buffers, ms per
// call with the current kernels: E = 4 4.969, 8 4.758, 16 4.855, 32 5.034.
#ifndef WPBR_PIPE_EDGE
#define WPBR_PIPE_EDGE 8
#endif

static wpbr_status collide_pipelined(wpbr_ctx* ctx, const float* rays, uint64_t n, float* hits, uint32_t mode) {
  if (!ctx->io_h2d) WPBR_CUDA(cudaStreamCreateWithFlags(&ctx->io_h2d, cudaStreamNonBlocking));
  if (!ctx->io_d2h) WPBR_CUDA(cudaStreamCreateWithFlags(&ctx->io_d2h, cudaStreamNonBlocking));
  if (!ctx->io_comp) WPBR_CUDA(cudaStreamCreateWithFlags(&ctx->io_comp, cudaStreamNonBlocking));
  for (cudaEvent_t& ev : ctx->io_ev)
    if (!ev) WPBR_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaStream_t st = ctx->stream;
  cudaStream_t comp[2] = {st, ctx->io_comp};
  // four chunks of 1/E, 1/2 - 1/E, 1/2 - 1/E, 1/E of the batch: the first
  // copy up and the last copy down, which nothing overlaps, are short
  const uint64_t edge = n / WPBR_PIPE_EDGE;
  uint64_t bounds[5] = {0, edge, n / 2, n - edge, n};
  // everything starts after the work already queued on the context's stream
  WPBR_CUDA(cudaEventRecord(ctx->io_ev[2], st));
  WPBR_CUDA(cudaStreamWaitEvent(ctx->io_h2d, ctx->io_ev[2], 0));
  WPBR_CUDA(cudaStreamWaitEvent(ctx->io_comp, ctx->io_ev[2], 0));
  // A failure inside the loop leaves the loop (never returns from it): the
  // copies already queued read `rays` and write `hits`, so all four streams
  // are drained before the call returns, whatever happened.
  wpbr_status s = WPBR_OK;
  cudaError_t ce = cudaSuccess;
  const char* what = "collide";
  for (int i = 0; i < 4; ++i) {
    uint64_t off = bounds[i], c = bounds[i + 1] - bounds[i];
    if (c == 0) continue;
    cudaStream_t cs = comp[i & 1];
    ce = cudaMemcpyAsync(ctx->io_rays.p + 2 * off, rays + 8 * off, 32 * c, cudaMemcpyHostToDevice, ctx->io_h2d);
    if (ce == cudaSuccess) ce = cudaEventRecord(ctx->io_ev[0], ctx->io_h2d);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(cs, ctx->io_ev[0], 0);
    if (ce != cudaSuccess) {
      what = "collide: rays to the device";
      break;
    }
    s = trace_rays(ctx, ctx->io_rays.p + 2 * off, c, ctx->io_hits.p + off, mode, nullptr, i & 1, cs);
    if (s != WPBR_OK) break;
    ce = cudaEventRecord(ctx->io_ev[1], cs);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(ctx->io_d2h, ctx->io_ev[1], 0);
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(hits + 4 * off, ctx->io_hits.p + off, 16 * c, cudaMemcpyDeviceToHost, ctx->io_d2h);
    if (ce != cudaSuccess) {
      what = "collide: hits to the host";
      break;
    }
  }
  cudaError_t e1 = cudaStreamSynchronize(ctx->io_h2d);
  cudaError_t e2 = cudaStreamSynchronize(ctx->io_comp);
  cudaError_t e3 = cudaStreamSynchronize(ctx->io_d2h);
  cudaError_t e4 = cudaStreamSynchronize(st);
  if (s != WPBR_OK) return s;
  if (ce != cudaSuccess) return cuda_err(ctx, ce, what);
  for (cudaError_t e : {e1, e2, e3, e4})
    if (e != cudaSuccess) return cuda_err(ctx, e, "collide");
  return WPBR_OK;
}

static wpbr_status collide_host(wpbr_ctx* ctx, const float* rays, uint64_t n, float* hits, uint32_t* stats,
                                uint32_t mode) {
  if (!ctx || (n && (!rays || !hits)) || mode > WPBR_TRACE_ANY) return WPBR_ERR_INVALID_ARG;
  if (n == 0) return WPBR_OK;
  // grow-only staging buffers owned by the context (no allocation per call)
  cudaStream_t st = ctx->stream;
  WPBR_CUDA(ctx->io_rays.ensure(2 * n));
  WPBR_CUDA(ctx->io_hits.ensure(n));
  if (!stats && n >= kPipeMin) return collide_pipelined(ctx, rays, n, hits, mode);
  if (stats) WPBR_CUDA(ctx->io_stats.ensure(2 * n));
  WPBR_CUDA(cudaMemcpyAsync(ctx->io_rays.p, rays, 32 * n, cudaMemcpyHostToDevice, st));
  wpbr_status s = trace_rays(ctx, ctx->io_rays.p, n, ctx->io_hits.p, mode, stats ? ctx->io_stats.p : nullptr);
  if (s != WPBR_OK) return s;
  WPBR_CUDA(cudaMemcpyAsync(hits, ctx->io_hits.p, 16 * n, cudaMemcpyDeviceToHost, st));
  if (stats) WPBR_CUDA(cudaMemcpyAsync(stats, ctx->io_stats.p, 8 * n, cudaMemcpyDeviceToHost, st));
  WPBR_CUDA(cudaStreamSynchronize(st));
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_set_kernel_timing(wpbr_ctx* ctx, uint32_t enable) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  ctx->kernel_timing = enable != 0;
  ctx->timed = 0;
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_kernel_timing(wpbr_ctx* ctx, float* total_ms, uint32_t* launches) {
  if (!ctx || !total_ms || !launches) return WPBR_ERR_INVALID_ARG;
  float sum = 0.0f;
  for (int i = 0; i < ctx->timed; ++i) {
    float ms = 0.0f;
    WPBR_CUDA(cudaEventSynchronize(ctx->tev[2 * i + 1]));
    WPBR_CUDA(cudaEventElapsedTime(&ms, ctx->tev[2 * i], ctx->tev[2 * i + 1]));
    sum += ms;
  }
  *total_ms = sum;
  *launches = (uint32_t)ctx->timed;
  ctx->timed = 0;
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_collide_launches(const wpbr_ctx* ctx, uint64_t n, uint32_t* launches) {
  if (!ctx || !launches) return WPBR_ERR_INVALID_ARG;
  if (!ctx->bvh.built) return WPBR_ERR_NOT_BUILT;
  *launches = trace_launches(ctx, n, false);
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_collide(wpbr_ctx* ctx, const float* rays, uint64_t n, float* hits, uint32_t mode) {
  return collide_host(ctx, rays, n, hits, nullptr, mode);
}

WPBR_API wpbr_status wpbr_collide_stats(wpbr_ctx* ctx, const float* rays, uint64_t n, float* hits, uint32_t* stats,
                                        uint32_t mode) {
  if (!stats) return WPBR_ERR_INVALID_ARG;
  return collide_host(ctx, rays, n, hits, stats, mode);
}

WPBR_API wpbr_status wpbr_render_setup(wpbr_ctx* ctx, uint32_t spp, uint32_t seed, uint32_t stream) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  return render_setup(ctx, spp, seed, stream);
}

WPBR_API wpbr_status wpbr_render_pass(wpbr_ctx* ctx, uint32_t pass) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  return render_pass_fused(ctx, pass);
}

WPBR_API wpbr_status wpbr_render(wpbr_ctx* ctx) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  if (!ctx->rs.ready) return set_err(ctx, WPBR_ERR_NOT_BUILT, "render: render_setup not called");
  wpbr_status s = render_frame(ctx);  // every pass, small films a group of passes at a time
  if (s != WPBR_OK) return s;
  return spectral_resolve(ctx);  // Sampled64: the film's toRGB, once per frame
}

WPBR_API wpbr_status wpbr_film_read(wpbr_ctx* ctx, float* acc_L, float* acc_w) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  RenderState& R = ctx->rs;
  if (!R.ready) return set_err(ctx, WPBR_ERR_NOT_BUILT, "film_read: render_setup not called");
  wpbr_status rs = spectral_resolve(ctx);
  if (rs != WPBR_OK) return rs;
  size_t n = (size_t)R.W * R.H;
  std::vector<float> a(n * 4);
  WPBR_CUDA(cudaMemcpyAsync(a.data(), R.acc.p, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost, ctx->stream));
  WPBR_CUDA(cudaStreamSynchronize(ctx->stream));
  for (size_t i = 0; i < n; ++i) {
    if (acc_L) {
      acc_L[3 * i] = a[4 * i];
      acc_L[3 * i + 1] = a[4 * i + 1];
      acc_L[3 * i + 2] = a[4 * i + 2];
    }
    if (acc_w) acc_w[i] = a[4 * i + 3];
  }
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_film_tonemap(wpbr_ctx* ctx, uint8_t* rgb8) {
  if (!ctx || !rgb8) return WPBR_ERR_INVALID_ARG;
  return film_tonemap(ctx, rgb8);
}

WPBR_API wpbr_status wpbr_job_run(wpbr_ctx* ctx, uint32_t job, uint32_t pass) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  return job_run(ctx, job, pass);
}

WPBR_API wpbr_status wpbr_job_record(wpbr_ctx* ctx, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                                     wpbr_pass_record* rec) {
  if (!ctx) return WPBR_ERR_INVALID_ARG;
  return job_record(ctx, x0, y0, x1, y1, rec);
}

}  // extern "C"
