// ctx.hpp — the per-GPU context behind the C ABI (wpbr_ctx) and its device
// buffers. Host code only.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <string>
#include <vector>

#include "camera.cuh"
#include "views.cuh"
#include "wpbr_gpu.h"

namespace wpbr {

// Allocation fault injection (wpbr_debug_fail_allocations): while the
// budget is >= 0, that many further device allocations succeed and every
// later one fails as out-of-memory without reaching cudaMalloc. Process-wide;
// -1 (the default) disables it.
extern std::atomic<long long> g_alloc_budget;
inline cudaError_t dev_malloc(void** p, size_t bytes) {
  long long b = g_alloc_budget.load();
  while (b >= 0) {
    if (b == 0) return cudaErrorMemoryAllocation;
    if (g_alloc_budget.compare_exchange_weak(b, b - 1)) break;
  }
  return cudaMalloc(p, bytes);
}

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t count) {
    if (count <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    size_t bytes = (count ? count : 1) * sizeof(T);
    cudaError_t e = dev_malloc((void**)&p, bytes);
    if (e == cudaSuccess) n = count;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// Build products and scratch of the LBVH build (bvh_build.cu).
struct BvhState {
  bool built = false;
  uint32_t N = 0, T = 0, M = 0, n_int = 0, max_depth = 0;
  // per primitive (input order)
  DevBuf<float4> pb_lo, pb_hi, centroid;
  DevBuf<uint32_t> codes;
  DevBuf<uint32_t> cb_enc;  // 6 encoded centroid-bound words
  // sort
  DevBuf<uint32_t> k0, k1, v0, v1, hist, scan_tmp;
  uint32_t* skey = nullptr;   // sorted codes (points into k0/k1)
  uint32_t* sprim = nullptr;  // sorted primitive ids
  // treelets / Karras
  DevBuf<uint32_t> tid, tstart, troot;
  DevBuf<uint32_t> rng_lo, rng_hi, child0, child1;  // unified-id arrays
  DevBuf<uint32_t> parent, visits, size;            // size 2N+T
  DevBuf<float4> nb_lo, nb_hi;                      // node bounds, unified ids
  // SAH (k_sah_levels): per position, two buffers each (cur / nxt hold the roots)
  DevBuf<uint32_t> cur, nxt, seg_of, posF, posT, rnk;
  DevBuf<float4> pos_lo, pos_hi;
  DevBuf<uint8_t> bucket;
  DevBuf<unsigned long long> ftl;  // prefix of the partition flags (true << 32 | false) within each chunk
  // per large segment, two sets (a level's and the next level's)
  DevBuf<uint32_t> seg_start, seg_end, seg_node, seg_acc, seg_bk, seg_best;
  DevBuf<uint4> seg_dec;
  DevBuf<unsigned long long> seg_pre, chunk_tot;  // children prefixes per segment, totals per chunk
  DevBuf<uint32_t> lvl, bar;                      // level words, grid barrier
  DevBuf<uint32_t> small_start, small_end, small_node, counters;
  DevBuf<uint32_t> med_start, med_end, med_node;  // segments of 33..4096 treelet roots
  DevBuf<uint32_t> sah_rng, tpos;  // SAH node position ranges; treelet sizes by position, scanned
  DevBuf<uint32_t> sah_ld, t_ld, tinv, seg_ld, med_ld, small_ld;  // depths and child-0 steps; treelet positions
  DevBuf<uint8_t> role;  // per radix node: 0 outside the flattened tree, 1 ref leaf, 2 ref interior
  DevBuf<uint32_t> dinfo;       // sizes found on the device (treelets, root, nodes, summary)
  uint32_t* h_info = nullptr;   // pinned copy of dinfo's summary
  DevBuf<uint32_t> sah_axis;
  // flattened tree (CSceneTreeLBVH) + traversal layout
  DevBuf<uint32_t> lin_node;  // M*3: offset, n_shapes, axis
  DevBuf<float> lin_bounds;   // M*6
  DevBuf<uint32_t> is_int, int_index, depth_max;
  DevBuf<uint32_t> int_kids, int_slot;  // traversal-layout order of the interior nodes
  DevBuf<Node2> nodes2;
  DevBuf<Node2> nodes_split;             // leaf-split layout: nodes2 + the records splitting large leaves
  DevBuf<uint32_t> split_off;  // offsets of each child slot's range-tree records
  DevBuf<float4> prims;
  BvhView view{};
};

// Words of RenderState::counters (zeroed at the start of every pass).
constexpr uint32_t kQueueCounter = 24;
constexpr uint32_t kPassCounters = 25;

struct RenderState {
  bool ready = false;
  uint32_t spp = 0, seed = 0, stream = 0;
  uint32_t W = 0, H = 0;
  DevBuf<float> acc;  // W*H*4 (L rgb, weight)
  // fused-path per-pixel state
  DevBuf<uint32_t> hit_prim;
  DevBuf<float4> shadow_rays;   // the pass's queued shadow rays (2 float4 each), at most 2 per pixel
  DevBuf<uint32_t> shadow_map;  // result slot (2 * pixel + branch) of each queued shadow ray
  DevBuf<uint32_t> shadow_hit;  // 2 per pixel
  DevBuf<float4> pstate;        // compact shading state, kStateF4 per pixel
  DevBuf<float4> Lbuf;          // per pixel L (xyz) + pFilm packed in w? separate:
  DevBuf<float2> pfilm;
  // staged-path (job-by-job) state: one slot per wpbr_pass_record field
  DevBuf<float> f[32];
  DevBuf<uint32_t> u[8];
  bool graph_ok = false;
  cudaGraphExec_t graph = nullptr;
  uint64_t graph_key = 0;
  DevBuf<uint32_t> pass_dev;  // pass index read by the captured kernels
  DevBuf<uint32_t> counters;  // kPassCounters words: ray-fetch counters of the pass's two traversal
                              // launches, the per-category pixel counts and cursors of the
                              // material-sorted order, and (kQueueCounter) the queued shadow rays
  DevBuf<uint32_t> order;     // the pass's pixels grouped by material category (k_cat_scatter)
  // Sampled64 mode: material / light spectra, per-pixel sample spectra, film spectra
  DevBuf<float> spec_mats, spec_le, spec_L, spec_acc;
  bool spec_dirty = false;  // Sampled64 passes ran since the last toRGB of the film
  const uint32_t* pass_ptr = nullptr;  // shared pass index (batches); null: pass_dev
  uint32_t trace_grid = 0;             // persistent traversal grid cap (0: full)
  // pass groups (render_frame, small RGB films): kMaxGroup branches of one
  // fork/join graph, each on its own stream, state slice and pass index word
  static constexpr uint32_t kMaxGroup = 8;
  uint32_t group = 0;  // passes per group of the captured group graph
  cudaGraphExec_t ggraph = nullptr;
  uint64_t ggraph_key = 0;
  // Sampled64 frames: one graph of `sgroup` sequential passes (sample slots
  // 0 .. sgroup - 1) and one film gather over them
  cudaGraphExec_t sgraph = nullptr;
  uint64_t sgraph_key = 0;
  uint32_t sgroup = 0;
  cudaStream_t gstream[kMaxGroup] = {};
  cudaEvent_t gfork = nullptr, gjoin[kMaxGroup] = {};
};

// State of the differentiable estimator (adjoint.cu): sampling (_s) and
// evaluation (_e) parameters, per-pixel replay state, gradients.
struct AdjState {
  bool ready = false;
  uint32_t spp = 0, seed = 0, stream = 0, W = 0, H = 0, nmat = 0;
  size_t n_texels = 0;
  uint64_t param_gen = 0, fwd_gen = 0;
  float Z_s = 0.0f, Z_e = 0.0f;
  std::vector<wpbr_material> h_mats;
  DevBuf<wpbr_material> mats_s, mats_e;
  DevBuf<float4> rgb_s, rgb_e;
  DevBuf<float> s_func, s_cdf, s_int, s_mfunc, s_mcdf, s_mint;
  DevBuf<float> e_func, e_cdf, e_int, e_mfunc, e_mcdf, e_mint;
  DevBuf<float> mat_prm, env_prm, target, image, g_env, g_func;
  DevBuf<double> g_mat, g_scalar;
  DevBuf<float4> state, rays, Lb, acc, gpix;
  DevBuf<float2> pf;
  DevBuf<uint32_t> hit_prim, shadow_hit, shadow_map, pass_dev, counters;  // counters: 2 ray fetches, queued shadow rays
  void release() {
    mats_s.release(); mats_e.release(); rgb_s.release(); rgb_e.release();
    s_func.release(); s_cdf.release(); s_int.release(); s_mfunc.release(); s_mcdf.release(); s_mint.release();
    e_func.release(); e_cdf.release(); e_int.release(); e_mfunc.release(); e_mcdf.release(); e_mint.release();
    mat_prm.release(); env_prm.release(); target.release(); image.release(); g_env.release(); g_func.release();
    g_mat.release(); g_scalar.release(); state.release(); rays.release(); Lb.release(); acc.release();
    gpix.release(); pf.release(); hit_prim.release(); shadow_hit.release(); shadow_map.release(); pass_dev.release();
    counters.release();
    ready = false;
  }
};

}  // namespace wpbr

struct wpbr_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  uint32_t quirks = 0;
  uint64_t epoch = 0;  // bumped by every scene upload, BVH build, quirk or traversal change
  uint32_t traversal = 0;  // wpbr_traversal: 0 binary (leaf-split), 2 binary over the reference's leaves
  uint32_t lim_stack = 0, lim_steps = 0;  // wpbr_set_traversal_limits (0: the defaults)
  uint32_t spectrum = 0;   // wpbr_spectrum: 0 RGB, 1 Sampled64
  wpbr::DevBuf<uint32_t> d_err;
  // scene
  bool has_scene = false;
  uint32_t ns = 0, nt = 0, nv = 0, N = 0;
  wpbr::DevBuf<wpbr::Xf> sph_o2w, sph_w2o;
  wpbr::DevBuf<float> sph_r, pos, nrm, tan, uv;
  wpbr::DevBuf<uint32_t> sph_mat, idx, tri_mat, tri_flags;
  bool has_nrm = false, has_uv = false;
  wpbr::DevBuf<wpbr_material> mats;
  uint32_t nmat = 0;
  // MIP-mapped textures (all levels of all textures) and the EWA filter table
  wpbr::DevBuf<float4> tex_texels;
  wpbr::DevBuf<wpbr::TexLevel> tex_levels;
  wpbr::DevBuf<wpbr::TexInfo> tex_info;
  wpbr::DevBuf<float> tex_gauss;
  uint32_t ntex = 0;
  bool has_metal = false;
  wpbr::DevBuf<wpbr_light> lights;
  std::vector<wpbr_light> h_lights;
  bool has_env = false;
  // every light is an environment light: a shadow ray is unoccluded iff it
  // hits nothing, so the fused pass traces shadow rays any-hit
  bool env_lights_only = false;
  int envW = 0, envH = 0;
  wpbr::DevBuf<float4> env_rgb;
  wpbr::DevBuf<float> cond_func, cond_cdf, cond_int, marg_func, marg_cdf, marg_int, env_lum;
  wpbr::Xf env_l2w, env_w2l;
  wpbr::RGB3 env_le{1, 1, 1};
  float env_marg_int = 0.0f;
  wpbr::CameraParams cam{};
  wpbr::BvhState bvh;
  wpbr::RenderState rs;
  wpbr::AdjState adj;
  // staging for the host-buffer collide entry points
  wpbr::DevBuf<float4> io_rays, io_hits;
  wpbr::DevBuf<uint32_t> io_stats;
  // copy streams and events of the chunked host-buffer collide (created on
  // first use): rays of chunk i+1 go up and hits of chunk i-1 come down while
  // chunk i is traced on the context's stream
  cudaStream_t io_h2d = nullptr, io_d2h = nullptr;
  cudaEvent_t io_ev[3] = {nullptr, nullptr, nullptr};
  // wpbr_set_kernel_timing: CUDA events around each collide traversal launch
  static constexpr int kTimedMax = 64;
  bool kernel_timing = false;
  int timed = 0;  // event pairs recorded since the last wpbr_kernel_timing
  cudaEvent_t tev[2 * kTimedMax] = {};
  // per-collide scratch: the persistent traversal's ray-fetch counter and the
  // ray reordering of large batches (keys, permutation, radix scratch). Set 1
  // belongs to io_comp, the second traversal stream of the chunked host
  // collide, so two chunks can be traced at once.
  struct TraceScratch {
    wpbr::DevBuf<uint32_t> counter, k0, v0, k1, v1, hist, scan;
    void release() {
      counter.release(); k0.release(); v0.release(); k1.release(); v1.release(); hist.release(); scan.release();
    }
  };
  TraceScratch tscr[2];
  cudaStream_t io_comp = nullptr;
  uint32_t ray_sort = 8;  // bits per axis of the origin grid (0: input order)
};

namespace wpbr {
// The BVH view the traversal kernels receive: the child-pair records of the
// reference's leaves as they are for WPBR_TRAVERSAL_BINARY_FULL_LEAVES, else
// the leaf-split child-pair layout.
inline BvhView traversal_view(const wpbr_ctx* ctx) {
  BvhView v = ctx->bvh.view;
  if (ctx->traversal == WPBR_TRAVERSAL_BINARY_FULL_LEAVES) v = reference_leaves_view(v);
  if (ctx->lim_stack) v.stack_cap = ctx->lim_stack;
  if (ctx->lim_steps) v.step_cap = ctx->lim_steps;
  return v;
}
// The view of the render passes' traversals (camera and shadow rays of the
// fused, staged, Sampled64 and differentiable passes): the reference's leaves
// as they are. The leaf split speeds up collide batches (8.4M-ray closest hit
// 4.27 -> 4.19 ms) but slows the passes' traversals, whose warps mostly share
// leaves (1080p x 64 spp full frame: 1,261 Msamples/s over the reference's
// leaves, 1,250 with split camera rays, 1,228 with split shadow rays, 1,214
// with both). A batch's arena keeps only the split layout, which its passes
// then traverse (32 scenes: 941 against 930 Msamples/s unsplit).
inline BvhView render_traversal_view(const wpbr_ctx* ctx) { return reference_leaves_view(traversal_view(ctx)); }
wpbr_status set_err(wpbr_ctx* ctx, wpbr_status st, const std::string& msg);
wpbr_status cuda_err(wpbr_ctx* ctx, cudaError_t e, const char* what);
SceneView scene_view(const wpbr_ctx* ctx);
wpbr_status bvh_build(wpbr_ctx* ctx);
// Keys per block of the radix sort's kernels (its histograms are kept per
// tile of this many keys, digit-major).
constexpr uint32_t kSortTile = 2048;
// first_hist: the first pass's tile histograms are already in hist (written
// by the kernel that produced the keys); index_values: sort the keys'
// positions (v0 need not be filled).
cudaError_t radix_sort_pairs(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, uint32_t n, int bits,
                             DevBuf<uint32_t>& hist, DevBuf<uint32_t>& scan_tmp, cudaStream_t st, uint32_t** kres,
                             uint32_t** vres, bool first_hist = false, bool index_values = false);
// Traces on `stream` (the context's when null) with scratch set `scratch`.
wpbr_status trace_rays(wpbr_ctx* ctx, const float4* d_rays, uint64_t n, float4* d_hits, uint32_t mode,
                       uint32_t* d_stats, int scratch = 0, cudaStream_t stream = nullptr);
wpbr_status env_preprocess(wpbr_ctx* ctx);
// Distribution2D of an environment image (JobLightInfiniteAreaPreprocessSampling)
// into caller-owned arrays: cond_func/cond_cdf/cond_int of H rows of W, marg_* of H.
struct EnvDist {
  float *cond_func, *cond_cdf, *cond_int, *marg_func, *marg_cdf, *marg_int;
};
wpbr_status env_distribution_build(wpbr_ctx* ctx, const float4* rgb, const EnvDist& out, float* marg_int_host);
wpbr_status render_setup(wpbr_ctx* ctx, uint32_t spp, uint32_t seed, uint32_t stream);
wpbr_status render_pass_fused(wpbr_ctx* ctx, uint32_t pass);
wpbr_status render_pass_launch(wpbr_ctx* ctx);
wpbr_status render_frame(wpbr_ctx* ctx);
wpbr_status spectral_setup(wpbr_ctx* ctx);
// Sampled64 pieces of render_pass_launch: the scalar spawn (replaces the
// RGB spawn) and the per-bin finish + film (replace the RGB finish + film).
// `order`: the material-sorted pixel order (null: film order).
// Sample slots: a Sampled64 frame writes `slots` passes' film positions and
// spectra side by side and gathers them into the film at once.
cudaError_t spectral_slots(wpbr_ctx* ctx, uint32_t slots);
cudaError_t spectral_spawn_launch(wpbr_ctx* ctx, const uint32_t* pass_ptr, const uint32_t* order, uint32_t slot);
cudaError_t spectral_finish_launch(wpbr_ctx* ctx, const uint32_t* order, uint32_t slot, uint32_t film_slots);
wpbr_status spectral_resolve(wpbr_ctx* ctx);
// float4 per pixel of the fused pass's state buffer (RenderState::pstate);
// the RGB and the Sampled64 spawn records both fit in it.
constexpr int kPassStateF4 = 7;
uint32_t persistent_full_grid();
void bvh_release(wpbr_ctx* ctx, bool keep_traversal);
wpbr_status job_run(wpbr_ctx* ctx, uint32_t job, uint32_t pass);
wpbr_status job_record(wpbr_ctx* ctx, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1, wpbr_pass_record* rec);
wpbr_status film_tonemap(wpbr_ctx* ctx, uint8_t* out);
wpbr_status adjoint_setup(wpbr_ctx* ctx, uint32_t spp, uint32_t seed, uint32_t stream);
wpbr_status adjoint_get_params(wpbr_ctx* ctx, float* mat, float* env);
wpbr_status adjoint_set_params(wpbr_ctx* ctx, const float* mat, const float* env, bool device);
wpbr_status adjoint_freeze(wpbr_ctx* ctx);
wpbr_status adjoint_forward(wpbr_ctx* ctx, const float* target, float* image, double* loss, bool device);
wpbr_status adjoint_backward(wpbr_ctx* ctx, float* grad_mat, float* grad_env, bool device);
// scan helper (exclusive, in place allowed): out[i] = sum in[0..i); returns total in *total_dev (device, may be null)
cudaError_t scan_exclusive(const uint32_t* in, uint32_t* out, uint32_t n, DevBuf<uint32_t>& tmp, cudaStream_t s);
uint32_t scan_launches(uint32_t n);
uint32_t radix_sort_launches(uint32_t n, int bits);
uint32_t trace_launches(const wpbr_ctx* ctx, uint64_t n, bool stats);
wpbr_status ray_order_debug(wpbr_ctx* ctx, const float* rays, uint64_t n, uint32_t* keys, uint32_t* perm);
}  // namespace wpbr

#define WPBR_CUDA(call)                                          \
  do {                                                           \
    cudaError_t e_ = (call);                                     \
    if (e_ != cudaSuccess) return wpbr::cuda_err(ctx, e_, #call); \
  } while (0)
