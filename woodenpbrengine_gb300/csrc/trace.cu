// trace.cu — the collision kernel behind wpbr_collide (runCollisionSystem,
// WoodenPBREngine/MEngine.cpp:352-361) over a caller-supplied ray batch.
#include "common.cuh"
#include "ctx.hpp"
#include "traverse.cuh"
#include "traverse_persistent.cuh"

namespace wpbr {

namespace {

constexpr uint64_t kRaySortMin = 1u << 18;  // batches below this are traced in input order

template <bool ANY, bool STATS, int STACK>
__global__ void __launch_bounds__(128) k_trace(SceneView S, BvhView Bv, const float4* __restrict__ rays, uint64_t n,
                                               float4* __restrict__ hits, uint32_t* __restrict__ stats,
                                               uint32_t* err) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 ro = __ldg(&rays[2 * i]);
  float4 rd = __ldg(&rays[2 * i + 1]);
  uint32_t nv = 0, np = 0;
  HitRec h = trace_ray<ANY, STACK>(S, Bv, V3{ro.x, ro.y, ro.z}, V3{rd.x, rd.y, rd.z}, rd.w, STATS ? &nv : nullptr,
                                   STATS ? &np : nullptr, err);
  hits[i] = make_float4(h.t, __uint_as_float(h.prim), h.b1, h.b2);
  if (STATS) {
    stats[2 * i] = nv;
    stats[2 * i + 1] = np;
  }
}

// Sort key of a ray: Morton code of its origin on a 2^b grid per axis over
// the scene bounds (clamped), 3b bits; the index is the payload.
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
  v &= 0x3FFu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}
// One block per kSortTile rays: the keys, and the tile's histogram of the
// sort's first digit (the low 8 bits), in the layout of the sort's own
// histogram kernel (digit-major, tile-minor), which the sort then skips. A
// thread loads its rays' origins before it counts any (its loads in flight
// together); a warp whose 32 keys share the digit adds them with one atomic.
// The sort's first pass makes the indices itself.
constexpr int kKeyBlock = 256;
constexpr int kKeyItems = (int)kSortTile / kKeyBlock;
__global__ void __launch_bounds__(kKeyBlock) k_ray_keys(const float4* rays, uint32_t n, float3 lo, float3 scale,
                                                        uint32_t cells, uint32_t* keys, uint32_t* hist,
                                                        uint32_t ntiles) {
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  const float top = (float)(cells - 1);
  const uint32_t base = blockIdx.x * kSortTile;
  float4 o[kKeyItems];
#pragma unroll
  for (int k = 0; k < kKeyItems; ++k) {
    const uint32_t i = base + k * kKeyBlock + threadIdx.x;
    o[k] = i < n ? __ldg(&rays[2 * (size_t)i]) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kKeyItems; ++k) {
    const uint32_t i = base + k * kKeyBlock + threadIdx.x;
    uint32_t d = 0xFFFFFFFFu;
    if (i < n) {
      float q[3] = {(o[k].x - lo.x) * scale.x, (o[k].y - lo.y) * scale.y, (o[k].z - lo.z) * scale.z};
      uint32_t c[3];
      for (int a = 0; a < 3; ++a) c[a] = q[a] > 0.0f ? (q[a] < top ? (uint32_t)q[a] : cells - 1) : 0u;
      const uint32_t key = spread10(c[0]) | (spread10(c[1]) << 1) | (spread10(c[2]) << 2);
      keys[i] = key;
      d = key & 0xFFu;
    }
    if (__all_sync(0xFFFFFFFFu, d == __shfl_sync(0xFFFFFFFFu, d, 0) && d != 0xFFFFFFFFu)) {
      if ((threadIdx.x & 31u) == 0) atomicAdd(&cnt[d], 32u);
    } else if (d != 0xFFFFFFFFu) {
      atomicAdd(&cnt[d], 1u);
    }
  }
  __syncthreads();
  hist[threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

// The ray order of a batch: keys with the first digit's tile histograms,
// then the rest of the stable LSD sort of the ray indices; *perm receives
// sorted position -> input index. keys_host, when given, receives the keys
// in input order (a testing aid).
cudaError_t ray_order(wpbr_ctx* ctx, wpbr_ctx::TraceScratch& X, const BvhView& Bv, const float4* d_rays, uint32_t n,
                      cudaStream_t st, const uint32_t** perm, uint32_t* keys_host) {
  cudaError_t e = cudaSuccess;
  for (DevBuf<uint32_t>* b : {&X.k0, &X.v0, &X.k1, &X.v1})
    if (e == cudaSuccess) e = b->ensure(n);
  if (e != cudaSuccess) return e;
  const float3 lo = make_float3(Bv.root_lo[0], Bv.root_lo[1], Bv.root_lo[2]);
  const float ex[3] = {Bv.root_hi[0] - Bv.root_lo[0], Bv.root_hi[1] - Bv.root_lo[1], Bv.root_hi[2] - Bv.root_lo[2]};
  const uint32_t b = ctx->ray_sort;  // bits per axis
  const int key_bits = 3 * (int)b;
  const float cells = (float)(1u << b);
  const float3 sc = make_float3(ex[0] > 0.0f ? cells / ex[0] : 0.0f, ex[1] > 0.0f ? cells / ex[1] : 0.0f,
                                ex[2] > 0.0f ? cells / ex[2] : 0.0f);
  const uint32_t ntiles = div_up(n, kSortTile);
  e = X.hist.ensure((size_t)256 * ntiles);
  if (e != cudaSuccess) return e;
  k_ray_keys<<<ntiles, kKeyBlock, 0, st>>>(d_rays, n, lo, sc, 1u << b, X.k0.p, X.hist.p, ntiles);
  if (keys_host) e = cudaMemcpyAsync(keys_host, X.k0.p, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  uint32_t *kr = nullptr, *vr = nullptr;
  if (e == cudaSuccess)
    e = radix_sort_pairs(X.k0.p, X.v0.p, X.k1.p, X.v1.p, n, key_bits, X.hist, X.scan, st, &kr, &vr, true, true);
  *perm = vr;
  return e;
}

template <bool ANY, bool STATS>
cudaError_t launch(const SceneView& S, const BvhView& Bv, const float4* rays, uint64_t n, float4* hits,
                   uint32_t* stats, uint32_t* err, cudaStream_t st) {
  unsigned blocks = div_up(n, 128);
  if (Bv.max_depth < 60)
    k_trace<ANY, STATS, 64><<<blocks, 128, 0, st>>>(S, Bv, rays, n, hits, stats, err);
  else
    k_trace<ANY, STATS, 256><<<blocks, 128, 0, st>>>(S, Bv, rays, n, hits, stats, err);
  return cudaGetLastError();
}

}  // namespace

// Kernel launches of one trace_rays call (the memset of the work counter is
// not a kernel): the traversal, plus the key kernel and the radix sort of
// the ray order for large batches.
uint32_t trace_launches(const wpbr_ctx* ctx, uint64_t n, bool stats) {
  if (n == 0) return 0;
  if (stats) return 1;
  const BvhView Bv = traversal_view(ctx);
  // the key kernel also counts the sort's first digit, so the sort skips one histogram launch
  if (ctx->ray_sort && n >= kRaySortMin && !Bv.empty) return 1 + radix_sort_launches((uint32_t)n, 3 * (int)ctx->ray_sort);
  return 1;
}

wpbr_status trace_rays(wpbr_ctx* ctx, const float4* d_rays, uint64_t n, float4* d_hits, uint32_t mode,
                       uint32_t* d_stats, int scratch, cudaStream_t stream) {
  cudaStream_t st = stream ? stream : ctx->stream;
  wpbr_ctx::TraceScratch& X = ctx->tscr[scratch];
  if (!ctx->bvh.built) return set_err(ctx, WPBR_ERR_NOT_BUILT, "collide: BVH not built");
  if (ctx->bvh.view.max_depth >= 250) return set_err(ctx, WPBR_ERR_TRAVERSAL_LIMIT, "collide: BVH deeper than 250");
  if (n == 0) return WPBR_OK;
  SceneView S = scene_view(ctx);
  const BvhView Bv = traversal_view(ctx);
  cudaError_t e;
  if (d_stats) {
    // statistics count the box and primitive tests over the reference's leaves
    const BvhView Br = reference_leaves_view(Bv);
    e = (mode == WPBR_TRACE_ANY) ? launch<true, true>(S, Br, d_rays, n, d_hits, d_stats, ctx->d_err.p, st)
                                 : launch<false, true>(S, Br, d_rays, n, d_hits, d_stats, ctx->d_err.p, st);
  } else {
    if (n >= 0xFFFFFFFFull) return set_err(ctx, WPBR_ERR_INVALID_ARG, "collide: more than 2^32-1 rays per call");
    // large batches are traced in the order of their origins' Morton cells:
    // neighbouring rays of a warp then share nodes (hits are per ray, so the
    // order does not change them)
    const bool sorted = ctx->ray_sort && n >= kRaySortMin && !Bv.empty;
    e = X.counter.ensure(1);
    if (e == cudaSuccess) {
      uint32_t* c = X.counter.p;
      e = cudaMemsetAsync(c, 0, sizeof(uint32_t), st);
      const uint32_t* perm = nullptr;
      if (e == cudaSuccess && sorted) e = ray_order(ctx, X, Bv, d_rays, (uint32_t)n, st, &perm, nullptr);
      // optional CUDA events around the traversal launch (wpbr_set_kernel_timing)
      int slot = -1;
      if (e == cudaSuccess && ctx->kernel_timing && ctx->timed < wpbr_ctx::kTimedMax) {
        slot = ctx->timed;
        for (int k = 0; k < 2 && e == cudaSuccess; ++k)
          if (!ctx->tev[2 * slot + k]) e = cudaEventCreate(&ctx->tev[2 * slot + k]);
        if (e == cudaSuccess) e = cudaEventRecord(ctx->tev[2 * slot], st);
      }
      if (e == cudaSuccess) {
        if (perm) {
          PermSrc src{d_rays, perm};
          PermHitSink4 sink{d_hits, perm};
          if (mode == WPBR_TRACE_ANY)
            launch_traversal<true>(S, Bv, src, sink, (uint32_t)n, c, ctx->d_err.p, st);
          else
            launch_traversal<false>(S, Bv, src, sink, (uint32_t)n, c, ctx->d_err.p, st);
        } else {
          BufferSrc src{d_rays};
          HitSink4 sink{d_hits};
          if (mode == WPBR_TRACE_ANY)
            launch_traversal<true>(S, Bv, src, sink, (uint32_t)n, c, ctx->d_err.p, st);
          else
            launch_traversal<false>(S, Bv, src, sink, (uint32_t)n, c, ctx->d_err.p, st);
        }
        e = cudaGetLastError();
      }
      if (e == cudaSuccess && slot >= 0) {
        e = cudaEventRecord(ctx->tev[2 * slot + 1], st);
        if (e == cudaSuccess) ctx->timed = slot + 1;
      }
    }
  }
  if (e != cudaSuccess) return cuda_err(ctx, e, "collide kernel");
  return WPBR_OK;
}

wpbr_status ray_order_debug(wpbr_ctx* ctx, const float* rays, uint64_t n, uint32_t* keys, uint32_t* perm) {
  if (!ctx->bvh.built) return set_err(ctx, WPBR_ERR_NOT_BUILT, "ray order: BVH not built");
  if (n == 0) return WPBR_OK;
  const BvhView Bv = traversal_view(ctx);
  if (!ctx->ray_sort || Bv.empty || n >= 0xFFFFFFFFull)
    return set_err(ctx, WPBR_ERR_INVALID_ARG, "ray order: sorting off, empty scene or 2^32-1 rays and more");
  cudaStream_t st = ctx->stream;
  wpbr_ctx::TraceScratch& X = ctx->tscr[0];
  DevBuf<float4> d_rays;
  cudaError_t e = d_rays.ensure(2 * n);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_rays.p, rays, n * 32, cudaMemcpyHostToDevice, st);
  const uint32_t* d_perm = nullptr;
  if (e == cudaSuccess) e = ray_order(ctx, X, Bv, d_rays.p, (uint32_t)n, st, &d_perm, keys);
  if (e == cudaSuccess) e = cudaMemcpyAsync(perm, d_perm, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  d_rays.release();
  if (e != cudaSuccess) return cuda_err(ctx, e, "ray order");
  return WPBR_OK;
}

}  // namespace wpbr
