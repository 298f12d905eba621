// trace.cu — the collision kernel behind wpbr_collide (runCollisionSystem,
// WoodenPBREngine/MEngine.cpp:352-361) over a caller-supplied ray batch.
#include "common.cuh"
#include "ctx.hpp"
#include "traverse.cuh"
#include "traverse_persistent.cuh"

namespace wpbr {

namespace {

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

wpbr_status trace_rays(wpbr_ctx* ctx, const float4* d_rays, uint64_t n, float4* d_hits, uint32_t mode,
                       uint32_t* d_stats) {
  if (!ctx->bvh.built) return set_err(ctx, WPBR_ERR_NOT_BUILT, "collide: BVH not built");
  if (ctx->bvh.view.max_depth >= 250) return set_err(ctx, WPBR_ERR_TRAVERSAL_LIMIT, "collide: BVH deeper than 250");
  if (n == 0) return WPBR_OK;
  SceneView S = scene_view(ctx);
  const BvhView Bv = traversal_view(ctx);
  cudaError_t e;
  if (d_stats) {
    e = (mode == WPBR_TRACE_ANY) ? launch<true, true>(S, Bv, d_rays, n, d_hits, d_stats, ctx->d_err.p, ctx->stream)
                                 : launch<false, true>(S, Bv, d_rays, n, d_hits, d_stats, ctx->d_err.p, ctx->stream);
  } else {
    if (n >= 0xFFFFFFFFull) return set_err(ctx, WPBR_ERR_INVALID_ARG, "collide: more than 2^32-1 rays per call");
    e = ctx->trace_counter.ensure(4);
    if (e == cudaSuccess) {
      uint32_t* c = ctx->trace_counter.p;
      e = cudaMemsetAsync(c, 0, sizeof(uint32_t), ctx->stream);
      if (e == cudaSuccess) {
        BufferSrc src{d_rays};
        HitSink4 sink{d_hits};
        if (mode == WPBR_TRACE_ANY)
          launch_traversal<true>(S, Bv, src, sink, (uint32_t)n, c, ctx->d_err.p, ctx->stream);
        else
          launch_traversal<false>(S, Bv, src, sink, (uint32_t)n, c, ctx->d_err.p, ctx->stream);
        e = cudaGetLastError();
      }
    }
  }
  if (e != cudaSuccess) return cuda_err(ctx, e, "collide kernel");
  return WPBR_OK;
}

}  // namespace wpbr
