// traverse_persistent.cuh — persistent while-while traversal kernel
// (Aila & Laine, "Understanding the Efficiency of Ray Traversal on GPUs",
// HPG 2009, with speculative traversal and dynamic ray fetching).
//
// Each warp keeps its 32 lanes busy: lanes whose ray finished take new ray
// indices from a global counter (one atomic per warp, __ballot_sync
// compaction of the idle lanes). Traversal alternates an interior-node loop
// and a leaf loop; a lane that reaches a leaf postpones it and keeps
// descending until every lane of the warp holds a leaf, then all lanes test
// primitives together. Leaves are still tested in depth-first near-first
// order, and a postponed leaf only delays the update of the best t, which
// makes pruning more conservative — the hit is the one trace_ray returns.
#pragma once

#include "common.cuh"
#include "traverse.cuh"

namespace wpbr {

constexpr int kEnd = (int)0x80000000;  // no node (empty stack)
constexpr int kPersistBlock = 128;

template <bool ANY, int STACK, class Src, class Sink>
__global__ void __launch_bounds__(kPersistBlock) k_trace_persistent(SceneView S, BvhView Bv, Src src, Sink sink,
                                                                    uint32_t n, uint32_t* counter, uint32_t* err) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t lt_mask = (1u << lane) - 1u;
  V3 o{0, 0, 0}, d{0, 0, 0}, inv{0, 0, 0};
  int neg[3] = {0, 0, 0};
  RayTri R{};
  float tmax = 0.0f, tb = 0.0f;
  HitRec h{0.0f, kNoHit, 0.0f, 0.0f};
  int ref = kEnd;
  uint32_t cnt = 0;
  int lref = kEnd;
  uint32_t lcnt = 0;
  int sp = 0;
  int st_ref[STACK];
  uint32_t st_cnt[STACK];
  float st_t[STACK];
  uint32_t rid = 0;
  bool active = false;
  bool exhausted = false;
  uint32_t guard = 0;

  while (true) {
    // ---- refill idle lanes ------------------------------------------------
    __syncwarp();
    uint32_t idle = __ballot_sync(0xFFFFFFFFu, !active && !exhausted);
    if (idle) {
      uint32_t leader = __ffs(idle) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(idle));
      base = __shfl_sync(0xFFFFFFFFu, base, leader);
      if (!active && !exhausted) {
        uint32_t r = base + __popc(idle & lt_mask);
        if (r >= n) {
          exhausted = true;
        } else {
          rid = r;
          float4 ro, rd;
          src.load(r, &ro, &rd);
          o = V3{ro.x, ro.y, ro.z};
          d = V3{rd.x, rd.y, rd.z};
          tmax = rd.w;
          inv = V3{1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
          neg[0] = inv.x < 0.0f;
          neg[1] = inv.y < 0.0f;
          neg[2] = inv.z < 0.0f;
          R = ray_tri_setup(o, d, S.quirks);
          tb = inf_();
          h = HitRec{inf_(), kNoHit, 0.0f, 0.0f};
          sp = 0;
          lref = kEnd;
          ref = kEnd;
          float te;
          if (!Bv.empty &&
              slab_test(V3{Bv.root_lo[0], Bv.root_lo[1], Bv.root_lo[2]},
                        V3{Bv.root_hi[0], Bv.root_hi[1], Bv.root_hi[2]}, o, inv, neg, tmax, &te)) {
            ref = Bv.root_ref;
            cnt = Bv.root_count;
          }
          active = true;
        }
      }
    }
    if (__all_sync(0xFFFFFFFFu, !active && exhausted)) break;
    if (++guard > (1u << 26)) {
      if (lane == 0) atomicOr(err, kErrLoopLimit);
      break;
    }

    if (active) {
      // ---- interior loop (speculative) --------------------------------------
      while (ref >= 0) {
        if ((uint32_t)ref >= Bv.n_int) {
          atomicOr(err, kErrBuild);
          ref = kEnd;
          break;
        }
        const Node2* np_ = Bv.nodes + ref;
        float4 b0 = __ldg(&np_->b0), b1 = __ldg(&np_->b1), bz = __ldg(&np_->bz);
        int4 m = __ldg(&np_->meta);
        float t0, t1;
        bool h0 = slab_test(V3{b0.x, b0.z, bz.x}, V3{b0.y, b0.w, bz.y}, o, inv, neg, tmax, &t0) &&
                  !(t0 > tb * kPruneScale);
        bool h1 = slab_test(V3{b1.x, b1.z, bz.z}, V3{b1.y, b1.w, bz.w}, o, inv, neg, tmax, &t1) &&
                  !(t1 > tb * kPruneScale);
        uint32_t axis = ((uint32_t)m.w) >> 30;
        uint32_t c0n = (uint32_t)m.z, c1n = ((uint32_t)m.w) & 0x3FFFFFFFu;
        if (h0 && h1) {
          bool first1 = neg[axis] != 0;
          if (sp >= STACK) {
            atomicOr(err, kErrStackOverflow);
            ref = kEnd;
            break;
          }
          st_ref[sp] = first1 ? m.x : m.y;
          st_cnt[sp] = first1 ? c0n : c1n;
          st_t[sp] = first1 ? t0 : t1;
          ++sp;
          ref = first1 ? m.y : m.x;
          cnt = first1 ? c1n : c0n;
        } else if (h0) {
          ref = m.x;
          cnt = c0n;
        } else if (h1) {
          ref = m.y;
          cnt = c1n;
        } else {
          ref = kEnd;
          while (sp > 0) {
            --sp;
            if (!(st_t[sp] > tb * kPruneScale)) {
              ref = st_ref[sp];
              cnt = st_cnt[sp];
              break;
            }
          }
        }
        // postpone the first leaf found, keep descending for the next one
        if (ref < 0 && ref != kEnd && lref == kEnd) {
          lref = ref;
          lcnt = cnt;
          ref = kEnd;
          while (sp > 0) {
            --sp;
            if (!(st_t[sp] > tb * kPruneScale)) {
              ref = st_ref[sp];
              cnt = st_cnt[sp];
              break;
            }
          }
        }
        if (!__any_sync(__activemask(), lref == kEnd)) break;
      }
      // the current node may itself be a leaf reached without postponing
      if (lref == kEnd && ref < 0 && ref != kEnd) {
        lref = ref;
        lcnt = cnt;
        ref = kEnd;
        while (sp > 0) {
          --sp;
          if (!(st_t[sp] > tb * kPruneScale)) {
            ref = st_ref[sp];
            cnt = st_cnt[sp];
            break;
          }
        }
      }
      // ---- leaf loop ---------------------------------------------------------
      bool done_any = false;
      while (lref != kEnd) {
        uint32_t first = (uint32_t)(~lref);
        if (first >= Bv.n_prims || lcnt > Bv.n_prims - first) {
          atomicOr(err, kErrBuild);
          lref = kEnd;
          ref = kEnd;
          break;
        }
        for (uint32_t k = 0; k < lcnt; ++k) {
          uint32_t prim;
          float b1, b2;
          float t = prim_test(S, Bv.prims, first + k, o, d, R, &prim, &b1, &b2);
          if (t == 0.0f || !(t < tmax)) continue;
          if (tb > t) {
            tb = t;
            h = HitRec{t, prim, b1, b2};
            if (ANY) {
              done_any = true;
              break;
            }
          }
        }
        if (done_any) {
          lref = kEnd;
          ref = kEnd;
          break;
        }
        lref = kEnd;
        if (ref < 0 && ref != kEnd) {  // next node is a leaf too: test it now
          lref = ref;
          lcnt = cnt;
          ref = kEnd;
          while (sp > 0) {
            --sp;
            if (!(st_t[sp] > tb * kPruneScale)) {
              ref = st_ref[sp];
              cnt = st_cnt[sp];
              break;
            }
          }
        }
      }
      if (ref == kEnd && lref == kEnd) {
        sink.store(rid, h);
        active = false;
      }
    }
  }
}

// ---- ray sources and hit sinks -------------------------------------------------
struct BufferSrc {
  const float4* rays;  // 2 float4 per ray: (o, unused), (d, tmax)
  __device__ __forceinline__ void load(uint32_t i, float4* o, float4* d) const {
    *o = __ldg(&rays[2 * (size_t)i]);
    *d = __ldg(&rays[2 * (size_t)i + 1]);
  }
};
struct HitSink4 {
  float4* hits;
  __device__ __forceinline__ void store(uint32_t i, const HitRec& h) const {
    hits[i] = make_float4(h.t, __uint_as_float(h.prim), h.b1, h.b2);
  }
};
struct PrimSink {
  uint32_t* prims;
  __device__ __forceinline__ void store(uint32_t i, const HitRec& h) const { prims[i] = h.prim; }
};

}  // namespace wpbr
