// traverse.cuh — closest-hit / any-hit traversal of the flattened
// CSceneTreeLBVH in its child-pair layout.
//
// Result equals JobProcessRayCasts + the per-shape interaction jobs +
// JobProcessRayCastsResults (WoodenPBREngine/SLBVH.cpp:9-162): the closest
// non-zero t over all candidate primitives, the first candidate in near-first
// order winning ties. Children are visited in the reference's order (the
// child on the ray's negative side of the parent's split axis first, via
// dirIsNeg[axis]); primitives of a leaf in sorted order. Unlike the reference
// the traversal prunes boxes whose entry distance exceeds the current best t
// by more than 2^-10 relative: no primitive inside such a box can undercut the
// best hit, and a later candidate with an equal t never replaces an earlier
// one, so the hit is unchanged. In the leaf-split layout a large leaf is a
// small tree over ranges of its sorted positions, visited lowest range first:
// its primitives are still tested in sorted order, the boxes of the ranges
// only let a ray skip primitives whose box it misses.
#pragma once

#include "common.cuh"
#include "intersect.cuh"
#include "views.cuh"

namespace wpbr {

constexpr float kPruneScale = 1.0f + 0x1p-10f;

struct HitRec {
  float t;
  uint32_t prim;
  float b1, b2;
};

// Order of a child-pair record's two children: axis 0-2 visits the child on
// the ray's negative side of that split axis first (dirIsNeg[axis],
// SLBVH.cpp:133-145); axis code 3 (the records splitting one large leaf)
// visits child 0, the lower sorted positions, first.
__device__ __forceinline__ bool second_child_first(const int neg[3], uint32_t axis) {
  return axis == 0 ? neg[0] != 0 : (axis == 1 ? neg[1] != 0 : (axis == 2 ? neg[2] != 0 : false));
}

__device__ __forceinline__ float prim_test(const SceneView& S, const float4* prims, uint32_t pos, V3 o, V3 d,
                                           const RayTri& R, uint32_t* prim_out, float* b1, float* b2) {
  const float4* r = prims + (size_t)pos * 3;
  float4 r0 = __ldg(r), r1 = __ldg(r + 1);
  *prim_out = __float_as_uint(r0.w);
  if (__float_as_uint(r1.w) == 1u) {
    uint32_t s = __float_as_uint(r1.x);
    V3 rlo, rld, ph;
    float t = sphere_intersect(S.sph_w2o[s], S.sph_r[s], o, d, &rlo, &rld, &ph);
    *b1 = 0.0f;
    *b2 = 0.0f;
    return t;
  }
  float4 r2 = __ldg(r + 2);
  float c0, c1, c2;
  float t = tri_intersect_pre(V3{r0.x, r0.y, r0.z}, V3{r1.x, r1.y, r1.z}, V3{r2.x, r2.y, r2.z}, R, &c0, &c1, &c2);
  *b1 = c1;
  *b2 = c2;
  return t;
}

template <bool ANY, int STACK>
__device__ HitRec trace_ray(const SceneView& S, const BvhView& Bv, V3 o, V3 d, float tmax, uint32_t* nvisit,
                            uint32_t* ntest, uint32_t* err) {
  HitRec h{inf_(), kNoHit, 0.0f, 0.0f};
  uint32_t nv = 0, np = 0;
  if (Bv.empty) return h;
  V3 inv{1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
  int neg[3] = {inv.x < 0.0f, inv.y < 0.0f, inv.z < 0.0f};
  const RayTri R = ray_tri_setup(o, d, S.quirks);
  float te;
  ++nv;
  if (!slab_test(V3{Bv.root_lo[0], Bv.root_lo[1], Bv.root_lo[2]}, V3{Bv.root_hi[0], Bv.root_hi[1], Bv.root_hi[2]}, o,
                 inv, neg, tmax, &te)) {
    if (nvisit) *nvisit = nv;
    if (ntest) *ntest = np;
    return h;
  }
  int st_ref[STACK];
  uint32_t st_cnt[STACK];
  float st_t[STACK];
  int sp = 0;
  int ref = Bv.root_ref;
  uint32_t cnt = Bv.root_count;
  float tb = inf_();
  uint32_t iters = 0;
  while (true) {
    bool go = false;
    if (++iters > Bv.step_cap) {  // a well-formed tree never gets here
      atomicOr(err, kErrLoopLimit);
      break;
    }
    if (ref >= 0) {
      if ((uint32_t)ref >= Bv.n_int) {
        atomicOr(err, kErrBuild);
        break;
      }
      const Node2* np_ = Bv.nodes + ref;
      float4 b0 = __ldg(&np_->b0), b1 = __ldg(&np_->b1), bz = __ldg(&np_->bz);
      int4 m = __ldg(&np_->meta);
      nv += 2;
      float t0, t1;
      bool h0 = slab_test(V3{b0.x, b0.z, bz.x}, V3{b0.y, b0.w, bz.y}, o, inv, neg, tmax, &t0) && !(t0 > tb * kPruneScale);
      bool h1 = slab_test(V3{b1.x, b1.z, bz.z}, V3{b1.y, b1.w, bz.w}, o, inv, neg, tmax, &t1) && !(t1 > tb * kPruneScale);
      uint32_t axis = ((uint32_t)m.w) >> 30;
      uint32_t c0n = (uint32_t)m.z, c1n = ((uint32_t)m.w) & 0x3FFFFFFFu;
      if (h0 && h1) {
        bool first1 = second_child_first(neg, axis);
        if (sp >= STACK || (uint32_t)sp >= Bv.stack_cap) {
          atomicOr(err, kErrStackOverflow);
          break;
        }
        st_ref[sp] = first1 ? m.x : m.y;
        st_cnt[sp] = first1 ? c0n : c1n;
        st_t[sp] = first1 ? t0 : t1;
        ++sp;
        ref = first1 ? m.y : m.x;
        cnt = first1 ? c1n : c0n;
        go = true;
      } else if (h0) {
        ref = m.x;
        cnt = c0n;
        go = true;
      } else if (h1) {
        ref = m.y;
        cnt = c1n;
        go = true;
      }
    } else {
      uint32_t first = (uint32_t)(~ref);
      if (first >= Bv.n_prims || cnt > Bv.n_prims - first) {
        atomicOr(err, kErrBuild);
        break;
      }
      for (uint32_t k = 0; k < cnt; ++k) {
        uint32_t prim;
        float b1, b2;
        ++np;
        float t = prim_test(S, Bv.prims, first + k, o, d, R, &prim, &b1, &b2);
        if (t == 0.0f || !(t < tmax)) continue;
        if (tb > t) {
          tb = t;
          h.t = t;
          h.prim = prim;
          h.b1 = b1;
          h.b2 = b2;
          if (ANY) break;
        }
      }
      if (ANY && h.prim != kNoHit) break;
    }
    if (go) continue;
    bool found = false;
    while (sp > 0) {
      --sp;
      if (!(st_t[sp] > tb * kPruneScale)) {
        ref = st_ref[sp];
        cnt = st_cnt[sp];
        found = true;
        break;
      }
    }
    if (!found) break;
  }
  if (nvisit) *nvisit = nv;
  if (ntest) *ntest = np;
  return h;
}

}  // namespace wpbr
