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
// A warp fetches new rays once at least this many of its lanes are idle (or
// none is busy): a refill costs the whole warp a detour, so batching them
// pays. 8.4M-ray microbenchmark, closest hit: 1 lane 4.77 ms, 8 4.66, 16
// 4.39, 20 4.35, 24 4.35, 28 4.42, 32 4.88; with the shared-memory stack
// entries (closest-hit step): 18 4.139, 20 4.128, 22 4.136 ms.
#ifndef WPBR_REFILL_MIN
#define WPBR_REFILL_MIN 20
#endif
// Resident blocks per SM each traversal instantiation is compiled for
// (Sink::kMinBlocks): 8 (64 registers, next to no spilling) for the collide
// kernels, whose lowest 8 stack entries live in shared memory, and for the
// render passes' kernels (camera rays generated in the source, prim-id
// sinks), where 10 cost 5%. With the whole stack in local memory the collide
// kernels had run best at 12 blocks (40 registers, registers and stack
// entries spilled to local memory, 2.1 M-ray launch: 63 M local loads).

// Ray data the warp's lanes read when they test primitives for another lane:
// a triangle test reads the first two float4s (two 16-byte shared loads), a
// sphere test also the direction, and takes the world origin back from the
// permuted one (the permutation only moves components, so it is exact).
struct __align__(16) SharedRay {
  float4 s;   // sx, sy, sz of the triangle test's shear; w: the ray's tmax
  float4 po;  // origin permuted to (kx, ky, kz); w: kx | ky << 2 | kz << 4 | miss_all << 6
  float4 d;   // world direction (sphere tests)
};

__device__ __forceinline__ RayTri unpack_ray_tri(float4 s, float4 po) {
  uint32_t kp = __float_as_uint(po.w);
  RayTri R;
  R.kx = (int)(kp & 3u);
  R.ky = (int)((kp >> 2) & 3u);
  R.kz = (int)((kp >> 4) & 3u);
  R.miss_all = (kp >> 6) & 1u;
  R.sx = s.x;
  R.sy = s.y;
  R.sz = s.z;
  R.ox = po.x;
  R.oy = po.y;
  R.oz = po.z;
  return R;
}

// prim_test for another lane's ray: the world origin and direction are read
// on the sphere branch only.
__device__ __forceinline__ float prim_test_shared(const SceneView& S, const float4* prims, uint32_t pos,
                                                  const SharedRay& sr, const RayTri& R, uint32_t* prim_out,
                                                  float* b1, float* b2) {
  const float4* r = prims + (size_t)pos * 3;
  float4 r0 = __ldg(r), r1 = __ldg(r + 1);
  *prim_out = __float_as_uint(r0.w);
  if (__float_as_uint(r1.w) == 1u) {
    uint32_t s = __float_as_uint(r1.x);
    float4 dd = sr.d;
    // (kx, ky, kz) is a permutation of (0, 1, 2): o[kx] = R.ox, o[ky] = R.oy, o[kz] = R.oz
    V3 o{R.kx == 0 ? R.ox : (R.ky == 0 ? R.oy : R.oz), R.kx == 1 ? R.ox : (R.ky == 1 ? R.oy : R.oz),
         R.kx == 2 ? R.ox : (R.ky == 2 ? R.oy : R.oz)};
    V3 rlo, rld, ph;
    float t = sphere_intersect(S.sph_w2o[s], S.sph_r[s], o, V3{dd.x, dd.y, dd.z}, &rlo, &rld, &ph);
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

// Traversal stack of one lane: the far children pushed on the way down, with
// their leaf counts and entry distances. The collide kernels (Sink::kCollide)
// keep (entry distance, ref) in one 8-byte word, so testing a popped entry
// against the best hit is one local load; the render passes' kernels keep
// separate arrays, which measured faster at their 64 registers.
template <int STACK, bool PACKED>
struct TravStack;
template <int STACK>
struct TravStack<STACK, true> {
  unsigned long long tr[STACK];  // (entry distance bits << 32) | ref
  uint32_t c[STACK];
  __device__ __forceinline__ void put(int i, int ref, uint32_t cnt, float t) {
    tr[i] = ((unsigned long long)__float_as_uint(t) << 32) | (uint32_t)ref;
    c[i] = cnt;
  }
  __device__ __forceinline__ bool take(int i, float limit, int* ref, uint32_t* cnt) const {
    unsigned long long e = tr[i];
    if (__uint_as_float((uint32_t)(e >> 32)) > limit) return false;
    *ref = (int)(uint32_t)e;
    *cnt = c[i];
    return true;
  }
};
template <int STACK>
struct TravStack<STACK, false> {
  int r[STACK];
  uint32_t c[STACK];
  float t[STACK];
  __device__ __forceinline__ void put(int i, int ref, uint32_t cnt, float tt) {
    r[i] = ref;
    c[i] = cnt;
    t[i] = tt;
  }
  __device__ __forceinline__ bool take(int i, float limit, int* ref, uint32_t* cnt) const {
    if (t[i] > limit) return false;
    *ref = r[i];
    *cnt = c[i];
    return true;
  }
};
// The same stack with its lowest KS entries in shared memory (the block's
// entries stored entry-major, so a warp's 32 lanes touch consecutive words)
// and the rest in local memory. The collide kernels keep 8 entries there
// (12 KB per block). 8.4M-ray microbenchmark, closest-hit step / any-hit
// step, ms: all local at 12 blocks 4.307 / 3.963; 8 shared entries at 8
// blocks 4.228 / 3.855, 10 at 8 4.232 / 3.858, 12 at 8 4.258 / 3.871, 14 at 8
// (7 blocks fit) 4.476 / 4.079, none at 8 4.351 / 3.975; 6 or 8 at 9 blocks
// 4.27 / 3.91; 4-8 at 12 blocks 4.56-4.72 (the L1 left is too small), 12 at
// 7 blocks 4.437; hits identical in every case. Again once the far-child
// prefetch was gone and rays and hits streamed: 6 entries 4.151, 8 4.128,
// 10 4.129 ms.
template <int STACK, int KS>
struct TravStackSh {
  unsigned long long* s_tr;  // this lane's column: entry i at s_tr[i * kPersistBlock]
  uint32_t* s_c;
  unsigned long long tr[STACK - KS];
  uint32_t c[STACK - KS];
  __device__ __forceinline__ void put(int i, int ref, uint32_t cnt, float t) {
    const unsigned long long e = ((unsigned long long)__float_as_uint(t) << 32) | (uint32_t)ref;
    if (i < KS) {
      s_tr[i * kPersistBlock] = e;
      s_c[i * kPersistBlock] = cnt;
    } else {
      tr[i - KS] = e;
      c[i - KS] = cnt;
    }
  }
  __device__ __forceinline__ bool take(int i, float limit, int* ref, uint32_t* cnt) const {
    const unsigned long long e = i < KS ? s_tr[i * kPersistBlock] : tr[i - KS];
    if (__uint_as_float((uint32_t)(e >> 32)) > limit) return false;
    *ref = (int)(uint32_t)e;
    *cnt = i < KS ? s_c[i * kPersistBlock] : c[i - KS];
    return true;
  }
};
#ifndef WPBR_SHARED_STACK
#define WPBR_SHARED_STACK 8
#endif
// The render passes' kernels keep their stacks in local memory: 4, 8 or 12
// shared entries changed the 1080p full frame by -0.5, +0.2 and -1.4 %, the
// textured-metal frame by -1.0, -0.9 and -1.3 %.
#ifndef WPBR_SHARED_STACK_RENDER
#define WPBR_SHARED_STACK_RENDER 0
#endif
template <int STACK, bool PACKED, int KS>
struct StackSel {
  using type = TravStackSh<STACK, KS>;
};
template <int STACK, bool PACKED>
struct StackSel<STACK, PACKED, 0> {
  using type = TravStack<STACK, PACKED>;
};
template <int STACK, int KS>
__device__ __forceinline__ void stack_bind(TravStackSh<STACK, KS>& st, unsigned long long* tr, uint32_t* c) {
  st.s_tr = tr;
  st.s_c = c;
}
template <int STACK, bool PACKED>
__device__ __forceinline__ void stack_bind(TravStack<STACK, PACKED>&, unsigned long long*, uint32_t*) {}

// Pops until an entry whose entry distance does not exceed the best hit by
// more than the pruning margin; kEnd when the stack runs out.
template <class Stack>
__device__ __forceinline__ int pop_unpruned(const Stack& st, int& sp, float tb, uint32_t* cnt) {
  int r = kEnd;
  while (sp > 0) {
    --sp;
    if (st.take(sp, tb * kPruneScale, &r, cnt)) return r;
  }
  return kEnd;
}

template <bool ANY, int STACK, class Src, class Sink>
__global__ void __launch_bounds__(kPersistBlock, Sink::kMinBlocks) k_trace_persistent(SceneView S, BvhView Bv,
                                                                                           Src src, Sink sink,
                                                                    uint32_t n, uint32_t* counter, uint32_t* err) {
  __shared__ SharedRay s_ray[kPersistBlock / 32][32];
  __shared__ unsigned long long s_key[kPersistBlock / 32][32];
  __shared__ uint32_t s_hprim[kPersistBlock / 32][32];  // primitive and barycentrics of s_key's hit
  __shared__ float2 s_hbary[kPersistBlock / 32][32];
  constexpr int KS = Sink::kCollide ? WPBR_SHARED_STACK : WPBR_SHARED_STACK_RENDER;
  __shared__ unsigned long long s_stk_tr[KS > 0 ? KS : 1][kPersistBlock];
  __shared__ uint32_t s_stk_c[KS > 0 ? KS : 1][kPersistBlock];
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t wid = threadIdx.x >> 5;
  const uint32_t lt_mask = (1u << lane) - 1u;
  V3 o{0, 0, 0}, inv{0, 0, 0};
  int neg[3] = {0, 0, 0};
  float tmax = 0.0f, tb = 0.0f;
  // The render passes' kernels keep the hit record the cooperative leaf
  // tests leave in shared memory; the collide kernels keep only the winning
  // primitive's sorted position and test it once more when the ray is done
  // (the direction then comes back from the ray's shared record), which
  // keeps four registers and the direction out of the traversal loops.
  HitRec h{0.0f, kNoHit, 0.0f, 0.0f};
  uint32_t hpos = kNoHit;
  int ref = kEnd;
  uint32_t cnt = 0;
  int lref = kEnd;
  uint32_t lcnt = 0;
  int sp = 0;
  typename StackSel<STACK, Sink::kCollide, KS>::type stk;
  stack_bind(stk, &s_stk_tr[0][threadIdx.x], &s_stk_c[0][threadIdx.x]);
  uint32_t rid = 0;
  bool active = false;
  bool exhausted = false;
  uint32_t guard = 0;
  n = src.limit(n);  // a queue source reads its length from device memory

  while (true) {
    // ---- refill idle lanes ------------------------------------------------
    __syncwarp();
    uint32_t idle = __ballot_sync(0xFFFFFFFFu, !active && !exhausted);
    if (idle && (__popc(idle) >= WPBR_REFILL_MIN || !__any_sync(0xFFFFFFFFu, active))) {
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
          const V3 d{rd.x, rd.y, rd.z};
          tmax = rd.w;
          inv = V3{1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
          neg[0] = inv.x < 0.0f;
          neg[1] = inv.y < 0.0f;
          neg[2] = inv.z < 0.0f;
          RayTri R = ray_tri_setup(o, d, S.quirks);
          SharedRay& sr = s_ray[wid][lane];
          uint32_t kpack =
              (uint32_t)R.kx | ((uint32_t)R.ky << 2) | ((uint32_t)R.kz << 4) | ((R.miss_all ? 1u : 0u) << 6);
          sr.s = make_float4(R.sx, R.sy, R.sz, tmax);
          sr.po = make_float4(R.ox, R.oy, R.oz, __uint_as_float(kpack));
          sr.d = make_float4(d.x, d.y, d.z, 0.0f);
          tb = inf_();
          h = HitRec{inf_(), kNoHit, 0.0f, 0.0f};
          hpos = kNoHit;
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
    if (++guard > Bv.step_cap) {
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
        float tbs = tb * kPruneScale;
        bool h0 = slab_test_flat(V3{b0.x, b0.z, bz.x}, V3{b0.y, b0.w, bz.y}, o, inv, neg, tmax, &t0) && !(t0 > tbs);
        bool h1 = slab_test_flat(V3{b1.x, b1.z, bz.z}, V3{b1.y, b1.w, bz.w}, o, inv, neg, tmax, &t1) && !(t1 > tbs);
        uint32_t axis = ((uint32_t)m.w) >> 30;
        uint32_t c0n = (uint32_t)m.z, c1n = ((uint32_t)m.w) & 0x3FFFFFFFu;
        if (h0 && h1) {
          bool first1 = second_child_first(neg, axis);
          if ((uint32_t)sp >= Bv.stack_cap) {  // stack_cap <= STACK (launch_traversal clamps it)
            atomicOr(err, kErrStackOverflow);
            ref = kEnd;
            break;
          }
          // (an L2 prefetch of the far child's record here, -1.1 % with the
          // stack in local memory, cost 1.5 % once the kernels were issue-bound)
          stk.put(sp, first1 ? m.x : m.y, first1 ? c0n : c1n, first1 ? t0 : t1);
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
          ref = pop_unpruned(stk, sp, tb, &cnt);
        }
        // postpone the first leaf found, keep descending for the next one
        if (ref < 0 && ref != kEnd && lref == kEnd) {
          lref = ref;
          lcnt = cnt;
          ref = pop_unpruned(stk, sp, tb, &cnt);
        }
        if (!__any_sync(__activemask(), lref == kEnd)) break;
      }
      // the current node may itself be a leaf reached without postponing
      if (lref == kEnd && ref < 0 && ref != kEnd) {
        lref = ref;
        lcnt = cnt;
        ref = pop_unpruned(stk, sp, tb, &cnt);
      }
    }

    // ---- leaf phase: the warp tests all its lanes' leaf primitives together ----
    // Each round every lane with a leaf contributes its primitive range; the
    // 32 lanes take the primitives in turn (owner found by a binary search
    // over the exclusive prefix of the counts) and fold their hits into the
    // owner's key with a shared-memory atomicMin: (t, position) for the
    // closest hit — the smallest t, and among equal t the first position, as
    // the sequential leaf scan keeps — and (position, t) for any-hit. In the
    // render passes' kernels, after each step in which a lane hit, the lane
    // whose key is its owner's minimum (keys are unique: one position each)
    // records the primitive and barycentrics, so the owner takes its hit
    // without testing it again (1080p full frame +1.7 %, 256x256 spheres
    // scene +20 %, textured metal +11 %: a sphere test is costly); the
    // collide kernels test the winning primitive again, which measured
    // faster on the triangle-mesh microbenchmark (4.14 against 4.23 ms).
    while (__any_sync(0xFFFFFFFFu, lref != kEnd)) {
      uint32_t myc = 0, myfirst = 0;
      if (lref != kEnd) {
        myfirst = (uint32_t)(~lref);
        if (myfirst >= Bv.n_prims || lcnt > Bv.n_prims - myfirst) {
          atomicOr(err, kErrBuild);
          lref = kEnd;
          ref = kEnd;
        } else {
          myc = lcnt;
        }
      }
      uint32_t incl = myc;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, off);
        if (lane >= (uint32_t)off) incl += v;
      }
      uint32_t excl = incl - myc;
      uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
      s_key[wid][lane] = ~0ull;
      __syncwarp();
      for (uint32_t base = 0; base < total; base += 32) {
        uint32_t g = base + lane;
        uint32_t owner = 0;
#pragma unroll
        for (uint32_t step = 16; step > 0; step >>= 1) {
          uint32_t cand = owner + step;
          uint32_t e = __shfl_sync(0xFFFFFFFFu, excl, cand);
          if (e <= g) owner = cand;
        }
        uint32_t ofirst = __shfl_sync(0xFFFFFFFFu, myfirst, owner);
        uint32_t oexcl = __shfl_sync(0xFFFFFFFFu, excl, owner);
        bool hit = false;
        unsigned long long key = 0;
        uint32_t prim = 0;
        float b1 = 0.0f, b2 = 0.0f;
        if (g < total) {
          const SharedRay& sr = s_ray[wid][owner];
          float4 s4 = sr.s;
          RayTri R = unpack_ray_tri(s4, sr.po);
          uint32_t pos = ofirst + (g - oexcl);
          float t = prim_test_shared(S, Bv.prims, pos, sr, R, &prim, &b1, &b2);
          if (t != 0.0f && t < s4.w) {
            key = ANY ? (((unsigned long long)pos << 32) | __float_as_uint(t))
                      : (((unsigned long long)__float_as_uint(t) << 32) | pos);
            atomicMin(&s_key[wid][owner], key);
            hit = true;
          }
        }
        if (!Sink::kCollide && __any_sync(0xFFFFFFFFu, hit)) {
          __syncwarp();
          if (hit && s_key[wid][owner] == key) {
            s_hprim[wid][owner] = prim;
            s_hbary[wid][owner] = make_float2(b1, b2);
          }
        }
      }
      __syncwarp();
      bool done_any = false;
      if (myc) {
        unsigned long long key = s_key[wid][lane];
        if (key != ~0ull) {
          float t = __uint_as_float(ANY ? (uint32_t)(key & 0xFFFFFFFFull) : (uint32_t)(key >> 32));
          if (tb > t) {
            if (Sink::kCollide) {
              hpos = ANY ? (uint32_t)(key >> 32) : (uint32_t)(key & 0xFFFFFFFFull);
            } else {
              float2 bb = s_hbary[wid][lane];
              h = HitRec{t, s_hprim[wid][lane], bb.x, bb.y};
            }
            tb = t;
            if (ANY) done_any = true;
          }
        }
      }
      __syncwarp();
      if (lref != kEnd) {
        lref = kEnd;
        if (done_any) {
          ref = kEnd;
          sp = 0;
        } else if (ref < 0 && ref != kEnd) {  // next node is a leaf too: test it in the next round
          lref = ref;
          lcnt = cnt;
          ref = pop_unpruned(stk, sp, tb, &cnt);
        }
      }
    }
    if (active && ref == kEnd && lref == kEnd) {
      if (Sink::kCollide && hpos != kNoHit) {
        const float4 dd = s_ray[wid][lane].d;
        const V3 d{dd.x, dd.y, dd.z};
        RayTri R = ray_tri_setup(o, d, S.quirks);
        uint32_t prim;
        float b1, b2;
        float tt = prim_test(S, Bv.prims, hpos, o, d, R, &prim, &b1, &b2);
        h = HitRec{tt, prim, b1, b2};
      }
      sink.store(rid, h);
      active = false;
    }
  }
}

// ---- ray sources and hit sinks -------------------------------------------------
// The collide kernels load each ray and store each hit once: the
// cache-streaming forms leave L2 to the tree (8.4M rays, 268 MB of rays and
// 134 MB of hits against a 93 MB tree: closest-hit step -0.2 %).
__device__ __forceinline__ float4 ray_load(const float4* p) { return __ldcs(p); }
__device__ __forceinline__ void hit_store(float4* p, float4 v) { __stcs(p, v); }
struct BufferSrc {
  const float4* rays;  // 2 float4 per ray: (o, unused), (d, tmax)
  __device__ __forceinline__ uint32_t limit(uint32_t n) const { return n; }
  __device__ __forceinline__ void load(uint32_t i, float4* o, float4* d) const {
    *o = ray_load(&rays[2 * (size_t)i]);
    *d = ray_load(&rays[2 * (size_t)i + 1]);
  }
};
// The rays a kernel queued (ShadowQueue): as many as *count says, at most
// the launch's n.
struct QueueSrc {
  const float4* rays;
  const uint32_t* count;
  __device__ __forceinline__ uint32_t limit(uint32_t n) const {
    const uint32_t c = *count;
    return c < n ? c : n;
  }
  __device__ __forceinline__ void load(uint32_t i, float4* o, float4* d) const {
    *o = __ldg(&rays[2 * (size_t)i]);
    *d = __ldg(&rays[2 * (size_t)i + 1]);
  }
};
#ifndef WPBR_COLLIDE_BLOCKS
#define WPBR_COLLIDE_BLOCKS 8
#endif
struct HitSink4 {
  static constexpr int kMinBlocks = WPBR_COLLIDE_BLOCKS;
  static constexpr bool kCollide = true;
  float4* hits;
  __device__ __forceinline__ void store(uint32_t i, const HitRec& h) const {
    hit_store(&hits[i], make_float4(h.t, __uint_as_float(h.prim), h.b1, h.b2));
  }
};
// Rays visited in the order of a permutation (sorted position -> input
// index); hits land at the input index.
struct PermSrc {
  const float4* rays;
  const uint32_t* perm;
  __device__ __forceinline__ uint32_t limit(uint32_t n) const { return n; }
  __device__ __forceinline__ void load(uint32_t i, float4* o, float4* d) const {
    size_t j = __ldg(&perm[i]);
    *o = ray_load(&rays[2 * j]);
    *d = ray_load(&rays[2 * j + 1]);
  }
};
struct PermHitSink4 {
  static constexpr int kMinBlocks = WPBR_COLLIDE_BLOCKS;
  static constexpr bool kCollide = true;
  float4* hits;
  const uint32_t* perm;
  __device__ __forceinline__ void store(uint32_t i, const HitRec& h) const {
    hit_store(&hits[__ldg(&perm[i])], make_float4(h.t, __uint_as_float(h.prim), h.b1, h.b2));
  }
};
// The render passes' camera (PrimSink) and shadow-queue (MapSink) traversals
// at 8 resident blocks per SM. 1080p full frame x 16 spp, camera/shadow
// blocks: 8/8 1,815 Msamples/s, 8/10 1,786, 8/12 1,772, 10/10 1,739, 12/12
// 1,688 (textured metal and the 256x256 frame in the same order).
struct PrimSink {
  static constexpr int kMinBlocks = 8;
  static constexpr bool kCollide = false;
  uint32_t* prims;
  __device__ __forceinline__ void store(uint32_t i, const HitRec& h) const { prims[i] = h.prim; }
};
// Hit primitive of queued ray i at the result slot the queue recorded for it.
struct MapSink {
  static constexpr int kMinBlocks = 8;
  static constexpr bool kCollide = false;
  uint32_t* prims;
  const uint32_t* map;
  __device__ __forceinline__ void store(uint32_t i, const HitRec& h) const { prims[__ldg(&map[i])] = h.prim; }
};


// Launches the traversal whose stack fits the tree: a lane's stack never
// holds more entries than the tree is deep, so trees shallower than 60
// levels take the 64-entry kernel and deeper ones (the callers refuse depths
// of 250 and more) the 256-entry kernel of the reference's nodesToVisit[256]
// (SLBVH.cpp:101); grid_cap limits the persistent grid (0: one full wave of
// resident blocks).
template <bool ANY, class Src, class Sink>
inline void launch_traversal(const SceneView& S, const BvhView& Bv, const Src& src, const Sink& sink, uint32_t n,
                             uint32_t* counter, uint32_t* err, cudaStream_t st, uint32_t grid_cap = 0) {
  auto go = [&](auto kern, uint32_t stack) {
    unsigned full = persistent_grid((const void*)kern, kPersistBlock);
    unsigned g = (grid_cap && grid_cap < full) ? grid_cap : full;
    BvhView B = Bv;
    if (B.stack_cap > stack) B.stack_cap = stack;
    kern<<<g, kPersistBlock, 0, st>>>(S, B, src, sink, n, counter, err);
  };
  if (Bv.max_depth < 60)
    go(k_trace_persistent<ANY, 64, Src, Sink>, 64u);
  else
    go(k_trace_persistent<ANY, 256, Src, Sink>, 256u);
}

}  // namespace wpbr
