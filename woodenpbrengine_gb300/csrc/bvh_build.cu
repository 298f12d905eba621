// bvh_build.cu — GPU build of the reference's SLBVH (MEngine::buildLBVH,
// WoodenPBREngine/MEngine.cpp:341-350; SLBVH.cpp), producing the identical
// flattened CSceneTreeLBVH (node order, bounds, axes, leaf ranges) and the
// child-pair traversal layout.
//
// Stages (reference job -> kernels):
//   JobUpdateBoundsAndCentroid{Sphere,Triangle}  k_prim_bounds
//   JobGenerateShapesCentroidBound               k_prim_bounds (block + atomic reduce)
//   JobGenerateShapesMortonCode                  k_morton
//   JobSortsShapesByMortonCode                   8-bit LSD radix sort (k_radix_*), stable, so
//                                                the permutation equals the reference's 6-bit
//                                                passes; treelet split k_treelet_*
//   JobEmitLBVH                                  Karras radix tree per treelet (k_karras) + the
//                                                reference's leaf rule (n < 30 or equal codes),
//                                                bottom-up bounds (k_refit)
//   JobBuildUpperSAH                             level-synchronous segmented 12-bucket SAH over
//                                                treelet roots (k_seg_*), std::partition's
//                                                two-pointer swap order reproduced with ranks;
//                                                segments of <= 32 roots finish in one warp
//                                                (k_small_sah)
//   flattenBVHTree                               preorder index by walking up subtree sizes
//                                                (k_flatten), then k_node2 / k_prims
//
// Unified node ids: [0, N-1) radix-tree internal nodes, [N, 2N) single
// primitives (sorted position + N), [2N, 2N + T) SAH nodes.
#include <algorithm>
#include <cstdio>

#include "common.cuh"
#include "ctx.hpp"
#include "intersect.cuh"

namespace wpbr {

namespace {

constexpr uint32_t kTreeletMask = 0b00111111111111000000000000000000u;  // SLBVH.cpp:301
constexpr int kLeafMax = 30;                                          // SLBVH.cpp:356
constexpr uint32_t kSmallSeg = 32;
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kB = 256;

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }

// ---------------------------------------------------------------------------
// exclusive scan (tile scan + recursive block sums) of 32-bit counts, or of
// 64-bit words that pack two 32-bit counts whose sums stay below 2^32 (no
// carry crosses the halves, so one scan gives both prefix sums)
// ---------------------------------------------------------------------------
template <class V>
__global__ void k_scan_tile(const V* in, V* out, uint32_t n, V* bsum) {
  __shared__ V sh[kScanTile];
  __shared__ V wsum[kScanBlock / 32];
  const uint32_t base = blockIdx.x * kScanTile;
  for (int k = 0; k < kScanItems; ++k) {
    uint32_t i = base + threadIdx.x + k * kScanBlock;
    sh[threadIdx.x + k * kScanBlock] = i < n ? in[i] : V(0);
  }
  __syncthreads();
  V v[kScanItems];
  V sum = 0;
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = sh[threadIdx.x * kScanItems + k];
    sum += v[k];
  }
  uint32_t lane = lane_id(), w = threadIdx.x >> 5;
  V x = sum;
  for (int o = 1; o < 32; o <<= 1) {
    V y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    V ws = lane < kScanBlock / 32 ? wsum[lane] : V(0);
    V inc = ws;
    for (int o = 1; o < 32; o <<= 1) {
      V y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
      if (lane >= (uint32_t)o) inc += y;
    }
    if (lane < kScanBlock / 32) wsum[lane] = inc - ws;
  }
  __syncthreads();
  V run = (x - sum) + wsum[w];
  V total_before = run;
  for (int k = 0; k < kScanItems; ++k) {
    sh[threadIdx.x * kScanItems + k] = run;
    run += v[k];
  }
  __syncthreads();
  for (int k = 0; k < kScanItems; ++k) {
    uint32_t i = base + threadIdx.x + k * kScanBlock;
    if (i < n) out[i] = sh[threadIdx.x + k * kScanBlock];
  }
  if (threadIdx.x == kScanBlock - 1 && bsum) bsum[blockIdx.x] = total_before + sum;
}

template <class V>
__global__ void k_scan_add(V* out, uint32_t n, const V* boff) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += boff[i / kScanTile];
}

template <class V>
cudaError_t scan_exclusive_t(const V* in, V* out, uint32_t n, V* tmp, size_t tmp_n, cudaStream_t s) {
  struct Lvl {
    const V* in;
    V* out;
    uint32_t n;
    V* sums;
  };
  Lvl lv[8];
  int L = 0;
  size_t off = 0;
  const V* cin = in;
  V* cout = out;
  uint32_t m = n;
  while (true) {
    uint32_t nb = div_up(m, kScanTile);
    V* sums = nb > 1 ? tmp + off : nullptr;
    lv[L++] = Lvl{cin, cout, m, sums};
    if (nb <= 1) break;
    off += nb + 1;
    if (off > tmp_n) return cudaErrorInvalidValue;
    cin = sums;
    cout = sums;
    m = nb;
    if (L >= 8) return cudaErrorInvalidValue;
  }
  for (int i = 0; i < L; ++i) {
    uint32_t nb = div_up(lv[i].n, kScanTile);
    k_scan_tile<V><<<nb, kScanBlock, 0, s>>>(lv[i].in, lv[i].out, lv[i].n, lv[i].sums);
  }
  for (int i = L - 2; i >= 0; --i) {
    k_scan_add<V><<<div_up(lv[i].n, 256), 256, 0, s>>>(lv[i].out, lv[i].n, lv[i].sums);
  }
  return cudaGetLastError();
}

size_t scan_tmp_need(uint32_t n) {
  size_t need = 0;
  for (uint32_t m = n; m > (uint32_t)kScanTile; m = div_up(m, kScanTile)) need += div_up(m, kScanTile) + 1;
  return need;
}

// Both partition counts of the SAH levels in one pass (two 32-bit prefix sums
// packed in 64-bit words); tmp holds the block sums as 32-bit words, two each.
cudaError_t scan_exclusive_pair(const unsigned long long* in, unsigned long long* out, uint32_t n,
                                DevBuf<uint32_t>& tmp, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  size_t need = scan_tmp_need(n);
  cudaError_t e = tmp.ensure(2 * need + 16);
  if (e != cudaSuccess) return e;
  unsigned long long* t64 = reinterpret_cast<unsigned long long*>(tmp.p);
  return scan_exclusive_t(in, out, n, t64, need + 8, s);
}

}  // namespace

// Kernel launches of scan_exclusive over n elements: one tile scan per
// level, one add per level but the last.
uint32_t scan_launches(uint32_t n) {
  if (n == 0) return 0;
  uint32_t levels = 1;
  for (uint32_t m = n; m > (uint32_t)kScanTile; m = div_up(m, kScanTile)) ++levels;
  return 2 * levels - 1;
}

cudaError_t scan_exclusive(const uint32_t* in, uint32_t* out, uint32_t n, DevBuf<uint32_t>& tmp, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  // tmp layout: level-1 sums, level-2 sums, ...
  size_t need = scan_tmp_need(n);
  cudaError_t e = tmp.ensure(need + 8);
  if (e != cudaSuccess) return e;
  return scan_exclusive_t(in, out, n, tmp.p, need + 8, s);
}

namespace {

// ---------------------------------------------------------------------------
// A3/A4: primitive bounds, centroids, centroid bounds
// ---------------------------------------------------------------------------
__global__ void k_prim_bounds(SceneView S, float4* pb_lo, float4* pb_hi, float4* cen, uint32_t* cb_enc) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t e[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
  if (i < S.N) {
    Bounds b;
    if (i < S.ns) {
      float r = S.sph_r[i];
      Xf M = S.sph_o2w[i];
      for (int c = 0; c < 8; ++c) {
        V3 p{(c & 1) ? r : -r, (c & 2) ? r : -r, (c & 4) ? r : -r};
        V3 q = xpoint(M, p);
        b = (c == 0) ? Bounds{q, q} : bunionp(b, q);
      }
    } else {
      uint32_t t = i - S.ns;
      const uint32_t* ix = S.idx + 3 * t;
      V3 a{S.pos[3 * ix[0]], S.pos[3 * ix[0] + 1], S.pos[3 * ix[0] + 2]};
      V3 bb{S.pos[3 * ix[1]], S.pos[3 * ix[1] + 1], S.pos[3 * ix[1] + 2]};
      V3 c{S.pos[3 * ix[2]], S.pos[3 * ix[2] + 1], S.pos[3 * ix[2] + 2]};
      b = Bounds{vmin(a, bb), vmax(a, bb)};
      b = bunionp(b, c);
    }
    V3 ce = bcentroid(b);
    pb_lo[i] = make_float4(b.lo.x, b.lo.y, b.lo.z, 0.0f);
    pb_hi[i] = make_float4(b.hi.x, b.hi.y, b.hi.z, 0.0f);
    cen[i] = make_float4(ce.x, ce.y, ce.z, 0.0f);
    e[0] = fenc(ce.x); e[1] = fenc(ce.y); e[2] = fenc(ce.z);
    e[3] = e[0]; e[4] = e[1]; e[5] = e[2];
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int k = 0; k < 6; ++k) {
      uint32_t y = __shfl_xor_sync(0xFFFFFFFFu, e[k], o);
      e[k] = k < 3 ? min(e[k], y) : max(e[k], y);
    }
  __shared__ uint32_t sh[kB / 32][6];
  if (lane_id() == 0)
    for (int k = 0; k < 6; ++k) sh[threadIdx.x >> 5][k] = e[k];
  __syncthreads();
  if (threadIdx.x < 6) {
    uint32_t k = threadIdx.x;
    uint32_t v = sh[0][k];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = k < 3 ? min(v, sh[w][k]) : max(v, sh[w][k]);
    if (k < 3) atomicMin(&cb_enc[k], v);
    else atomicMax(&cb_enc[k], v);
  }
}

// A5: JobGenerateShapesMortonCode + leftShift3 (SLBVH.cpp:186-227)
__device__ __forceinline__ uint32_t left_shift3(uint32_t x) {
  if (x == (1u << 10)) --x;
  x = (x | (x << 16)) & 0b00000011000000000000000011111111u;
  x = (x | (x << 8)) & 0b00000011000000001111000000001111u;
  x = (x | (x << 4)) & 0b00000011000011000011000011000011u;
  x = (x | (x << 2)) & 0b00001001001001001001001001001001u;
  return x;
}
__device__ __forceinline__ uint32_t f2u_trunc(float v) { return (v >= 0.0f) ? (uint32_t)v : 0u; }

__global__ void k_morton(uint32_t N, const float4* cen, const uint32_t* cb_enc, uint32_t* codes, uint32_t* keys,
                         uint32_t* vals) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  float lx = fdec(cb_enc[0]), ly = fdec(cb_enc[1]), lz = fdec(cb_enc[2]);
  float hx = fdec(cb_enc[3]), hy = fdec(cb_enc[4]), hz = fdec(cb_enc[5]);
  float4 c = cen[i];
  float nx = (c.x - lx) / (hx - lx), ny = (c.y - ly) / (hy - ly), nz = (c.z - lz) / (hz - lz);
  uint32_t code = (left_shift3(f2u_trunc(nz * 1024.0f)) << 2) | (left_shift3(f2u_trunc(ny * 1024.0f)) << 1) |
                  left_shift3(f2u_trunc(nx * 1024.0f));
  codes[i] = code;
  keys[i] = code;
  vals[i] = i;
}

// ---------------------------------------------------------------------------
// A6: stable LSD radix sort, 8-bit digits, 2048 keys per block
// ---------------------------------------------------------------------------
constexpr int kRadixItems = 8;
constexpr int kRadixTile = kB * kRadixItems;

__global__ void k_radix_hist(const uint32_t* keys, uint32_t n, int shift, uint32_t dmask, uint32_t* hist,
                             uint32_t nblocks) {
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  uint32_t base = blockIdx.x * kRadixTile;
  for (int k = 0; k < kRadixItems; ++k) {
    uint32_t i = base + threadIdx.x + k * kB;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & dmask], 1u);
  }
  __syncthreads();
  hist[threadIdx.x * nblocks + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void k_radix_scatter(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout,
                                uint32_t n, int shift, uint32_t dmask, const uint32_t* offs, uint32_t nblocks) {
  __shared__ uint32_t s_off[256];
  __shared__ uint32_t s_wcnt[kB / 32][256];
  __shared__ uint32_t s_round[256];
  s_off[threadIdx.x] = offs[threadIdx.x * nblocks + blockIdx.x];
  const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  uint32_t base = blockIdx.x * kRadixTile;
  for (int r = 0; r < kRadixItems; ++r) {
    for (int q = 0; q < kB / 32; ++q) s_wcnt[q][threadIdx.x] = 0;
    __syncthreads();
    uint32_t i = base + r * kB + threadIdx.x;
    bool valid = i < n;
    uint32_t key = valid ? kin[i] : 0u;
    uint32_t val = valid ? vin[i] : 0u;
    uint32_t d = valid ? ((key >> shift) & dmask) : (256u + lane);
    uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
    uint32_t rank = __popc(peers & lt);
    if (valid && rank == 0) s_wcnt[w][d] = __popc(peers);
    __syncthreads();
    {
      uint32_t dd = threadIdx.x, acc = 0;
      for (int q = 0; q < kB / 32; ++q) {
        uint32_t c = s_wcnt[q][dd];
        s_wcnt[q][dd] = acc;
        acc += c;
      }
      s_round[dd] = acc;
    }
    __syncthreads();
    if (valid) {
      uint32_t pos = s_off[d] + s_wcnt[w][d] + rank;
      kout[pos] = key;
      vout[pos] = val;
    }
    __syncthreads();
    s_off[threadIdx.x] += s_round[threadIdx.x];
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// treelets (top 12 bits of the code)
// ---------------------------------------------------------------------------
__global__ void k_treelet_flags(const uint32_t* skey, uint32_t N, uint32_t* flags) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  flags[i] = (i == 0 || ((skey[i] ^ skey[i - 1]) & kTreeletMask) != 0) ? 1u : 0u;
}
__global__ void k_treelet_ids(const uint32_t* flags, uint32_t* tid, uint32_t* tstart, uint32_t N) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  uint32_t t = tid[i] + flags[i] - 1u;  // inclusive - 1
  tid[i] = t;
  if (flags[i]) tstart[t] = i;
}
__global__ void k_treelet_sizes(const uint32_t* tstart, uint32_t* tsize, uint32_t T, uint32_t N) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  tsize[t] = (t + 1 < T ? tstart[t + 1] : N) - tstart[t];
}

// ---------------------------------------------------------------------------
// A7: radix tree per treelet (Karras 2012) with the reference's leaf rule
// ---------------------------------------------------------------------------
struct KarrasCtx {
  const uint32_t* skey;
  uint32_t ts, te;
  __device__ int delta(int a, int b) const {
    if (b < (int)ts || b > (int)te) return -1;
    uint32_t ka = skey[a], kb = skey[b];
    if (ka != kb) return __clz(ka ^ kb);
    return 32 + __clz((uint32_t)a ^ (uint32_t)b);
  }
};

__global__ void k_karras(const uint32_t* skey, const uint32_t* tid, const uint32_t* tstart, const uint32_t* tsize,
                         uint32_t N, uint32_t* rng_lo, uint32_t* rng_hi, uint32_t* child0, uint32_t* child1,
                         uint32_t* parent) {
  int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= (int)N - 1) return;
  uint32_t t = tid[i];
  KarrasCtx K{skey, tstart[t], tstart[t] + tsize[t] - 1};
  if ((uint32_t)i == K.te) return;  // last primitive of the treelet: no internal node here
  int d = (K.delta(i, i + 1) - K.delta(i, i - 1)) > 0 ? 1 : -1;
  int dmin = K.delta(i, i - d);
  int lmax = 2;
  while (K.delta(i, i + lmax * d) > dmin) lmax *= 2;
  int l = 0;
  for (int s = lmax / 2; s >= 1; s /= 2)
    if (K.delta(i, i + (l + s) * d) > dmin) l += s;
  int j = i + l * d;
  int dnode = K.delta(i, j);
  int s = 0;
  int step = l;
  do {
    step = (step + 1) >> 1;
    if (K.delta(i, i + (s + step) * d) > dnode) s += step;
  } while (step > 1);
  int gamma = i + s * d + min(d, 0);
  uint32_t lo = (uint32_t)min(i, j), hi = (uint32_t)max(i, j);
  uint32_t c0 = (lo == (uint32_t)gamma) ? N + (uint32_t)gamma : (uint32_t)gamma;
  uint32_t c1 = (hi == (uint32_t)gamma + 1) ? N + (uint32_t)gamma + 1 : (uint32_t)gamma + 1;
  rng_lo[i] = lo;
  rng_hi[i] = hi;
  child0[i] = c0;
  child1[i] = c1;
  parent[c0] = ((uint32_t)i << 1) | 0u;
  parent[c1] = ((uint32_t)i << 1) | 1u;
}

__device__ __forceinline__ bool ref_interior(uint32_t x, uint32_t N, const uint32_t* rng_lo, const uint32_t* rng_hi,
                                             const uint32_t* skey) {
  if (x >= N) return false;
  uint32_t lo = rng_lo[x], hi = rng_hi[x];
  return (hi - lo + 1 >= (uint32_t)kLeafMax) && (skey[lo] != skey[hi]);
}

// treelet root of the treelet containing sorted position p
__device__ __forceinline__ uint32_t treelet_root(uint32_t t, const uint32_t* tstart, const uint32_t* tsize, uint32_t N) {
  return tsize[t] >= 2 ? tstart[t] : N + tstart[t];
}

// Ref leaves compute their bounds; the second child to finish builds each
// parent (atomic arrival counter), up to the treelet root.
__global__ void k_refit(uint32_t N, const uint32_t* skey, const uint32_t* sprim, const uint32_t* tid,
                        const uint32_t* tstart, const uint32_t* tsize, const uint32_t* rng_lo, const uint32_t* rng_hi,
                        const uint32_t* child0, const uint32_t* child1, const uint32_t* parent, uint32_t* visits,
                        uint32_t* size, float4* nb_lo, float4* nb_hi, const float4* pb_lo, const float4* pb_hi,
                        uint32_t* troot, uint32_t* err) {
  uint32_t X = blockIdx.x * blockDim.x + threadIdx.x;
  if (X >= 2 * N) return;
  uint32_t lo, hi, t;
  if (X < N) {
    if (X + 1 >= N) return;
    t = tid[X];
    if (tid[X + 1] != t) return;  // not an internal node
    lo = rng_lo[X];
    hi = rng_hi[X];
  } else {
    lo = hi = X - N;
    t = tid[lo];
  }
  uint32_t root = treelet_root(t, tstart, tsize, N);
  bool is_root = (X == root);
  if (!is_root) {
    uint32_t p = parent[X] >> 1;
    if (!ref_interior(p, N, rng_lo, rng_hi, skey)) return;  // inside a leaf
  }
  if (ref_interior(X, N, rng_lo, rng_hi, skey)) return;  // interior: built by its children
  // ref leaf: union of its primitives' bounds in sorted order
  float4 l = pb_lo[sprim[lo]], h = pb_hi[sprim[lo]];
  V3 blo{l.x, l.y, l.z}, bhi{h.x, h.y, h.z};
  for (uint32_t q = lo + 1; q <= hi; ++q) {
    float4 a = pb_lo[sprim[q]], b = pb_hi[sprim[q]];
    blo = vmin(blo, V3{a.x, a.y, a.z});
    bhi = vmax(bhi, V3{b.x, b.y, b.z});
  }
  nb_lo[X] = make_float4(blo.x, blo.y, blo.z, 0.0f);
  nb_hi[X] = make_float4(bhi.x, bhi.y, bhi.z, 0.0f);
  size[X] = 1;
  uint32_t cur = X;
  uint32_t guard = 0;
  while (cur != root) {
    if (++guard > 64) {
      atomicOr(err, kErrLoopLimit);
      return;
    }
    uint32_t p = parent[cur] >> 1;
    __threadfence();
    if (atomicAdd(&visits[p], 1u) == 0u) return;
    __threadfence();
    uint32_t c0 = child0[p], c1 = child1[p];
    float4 a0 = __ldcg(&nb_lo[c0]), a1 = __ldcg(&nb_lo[c1]);
    float4 b0 = __ldcg(&nb_hi[c0]), b1 = __ldcg(&nb_hi[c1]);
    V3 plo = vmin(V3{a0.x, a0.y, a0.z}, V3{a1.x, a1.y, a1.z});
    V3 phi = vmax(V3{b0.x, b0.y, b0.z}, V3{b1.x, b1.y, b1.z});
    nb_lo[p] = make_float4(plo.x, plo.y, plo.z, 0.0f);
    nb_hi[p] = make_float4(phi.x, phi.y, phi.z, 0.0f);
    size[p] = 1u + __ldcg(&size[c0]) + __ldcg(&size[c1]);
    cur = p;
  }
  troot[t] = root;
}

// ---------------------------------------------------------------------------
// A8: segmented SAH over treelet roots
// ---------------------------------------------------------------------------
struct SahArgs {
  uint32_t N, T;
  const uint32_t* troot;
  const float4* nb_lo;
  const float4* nb_hi;
};

__device__ __forceinline__ void item_bounds(const SahArgs& A, uint32_t item, V3* lo, V3* hi) {
  uint32_t r = A.troot[item];
  float4 l = A.nb_lo[r], h = A.nb_hi[r];
  *lo = V3{l.x, l.y, l.z};
  *hi = V3{h.x, h.y, h.z};
}

__global__ void k_fill(uint32_t* p, uint32_t n, uint32_t v) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// Segment of every position (kNone outside the level's large segments): a
// binary search over the segment starts, which are in ascending order.
// The SAH levels' kernels read the level's count of large segments from
// device memory (nseg_p), so the host can queue a level before the previous
// one has finished.
__global__ void k_pos_seg(uint32_t T, const uint32_t* nseg_p, const uint32_t* seg_start, const uint32_t* seg_end,
                          uint32_t* pos_seg) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= T) return;
  const uint32_t nseg = *nseg_p;
  uint32_t lo = 0, hi = nseg;
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (__ldg(seg_start + mid) <= p)
      lo = mid + 1;
    else
      hi = mid;
  }
  pos_seg[p] = (lo > 0 && p <= __ldg(seg_end + lo - 1)) ? lo - 1 : kNone;
}

__global__ void k_seg_init(const uint32_t* nseg_p, uint32_t* benc, uint32_t* cenc, uint32_t* bcnt, uint32_t* bkenc) {
  uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= *nseg_p) return;
  for (int k = 0; k < 6; ++k) {
    benc[s * 6 + k] = k < 3 ? 0xFFFFFFFFu : 0u;
    cenc[s * 6 + k] = k < 3 ? 0xFFFFFFFFu : 0u;
  }
  for (int b = 0; b < 12; ++b) {
    bcnt[s * 12 + b] = 0;
    for (int k = 0; k < 6; ++k) bkenc[(s * 12 + b) * 6 + k] = k < 3 ? 0xFFFFFFFFu : 0u;
  }
}

// Bounds and centroid bounds per segment: warp-segmented reduce over the
// contiguous runs, then per block: the runs of the block's first kSegSlots
// segments meet in shared memory and leave one global atomic per block and
// segment (near the root a level has a handful of segments, and one atomic per
// warp on the same words serialised in L2); runs of later segments go to
// global memory directly. Min and max are order-independent, so the bounds
// are exact whatever the grouping.
constexpr int kSegSlots = 16;
__global__ void k_seg_reduce(SahArgs A, const uint32_t* cur, const uint32_t* pos_seg, uint32_t* benc, uint32_t* cenc) {
  __shared__ uint32_t s_min;
  __shared__ uint32_t s_red[kSegSlots * 12];  // slot * 12 + (lo xyz, hi xyz, centroid lo xyz, centroid hi xyz)
  if (threadIdx.x == 0) s_min = kNone;
  for (int k = threadIdx.x; k < kSegSlots * 12; k += blockDim.x) s_red[k] = ((k % 12) / 3) % 2 == 0 ? 0xFFFFFFFFu : 0u;
  __syncthreads();
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t s = (p < A.T) ? pos_seg[p] : kNone;
  uint32_t wmin = __reduce_min_sync(0xFFFFFFFFu, s);
  if (lane_id() == 0 && wmin != kNone) atomicMin(&s_min, wmin);
  __syncthreads();
  const uint32_t smin = s_min;
  uint32_t e[12];
  if (s != kNone) {
    V3 lo, hi;
    item_bounds(A, cur[p], &lo, &hi);
    V3 c = mul(add(lo, hi), 0.5f);
    e[0] = fenc(lo.x); e[1] = fenc(lo.y); e[2] = fenc(lo.z);
    e[3] = fenc(hi.x); e[4] = fenc(hi.y); e[5] = fenc(hi.z);
    e[6] = fenc(c.x); e[7] = fenc(c.y); e[8] = fenc(c.z);
    e[9] = e[6]; e[10] = e[7]; e[11] = e[8];
  } else {
    for (int k = 0; k < 12; ++k) e[k] = 0;
  }
  uint32_t lane = lane_id();
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t so = __shfl_down_sync(0xFFFFFFFFu, s, o);
    bool take = (lane + o < 32) && (so == s) && (s != kNone);
    for (int k = 0; k < 12; ++k) {
      uint32_t y = __shfl_down_sync(0xFFFFFFFFu, e[k], o);
      if (take) {
        bool mn = (k < 3) || (k >= 6 && k < 9);
        e[k] = mn ? min(e[k], y) : max(e[k], y);
      }
    }
  }
  uint32_t sp = __shfl_up_sync(0xFFFFFFFFu, s, 1);
  bool head = (s != kNone) && (lane == 0 || sp != s);
  if (head) {
    uint32_t slot = s - smin;  // s >= smin for every s != kNone of the block
    if (slot < (uint32_t)kSegSlots) {
      uint32_t* r = s_red + slot * 12;
      for (int k = 0; k < 3; ++k) atomicMin(&r[k], e[k]);
      for (int k = 3; k < 6; ++k) atomicMax(&r[k], e[k]);
      for (int k = 6; k < 9; ++k) atomicMin(&r[k], e[k]);
      for (int k = 9; k < 12; ++k) atomicMax(&r[k], e[k]);
    } else {
      for (int k = 0; k < 3; ++k) atomicMin(&benc[s * 6 + k], e[k]);
      for (int k = 3; k < 6; ++k) atomicMax(&benc[s * 6 + k], e[k]);
      for (int k = 0; k < 3; ++k) atomicMin(&cenc[s * 6 + k], e[6 + k]);
      for (int k = 0; k < 3; ++k) atomicMax(&cenc[s * 6 + 3 + k], e[9 + k]);
    }
  }
  __syncthreads();
  if (smin == kNone) return;
  for (int k = threadIdx.x; k < kSegSlots * 12; k += blockDim.x) {
    uint32_t v = s_red[k];
    int j = k % 12;
    bool is_min = (j / 3) % 2 == 0;
    if (v == (is_min ? 0xFFFFFFFFu : 0u)) continue;  // no run of this slot's segment in the block
    uint32_t seg = smin + (uint32_t)(k / 12);
    uint32_t* dst = (j < 6 ? benc : cenc) + seg * 6 + (j < 6 ? j : j - 6);
    if (is_min)
      atomicMin(dst, v);
    else
      atomicMax(dst, v);
  }
}

__device__ __forceinline__ Bounds dec_bounds(const uint32_t* e) {
  return Bounds{V3{fdec(e[0]), fdec(e[1]), fdec(e[2])}, V3{fdec(e[3]), fdec(e[4]), fdec(e[5])}};
}

// Bucket of every root (JobBuildUpperSAH, SLBVH.cpp:484-502) and per-bucket
// counts / bounds, pre-aggregated in shared memory per block.
__global__ void k_seg_bucket(SahArgs A, const uint32_t* cur, const uint32_t* pos_seg, const uint32_t* cenc,
                             uint32_t* bucket, uint32_t* bcnt, uint32_t* bkenc) {
  __shared__ uint32_t s_min;
  __shared__ uint32_t s_cnt[kSegSlots * 12];
  __shared__ uint32_t s_enc[kSegSlots * 12 * 6];
  if (threadIdx.x == 0) s_min = kNone;
  for (int k = threadIdx.x; k < kSegSlots * 12; k += blockDim.x) s_cnt[k] = 0;
  for (int k = threadIdx.x; k < kSegSlots * 12 * 6; k += blockDim.x) s_enc[k] = (k % 6) < 3 ? 0xFFFFFFFFu : 0u;
  __syncthreads();
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t s = (p < A.T) ? pos_seg[p] : kNone;
  if (s != kNone) atomicMin(&s_min, s);
  __syncthreads();
  if (s != kNone) {
    V3 lo, hi;
    item_bounds(A, cur[p], &lo, &hi);
    Bounds cb = dec_bounds(cenc + s * 6);
    int dim = bmax_extent(cb);
    float dist = comp(cb.hi, dim) - comp(cb.lo, dim);
    float c = (comp(lo, dim) + comp(hi, dim)) * 0.5f;
    float t = (c - comp(cb.lo, dim)) / dist;
    float bt = 12.0f * t;
    uint32_t ib = (bt >= 0.0f) ? (uint32_t)bt : 0u;
    if (ib >= 12u) ib = 11u;
    bucket[p] = ib;
    uint32_t e[6] = {fenc(lo.x), fenc(lo.y), fenc(lo.z), fenc(hi.x), fenc(hi.y), fenc(hi.z)};
    uint32_t slot = s - s_min;
    if (slot < (uint32_t)kSegSlots) {
      atomicAdd(&s_cnt[slot * 12 + ib], 1u);
      uint32_t* d = &s_enc[(slot * 12 + ib) * 6];
      for (int k = 0; k < 3; ++k) atomicMin(&d[k], e[k]);
      for (int k = 3; k < 6; ++k) atomicMax(&d[k], e[k]);
    } else {
      atomicAdd(&bcnt[s * 12 + ib], 1u);
      uint32_t* d = &bkenc[(s * 12 + ib) * 6];
      for (int k = 0; k < 3; ++k) atomicMin(&d[k], e[k]);
      for (int k = 3; k < 6; ++k) atomicMax(&d[k], e[k]);
    }
  }
  __syncthreads();
  if (s_min == kNone) return;
  for (int k = threadIdx.x; k < kSegSlots * 12; k += blockDim.x) {
    uint32_t c = s_cnt[k];
    if (c == 0) continue;
    uint32_t gs = s_min + (uint32_t)(k / 12), b = (uint32_t)(k % 12);
    atomicAdd(&bcnt[gs * 12 + b], c);
    uint32_t* d = &bkenc[(gs * 12 + b) * 6];
    for (int q = 0; q < 3; ++q) atomicMin(&d[q], s_enc[k * 6 + q]);
    for (int q = 3; q < 6; ++q) atomicMax(&d[q], s_enc[k * 6 + q]);
  }
}

// Cost of the 11 candidate splits, SLBVH.cpp:504-538, and the child layout.
// The two sides of split i are the unions of the non-empty buckets 0..i and
// i+1..11 (JobBuildUpperSAH's two inner loops): the right sides are built
// once as suffix unions and the left sides accumulated in bucket order, 24
// bucket decodes instead of 132 (one thread decides a segment; near the root
// that chain of dependent loads was the level's longest kernel). Min and max
// of finite coordinates do not depend on the grouping; only a zero's sign
// could, which no area or cost sees.
__device__ void sah_decide(const uint32_t* bcnt, const uint32_t* bkenc, const Bounds& bounds, uint32_t n, int* best_out,
                           uint32_t* k_out) {
  float barea_ = barea(bounds);
  float cost_min = 0.0f;
  int best = 0;
  uint32_t c[12];
#pragma unroll
  for (int j = 0; j < 12; ++j) c[j] = bcnt[j];
  Bounds suf[11];
  uint32_t nsuf[11];
  suf[10] = bempty();
  nsuf[10] = 0;
  if (c[11]) {
    suf[10] = bunion(suf[10], dec_bounds(bkenc + 11 * 6));
    nsuf[10] = c[11];
  }
#pragma unroll
  for (int i = 9; i >= 0; --i) {
    suf[i] = suf[i + 1];
    nsuf[i] = nsuf[i + 1];
    if (c[i + 1]) {
      suf[i] = bunion(suf[i], dec_bounds(bkenc + (i + 1) * 6));
      nsuf[i] += c[i + 1];
    }
  }
  Bounds b0 = bempty();
  uint32_t n0 = 0;
#pragma unroll
  for (int i = 0; i < 11; ++i) {
    if (c[i]) {
      b0 = bunion(b0, dec_bounds(bkenc + i * 6));
      n0 += c[i];
    }
    const Bounds& b1 = suf[i];
    uint32_t n1 = nsuf[i];
    float l = (n0 == 0) ? 0.0f : (float)n0 * barea(b0);
    float r = (n1 == 0) ? 0.0f : (float)n1 * barea(b1);
    float cost = (float)(0.125 + (double)((l + r) / barea_));
    if (i == 0 || cost < cost_min) {
      cost_min = cost;
      best = i;
    }
  }
  uint32_t k = 0;
  for (int j = 0; j <= best; ++j) k += c[j];
  (void)n;
  *best_out = best;
  *k_out = k;
}

struct SegLevel {
  const uint32_t* start;
  const uint32_t* end;
  const uint32_t* node;
};

__global__ void k_seg_split(const uint32_t* nseg_p, uint32_t nscan, SegLevel L, const uint32_t* benc, const uint32_t* cenc,
                            const uint32_t* bcnt, const uint32_t* bkenc, uint32_t* seg_k, uint32_t* seg_best,
                            uint32_t* seg_mid, uint32_t* seg_cl, uint32_t* seg_cr, uint32_t* counters,
                            uint32_t* sah_axis, float4* nb_lo, float4* nb_hi, uint32_t* child0, uint32_t* child1,
                            uint32_t* parent, uint32_t* nlarge_cnt, uint32_t* small_start, uint32_t* small_end,
                            uint32_t* small_node, uint32_t N2) {
  uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= *nseg_p) {
    if (s < nscan) nlarge_cnt[s] = 0u;  // the scan of the counts runs over nscan entries
    return;
  }
  uint32_t a = L.start[s], b = L.end[s], nd = L.node[s];
  uint32_t n = b - a + 1;
  Bounds bb = dec_bounds(benc + s * 6);
  Bounds cb = dec_bounds(cenc + s * 6);
  int dim = bmax_extent(cb);
  int best;
  uint32_t k;
  sah_decide(bcnt + s * 12, bkenc + s * 12 * 6, bb, n, &best, &k);
  uint32_t mid = (k == n) ? a + n / 2 : a + k;
  seg_k[s] = a + k;
  seg_best[s] = (uint32_t)best;
  seg_mid[s] = mid;
  uint32_t me = N2 + nd;
  sah_axis[nd] = (uint32_t)dim;
  nb_lo[me] = make_float4(bb.lo.x, bb.lo.y, bb.lo.z, 0.0f);
  nb_hi[me] = make_float4(bb.hi.x, bb.hi.y, bb.hi.z, 0.0f);
  uint32_t ln = mid - a, rn = b - mid + 1;
  uint32_t cl = kNone, cr = kNone;
  uint32_t nl = 0;
  // node ids and small-segment slots: one atomic per warp (the ids only
  // label nodes; the flattened tree follows the child links). Deep levels
  // have ~10^4 segments, whose per-child atomics on one counter serialised.
  const uint32_t act = __activemask(), lt = act & ((1u << lane_id()) - 1u);
  const uint32_t leader = __ffs(act) - 1;
  const bool l_node = ln >= 2, r_node = rn >= 2;
  const bool l_small = l_node && ln <= kSmallSeg, r_small = r_node && rn <= kSmallSeg;
  uint32_t bl = __ballot_sync(act, l_node), br = __ballot_sync(act, r_node);
  uint32_t sl = __ballot_sync(act, l_small), sr = __ballot_sync(act, r_small);
  uint32_t node_base = 0, small_base = 0;
  if (lane_id() == leader) {
    uint32_t nn = __popc(bl) + __popc(br), ns = __popc(sl) + __popc(sr);
    if (nn) node_base = atomicAdd(&counters[0], nn);
    if (ns) small_base = atomicAdd(&counters[2], ns);
  }
  node_base = __shfl_sync(act, node_base, leader) + __popc(bl & lt) + __popc(br & lt);
  small_base = __shfl_sync(act, small_base, leader) + __popc(sl & lt) + __popc(sr & lt);
  if (l_node) {
    cl = node_base++;
    child0[me] = N2 + cl;
    parent[N2 + cl] = (me << 1) | 0u;
    if (!l_small) ++nl;
    else {
      uint32_t q = small_base++;
      small_start[q] = a; small_end[q] = mid - 1; small_node[q] = cl;
    }
  }
  if (r_node) {
    cr = node_base;
    child1[me] = N2 + cr;
    parent[N2 + cr] = (me << 1) | 1u;
    if (!r_small) ++nl;
    else {
      uint32_t q = small_base;
      small_start[q] = mid; small_end[q] = b; small_node[q] = cr;
    }
  }
  seg_cl[s] = cl;
  seg_cr[s] = cr;
  nlarge_cnt[s] = nl;
}

// std::partition(first, last, bucket <= best) — the two-pointer swap scheme:
// the r-th "false" element left of the partition point (from the left) trades
// places with the r-th "true" element right of it (from the right).
// The two flags of a position packed as (true << 32) | false, and their
// prefix sums packed the same way (one scan for both).
__device__ __forceinline__ uint32_t lo32(unsigned long long v) { return (uint32_t)(v & 0xFFFFFFFFull); }
__device__ __forceinline__ uint32_t hi32(unsigned long long v) { return (uint32_t)(v >> 32); }
__global__ void k_part_flags(uint32_t T, const uint32_t* pos_seg, const uint32_t* bucket, const uint32_t* seg_k,
                             const uint32_t* seg_best, unsigned long long* ft) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= T) return;
  uint32_t s = pos_seg[p];
  uint32_t f = 0, t = 0;
  if (s != kNone) {
    bool pred = bucket[p] <= seg_best[s];
    uint32_t sp = seg_k[s];
    f = (p < sp && !pred) ? 1u : 0u;
    t = (p >= sp && pred) ? 1u : 0u;
  }
  ft[p] = ((unsigned long long)t << 32) | f;
}
__global__ void k_part_ranks(uint32_t T, SegLevel L, const uint32_t* pos_seg, const unsigned long long* ft,
                             const unsigned long long* ftscan, uint32_t* posF, uint32_t* posT) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= T) return;
  uint32_t s = pos_seg[p];
  if (s == kNone) return;
  uint32_t a = L.start[s], b = L.end[s];
  unsigned long long fp = ft[p], sp = ftscan[p];
  if (lo32(fp)) posF[a + (lo32(sp) - lo32(ftscan[a]))] = p;
  if (hi32(fp)) posT[a + ((hi32(ftscan[b]) + hi32(ft[b])) - (hi32(sp) + 1u))] = p;
}
__global__ void k_part_scatter(uint32_t T, SegLevel L, const uint32_t* pos_seg, const unsigned long long* ft,
                               const unsigned long long* ftscan, const uint32_t* posF, const uint32_t* posT,
                               const uint32_t* cur, uint32_t* nxt) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= T) return;
  uint32_t s = pos_seg[p];
  uint32_t dst = p;
  if (s != kNone) {
    uint32_t a = L.start[s], b = L.end[s];
    unsigned long long fp = ft[p], sp = ftscan[p];
    if (lo32(fp)) dst = posT[a + (lo32(sp) - lo32(ftscan[a]))];
    else if (hi32(fp)) dst = posF[a + ((hi32(ftscan[b]) + hi32(ft[b])) - (hi32(sp) + 1u))];
  }
  nxt[dst] = cur[p];
}

// Size-1 children (a single treelet root) and the next level's large segments.
// nseg_next receives the next level's count: the exclusive scan's last entry
// (nscan exceeds every level's count, so that entry's own count is 0).
__global__ void k_seg_children(const uint32_t* nseg_p, uint32_t nscan, uint32_t* nseg_next, SegLevel L,
                               const uint32_t* seg_mid, const uint32_t* seg_cl, const uint32_t* seg_cr,
                               const uint32_t* nlarge_scan, const uint32_t* cur, const uint32_t* troot,
                               uint32_t* child0, uint32_t* child1, uint32_t* parent, uint32_t* ns_start,
                               uint32_t* ns_end, uint32_t* ns_node, uint32_t N2) {
  uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) *nseg_next = nlarge_scan[nscan - 1];
  if (s >= *nseg_p) return;
  uint32_t a = L.start[s], b = L.end[s], mid = seg_mid[s];
  uint32_t me = N2 + L.node[s];
  uint32_t ln = mid - a, rn = b - mid + 1;
  if (ln == 1) {
    uint32_t r = troot[cur[a]];
    child0[me] = r;
    parent[r] = (me << 1) | 0u;
  }
  if (rn == 1) {
    uint32_t r = troot[cur[b]];
    child1[me] = r;
    parent[r] = (me << 1) | 1u;
  }
  uint32_t q = nlarge_scan[s];
  if (ln > kSmallSeg) {
    ns_start[q] = a; ns_end[q] = mid - 1; ns_node[q] = seg_cl[s];
    ++q;
  }
  if (rn > kSmallSeg) {
    ns_start[q] = mid; ns_end[q] = b; ns_node[q] = seg_cr[s];
  }
}

// Bounds of another lane (shuffled component by component).
__device__ __forceinline__ Bounds shfl_bounds_up(const Bounds& b, uint32_t o) {
  const uint32_t F = 0xFFFFFFFFu;
  return Bounds{V3{__shfl_up_sync(F, b.lo.x, o), __shfl_up_sync(F, b.lo.y, o), __shfl_up_sync(F, b.lo.z, o)},
                V3{__shfl_up_sync(F, b.hi.x, o), __shfl_up_sync(F, b.hi.y, o), __shfl_up_sync(F, b.hi.z, o)}};
}
__device__ __forceinline__ Bounds shfl_bounds_down(const Bounds& b, uint32_t o) {
  const uint32_t F = 0xFFFFFFFFu;
  return Bounds{V3{__shfl_down_sync(F, b.lo.x, o), __shfl_down_sync(F, b.lo.y, o), __shfl_down_sync(F, b.lo.z, o)},
                V3{__shfl_down_sync(F, b.hi.x, o), __shfl_down_sync(F, b.hi.y, o), __shfl_down_sync(F, b.hi.z, o)}};
}

// Segments of 2..32 roots: the whole SAH recursion inside one warp. Bounds
// by warp reductions, buckets by shared-memory atomics, the 11 split costs
// one per lane (sah_decide's float operations on the same boxes) and the sequential
// first-minimum rule by a lexicographic (cost, split) reduction. The
// segment's n - 2 new SAH node ids are reserved with one atomic.
__global__ void k_small_sah(SahArgs A, uint32_t nsmall, const uint32_t* sm_start, const uint32_t* sm_end,
                            const uint32_t* sm_node, uint32_t* cur, uint32_t* counters, uint32_t* sah_axis,
                            float4* nb_lo, float4* nb_hi, uint32_t* child0, uint32_t* child1, uint32_t* parent,
                            uint32_t N2, uint32_t* err) {
  __shared__ uint32_t sh_bcnt[kB / 32][12];
  __shared__ uint32_t sh_benc[kB / 32][12 * 6];
  __shared__ uint32_t sh_stack[kB / 32][3 * 64];
  const uint32_t FULL = 0xFFFFFFFFu;
  const uint32_t w = threadIdx.x >> 5, lane = lane_id();
  uint32_t seg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (seg >= nsmall) return;
  const uint32_t base = sm_start[seg];
  const uint32_t n = sm_end[seg] - base + 1;
  uint32_t item = lane < n ? cur[base + lane] : 0u;
  V3 lo{0, 0, 0}, hi{0, 0, 0};
  if (lane < n) item_bounds(A, item, &lo, &hi);
  uint32_t id_base = 0, id_next = 0;
  if (lane == 0 && n > 2) id_base = atomicAdd(&counters[0], n - 2);
  id_base = __shfl_sync(FULL, id_base, 0);
  uint32_t* stk = sh_stack[w];
  int sp = 0;
  if (lane == 0) {
    stk[0] = 0;
    stk[1] = n - 1;
    stk[2] = sm_node[seg];
  }
  sp = 1;
  __syncwarp();
  uint32_t guard = 0;
  while (sp > 0) {
    if (++guard > 64) {
      if (lane == 0) atomicOr(err, kErrLoopLimit);
      break;
    }
    --sp;
    uint32_t a = stk[3 * sp], b = stk[3 * sp + 1], nd = stk[3 * sp + 2];
    __syncwarp();
    bool act = lane >= a && lane <= b;
    uint32_t cnt = b - a + 1;
    V3 c = mul(add(lo, hi), 0.5f);
    Bounds bb{V3{fdec(__reduce_min_sync(FULL, act ? fenc(lo.x) : 0xFFFFFFFFu)),
                 fdec(__reduce_min_sync(FULL, act ? fenc(lo.y) : 0xFFFFFFFFu)),
                 fdec(__reduce_min_sync(FULL, act ? fenc(lo.z) : 0xFFFFFFFFu))},
              V3{fdec(__reduce_max_sync(FULL, act ? fenc(hi.x) : 0u)), fdec(__reduce_max_sync(FULL, act ? fenc(hi.y) : 0u)),
                 fdec(__reduce_max_sync(FULL, act ? fenc(hi.z) : 0u))}};
    Bounds cb{V3{fdec(__reduce_min_sync(FULL, act ? fenc(c.x) : 0xFFFFFFFFu)),
                 fdec(__reduce_min_sync(FULL, act ? fenc(c.y) : 0xFFFFFFFFu)),
                 fdec(__reduce_min_sync(FULL, act ? fenc(c.z) : 0xFFFFFFFFu))},
              V3{fdec(__reduce_max_sync(FULL, act ? fenc(c.x) : 0u)), fdec(__reduce_max_sync(FULL, act ? fenc(c.y) : 0u)),
                 fdec(__reduce_max_sync(FULL, act ? fenc(c.z) : 0u))}};
    int dim = bmax_extent(cb);
    float dist = comp(cb.hi, dim) - comp(cb.lo, dim);
    uint32_t ib = 0;
    if (act) {
      float cc = (comp(lo, dim) + comp(hi, dim)) * 0.5f;
      float t = (cc - comp(cb.lo, dim)) / dist;
      float bt = 12.0f * t;
      ib = (bt >= 0.0f) ? (uint32_t)bt : 0u;
      if (ib >= 12u) ib = 11u;
    }
    // per-bucket counts and bounds
    uint32_t* bcnt = sh_bcnt[w];
    uint32_t* benc = sh_benc[w];
    if (lane < 12) {
      bcnt[lane] = 0;
      for (int k = 0; k < 6; ++k) benc[lane * 6 + k] = k < 3 ? 0xFFFFFFFFu : 0u;
    }
    __syncwarp();
    if (act) {
      atomicAdd(&bcnt[ib], 1u);
      uint32_t* be = benc + ib * 6;
      atomicMin(be + 0, fenc(lo.x));
      atomicMin(be + 1, fenc(lo.y));
      atomicMin(be + 2, fenc(lo.z));
      atomicMax(be + 3, fenc(hi.x));
      atomicMax(be + 4, fenc(hi.y));
      atomicMax(be + 5, fenc(hi.z));
    }
    __syncwarp();
    // SAH cost of split `lane` (sah_decide's loop body). Lane j < 12 holds
    // bucket j; shuffle scans give each lane the union and count of buckets
    // 0..j (prefix) and j..11 (suffix), so split i takes lane i's prefix and
    // lane i+1's suffix. Min and max of finite coordinates do not depend on
    // the grouping (only a zero's sign could, which no area or cost sees).
    uint32_t cj = lane < 12 ? bcnt[lane] : 0u;
    Bounds pre = (lane < 12 && cj) ? dec_bounds(benc + lane * 6) : bempty();
    Bounds suf = pre;
    uint32_t npre = cj, nsuf = cj;
#pragma unroll
    for (uint32_t o = 1; o < 16; o <<= 1) {
      Bounds u = shfl_bounds_up(pre, o);
      uint32_t nu = __shfl_up_sync(FULL, npre, o);
      Bounds v = shfl_bounds_down(suf, o);
      uint32_t nv = __shfl_down_sync(FULL, nsuf, o);
      if (lane >= o) {
        pre = bunion(u, pre);
        npre += nu;
      }
      if (lane + o < 12) {
        suf = bunion(suf, v);
        nsuf += nv;
      }
    }
    Bounds b1 = shfl_bounds_down(suf, 1);
    uint32_t n1 = __shfl_down_sync(FULL, nsuf, 1);
    float cost = 0.0f;
    if (lane < 11) {
      const Bounds& b0 = pre;
      uint32_t n0 = npre;
      float l = (n0 == 0) ? 0.0f : (float)n0 * barea(b0);
      float r = (n1 == 0) ? 0.0f : (float)n1 * barea(b1);
      cost = (float)(0.125 + (double)((l + r) / barea(bb)));
    }
    // first index of the minimum; a NaN never wins, and a NaN at split 0 keeps split 0
    float c0 = __shfl_sync(FULL, cost, 0);
    float bc = (lane < 11 && !isnan(cost)) ? cost : __int_as_float(0x7f800000);
    uint32_t bi = lane;
    for (int o = 16; o > 0; o >>= 1) {
      float oc = __shfl_xor_sync(FULL, bc, o);
      uint32_t oi = __shfl_xor_sync(FULL, bi, o);
      if (oc < bc || (oc == bc && oi < bi)) {
        bc = oc;
        bi = oi;
      }
    }
    int best = isnan(c0) ? 0 : (int)bi;
    uint32_t k = 0;
    for (int j = 0; j <= best; ++j) k += bcnt[j];
    // two-pointer partition of [a, b] by ib <= best
    uint32_t spt = a + k;
    bool pred = ib <= (uint32_t)best;
    uint32_t fmask = __ballot_sync(FULL, act && lane < spt && !pred);
    uint32_t tmask = __ballot_sync(FULL, act && lane >= spt && pred);
    uint32_t src = lane;
    if (act && lane < spt && !pred) {
      uint32_t r = __popc(fmask & ((1u << lane) - 1u));
      uint32_t m = __brev(tmask);  // r-th highest set bit of tmask
      for (uint32_t q = 0; q < r; ++q) m &= m - 1u;
      src = 31u - (uint32_t)(__ffs(m) - 1);
    } else if (act && lane >= spt && pred) {
      uint32_t r = __popc(tmask & ~((2u << lane) - 1u));  // trues above this lane
      if (lane == 31) r = 0;
      uint32_t m = fmask;
      for (uint32_t q = 0; q < r; ++q) m &= m - 1u;
      src = (uint32_t)(__ffs(m) - 1);
    }
    item = __shfl_sync(FULL, item, src);
    lo.x = __shfl_sync(FULL, lo.x, src); lo.y = __shfl_sync(FULL, lo.y, src);
    lo.z = __shfl_sync(FULL, lo.z, src); hi.x = __shfl_sync(FULL, hi.x, src);
    hi.y = __shfl_sync(FULL, hi.y, src); hi.z = __shfl_sync(FULL, hi.z, src);
    uint32_t mid = (k == cnt) ? a + cnt / 2 : a + k;
    uint32_t me = N2 + nd;
    if (lane == 0) {
      sah_axis[nd] = (uint32_t)dim;
      nb_lo[me] = make_float4(bb.lo.x, bb.lo.y, bb.lo.z, 0.0f);
      nb_hi[me] = make_float4(bb.hi.x, bb.hi.y, bb.hi.z, 0.0f);
    }
    uint32_t ln = mid - a, rn = b - mid + 1;
    uint32_t litem = __shfl_sync(FULL, item, a);
    uint32_t ritem = __shfl_sync(FULL, item, b);
    if (lane == 0) {
      if (ln == 1) {
        uint32_t r = A.troot[litem];
        child0[me] = r;
        parent[r] = (me << 1) | 0u;
      } else {
        uint32_t cl = id_base + id_next++;
        child0[me] = N2 + cl;
        parent[N2 + cl] = (me << 1) | 0u;
        stk[3 * sp] = a; stk[3 * sp + 1] = mid - 1; stk[3 * sp + 2] = cl;
        ++sp;
      }
      if (rn == 1) {
        uint32_t r = A.troot[ritem];
        child1[me] = r;
        parent[r] = (me << 1) | 1u;
      } else {
        uint32_t cr = id_base + id_next++;
        child1[me] = N2 + cr;
        parent[N2 + cr] = (me << 1) | 1u;
        stk[3 * sp] = mid; stk[3 * sp + 1] = b; stk[3 * sp + 2] = cr;
        ++sp;
      }
    }
    sp = __shfl_sync(FULL, sp, 0);
    __syncwarp();
  }
  if (lane < n) cur[base + lane] = item;
}

// Subtree node counts of SAH nodes, bottom-up from the treelet roots.
__global__ void k_sah_sizes(uint32_t T, const uint32_t* troot, const uint32_t* parent, uint32_t* visits, uint32_t* size,
                            const uint32_t* child0, const uint32_t* child1, uint32_t root, uint32_t* err) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  uint32_t cur = troot[t];
  uint32_t guard = 0;
  while (cur != root) {
    if (++guard > (1u << 22)) {
      atomicOr(err, kErrLoopLimit);
      return;
    }
    uint32_t p = parent[cur] >> 1;
    __threadfence();
    if (atomicAdd(&visits[p], 1u) == 0u) return;
    __threadfence();
    size[p] = 1u + __ldcg(&size[child0[p]]) + __ldcg(&size[child1[p]]);
    cur = p;
  }
}

// ---------------------------------------------------------------------------
// A9: flattenBVHTree — depth-first preorder index of every reference node
// ---------------------------------------------------------------------------
__global__ void k_flatten(uint32_t N, uint32_t nsah, uint32_t root, uint32_t M, const uint32_t* skey, const uint32_t* tid,
                          const uint32_t* tstart, const uint32_t* tsize, const uint32_t* rng_lo,
                          const uint32_t* rng_hi, const uint32_t* child0, const uint32_t* parent,
                          const uint32_t* size, const uint32_t* sah_axis, const float4* nb_lo, const float4* nb_hi,
                          uint32_t* lin_node, float* lin_bounds, uint32_t* is_int, uint32_t* depth_max,
                          uint32_t* err) {
  uint32_t X = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t N2 = 2 * N;
  if (X >= N2 + nsah) return;
  uint32_t kind;  // 0 radix interior, 1 leaf, 2 SAH
  uint32_t lo = 0, hi = 0;
  if (X >= N2) {
    kind = 2;
  } else {
    uint32_t t;
    if (X < N) {
      if (X + 1 >= N) return;
      t = tid[X];
      if (tid[X + 1] != t) return;
      lo = rng_lo[X];
      hi = rng_hi[X];
    } else {
      lo = hi = X - N;
      t = tid[lo];
    }
    uint32_t troot_ = treelet_root(t, tstart, tsize, N);
    if (X != troot_) {
      uint32_t p = parent[X] >> 1;
      if (!ref_interior(p, N, rng_lo, rng_hi, skey)) return;
    }
    kind = ref_interior(X, N, rng_lo, rng_hi, skey) ? 0u : 1u;
  }
  uint32_t idx = 0, depth = 0, cur = X;
  while (cur != root) {
    if (++depth > (1u << 22)) {
      atomicOr(err, kErrLoopLimit);
      return;
    }
    uint32_t pw = parent[cur];
    uint32_t p = pw >> 1;
    idx += (pw & 1u) ? 1u + size[child0[p]] : 1u;
    cur = p;
  }
  if (idx >= M) {
    atomicOr(err, kErrBuild);
    return;
  }
  atomicMax(depth_max, depth);
  float4 bl = nb_lo[X], bh = nb_hi[X];
  float* B = lin_bounds + (size_t)idx * 6;
  B[0] = bl.x; B[1] = bl.y; B[2] = bl.z; B[3] = bh.x; B[4] = bh.y; B[5] = bh.z;
  uint32_t* L = lin_node + (size_t)idx * 3;
  if (kind == 1) {
    L[0] = lo;
    L[1] = hi - lo + 1;
    L[2] = 0;
    is_int[idx] = 0;
  } else {
    L[0] = idx + 1 + size[child0[X]];
    L[1] = 0;
    L[2] = (kind == 0) ? (uint32_t)((31 - __clz(skey[lo] ^ skey[hi])) % 3) : sah_axis[X - N2];
    is_int[idx] = 1;
  }
}

// Traversal-layout order of the interior nodes: the root first, then, for
// each interior node in preorder, its interior children side by side. The
// two children a traversal step chooses between share a cache line, and a
// left subtree's records follow its parent's closely. kids[r] counts the
// interior children of the interior node of preorder rank r.
__global__ void k_int_kids(uint32_t M, const uint32_t* lin_node, const uint32_t* is_int, const uint32_t* int_index,
                           uint32_t* kids) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M || !is_int[i]) return;
  uint32_t c1 = lin_node[(size_t)i * 3];
  uint32_t k = (i + 1 < M ? is_int[i + 1] : 0u) + (c1 < M ? is_int[c1] : 0u);
  kids[int_index[i]] = k;
}
// slot[rank] = the node's index in the traversal layout; off = exclusive scan of kids
__global__ void k_int_slots(uint32_t M, const uint32_t* lin_node, const uint32_t* is_int, const uint32_t* int_index,
                            const uint32_t* off, uint32_t* slot) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M || !is_int[i]) return;
  uint32_t r = int_index[i];
  if (r == 0) slot[0] = 0;
  uint32_t s = 1 + off[r];
  uint32_t c0 = i + 1, c1 = lin_node[(size_t)i * 3];
  if (c0 < M && is_int[c0]) slot[int_index[c0]] = s++;
  if (c1 < M && is_int[c1]) slot[int_index[c1]] = s;
}

// Child-pair traversal layout.
__global__ void k_node2(uint32_t M, const uint32_t* lin_node, const float* lin_bounds, const uint32_t* is_int,
                        const uint32_t* int_index, const uint32_t* slot, Node2* out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M || !is_int[i]) return;
  uint32_t c[2] = {i + 1, lin_node[(size_t)i * 3]};
  if (c[0] >= M || c[1] >= M) return;  // malformed tree: traversal guards report it
  int ref[2];
  uint32_t cnt[2];
  float b[2][6];
  for (int k = 0; k < 2; ++k) {
    uint32_t ci = c[k];
    for (int q = 0; q < 6; ++q) b[k][q] = lin_bounds[(size_t)ci * 6 + q];
    if (is_int[ci]) {
      ref[k] = (int)slot[int_index[ci]];
      cnt[k] = 0;
    } else {
      ref[k] = ~(int)lin_node[(size_t)ci * 3];
      cnt[k] = lin_node[(size_t)ci * 3 + 1];
    }
  }
  Node2 nd;
  nd.b0 = make_float4(b[0][0], b[0][3], b[0][1], b[0][4]);
  nd.b1 = make_float4(b[1][0], b[1][3], b[1][1], b[1][4]);
  nd.bz = make_float4(b[0][2], b[0][5], b[1][2], b[1][5]);
  nd.meta = make_int4(ref[0], ref[1], (int)cnt[0], (int)((lin_node[(size_t)i * 3 + 2] << 30) | (cnt[1] & 0x3FFFFFFFu)));
  out[slot[int_index[i]]] = nd;
}

// Primitive records in leaf order: triangles carry their vertices, spheres
// their index (traversal reads the sphere's transform separately).
__global__ void k_prims(SceneView S, const uint32_t* sprim, float4* prims) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= S.N) return;
  uint32_t prim = sprim[p];
  float4* o = prims + (size_t)p * 3;
  if (prim < S.ns) {
    o[0] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(prim));
    o[1] = make_float4(__uint_as_float(prim), 0.0f, 0.0f, __uint_as_float(1u));
    o[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  } else {
    const uint32_t* ix = S.idx + 3 * (size_t)(prim - S.ns);
    const float* a = S.pos + 3 * (size_t)ix[0];
    const float* b = S.pos + 3 * (size_t)ix[1];
    const float* c = S.pos + 3 * (size_t)ix[2];
    o[0] = make_float4(a[0], a[1], a[2], __uint_as_float(prim));
    o[1] = make_float4(b[0], b[1], b[2], __uint_as_float(0u));
    o[2] = make_float4(c[0], c[1], c[2], 0.0f);
  }
}

// ---------------------------------------------------------------------------
// leaf-split traversal layout
// ---------------------------------------------------------------------------
// The reference's leaves hold up to 29 primitives (more where Morton codes
// repeat), so a closest-hit ray tests about 20 primitives. For traversal,
// every leaf of more than kSplitLeaf (and at most kSplitMax) primitives is
// replaced by a complete binary tree of depth d over 2^d equal ranges of its
// sorted positions, d the least depth whose ranges hold at most kSplitLeaf.
// Its records carry axis code 3, which visits child 0 (the lower positions)
// first whatever the ray's direction: the leaf's primitives are tested in
// sorted order as before, so a tie in t still goes to the first position
// and any-hit still finds the first hit of the sequential scan; a range is
// skipped only when the ray misses its box. The records of one leaf are
// stored in heap order (children of record h at 2h+1, 2h+2) after the
// reference layout's records, which are copied unchanged except for the
// child slot that now refers to the range tree's root. 8.4M-ray closest-hit
// microbenchmark (traversal launch): unsplit 4.29 ms; ranges of at most 2
// primitives 4.50, 4 4.32, 6 4.24, 8 4.20, 10 4.20, 12 4.21, 16 4.21 ms (the
// warp-cooperative leaf tests already use the lanes well on large leaves, so
// only coarse ranges pay for their extra box tests).
#ifndef WPBR_SPLIT_LEAF
#define WPBR_SPLIT_LEAF 8
#endif
constexpr uint32_t kSplitLeaf = WPBR_SPLIT_LEAF;
constexpr uint32_t kSplitMax = 4096;
static_assert(kSplitLeaf >= 2, "ranges of the leaf split must not be empty");

__host__ __device__ inline uint32_t split_depth(uint32_t c) {
  if (c <= kSplitLeaf || c > kSplitMax) return 0;
  uint32_t d = 1;
  while (((c + (1u << d) - 1u) >> d) > kSplitLeaf) ++d;
  return d;
}

// Records each child slot of the reference layout adds (slot s = 2 * record + child).
__global__ void k_split_count(uint32_t n_int, const Node2* nodes, uint32_t* cnt, uint32_t* max_d) {
  uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= 2 * n_int) return;
  int4 m = nodes[s >> 1].meta;
  int ref = (s & 1) ? m.y : m.x;
  uint32_t c = (s & 1) ? ((uint32_t)m.w & 0x3FFFFFFFu) : (uint32_t)m.z;
  uint32_t d = ref < 0 ? split_depth(c) : 0u;
  cnt[s] = d ? (1u << d) - 1u : 0u;
  if (d) atomicMax(max_d, d);
}

// One thread per child slot: redirects the slot to its range tree and writes
// the tree's records (boxes = union of the primitive bounds of each range).
// out holds a copy of the reference layout's n_int records on entry.
__global__ void k_split_emit(uint32_t n_int, const Node2* nodes, const uint32_t* off, const uint32_t* sprim,
                             const float4* pb_lo, const float4* pb_hi, uint32_t n_prims, Node2* out, uint32_t n_out,
                             uint32_t* err) {
  uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= 2 * n_int) return;
  uint32_t i = s >> 1, k = s & 1;
  int4 m = nodes[i].meta;
  int ref = k ? m.y : m.x;
  uint32_t c = k ? ((uint32_t)m.w & 0x3FFFFFFFu) : (uint32_t)m.z;
  uint32_t d = ref < 0 ? split_depth(c) : 0u;
  if (!d) return;
  uint32_t first = (uint32_t)(~ref);
  uint32_t nsub = (1u << d) - 1u;
  uint32_t base = n_int + off[s];
  if (first >= n_prims || c > n_prims - first || base > n_out || nsub > n_out - base) {
    atomicOr(err, kErrBuild);
    return;
  }
  // the two children of record i are written by two threads: each one
  // touches only its own words of the meta
  int* pm = reinterpret_cast<int*>(&out[i].meta);
  if (k == 0) {
    pm[0] = (int)base;
    pm[2] = 0;
  } else {
    pm[1] = (int)base;
    pm[3] = (int)((uint32_t)m.w & 0xC0000000u);
  }
  for (uint32_t h = 0; h < nsub; ++h) {
    uint32_t lvl = 31u - (uint32_t)__clz((int)(h + 1u));  // depth of record h, root 0
    uint32_t j = h + 1u - (1u << lvl);
    uint32_t sh = lvl + 1u;  // depth of its children
    float b[2][6];
    int cref[2];
    uint32_t ccnt[2];
    for (uint32_t q = 0; q < 2; ++q) {
      uint32_t piece = 2u * j + q;
      uint32_t lo = (uint32_t)(((uint64_t)piece * c) >> sh);
      uint32_t hi = (uint32_t)(((uint64_t)(piece + 1u) * c) >> sh);
      float bl[3] = {inf_(), inf_(), inf_()}, bh[3] = {-inf_(), -inf_(), -inf_()};
      for (uint32_t p = first + lo; p < first + hi; ++p) {
        uint32_t pr = sprim[p];
        float4 a = pb_lo[pr], z = pb_hi[pr];
        bl[0] = fminf(bl[0], a.x);
        bl[1] = fminf(bl[1], a.y);
        bl[2] = fminf(bl[2], a.z);
        bh[0] = fmaxf(bh[0], z.x);
        bh[1] = fmaxf(bh[1], z.y);
        bh[2] = fmaxf(bh[2], z.z);
      }
      for (int a = 0; a < 3; ++a) {
        b[q][a] = bl[a];
        b[q][3 + a] = bh[a];
      }
      if (sh == d) {
        cref[q] = ~(int)(first + lo);
        ccnt[q] = hi - lo;
      } else {
        cref[q] = (int)(base + 2u * h + 1u + q);
        ccnt[q] = 0;
      }
    }
    Node2 nd;
    nd.b0 = make_float4(b[0][0], b[0][3], b[0][1], b[0][4]);
    nd.b1 = make_float4(b[1][0], b[1][3], b[1][1], b[1][4]);
    nd.bz = make_float4(b[0][2], b[0][5], b[1][2], b[1][5]);
    nd.meta = make_int4(cref[0], cref[1], (int)ccnt[0], (int)((3u << 30) | ccnt[1]));
    out[base + h] = nd;
  }
}

}  // namespace

// Kernel launches of radix_sort_pairs: per 8-bit pass a histogram, the
// scan of the block histograms and a scatter.
uint32_t radix_sort_launches(uint32_t n, int bits) {
  if (n <= 1) return 0;
  uint32_t passes = (uint32_t)((bits + 7) / 8);
  return passes * (2 + scan_launches(256 * div_up(n, kRadixTile)));
}

// Stable LSD radix sort of (key, value) pairs by key bits [0, bits), 8 bits
// per pass (the build's sort kernels); *kres / *vres point at the buffer
// pair that holds the result.
cudaError_t radix_sort_pairs(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, uint32_t n, int bits,
                             DevBuf<uint32_t>& hist, DevBuf<uint32_t>& scan_tmp, cudaStream_t st, uint32_t** kres,
                             uint32_t** vres) {
  uint32_t nblk = div_up(n, kRadixTile);
  cudaError_t e = hist.ensure((size_t)256 * nblk);
  if (e != cudaSuccess) return e;
  uint32_t *kin = k0, *vin = v0, *kout = k1, *vout = v1;
  for (int shift = 0; shift < bits && n > 1; shift += 8) {
    int w = bits - shift < 8 ? bits - shift : 8;
    uint32_t dmask = (1u << w) - 1u;
    k_radix_hist<<<nblk, kB, 0, st>>>(kin, n, shift, dmask, hist.p, nblk);
    e = scan_exclusive(hist.p, hist.p, 256 * nblk, scan_tmp, st);
    if (e != cudaSuccess) return e;
    k_radix_scatter<<<nblk, kB, 0, st>>>(kin, vin, kout, vout, n, shift, dmask, hist.p, nblk);
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  *kres = kin;
  *vres = vin;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------
static wpbr_status bvh_build_tree(wpbr_ctx* ctx);

// A build that fails part way may have reallocated the traversal buffers
// that a render or adjoint setup captured; those setups stop being ready.
wpbr_status bvh_build(wpbr_ctx* ctx) {
  wpbr_status st = bvh_build_tree(ctx);
  if (st != WPBR_OK) {
    ctx->rs.ready = false;
    ctx->adj.ready = false;
  }
  return st;
}

static wpbr_status bvh_build_tree(wpbr_ctx* ctx) {
  if (!ctx->has_scene) return set_err(ctx, WPBR_ERR_NOT_BUILT, "bvh_build: no scene uploaded");
  BvhState& B = ctx->bvh;
  cudaStream_t st = ctx->stream;
  const uint32_t N = ctx->N;
  B.built = false;
  ++ctx->epoch;
  B.N = N;
  SceneView S = scene_view(ctx);
  if (N == 0) {
    B.T = B.M = B.n_int = B.max_depth = 0;
    B.view = BvhView{};
    B.view.empty = 1;
    B.view.stack_cap = kDefaultStackCap;
    B.view.step_cap = kDefaultStepCap;
    B.built = true;
    return WPBR_OK;
  }
  const bool full = (ctx->quirks & WPBR_Q_FULL_MORTON_SORT) != 0;
  const uint32_t NU = 2 * N + N;  // unified id space upper bound (T <= N)
  WPBR_CUDA(B.pb_lo.ensure(N));
  WPBR_CUDA(B.pb_hi.ensure(N));
  WPBR_CUDA(B.centroid.ensure(N));
  WPBR_CUDA(B.codes.ensure(N));
  WPBR_CUDA(B.cb_enc.ensure(8));
  WPBR_CUDA(B.k0.ensure(N));
  WPBR_CUDA(B.k1.ensure(N));
  WPBR_CUDA(B.v0.ensure(N));
  WPBR_CUDA(B.v1.ensure(N));
  uint32_t nblk = div_up(N, kRadixTile);
  WPBR_CUDA(B.hist.ensure((size_t)256 * nblk));
  WPBR_CUDA(B.flags.ensure(N));
  WPBR_CUDA(B.tid.ensure(N));
  WPBR_CUDA(B.tstart.ensure(N));
  WPBR_CUDA(B.tsize.ensure(N));
  WPBR_CUDA(B.troot.ensure(N));
  WPBR_CUDA(B.rng_lo.ensure(N));
  WPBR_CUDA(B.rng_hi.ensure(N));
  WPBR_CUDA(B.child0.ensure(NU));
  WPBR_CUDA(B.child1.ensure(NU));
  WPBR_CUDA(B.parent.ensure(NU));
  WPBR_CUDA(B.visits.ensure(NU));
  WPBR_CUDA(B.size.ensure(NU));
  WPBR_CUDA(B.nb_lo.ensure(NU));
  WPBR_CUDA(B.nb_hi.ensure(NU));
  WPBR_CUDA(B.counters.ensure(8));
  WPBR_CUDA(B.depth_max.ensure(1));

  const unsigned g = div_up(N, kB);
  // A3/A4
  uint32_t cb_init[8] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u, 0u, 0u};
  WPBR_CUDA(cudaMemcpyAsync(B.cb_enc.p, cb_init, sizeof(cb_init), cudaMemcpyHostToDevice, st));
  k_prim_bounds<<<g, kB, 0, st>>>(S, B.pb_lo.p, B.pb_hi.p, B.centroid.p, B.cb_enc.p);
  // A5
  k_morton<<<g, kB, 0, st>>>(N, B.centroid.p, B.cb_enc.p, B.codes.p, B.k0.p, B.v0.p);
  // A6: stable radix sort by the low 24 bits (reference order) or all 30
  uint32_t* kin = B.k0.p;
  uint32_t* vin = B.v0.p;
  uint32_t* kout = B.k1.p;
  uint32_t* vout = B.v1.p;
  int passes = full ? 4 : 3;
  if (N > 1) {
    for (int ps = 0; ps < passes; ++ps) {
      int shift = ps * 8;
      uint32_t dmask = (ps == 3) ? 0x3Fu : 0xFFu;
      k_radix_hist<<<nblk, kB, 0, st>>>(kin, N, shift, dmask, B.hist.p, nblk);
      WPBR_CUDA(scan_exclusive(B.hist.p, B.hist.p, 256 * nblk, B.scan_tmp, st));
      k_radix_scatter<<<nblk, kB, 0, st>>>(kin, vin, kout, vout, N, shift, dmask, B.hist.p, nblk);
      std::swap(kin, kout);
      std::swap(vin, vout);
    }
  }
  B.skey = kin;
  B.sprim = vin;
  // treelets
  k_treelet_flags<<<g, kB, 0, st>>>(B.skey, N, B.flags.p);
  WPBR_CUDA(scan_exclusive(B.flags.p, B.tid.p, N, B.scan_tmp, st));
  uint32_t last_flag = 0, last_scan = 0;
  WPBR_CUDA(cudaMemcpyAsync(&last_flag, B.flags.p + N - 1, 4, cudaMemcpyDeviceToHost, st));
  WPBR_CUDA(cudaMemcpyAsync(&last_scan, B.tid.p + N - 1, 4, cudaMemcpyDeviceToHost, st));
  WPBR_CUDA(cudaStreamSynchronize(st));
  const uint32_t T = last_flag + last_scan;
  B.T = T;
  k_treelet_ids<<<g, kB, 0, st>>>(B.flags.p, B.tid.p, B.tstart.p, N);
  k_treelet_sizes<<<div_up(T, kB), kB, 0, st>>>(B.tstart.p, B.tsize.p, T, N);
  // A7
  WPBR_CUDA(cudaMemsetAsync(B.visits.p, 0, sizeof(uint32_t) * NU, st));
  WPBR_CUDA(cudaMemsetAsync(B.parent.p, 0xFF, sizeof(uint32_t) * NU, st));
  if (N > 1)
    k_karras<<<div_up(N - 1, kB), kB, 0, st>>>(B.skey, B.tid.p, B.tstart.p, B.tsize.p, N, B.rng_lo.p, B.rng_hi.p,
                                               B.child0.p, B.child1.p, B.parent.p);
  k_refit<<<div_up(2 * N, kB), kB, 0, st>>>(N, B.skey, B.sprim, B.tid.p, B.tstart.p, B.tsize.p, B.rng_lo.p,
                                            B.rng_hi.p, B.child0.p, B.child1.p, B.parent.p, B.visits.p, B.size.p,
                                            B.nb_lo.p, B.nb_hi.p, B.pb_lo.p, B.pb_hi.p, B.troot.p, ctx->d_err.p);
  // A8
  const uint32_t N2 = 2 * N;
  uint32_t nsah = 0;
  uint32_t root;
  if (T == 1) {
    WPBR_CUDA(cudaMemcpyAsync(&root, B.troot.p, 4, cudaMemcpyDeviceToHost, st));
    WPBR_CUDA(cudaStreamSynchronize(st));
  } else {
    root = N2;
    WPBR_CUDA(B.cur.ensure(T));
    WPBR_CUDA(B.nxt.ensure(T));
    WPBR_CUDA(B.pos_seg.ensure(T));
    WPBR_CUDA(B.bucket.ensure(T));
    WPBR_CUDA(B.fl.ensure(T));
    WPBR_CUDA(B.ft.ensure(T));
    WPBR_CUDA(B.ftscan.ensure(T));
    WPBR_CUDA(B.posF.ensure(T));
    WPBR_CUDA(B.posT.ensure(T));
    WPBR_CUDA(B.sah_axis.ensure(T));
    uint32_t maxseg = T / (kSmallSeg + 1) + 2;
    WPBR_CUDA(B.seg_start.ensure(2 * maxseg));
    WPBR_CUDA(B.seg_end.ensure(2 * maxseg));
    WPBR_CUDA(B.seg_node.ensure(2 * maxseg));
    WPBR_CUDA(B.seg_k.ensure(maxseg));
    WPBR_CUDA(B.seg_mid.ensure(maxseg));
    WPBR_CUDA(B.seg_dim.ensure(maxseg));  // best bucket
    WPBR_CUDA(B.seg_a.ensure(maxseg));    // left child node
    WPBR_CUDA(B.seg_b.ensure(maxseg));    // right child node
    WPBR_CUDA(B.seg_benc.ensure((size_t)6 * maxseg));
    WPBR_CUDA(B.seg_cenc.ensure((size_t)6 * maxseg));
    WPBR_CUDA(B.seg_bucket_cnt.ensure((size_t)12 * maxseg));
    WPBR_CUDA(B.seg_bucket_enc.ensure((size_t)72 * maxseg));
    WPBR_CUDA(B.small_start.ensure(T));
    WPBR_CUDA(B.small_end.ensure(T));
    WPBR_CUDA(B.small_node.ensure(T));
    WPBR_CUDA(B.flags.ensure(maxseg + 1));  // nlarge counts (reused)
    SahArgs A{N, T, B.troot.p, B.nb_lo.p, B.nb_hi.p};
    // iota
    {
      std::vector<uint32_t> dummy;
    }
    k_fill<<<div_up(T, kB), kB, 0, st>>>(B.pos_seg.p, T, 0);  // placeholder, replaced below
    // cur = 0..T-1
    {
      // write iota via scan of ones
      k_fill<<<div_up(T, kB), kB, 0, st>>>(B.fl.p, T, 1u);
      WPBR_CUDA(scan_exclusive(B.fl.p, B.cur.p, T, B.scan_tmp, st));
    }
    uint32_t h_counters[8] = {1u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
    uint32_t* L_start = B.seg_start.p;
    uint32_t* L_end = B.seg_end.p;
    uint32_t* L_node = B.seg_node.p;
    uint32_t* Nx_start = B.seg_start.p + maxseg;
    uint32_t* Nx_end = B.seg_end.p + maxseg;
    uint32_t* Nx_node = B.seg_node.p + maxseg;
    uint32_t nlarge = 0;
    if (T > kSmallSeg) {
      uint32_t init[3] = {0u, T - 1, 0u};
      WPBR_CUDA(cudaMemcpyAsync(L_start, &init[0], 4, cudaMemcpyHostToDevice, st));
      WPBR_CUDA(cudaMemcpyAsync(L_end, &init[1], 4, cudaMemcpyHostToDevice, st));
      WPBR_CUDA(cudaMemcpyAsync(L_node, &init[2], 4, cudaMemcpyHostToDevice, st));
      nlarge = 1;
    } else {
      uint32_t init[3] = {0u, T - 1, 0u};
      WPBR_CUDA(cudaMemcpyAsync(B.small_start.p, &init[0], 4, cudaMemcpyHostToDevice, st));
      WPBR_CUDA(cudaMemcpyAsync(B.small_end.p, &init[1], 4, cudaMemcpyHostToDevice, st));
      WPBR_CUDA(cudaMemcpyAsync(B.small_node.p, &init[2], 4, cudaMemcpyHostToDevice, st));
      h_counters[2] = 1;
    }
    WPBR_CUDA(cudaMemcpyAsync(B.counters.p, h_counters, sizeof(h_counters), cudaMemcpyHostToDevice, st));
    const unsigned gT = div_up(T, kB);
    const unsigned gS = div_up(maxseg, kB);
    // Level counts live in two device words (this level's and the next's);
    // each level's next count is also copied into a small pinned ring. Level
    // L is queued as soon as level L - 2's copy shows that level L - 1 has
    // large segments, so the GPU always has the next level queued instead of
    // idling through a host round trip per level; the level after the last
    // one is queued too and finds no segment.
    WPBR_CUDA(B.nseg.ensure(2));
    WPBR_CUDA(cudaMemcpyAsync(B.nseg.p, &nlarge, 4, cudaMemcpyHostToDevice, st));
    if (!B.h_nseg) WPBR_CUDA(cudaMallocHost((void**)&B.h_nseg, sizeof(uint32_t) * BvhState::kLevelRing));
    for (cudaEvent_t& ev : B.lev_ev)
      if (!ev) WPBR_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    int level = 0;
    while (nlarge > 0) {  // level 0 has a large segment; later levels end on the ring's counts
      if (level >= 2) {
        const int r = (level - 2) % BvhState::kLevelRing;
        WPBR_CUDA(cudaEventSynchronize(B.lev_ev[r]));
        if (B.h_nseg[r] == 0) break;  // level - 1 had no large segment
      }
      if (level >= 100000) return set_err(ctx, WPBR_ERR_CUDA, "bvh_build: SAH level limit");
      const uint32_t* nseg = B.nseg.p + (level & 1);
      uint32_t* nseg_next = B.nseg.p + ((level + 1) & 1);
      SegLevel L{L_start, L_end, L_node};
      k_pos_seg<<<gT, kB, 0, st>>>(T, nseg, L_start, L_end, B.pos_seg.p);
      k_seg_init<<<gS, kB, 0, st>>>(nseg, B.seg_benc.p, B.seg_cenc.p, B.seg_bucket_cnt.p, B.seg_bucket_enc.p);
      k_seg_reduce<<<gT, kB, 0, st>>>(A, B.cur.p, B.pos_seg.p, B.seg_benc.p, B.seg_cenc.p);
      k_seg_bucket<<<gT, kB, 0, st>>>(A, B.cur.p, B.pos_seg.p, B.seg_cenc.p, B.bucket.p, B.seg_bucket_cnt.p,
                                      B.seg_bucket_enc.p);
      k_seg_split<<<gS, kB, 0, st>>>(
          nseg, maxseg, L, B.seg_benc.p, B.seg_cenc.p, B.seg_bucket_cnt.p, B.seg_bucket_enc.p, B.seg_k.p, B.seg_dim.p,
          B.seg_mid.p, B.seg_a.p, B.seg_b.p, B.counters.p, B.sah_axis.p, B.nb_lo.p, B.nb_hi.p, B.child0.p,
          B.child1.p, B.parent.p, B.flags.p, B.small_start.p, B.small_end.p, B.small_node.p, N2);
      k_part_flags<<<gT, kB, 0, st>>>(T, B.pos_seg.p, B.bucket.p, B.seg_k.p, B.seg_dim.p, B.ft.p);
      WPBR_CUDA(scan_exclusive_pair(B.ft.p, B.ftscan.p, T, B.scan_tmp, st));
      k_part_ranks<<<gT, kB, 0, st>>>(T, L, B.pos_seg.p, B.ft.p, B.ftscan.p, B.posF.p, B.posT.p);
      k_part_scatter<<<gT, kB, 0, st>>>(T, L, B.pos_seg.p, B.ft.p, B.ftscan.p, B.posF.p, B.posT.p, B.cur.p,
                                        B.nxt.p);
      std::swap(B.cur, B.nxt);
      // next level list (ordered by start)
      WPBR_CUDA(scan_exclusive(B.flags.p, B.flags.p, maxseg, B.scan_tmp, st));
      k_seg_children<<<gS, kB, 0, st>>>(nseg, maxseg, nseg_next, L, B.seg_mid.p, B.seg_a.p, B.seg_b.p, B.flags.p,
                                        B.cur.p, B.troot.p, B.child0.p, B.child1.p, B.parent.p, Nx_start, Nx_end,
                                        Nx_node, N2);
      const int r = level % BvhState::kLevelRing;
      WPBR_CUDA(cudaMemcpyAsync(B.h_nseg + r, nseg_next, 4, cudaMemcpyDeviceToHost, st));
      WPBR_CUDA(cudaEventRecord(B.lev_ev[r], st));
      ++level;
      std::swap(L_start, Nx_start);
      std::swap(L_end, Nx_end);
      std::swap(L_node, Nx_node);
    }
    WPBR_CUDA(cudaMemcpyAsync(h_counters, B.counters.p, sizeof(h_counters), cudaMemcpyDeviceToHost, st));
    WPBR_CUDA(cudaStreamSynchronize(st));
    uint32_t nsmall = h_counters[2];
    if (nsmall > 0)
      k_small_sah<<<div_up((uint64_t)nsmall * 32, kB), kB, 0, st>>>(
          A, nsmall, B.small_start.p, B.small_end.p, B.small_node.p, B.cur.p, B.counters.p, B.sah_axis.p, B.nb_lo.p,
          B.nb_hi.p, B.child0.p, B.child1.p, B.parent.p, N2, ctx->d_err.p);
    WPBR_CUDA(cudaMemcpyAsync(h_counters, B.counters.p, sizeof(h_counters), cudaMemcpyDeviceToHost, st));
    WPBR_CUDA(cudaStreamSynchronize(st));
    nsah = h_counters[0];
    if (nsah != T - 1) return set_err(ctx, WPBR_ERR_CUDA, "bvh_build: SAH node count mismatch");
    k_sah_sizes<<<div_up(T, kB), kB, 0, st>>>(T, B.troot.p, B.parent.p, B.visits.p, B.size.p, B.child0.p,
                                              B.child1.p, root, ctx->d_err.p);
  }
  // A9
  uint32_t M = 0;
  WPBR_CUDA(cudaMemcpyAsync(&M, B.size.p + root, 4, cudaMemcpyDeviceToHost, st));
  WPBR_CUDA(cudaStreamSynchronize(st));
  B.M = M;
  WPBR_CUDA(B.lin_node.ensure((size_t)3 * M));
  WPBR_CUDA(B.lin_bounds.ensure((size_t)6 * M));
  WPBR_CUDA(B.is_int.ensure(M));
  WPBR_CUDA(B.int_index.ensure(M));
  WPBR_CUDA(cudaMemsetAsync(B.depth_max.p, 0, 4, st));
  k_flatten<<<div_up(N2 + nsah, kB), kB, 0, st>>>(N, nsah, root, M, B.skey, B.tid.p, B.tstart.p, B.tsize.p, B.rng_lo.p,
                                                   B.rng_hi.p, B.child0.p, B.parent.p, B.size.p, B.sah_axis.p,
                                                   B.nb_lo.p, B.nb_hi.p, B.lin_node.p, B.lin_bounds.p, B.is_int.p,
                                                   B.depth_max.p, ctx->d_err.p);
  WPBR_CUDA(scan_exclusive(B.is_int.p, B.int_index.p, M, B.scan_tmp, st));
  uint32_t last_int = 0, last_idx = 0, depth = 0;
  uint32_t node0[3];
  float b0[6];
  WPBR_CUDA(cudaMemcpyAsync(&last_int, B.is_int.p + M - 1, 4, cudaMemcpyDeviceToHost, st));
  WPBR_CUDA(cudaMemcpyAsync(&last_idx, B.int_index.p + M - 1, 4, cudaMemcpyDeviceToHost, st));
  WPBR_CUDA(cudaMemcpyAsync(&depth, B.depth_max.p, 4, cudaMemcpyDeviceToHost, st));
  WPBR_CUDA(cudaMemcpyAsync(node0, B.lin_node.p, 12, cudaMemcpyDeviceToHost, st));
  WPBR_CUDA(cudaMemcpyAsync(b0, B.lin_bounds.p, 24, cudaMemcpyDeviceToHost, st));
  WPBR_CUDA(cudaStreamSynchronize(st));
  B.n_int = last_int + last_idx;
  B.max_depth = depth;
  WPBR_CUDA(B.nodes2.ensure(B.n_int ? B.n_int : 1));
  WPBR_CUDA(B.prims.ensure((size_t)3 * N));
  if (B.n_int) {
    WPBR_CUDA(B.int_kids.ensure(B.n_int));
    WPBR_CUDA(B.int_slot.ensure(B.n_int));
    k_int_kids<<<div_up(M, kB), kB, 0, st>>>(M, B.lin_node.p, B.is_int.p, B.int_index.p, B.int_kids.p);
    WPBR_CUDA(scan_exclusive(B.int_kids.p, B.int_kids.p, B.n_int, B.scan_tmp, st));
    k_int_slots<<<div_up(M, kB), kB, 0, st>>>(M, B.lin_node.p, B.is_int.p, B.int_index.p, B.int_kids.p,
                                              B.int_slot.p);
    k_node2<<<div_up(M, kB), kB, 0, st>>>(M, B.lin_node.p, B.lin_bounds.p, B.is_int.p, B.int_index.p,
                                          B.int_slot.p, B.nodes2.p);
  }
  k_prims<<<g, kB, 0, st>>>(S, B.sprim, B.prims.p);
  WPBR_CUDA(cudaGetLastError());
  // leaf-split layout (the default binary traversal); a tree whose root is a
  // leaf keeps the reference layout
  uint32_t n_split = 0, split_d = 0;
  if (B.n_int) {
    WPBR_CUDA(B.counters.ensure(8));
    WPBR_CUDA(B.split_cnt.ensure(2 * (size_t)B.n_int));
    WPBR_CUDA(B.split_off.ensure(2 * (size_t)B.n_int));
    WPBR_CUDA(cudaMemsetAsync(B.counters.p + 6, 0, 4, st));
    k_split_count<<<div_up(2 * (size_t)B.n_int, kB), kB, 0, st>>>(B.n_int, B.nodes2.p, B.split_cnt.p,
                                                                  B.counters.p + 6);
    WPBR_CUDA(scan_exclusive(B.split_cnt.p, B.split_off.p, 2 * B.n_int, B.scan_tmp, st));
    uint32_t lastc = 0, lasto = 0;
    WPBR_CUDA(cudaMemcpyAsync(&lastc, B.split_cnt.p + 2 * B.n_int - 1, 4, cudaMemcpyDeviceToHost, st));
    WPBR_CUDA(cudaMemcpyAsync(&lasto, B.split_off.p + 2 * B.n_int - 1, 4, cudaMemcpyDeviceToHost, st));
    WPBR_CUDA(cudaMemcpyAsync(&split_d, B.counters.p + 6, 4, cudaMemcpyDeviceToHost, st));
    WPBR_CUDA(cudaStreamSynchronize(st));
    n_split = lastc + lasto;
    if (n_split) {
      if ((uint64_t)B.n_int + n_split > 0x7FFFFFFFull) return set_err(ctx, WPBR_ERR_OOM, "bvh_build: leaf split too large");
      WPBR_CUDA(B.nodes_split.ensure((size_t)B.n_int + n_split));
      WPBR_CUDA(cudaMemcpyAsync(B.nodes_split.p, B.nodes2.p, sizeof(Node2) * (size_t)B.n_int,
                                cudaMemcpyDeviceToDevice, st));
      k_split_emit<<<div_up(2 * (size_t)B.n_int, kB), kB, 0, st>>>(B.n_int, B.nodes2.p, B.split_off.p, B.sprim,
                                                                   B.pb_lo.p, B.pb_hi.p, N, B.nodes_split.p,
                                                                   B.n_int + n_split, ctx->d_err.p);
      WPBR_CUDA(cudaGetLastError());
    } else {
      split_d = 0;
    }
  }
  BvhView v{};
  v.nodes = n_split ? B.nodes_split.p : B.nodes2.p;
  v.nodes_ref = B.nodes2.p;
  v.n_ref_int = B.n_int;
  v.ref_depth = depth;
  v.prims = B.prims.p;
  v.empty = 0;
  bool root_leaf = node0[1] > 0;
  v.root_ref = root_leaf ? ~(int)node0[0] : 0;
  v.root_count = root_leaf ? node0[1] : 0;
  for (int k = 0; k < 3; ++k) {
    v.root_lo[k] = b0[k];
    v.root_hi[k] = b0[3 + k];
  }
  v.max_depth = depth + split_d;
  v.stack_cap = kDefaultStackCap;
  v.step_cap = kDefaultStepCap;
  v.n_prims = N;
  v.n_int = B.n_int + n_split;
  B.view = v;
  uint32_t derr = 0;
  WPBR_CUDA(cudaMemcpyAsync(&derr, ctx->d_err.p, 4, cudaMemcpyDeviceToHost, st));
  WPBR_CUDA(cudaStreamSynchronize(st));
  if (derr) return set_err(ctx, WPBR_ERR_CUDA, "bvh_build: device invariant violated");
  B.built = true;
  return WPBR_OK;
}

}  // namespace wpbr
