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
//                                                treelet roots: the levels of segments of more
//                                                than 4,096 roots in one cooperative launch
//                                                (k_sah_levels), std::partition's two-pointer
//                                                swap order reproduced with ranks; segments of
//                                                33..4,096 roots in one block each
//                                                (k_medium_sah), of <= 32 in one warp each
//                                                (k_small_sah)
//   flattenBVHTree                               subtree sizes from each SAH node's position
//                                                range (k_sah_sizes), preorder index from the
//                                                recorded depth and child-0 steps (k_flatten),
//                                                then k_node2 / k_prims
//
// Unified node ids: [0, N-1) radix-tree internal nodes, [N, 2N) single
// primitives (sorted position + N), [2N, 2N + T) SAH nodes.
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "common.cuh"
#include "ctx.hpp"
#include "intersect.cuh"

namespace wpbr {

namespace {

constexpr uint32_t kTreeletMask = 0b00111111111111000000000000000000u;  // SLBVH.cpp:301
constexpr int kLeafMax = 30;                                          // SLBVH.cpp:356
constexpr uint32_t kSmallSeg = 32;
// Segments of kSmallSeg + 1 .. kMedSeg treelet roots take their SAH levels in
// one block (k_medium_sah) instead of the cooperative grid.
// 1.31M-triangle build, device ms: 1024 1.775 (4 blocks of 256 per SM),
// 2048 1.718 (2 of 512), 4096 1.691 (1 of 1024).
#ifndef WPBR_MED_SEG
#define WPBR_MED_SEG 4096
#endif
constexpr uint32_t kMedSeg = WPBR_MED_SEG;
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kB = 256;

// Sizes the build finds on the device (read by its later kernels, and by the
// host once, at the end of the build): words of BvhState::dinfo.
enum : uint32_t {
  kInfoT = 0,      // treelets
  kInfoRoot = 1,   // unified id of the root
  kInfoM = 2,      // nodes of the flattened tree
  kInfoSum = 16,   // summary block copied to the host (k_build_summary)
  kInfoWords = 40
};

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ uint32_t div_up_d(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a + b - 1) / b); }

// ---------------------------------------------------------------------------
// exclusive scan (tile scan + recursive block sums) of 32-bit counts, or of
// 64-bit words that pack two 32-bit counts whose sums stay below 2^32 (no
// carry crosses the halves, so one scan gives both prefix sums)
// ---------------------------------------------------------------------------
// The scanned values come from an input functor: an array, or values made
// on the fly by the scan's first launch (no launch of their own).
template <class V>
struct ArrayIn {
  const V* p;
  __device__ __forceinline__ V operator()(uint32_t i) const { return p[i]; }
};
template <class V, class In>
__global__ void k_scan_tile(In in, V* out, uint32_t n, V* bsum) {
  __shared__ V sh[kScanTile];
  __shared__ V wsum[kScanBlock / 32];
  const uint32_t base = blockIdx.x * kScanTile;
  for (int k = 0; k < kScanItems; ++k) {
    uint32_t i = base + threadIdx.x + k * kScanBlock;
    sh[threadIdx.x + k * kScanBlock] = i < n ? in(i) : V(0);
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

// The second launch of a two-level scan: one block per scan tile adds the
// sum of the tile sums before it, reduced here from the unscanned sums (at
// most kScanTile of them) instead of by a scan launch of its own.
template <class V>
__global__ void __launch_bounds__(kScanBlock) k_scan_add_tiles(V* out, uint32_t n, const V* bsum) {
  __shared__ V wsum[kScanBlock / 32];
  const uint32_t j = blockIdx.x;
  if (j == 0) return;  // block-uniform: the first tile is already final
  V part = 0;
  for (uint32_t t = threadIdx.x; t < j; t += kScanBlock) part += bsum[t];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xFFFFFFFFu, part, o);
  if (lane_id() == 0) wsum[threadIdx.x >> 5] = part;
  __syncthreads();
  V off = 0;
#pragma unroll
  for (int q = 0; q < kScanBlock / 32; ++q) off += wsum[q];
  const uint32_t base = j * kScanTile;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const uint32_t i = base + threadIdx.x + k * kScanBlock;
    if (i < n) out[i] += off;
  }
}

template <class V, class In>
cudaError_t scan_exclusive_t(In in, V* out, uint32_t n, V* tmp, size_t tmp_n, cudaStream_t s) {
  struct Lvl {
    const V* in;  // levels above the first: the sums below
    V* out;
    uint32_t n;
    V* sums;
  };
  Lvl lv[8];
  int L = 0;
  size_t off = 0;
  const V* cin = nullptr;
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
  const uint32_t nb0 = div_up(n, kScanTile);
  k_scan_tile<V, In><<<nb0, kScanBlock, 0, s>>>(in, out, n, lv[0].sums);
  if (L == 2) {  // the tile sums fit one tile: two launches
    k_scan_add_tiles<V><<<nb0, kScanBlock, 0, s>>>(out, n, lv[0].sums);
    return cudaGetLastError();
  }
  for (int i = 1; i < L; ++i) {
    uint32_t nb = div_up(lv[i].n, kScanTile);
    k_scan_tile<V, ArrayIn<V>><<<nb, kScanBlock, 0, s>>>(ArrayIn<V>{lv[i].in}, lv[i].out, lv[i].n, lv[i].sums);
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

}  // namespace

// Kernel launches of scan_exclusive over n elements: one tile scan per
// level, one add per level but the last.
uint32_t scan_launches(uint32_t n) {
  if (n == 0) return 0;
  uint32_t levels = 1;
  for (uint32_t m = n; m > (uint32_t)kScanTile; m = div_up(m, kScanTile)) ++levels;
  return levels == 2 ? 2 : 2 * levels - 1;
}

namespace {
template <class In>
cudaError_t scan_exclusive_in(In in, uint32_t* out, uint32_t n, DevBuf<uint32_t>& tmp, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  // tmp layout: level-1 sums, level-2 sums, ...
  size_t need = scan_tmp_need(n);
  cudaError_t e = tmp.ensure(need + 8);
  if (e != cudaSuccess) return e;
  return scan_exclusive_t<uint32_t, In>(in, out, n, tmp.p, need + 8, s);
}
}  // namespace

cudaError_t scan_exclusive(const uint32_t* in, uint32_t* out, uint32_t n, DevBuf<uint32_t>& tmp, cudaStream_t s) {
  return scan_exclusive_in(ArrayIn<uint32_t>{in}, out, n, tmp, s);
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
static_assert(kRadixTile == (int)kSortTile, "the sort's tile size is shared with the key producers");

// Block histograms of one pass (digit-major, block-minor). Each thread
// loads its kRadixItems keys before it counts any (eight loads in flight: the
// kernel reads memory at a rate bound by loads in flight, and the shared
// atomics would otherwise order each load after the previous count). A warp
// whose 32 keys share one digit adds them with one atomic (coherent rays'
// origins often do), the others key by key.
__global__ void k_radix_hist(const uint32_t* keys, uint32_t n, int shift, uint32_t dmask, uint32_t* hist,
                             uint32_t nblocks) {
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  const uint32_t base = blockIdx.x * kRadixTile;
  uint32_t key[kRadixItems];
#pragma unroll
  for (int k = 0; k < kRadixItems; ++k) {
    const uint32_t i = base + threadIdx.x + k * kB;
    key[k] = i < n ? keys[i] : 0u;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kRadixItems; ++k) {
    const uint32_t i = base + threadIdx.x + k * kB;
    const bool valid = i < n;
    const uint32_t d = valid ? (key[k] >> shift) & dmask : 0xFFFFFFFFu;
    if (__all_sync(0xFFFFFFFFu, d == __shfl_sync(0xFFFFFFFFu, d, 0) && valid)) {
      if (lane_id() == 0) atomicAdd(&cnt[d], 32u);
    } else if (valid) {
      atomicAdd(&cnt[d], 1u);
    }
  }
  __syncthreads();
  hist[threadIdx.x * nblocks + blockIdx.x] = cnt[threadIdx.x];
}

// Stable scatter of one pass over tiles of kRadixTile keys. Warp w owns the
// tile's keys [w * 256, (w + 1) * 256) and takes them 32 at a time (lane l,
// round k: key w * 256 + 32 k + l): a __match_any_sync rank within the round
// plus the warp's running count of that digit (a warp-private row of counters
// in shared memory, updated by each digit group's first lane) ranks every key
// among the warp's keys of its digit. One block-wide pass then turns the
// warps' counts into offsets, warps in order, so the keys of one digit keep
// the tile's order, which is the input order. The keys go through a tile
// sorted by digit in shared memory, so each digit's run leaves the block as
// consecutive writes.
__global__ void __launch_bounds__(kB) k_radix_scatter(const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                                                      uint32_t* vout, uint32_t n, int shift, uint32_t dmask,
                                                      const uint32_t* offs, uint32_t nblocks) {
  __shared__ uint32_t s_wc[kB / 32][256];  // per warp and digit: keys, then the warp's offset in the block
  __shared__ uint32_t s_off[256];          // global start of each digit's run of this tile
  __shared__ uint32_t s_lst[256];          // start of each digit in the sorted tile
  __shared__ uint32_t s_wsum[kB / 32];
  __shared__ uint32_t s_key[kRadixTile], s_val[kRadixTile];
  const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
  for (int q = 0; q < kB / 32; ++q) s_wc[q][threadIdx.x] = 0;
  s_off[threadIdx.x] = offs[threadIdx.x * nblocks + blockIdx.x];
  __syncthreads();
  const uint32_t base = blockIdx.x * kRadixTile + w * (32 * kRadixItems);
  uint32_t key[kRadixItems], val[kRadixItems], rk[kRadixItems];
#pragma unroll
  for (int k = 0; k < kRadixItems; ++k) {
    const uint32_t i = base + k * 32 + lane;
    key[k] = i < n ? kin[i] : 0u;
    val[k] = i < n ? (vin ? vin[i] : i) : 0u;  // no values: the pass sorts the keys' positions
  }
  uint32_t* wc = s_wc[w];
#pragma unroll
  for (int k = 0; k < kRadixItems; ++k) {
    const bool valid = base + k * 32 + lane < n;
    const uint32_t d = valid ? ((key[k] >> shift) & dmask) : (256u + lane);
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
    const uint32_t leader = __ffs(peers) - 1;
    uint32_t before = 0;
    if (valid && lane == leader) {
      before = wc[d];
      wc[d] = before + __popc(peers);
    }
    before = __shfl_sync(0xFFFFFFFFu, before, leader);
    rk[k] = before + __popc(peers & lt);
    __syncwarp();
  }
  __syncthreads();
  {  // per digit: the warps' offsets in the block, then the digit's start in the sorted tile
    const uint32_t d = threadIdx.x;
    uint32_t acc = 0;
#pragma unroll
    for (int q = 0; q < kB / 32; ++q) {
      const uint32_t c = s_wc[q][d];
      s_wc[q][d] = acc;
      acc += c;
    }
    uint32_t x = acc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
      if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_wsum[w] = x;
    __syncthreads();
    uint32_t wb = 0;
    for (uint32_t q = 0; q < w; ++q) wb += s_wsum[q];
    s_lst[d] = wb + x - acc;
  }
  __syncthreads();
  // the tile sorted by digit in shared memory, then each digit's run written
  // to its global position by consecutive threads
#pragma unroll
  for (int k = 0; k < kRadixItems; ++k) {
    if (base + k * 32 + lane < n) {
      const uint32_t d = (key[k] >> shift) & dmask;
      const uint32_t lp = s_lst[d] + wc[d] + rk[k];
      s_key[lp] = key[k];
      s_val[lp] = val[k];
    }
  }
  __syncthreads();
  const uint32_t tile0 = blockIdx.x * kRadixTile;
  const uint32_t tile_n = min((uint32_t)kRadixTile, n - tile0);
  for (uint32_t t = threadIdx.x; t < tile_n; t += kB) {
    const uint32_t kt = s_key[t];
    const uint32_t d = (kt >> shift) & dmask;
    const uint32_t pos = s_off[d] + (t - s_lst[d]);
    kout[pos] = kt;
    vout[pos] = s_val[t];
  }
}

// ---------------------------------------------------------------------------
// treelets (top 12 bits of the code)
// ---------------------------------------------------------------------------
// A treelet starts where the top 12 bits of the code change (the scan's input).
struct TreeletFlagIn {
  const uint32_t* skey;
  __device__ __forceinline__ uint32_t operator()(uint32_t i) const {
    return (i == 0 || ((skey[i] ^ skey[i - 1]) & kTreeletMask) != 0) ? 1u : 0u;
  }
};
__global__ void k_treelet_ids(const uint32_t* skey, uint32_t* tid, uint32_t* tstart, uint32_t N, uint32_t* info) {
  const TreeletFlagIn flag{skey};
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const uint32_t f = flag(i);
  uint32_t t = tid[i] + f - 1u;  // inclusive - 1
  tid[i] = t;
  if (f) tstart[t] = i;
  if (i == N - 1) info[kInfoT] = t + 1u;
}
// Primitives of treelet t: from its start to the next treelet's (T treelets).
__device__ __forceinline__ uint32_t treelet_size(uint32_t t, const uint32_t* tstart, const uint32_t* info, uint32_t N) {
  const uint32_t T = info[kInfoT];
  return (t + 1 < T ? tstart[t + 1] : N) - tstart[t];
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

__global__ void k_karras(const uint32_t* skey, const uint32_t* tid, const uint32_t* tstart, const uint32_t* info,
                         uint32_t N, uint32_t* rng_lo, uint32_t* rng_hi, uint32_t* child0, uint32_t* child1,
                         uint32_t* parent) {
  int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= (int)N - 1) return;
  uint32_t t = tid[i];
  KarrasCtx K{skey, tstart[t], tstart[t] + treelet_size(t, tstart, info, N) - 1};
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
__device__ __forceinline__ uint32_t treelet_root(uint32_t t, const uint32_t* tstart, const uint32_t* info, uint32_t N) {
  return treelet_size(t, tstart, info, N) >= 2 ? tstart[t] : N + tstart[t];
}

// An arrival count with acquire-release ordering: the arriving thread's
// earlier writes are visible to the thread whose increment reads its value,
// and that thread's later reads see them.
__device__ __forceinline__ uint32_t arrive_acq_rel(uint32_t* a) {
  uint32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(a) : "memory");
  return old;
}

// Ref leaves compute their bounds; the second child to finish builds each
// parent (atomic arrival counter), up to the treelet root.
__global__ void k_refit(uint32_t N, const uint32_t* skey, const uint32_t* sprim, const uint32_t* tid,
                        const uint32_t* tstart, const uint32_t* info, const uint32_t* rng_lo, const uint32_t* rng_hi,
                        const uint32_t* child0, const uint32_t* child1, const uint32_t* parent, uint32_t* visits,
                        uint32_t* size, float4* nb_lo, float4* nb_hi, const float4* pb_lo, const float4* pb_hi,
                        uint32_t* troot, uint8_t* role, uint32_t* err) {
  uint32_t X = blockIdx.x * blockDim.x + threadIdx.x;
  if (X >= 2 * N) return;
  // role of X in the flattened tree (read by k_flatten): 0 none, 1 ref leaf,
  // 2 ref interior
  uint32_t lo, hi, t;
  if (X < N) {
    t = X + 1 < N ? tid[X] : kNone;
    if (X + 1 >= N || tid[X + 1] != t) {  // not an internal node
      role[X] = 0;
      return;
    }
    lo = rng_lo[X];
    hi = rng_hi[X];
  } else {
    lo = hi = X - N;
    t = tid[lo];
  }
  uint32_t root = treelet_root(t, tstart, info, N);
  bool is_root = (X == root);
  if (!is_root) {
    uint32_t p = parent[X] >> 1;
    if (!ref_interior(p, N, rng_lo, rng_hi, skey)) {  // inside a leaf
      role[X] = 0;
      return;
    }
  }
  if (ref_interior(X, N, rng_lo, rng_hi, skey)) {  // interior: built by its children
    role[X] = 2;
    return;
  }
  role[X] = 1;
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
    if (arrive_acq_rel(&visits[p]) == 0u) return;
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
// Where a node sits on its path from the root: (depth << 16) | the number of
// steps into a child 0. With a node's first final position a, its preorder
// index is that count + a + the treelet nodes of the roots before a (every
// subtree's roots fill a range of positions, child 0's range first).
__device__ __forceinline__ uint32_t ld_child(uint32_t ld, int q) { return ld + (1u << 16) + (q == 0 ? 1u : 0u); }

struct SahArgs {
  uint32_t N;
  const uint32_t* troot;
  const float4* nb_lo;
  const float4* nb_hi;
  uint32_t* sah_rng;  // per SAH node: its first final position and one past its last
  uint32_t* sah_ld;   // per SAH node: ld_child's packed depth and child-0 steps
  uint32_t* t_ld;     // per treelet: the same for its root
};

__device__ __forceinline__ void item_bounds(const SahArgs& A, uint32_t item, V3* lo, V3* hi) {
  uint32_t r = A.troot[item];
  float4 l = A.nb_lo[r], h = A.nb_hi[r];
  *lo = V3{l.x, l.y, l.z};
  *hi = V3{h.x, h.y, h.z};
}

__device__ __forceinline__ Bounds dec_bounds(const uint32_t* e) {
  return Bounds{V3{fdec(e[0]), fdec(e[1]), fdec(e[2])}, V3{fdec(e[3]), fdec(e[4]), fdec(e[5])}};
}
__device__ __forceinline__ Bounds dec_bounds_cg(const uint32_t* e) {
  uint32_t v[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) v[k] = __ldcg(e + k);
  return dec_bounds(v);
}

// Split decision of JobBuildUpperSAH (SLBVH.cpp:504-538) by one warp: lane
// j < 12 holds bucket j's count and bounds. One width-16 shuffle scan gives
// lanes 0..11 the union and count of buckets 0..j (prefix) and lanes 16..27,
// which hold the buckets in reverse order, those of buckets 11-m..11
// (suffix); lane i < 11 costs split i from its prefix and the suffix of
// bucket i+1 (lane 26 - i): the unions of the non-empty buckets on each side,
// as the reference's two inner loops form them. The sequential first-minimum
// rule is a lexicographic (cost, split) reduction: a NaN never wins, and a NaN
// at split 0 keeps split 0. Min and max of finite coordinates do not depend
// on the grouping or operand order; only a zero's sign could, which no area
// or cost sees. Returns the split bucket (warp-uniform); *k_out receives the
// count of buckets 0..best.
__device__ int warp_sah_split(uint32_t cj, const Bounds& bj, float area_all, uint32_t* k_out) {
  const uint32_t FULL = 0xFFFFFFFFu;
  const uint32_t lane = lane_id();
  const uint32_t src = lane < 16 ? lane : 27u - lane;  // lane 16 + m takes bucket 11 - m
  const bool holds = lane < 12 || (lane >= 16 && lane < 28);
  const uint32_t c = __shfl_sync(FULL, cj, src & 31u);
  const Bounds b{V3{__shfl_sync(FULL, bj.lo.x, src & 31u), __shfl_sync(FULL, bj.lo.y, src & 31u),
                    __shfl_sync(FULL, bj.lo.z, src & 31u)},
                 V3{__shfl_sync(FULL, bj.hi.x, src & 31u), __shfl_sync(FULL, bj.hi.y, src & 31u),
                    __shfl_sync(FULL, bj.hi.z, src & 31u)}};
  Bounds acc = (holds && c) ? b : bempty();
  uint32_t nacc = holds ? c : 0u;
#pragma unroll
  for (uint32_t o = 1; o < 16; o <<= 1) {
    const Bounds u{V3{__shfl_up_sync(FULL, acc.lo.x, o, 16), __shfl_up_sync(FULL, acc.lo.y, o, 16),
                      __shfl_up_sync(FULL, acc.lo.z, o, 16)},
                   V3{__shfl_up_sync(FULL, acc.hi.x, o, 16), __shfl_up_sync(FULL, acc.hi.y, o, 16),
                      __shfl_up_sync(FULL, acc.hi.z, o, 16)}};
    const uint32_t nu = __shfl_up_sync(FULL, nacc, o, 16);
    if ((lane & 15u) >= o) {
      acc = bunion(u, acc);
      nacc += nu;
    }
  }
  const uint32_t rs = lane < 11 ? 26u - lane : lane;  // the suffix of bucket lane + 1
  const Bounds b1{V3{__shfl_sync(FULL, acc.lo.x, rs), __shfl_sync(FULL, acc.lo.y, rs), __shfl_sync(FULL, acc.lo.z, rs)},
                  V3{__shfl_sync(FULL, acc.hi.x, rs), __shfl_sync(FULL, acc.hi.y, rs), __shfl_sync(FULL, acc.hi.z, rs)}};
  const uint32_t n1 = __shfl_sync(FULL, nacc, rs);
  float cost = 0.0f;
  if (lane < 11) {
    float l = (nacc == 0) ? 0.0f : (float)nacc * barea(acc);
    float r = (n1 == 0) ? 0.0f : (float)n1 * barea(b1);
    cost = (float)(0.125 + (double)((l + r) / area_all));
  }
  float c0 = __shfl_sync(FULL, cost, 0);
  float bc = (lane < 11 && !isnan(cost)) ? cost : __int_as_float(0x7f800000);
  uint32_t bi = lane;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float oc = __shfl_xor_sync(FULL, bc, o);
    uint32_t oi = __shfl_xor_sync(FULL, bi, o);
    if (oc < bc || (oc == bc && oi < bi)) {
      bc = oc;
      bi = oi;
    }
  }
  int best = isnan(c0) ? 0 : (int)bi;
  *k_out = __shfl_sync(FULL, nacc, best);
  return best;
}

// Bucket of a root (SLBVH.cpp:484-502): the centroid's position along the
// centroid bounds' longest axis in 12 equal parts.
__device__ __forceinline__ uint32_t sah_bucket(const V3& lo, const V3& hi, const Bounds& cb, int dim) {
  float dist = comp(cb.hi, dim) - comp(cb.lo, dim);
  float c = (comp(lo, dim) + comp(hi, dim)) * 0.5f;
  float t = (c - comp(cb.lo, dim)) / dist;
  float bt = 12.0f * t;
  uint32_t ib = (bt >= 0.0f) ? (uint32_t)bt : 0u;
  return ib >= 12u ? 11u : ib;
}

// ---------------------------------------------------------------------------
// A8, segments of more than kMedSeg treelet roots: their SAH levels in one
// cooperative launch (all blocks resident), phases separated by grid
// barriers:
//   A   (root level only) bounds and centroid bounds of the segment
//       (per-tile pre-reduction in shared memory, then global atomics on
//       order-preserving encodings); on later levels phase E of the level
//       before accumulates them by child segment;
//   B   the bucket of every root, bucket counts and bounds of every segment;
//   C1  the split decision of every segment (one warp decides, the same float
//       operations as the sequential loop) and the partition flags of
//       std::partition's two-pointer scheme, scanned within each block's
//       chunk of consecutive tiles, together with the children each segment
//       creates (counted at its first position);
//   C2  every block scans the chunk totals, which gives the global prefix of
//       any position: the select tables (the r-th "false" root left of the
//       partition point and the r-th "true" one right of it, from the right),
//       and, at each segment's first position, its SAH node, its children's
//       node ids, and the next level's segment slots (numbered in position
//       order) or the small-segment queue;
//   E   the swap: each pair trades places, the next level's position arrays
//       are written, single-root children are linked, and the next level's
//       segment bounds are accumulated.
// Segments of 33..kMedSeg roots go to the block-local queue (k_medium_sah),
// segments of 2..32 roots to the warp-local queue (k_small_sah). A tile is
// kCoopBlock consecutive positions. Every grid barrier is bounded: past the
// limit the kernel sets the error word and an abort flag, and every block
// leaves at its next barrier. Indices derived from scanned values are checked
// before use.
// ---------------------------------------------------------------------------
// 1.31M-triangle build, device ms: 512 threads (2 blocks per SM) 1.588,
// 1024 (1 per SM, half the grid barrier's arrivals) 1.575.
#ifndef WPBR_COOP_BLOCK
#define WPBR_COOP_BLOCK 1024
#endif
constexpr int kCoopBlock = WPBR_COOP_BLOCK;
constexpr int kCoopPerSM = 1024 / kCoopBlock;  // resident blocks per SM (64 registers a thread)
constexpr int kCoopWarps = kCoopBlock / 32;
constexpr uint32_t kMaxCoopGrid = 1024;  // blocks of the cooperative grid (chunk prefixes in shared memory)
static_assert(kMaxCoopGrid <= 2 * kCoopBlock, "block_scan_pairs scans two entries a thread");
constexpr uint32_t kSpinLimit = 1u << 24;   // barrier polls (100 ns apart) before giving up
constexpr uint32_t kSegWords = 12;          // bounds lo/hi, centroid bounds lo/hi (encoded)
constexpr uint32_t kBucketWords = 12 * 7;   // per bucket: count, lo xyz, hi xyz (encoded)

struct CoopSah {
  uint32_t N, N2;
  uint32_t maxseg;  // capacity of each set of per-segment arrays
  const uint32_t* T_p;  // treelet count
  const uint32_t* troot;
  float4* nb_lo;  // unified-id node bounds: treelet roots read, SAH nodes written
  float4* nb_hi;
  uint32_t* child0;
  uint32_t* child1;
  uint32_t* parent;
  uint32_t* sah_axis;
  uint32_t* sah_rng;  // per SAH node: first position, one past the last (positions of a segment never change)
  uint32_t* sah_ld;   // per SAH node: packed depth and child-0 steps
  uint32_t* t_ld;     // per treelet: the same for its root
  // per position (two buffers each, swapped every level)
  uint32_t* item[2];
  uint32_t* seg_of[2];
  float4* plo[2];
  float4* phi[2];
  uint8_t* bucket;
  unsigned long long* ftl;  // exclusive prefix of the flags (true << 32) | false within the block's chunk
  uint32_t* rnk;            // rank of a moving root among its segment's "false" (or "true") ones
  uint32_t* posF;
  uint32_t* posT;
  // per segment (two buffers: the level's and the next level's)
  uint32_t* sa[2];
  uint32_t* sb[2];
  uint32_t* snode[2];
  uint32_t* sld[2];   // the segment node's packed depth and child-0 steps
  uint32_t* sacc[2];  // kSegWords per segment
  uint32_t* sbk[2];   // kBucketWords per segment
  uint4* sdec;        // partition point, mid, left and right child segment (kNone: not large)
  uint32_t* sbest;
  unsigned long long* segpre;  // (large << 32 | new-node) children before the segment, within its chunk
  unsigned long long* btot;    // per block: its chunk's flag totals and children totals
  // level words, two sets: [0] large segments, [1] SAH nodes allocated before
  // the level
  uint32_t* lvl;
  uint32_t* small_start;
  uint32_t* small_end;
  uint32_t* small_node;
  uint32_t* med_start;
  uint32_t* med_end;
  uint32_t* med_node;
  uint32_t* med_ld;
  uint32_t* small_ld;
  uint32_t* counters;  // [0] SAH nodes allocated, [2] small segments queued, [3] medium segments queued
  uint32_t* root_out;  // unified id of the tree's root
  uint32_t* bar;       // grid barrier: [0] arrivals, [1] generation, [2] abort
  uint32_t* err;
};

__device__ __forceinline__ uint32_t ld_vol(const uint32_t* p) { return *(const volatile uint32_t*)p; }

// Grid-wide barrier of the cooperative launch. false: some block gave up
// waiting (abort set), and the caller leaves the kernel.
__device__ bool coop_sync(uint32_t* bar, uint32_t* err) {
  __shared__ uint32_t s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t gen = ld_vol(bar + 1);
    __threadfence();
    bool ok = true;
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      uint32_t spins = 0;
      while (ld_vol(bar + 1) == gen) {
        if (ld_vol(bar + 2)) {
          ok = false;
          break;
        }
        if (++spins > kSpinLimit) {
          atomicOr(bar + 2, 1u);
          atomicOr(err, kErrLoopLimit);
          ok = false;
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
    if (ld_vol(bar + 2)) ok = false;
    s_ok = ok ? 1u : 0u;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ unsigned long long warp_incl_scan64(unsigned long long v) {
  const uint32_t lane = lane_id();
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, v, o);
    if (lane >= (uint32_t)o) v += y;
  }
  return v;
}

// Exclusive scan of two 64-bit values over n <= 2 * blockDim.x entries of
// src (pairs, entry i at src[2i], src[2i + 1]) into shared arrays; returns the
// totals. Every thread of the block calls it.
__device__ void block_scan_pairs(const unsigned long long* src, uint32_t n, unsigned long long* o1,
                                 unsigned long long* o2, unsigned long long* w1, unsigned long long* w2,
                                 unsigned long long* tot) {
  const uint32_t lane = lane_id(), wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const uint32_t e0 = 2 * threadIdx.x, e1 = e0 + 1;
  unsigned long long a1 = e0 < n ? __ldcg(src + 2 * e0) : 0ull, a2 = e0 < n ? __ldcg(src + 2 * e0 + 1) : 0ull;
  unsigned long long b1 = e1 < n ? __ldcg(src + 2 * e1) : 0ull, b2 = e1 < n ? __ldcg(src + 2 * e1 + 1) : 0ull;
  unsigned long long x1 = warp_incl_scan64(a1 + b1), x2 = warp_incl_scan64(a2 + b2);
  if (lane == 31) {
    w1[wid] = x1;
    w2[wid] = x2;
  }
  __syncthreads();
  if (wid == 0) {
    unsigned long long v1 = lane < nw ? w1[lane] : 0ull, v2 = lane < nw ? w2[lane] : 0ull;
    unsigned long long y1 = warp_incl_scan64(v1), y2 = warp_incl_scan64(v2);
    if (lane < nw) {
      w1[lane] = y1 - v1;
      w2[lane] = y2 - v2;
    }
    if (lane == 31) {
      tot[0] = y1;
      tot[1] = y2;
    }
  }
  __syncthreads();
  const unsigned long long base1 = w1[wid] + x1 - (a1 + b1), base2 = w2[wid] + x2 - (a2 + b2);
  if (e0 < n) {
    o1[e0] = base1;
    o2[e0] = base2;
  }
  if (e1 < n) {
    o1[e1] = base1 + a1;
    o2[e1] = base2 + a2;
  }
  __syncthreads();
}

__device__ __forceinline__ void init_segment(uint32_t* acc, uint32_t* bk) {
  for (int k = 0; k < (int)kSegWords; ++k) acc[k] = ((k / 3) % 2 == 0) ? 0xFFFFFFFFu : 0u;
  for (int b = 0; b < 12; ++b) {
    bk[b * 7] = 0u;
    for (int k = 0; k < 6; ++k) bk[b * 7 + 1 + k] = k < 3 ? 0xFFFFFFFFu : 0u;
  }
}

// A large segment met by a block's batch of positions (shared memory). A
// batch of kBatch consecutive positions meets at most
// 2 + (kBatch - 2) / (kMedSeg + 1) large segments (each holds more than
// kMedSeg positions), and their ids are consecutive (segments are numbered in
// position order), so s & (kSlots - 1) names each one's slot without
// collisions; their large children, two at most each, take twice as many.
struct SlotSeg {
  uint32_t s, a, b, node;
  uint32_t spt, mid, best, kk;
  uint32_t cl, cr, ld;
  unsigned long long ga, ge;  // global flag prefixes at a and at b + 1 (phase C2)
  float cb[6];                // centroid bounds lo xyz, hi xyz (phase B)
};
constexpr int kBatchTiles = 4;
constexpr uint32_t kBatch = kBatchTiles * kCoopBlock;
constexpr uint32_t kSlots = 8;
static_assert(2 + (kBatch - 2) / (kMedSeg + 1) <= kSlots, "a batch meets at most kSlots large segments");

// Positions of the block's batch starting at `base` (k-th tile of the batch:
// base + k * kCoopBlock + thread) and their segments; marks the slots the
// batch meets. Leaves one __syncthreads after the marks.
__device__ __forceinline__ void batch_segments(const uint32_t* seg_of, uint32_t base, uint32_t end, uint32_t nseg,
                                               uint32_t* p, uint32_t* s, SlotSeg* sl) {
#pragma unroll
  for (int k = 0; k < kBatchTiles; ++k) {
    p[k] = base + k * kCoopBlock + threadIdx.x;
    uint32_t v = p[k] < end ? __ldcg(seg_of + p[k]) : kNone;
    s[k] = v < nseg ? v : kNone;
  }
  if (threadIdx.x < kSlots) sl[threadIdx.x].s = kNone;
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kBatchTiles; ++k)
    if (s[k] != kNone) sl[s[k] & (kSlots - 1)].s = s[k];
  __syncthreads();
}

__global__ void __launch_bounds__(kCoopBlock, kCoopPerSM) k_sah_levels(CoopSah C) {
  __shared__ SlotSeg sl[kSlots];
  __shared__ uint32_t s_acc[kSlots * kSegWords];
  __shared__ uint32_t s_nacc[2 * kSlots * kSegWords];  // phase E: the next level's bounds by child segment
  __shared__ uint32_t s_nid[2 * kSlots];
  __shared__ uint32_t s_bk[kSlots * kBucketWords];
  __shared__ unsigned long long s_w1[kBatchTiles][kCoopWarps], s_w2[kBatchTiles][kCoopWarps];
  __shared__ unsigned long long s_t1[kBatchTiles], s_t2[kBatchTiles];
  __shared__ unsigned long long s_tot[2];
  __shared__ unsigned long long s_bp1[kMaxCoopGrid], s_bp2[kMaxCoopGrid];  // chunk prefixes (phase C2)
  const uint32_t FULL = 0xFFFFFFFFu;
  const uint32_t T = *C.T_p;
  const uint32_t lane = lane_id(), wid = threadIdx.x >> 5;

  // ---- set-up: one treelet, a small segment, or level 0 over every root ----
  if (T <= 1) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      *C.root_out = T == 1 ? C.troot[0] : kNone;
      if (T == 1) C.t_ld[0] = 0u;
      C.counters[0] = 0u;
      C.counters[2] = 0u;
      C.counters[3] = 0u;
      C.counters[4] = 0u;
      C.counters[5] = 0u;
      C.counters[1] = 0u;
      C.counters[7] = 0u;
    }
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *C.root_out = C.N2;  // SAH node 0
  if (T <= kMedSeg) {  // the root segment is small or medium: no cooperative level
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < T; p += gridDim.x * blockDim.x) C.item[0][p] = p;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      uint32_t* st = T <= kSmallSeg ? C.small_start : C.med_start;
      uint32_t* en = T <= kSmallSeg ? C.small_end : C.med_end;
      uint32_t* nd = T <= kSmallSeg ? C.small_node : C.med_node;
      st[0] = 0u;
      en[0] = T - 1;
      nd[0] = 0u;
      (T <= kSmallSeg ? C.small_ld : C.med_ld)[0] = 0u;
      C.counters[0] = 1u;
      C.counters[2] = T <= kSmallSeg ? 1u : 0u;
      C.counters[3] = T <= kSmallSeg ? 0u : 1u;
      C.counters[4] = 0u;
      C.counters[5] = 0u;
      C.counters[1] = 0u;
      C.counters[7] = 0u;
    }
    return;
  }
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < T; p += gridDim.x * blockDim.x) {
    uint32_t r = C.troot[p];
    C.item[0][p] = p;
    C.seg_of[0][p] = 0u;
    C.plo[0][p] = C.nb_lo[r];
    C.phi[0][p] = C.nb_hi[r];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    C.sa[0][0] = 0u;
    C.sb[0][0] = T - 1;
    C.snode[0][0] = 0u;
    C.sld[0][0] = 0u;
    init_segment(C.sacc[0], C.sbk[0]);
    C.lvl[0] = 1u;  // one large segment
    C.lvl[1] = 1u;  // the root is SAH node 0
    C.counters[2] = 0u;  // the queues fill by atomics
    C.counters[3] = 0u;
    C.counters[4] = 0u;
    C.counters[5] = 0u;
    C.counters[1] = 0u;
    C.counters[7] = 0u;
  }
  if (!coop_sync(C.bar, C.err)) return;

  // every phase walks the block's chunk of consecutive positions in batches
  const uint32_t ntiles = div_up_d(T, kCoopBlock);
  const uint32_t chunk = div_up_d(ntiles, gridDim.x) * kCoopBlock;
  const uint32_t c0 = min(blockIdx.x * chunk, T), c1 = min(c0 + chunk, T);
  uint32_t par = 0;
  for (uint32_t level = 0;; ++level) {
    if (level > T) {  // every level splits each large segment: T levels at most
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(C.err, kErrLoopLimit);
      return;
    }
    const uint32_t nx = par ^ 1u;
    const uint32_t* Lc = C.lvl + 8 * par;
    uint32_t* Ln = C.lvl + 8 * nx;
    const uint32_t* seg_of = C.seg_of[par];
    const float4* plo = C.plo[par];
    const float4* phi = C.phi[par];
    uint32_t* sacc = C.sacc[par];
    uint32_t* sbk = C.sbk[par];
    const uint32_t* sa = C.sa[par];
    const uint32_t* sb = C.sb[par];
    const uint32_t* snode = C.snode[par];
    const uint32_t nseg = __ldcg(Lc);
    if (nseg > C.maxseg) {  // every block reads the same word: all leave together
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(C.err, kErrBuild);
      return;
    }
    uint32_t p[kBatchTiles], s[kBatchTiles];

    // ---- A: segment bounds and centroid bounds (the root level; later
    // levels' come from the swap phase before them) ----
    if (level == 0) {
      for (uint32_t base = c0; base < c1; base += kBatch) {
        batch_segments(seg_of, base, c1, nseg, p, s, sl);
        for (uint32_t k = threadIdx.x; k < kSlots * kSegWords; k += blockDim.x)
          s_acc[k] = (((k % kSegWords) / 3) % 2 == 0) ? 0xFFFFFFFFu : 0u;
        __syncthreads();
        float4 l[kBatchTiles], h[kBatchTiles];
  #pragma unroll
        for (int k = 0; k < kBatchTiles; ++k)
          if (s[k] != kNone) {
            l[k] = __ldcg(plo + p[k]);
            h[k] = __ldcg(phi + p[k]);
          }
  #pragma unroll 1
        for (int k = 0; k < kBatchTiles; ++k) {
          const uint32_t sk = s[k];
          if (!__any_sync(FULL, sk != kNone)) continue;
          uint32_t e[12];
          if (sk != kNone) {
            V3 lo{l[k].x, l[k].y, l[k].z}, hi{h[k].x, h[k].y, h[k].z};
            V3 c = mul(add(lo, hi), 0.5f);
            e[0] = fenc(lo.x); e[1] = fenc(lo.y); e[2] = fenc(lo.z);
            e[3] = fenc(hi.x); e[4] = fenc(hi.y); e[5] = fenc(hi.z);
            e[6] = fenc(c.x); e[7] = fenc(c.y); e[8] = fenc(c.z);
            e[9] = e[6]; e[10] = e[7]; e[11] = e[8];
          } else {
  #pragma unroll
            for (int q = 0; q < 12; ++q) e[q] = ((q / 3) % 2 == 0) ? 0xFFFFFFFFu : 0u;
          }
          const uint32_t s0 = __shfl_sync(FULL, sk, 0);
          if (__all_sync(FULL, sk == s0)) {  // one segment across the warp
  #pragma unroll
            for (int q = 0; q < 12; ++q)
              e[q] = ((q / 3) % 2 == 0) ? __reduce_min_sync(FULL, e[q]) : __reduce_max_sync(FULL, e[q]);
            if (lane == 0) {
              uint32_t* r = s_acc + (s0 & (kSlots - 1)) * kSegWords;
              for (int q = 0; q < 12; ++q) {
                if ((q / 3) % 2 == 0)
                  atomicMin(r + q, e[q]);
                else
                  atomicMax(r + q, e[q]);
              }
            }
          } else {  // runs of one segment meet at the run's first lane
  #pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
              uint32_t so = __shfl_down_sync(FULL, sk, o);
              bool take = (lane + o < 32) && (so == sk) && (sk != kNone);
  #pragma unroll
              for (int q = 0; q < 12; ++q) {
                uint32_t y = __shfl_down_sync(FULL, e[q], o);
                if (take) e[q] = ((q / 3) % 2 == 0) ? min(e[q], y) : max(e[q], y);
              }
            }
            uint32_t sp = __shfl_up_sync(FULL, sk, 1);
            if (sk != kNone && (lane == 0 || sp != sk)) {
              uint32_t* r = s_acc + (sk & (kSlots - 1)) * kSegWords;
              for (int q = 0; q < 12; ++q) {
                if ((q / 3) % 2 == 0)
                  atomicMin(r + q, e[q]);
                else
                  atomicMax(r + q, e[q]);
              }
            }
          }
        }
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < kSlots * kSegWords; k += blockDim.x) {
          const uint32_t seg = sl[k / kSegWords].s;
          if (seg == kNone) continue;
          const uint32_t v = s_acc[k];
          const bool mn = ((k % kSegWords) / 3) % 2 == 0;
          if (v == (mn ? 0xFFFFFFFFu : 0u)) continue;
          uint32_t* dst = sacc + (size_t)seg * kSegWords + (k % kSegWords);
          if (mn)
            atomicMin(dst, v);
          else
            atomicMax(dst, v);
        }
        __syncthreads();
      }
      if (!coop_sync(C.bar, C.err)) return;
    }

    // ---- B: buckets ----
    for (uint32_t base = c0; base < c1; base += kBatch) {
      batch_segments(seg_of, base, c1, nseg, p, s, sl);
      for (uint32_t k = threadIdx.x; k < kSlots * kBucketWords; k += blockDim.x)
        s_bk[k] = (k % 7 == 0) ? 0u : ((k % 7) <= 3 ? 0xFFFFFFFFu : 0u);
      if (threadIdx.x < kSlots * 6) {
        const uint32_t j = threadIdx.x / 6, q = threadIdx.x % 6;
        const uint32_t seg = sl[j].s;
        if (seg != kNone) sl[j].cb[q] = fdec(__ldcg(sacc + (size_t)seg * kSegWords + 6 + q));
      }
      __syncthreads();
      float4 l[kBatchTiles], h[kBatchTiles];
#pragma unroll
      for (int k = 0; k < kBatchTiles; ++k)
        if (s[k] != kNone) {
          l[k] = __ldcg(plo + p[k]);
          h[k] = __ldcg(phi + p[k]);
        }
#pragma unroll 1
      for (int k = 0; k < kBatchTiles; ++k) {
        const uint32_t sk = s[k];
        if (!__any_sync(FULL, sk != kNone)) continue;
        V3 lo{0, 0, 0}, hi{0, 0, 0};
        uint32_t ib = 0;
        if (sk != kNone) {
          lo = V3{l[k].x, l[k].y, l[k].z};
          hi = V3{h[k].x, h[k].y, h[k].z};
          const float* cbf = sl[sk & (kSlots - 1)].cb;
          Bounds cb{V3{cbf[0], cbf[1], cbf[2]}, V3{cbf[3], cbf[4], cbf[5]}};
          ib = sah_bucket(lo, hi, cb, bmax_extent(cb));
          C.bucket[p[k]] = (uint8_t)ib;
        }
        const uint32_t s0 = __shfl_sync(FULL, sk, 0);
        if (s0 != kNone && __all_sync(FULL, sk == s0)) {  // one segment: reduce per present bucket
          uint32_t present = __reduce_or_sync(FULL, 1u << ib);
          uint32_t* base_bk = s_bk + (s0 & (kSlots - 1)) * kBucketWords;
          while (present) {
            const uint32_t j = __ffs(present) - 1;
            present &= present - 1;
            const bool in = ib == j;
            const uint32_t cnt = __popc(__ballot_sync(FULL, in));
            uint32_t v0 = __reduce_min_sync(FULL, in ? fenc(lo.x) : 0xFFFFFFFFu);
            uint32_t v1 = __reduce_min_sync(FULL, in ? fenc(lo.y) : 0xFFFFFFFFu);
            uint32_t v2 = __reduce_min_sync(FULL, in ? fenc(lo.z) : 0xFFFFFFFFu);
            uint32_t v3 = __reduce_max_sync(FULL, in ? fenc(hi.x) : 0u);
            uint32_t v4 = __reduce_max_sync(FULL, in ? fenc(hi.y) : 0u);
            uint32_t v5 = __reduce_max_sync(FULL, in ? fenc(hi.z) : 0u);
            if (lane == 0) {
              uint32_t* d = base_bk + j * 7;
              atomicAdd(d, cnt);
              atomicMin(d + 1, v0);
              atomicMin(d + 2, v1);
              atomicMin(d + 3, v2);
              atomicMax(d + 4, v3);
              atomicMax(d + 5, v4);
              atomicMax(d + 6, v5);
            }
          }
        } else if (sk != kNone) {
          uint32_t* d = s_bk + (sk & (kSlots - 1)) * kBucketWords + ib * 7;
          atomicAdd(d, 1u);
          atomicMin(d + 1, fenc(lo.x));
          atomicMin(d + 2, fenc(lo.y));
          atomicMin(d + 3, fenc(lo.z));
          atomicMax(d + 4, fenc(hi.x));
          atomicMax(d + 5, fenc(hi.y));
          atomicMax(d + 6, fenc(hi.z));
        }
      }
      __syncthreads();
      for (uint32_t k = threadIdx.x; k < kSlots * 12; k += blockDim.x) {
        const uint32_t seg = sl[k / 12].s;
        const uint32_t* src = s_bk + k * 7;
        const uint32_t c = src[0];
        if (seg == kNone || c == 0) continue;
        uint32_t* d = sbk + (size_t)seg * kBucketWords + (k % 12) * 7;
        atomicAdd(d, c);
        for (int q = 1; q <= 3; ++q) atomicMin(d + q, src[q]);
        for (int q = 4; q <= 6; ++q) atomicMax(d + q, src[q]);
      }
      __syncthreads();
    }
    if (!coop_sync(C.bar, C.err)) return;

    // ---- C1: decisions, partition flags, scans within each block's chunk ----
    {
      unsigned long long carry1 = 0, carry2 = 0;
      for (uint32_t base = c0; base < c1; base += kBatch) {
        batch_segments(seg_of, base, c1, nseg, p, s, sl);
        // one decision per segment the batch meets, one warp each
        for (uint32_t j = wid; j < kSlots; j += kCoopWarps) {
          const uint32_t sv = sl[j].s;
          if (sv == kNone) continue;
          const uint32_t* bk = sbk + (size_t)sv * kBucketWords;
          uint32_t cj = 0;
          Bounds bj = bempty();
          if (lane < 12) {
            cj = __ldcg(bk + lane * 7);
            if (cj) bj = dec_bounds_cg(bk + lane * 7 + 1);
          }
          Bounds bb = dec_bounds_cg(sacc + (size_t)sv * kSegWords);
          uint32_t kv;
          int bv = warp_sah_split(cj, bj, barea(bb), &kv);
          if (lane == 0) {
            const uint32_t a = __ldcg(sa + sv), b = __ldcg(sb + sv);
            const uint32_t n = b - a + 1;
            sl[j].a = a;
            sl[j].b = b;
            sl[j].best = (uint32_t)bv;
            sl[j].kk = kv;
            sl[j].spt = a + kv;
            sl[j].mid = (kv == n) ? a + n / 2 : a + kv;
          }
        }
        __syncthreads();
        unsigned long long v1[kBatchTiles], v2[kBatchTiles], i1[kBatchTiles], i2[kBatchTiles];
        uint8_t bkt[kBatchTiles];
#pragma unroll
        for (int k = 0; k < kBatchTiles; ++k) bkt[k] = s[k] != kNone ? __ldcg(C.bucket + p[k]) : (uint8_t)0;
#pragma unroll
        for (int k = 0; k < kBatchTiles; ++k) {
          bool fF = false, fT = false;
          uint32_t nn = 0, nl = 0;
          if (s[k] != kNone) {
            const SlotSeg& g = sl[s[k] & (kSlots - 1)];
            const bool pred = bkt[k] <= g.best;
            fF = p[k] < g.spt && !pred;
            fT = p[k] >= g.spt && pred;
            if (p[k] == g.a) {
              const uint32_t ln = g.mid - g.a, rn = g.b - g.mid + 1;
              nn = (uint32_t)(ln >= 2) + (uint32_t)(rn >= 2);
              nl = (uint32_t)(ln > kMedSeg) + (uint32_t)(rn > kMedSeg);
            }
          }
          v1[k] = ((unsigned long long)fT << 32) | (unsigned long long)fF;
          v2[k] = ((unsigned long long)nl << 32) | (unsigned long long)nn;
          i1[k] = warp_incl_scan64(v1[k]);
          i2[k] = warp_incl_scan64(v2[k]);
          if (lane == 31) {
            s_w1[k][wid] = i1[k];
            s_w2[k][wid] = i2[k];
          }
        }
        __syncthreads();
        if (wid < (uint32_t)kBatchTiles) {  // warp k scans tile k's warp totals
          const uint32_t k = wid;
          unsigned long long w1 = lane < kCoopWarps ? s_w1[k][lane] : 0ull;
          unsigned long long w2 = lane < kCoopWarps ? s_w2[k][lane] : 0ull;
          unsigned long long x1 = warp_incl_scan64(w1), x2 = warp_incl_scan64(w2);
          if (lane < kCoopWarps) {
            s_w1[k][lane] = x1 - w1;
            s_w2[k][lane] = x2 - w2;
          }
          if (lane == 31) {
            s_t1[k] = x1;
            s_t2[k] = x2;
          }
        }
        __syncthreads();
        unsigned long long o1 = carry1, o2 = carry2;
#pragma unroll
        for (int k = 0; k < kBatchTiles; ++k) {
          if (p[k] < c1) C.ftl[p[k]] = o1 + s_w1[k][wid] + (i1[k] - v1[k]);
          if (s[k] != kNone) {
            const SlotSeg& g = sl[s[k] & (kSlots - 1)];
            if (p[k] == g.a) {
              C.segpre[s[k]] = o2 + s_w2[k][wid] + (i2[k] - v2[k]);
              C.sdec[s[k]] = make_uint4(g.spt, g.mid, kNone, kNone);
              C.sbest[s[k]] = g.best;
            }
          }
          o1 += s_t1[k];
          o2 += s_t2[k];
        }
        carry1 = o1;
        carry2 = o2;
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        C.btot[2 * blockIdx.x] = carry1;
        C.btot[2 * blockIdx.x + 1] = carry2;
      }
    }
    if (!coop_sync(C.bar, C.err)) return;

    // ---- C2: prefixes over the chunks, select tables, SAH nodes, children ----
    block_scan_pairs(C.btot, gridDim.x, s_bp1, s_bp2, &s_w1[0][0], &s_w2[0][0], s_tot);
    {
      const unsigned long long gtot1 = s_tot[0], gtot2 = s_tot[1];
      const uint32_t node_base = __ldcg(Lc + 1);
      if (blockIdx.x == 0 && threadIdx.x == 0) {  // the next level's words
        const uint32_t tot_nn = (uint32_t)(gtot2 & 0xFFFFFFFFull), tot_nl = (uint32_t)(gtot2 >> 32);
        Ln[0] = tot_nl;
        Ln[1] = node_base + tot_nn;
      }
      for (uint32_t base = c0; base < c1; base += kBatch) {
        batch_segments(seg_of, base, c1, nseg, p, s, sl);
        if (threadIdx.x < kSlots) {
          SlotSeg& g = sl[threadIdx.x];
          if (g.s != kNone) {
            g.a = __ldcg(sa + g.s);
            g.b = __ldcg(sb + g.s);
            g.spt = __ldcg(&C.sdec[g.s].x);
            g.mid = __ldcg(&C.sdec[g.s].y);
            g.best = __ldcg(C.sbest + g.s);
            const bool ok = g.a <= g.b && g.b < T;
            if (!ok) {
              atomicOr(C.err, kErrBuild);
              g.s = kNone;
            } else {
              g.ga = s_bp1[g.a / chunk] + __ldcg(C.ftl + g.a);
              g.ge = (g.b + 1 < T) ? s_bp1[(g.b + 1) / chunk] + __ldcg(C.ftl + g.b + 1) : gtot1;
            }
          }
        }
        __syncthreads();
#pragma unroll 1
        for (int k = 0; k < kBatchTiles; ++k) {
          if (s[k] == kNone) continue;
          const SlotSeg& g = sl[s[k] & (kSlots - 1)];
          if (g.s == kNone) continue;
          const uint32_t pk = p[k];
          const bool pred = __ldcg(C.bucket + pk) <= g.best;
          const bool fF = pk < g.spt && !pred, fT = pk >= g.spt && pred;
          const uint32_t n = g.b - g.a + 1;
          if (fF || fT) {
            const unsigned long long gp = s_bp1[pk / chunk] + __ldcg(C.ftl + pk);
            const uint32_t r = fF ? (uint32_t)(gp & 0xFFFFFFFFull) - (uint32_t)(g.ga & 0xFFFFFFFFull)
                                  : (uint32_t)(g.ge >> 32) - (uint32_t)(gp >> 32) - 1u;
            if (r < n) {
              (fF ? C.posF : C.posT)[g.a + r] = pk;
              C.rnk[pk] = r;
            } else {
              atomicOr(C.err, kErrBuild);
              C.rnk[pk] = kNone;
            }
          }
          if (pk != g.a) continue;
          // the segment's SAH node and its children
          const uint32_t sv = s[k];
          const unsigned long long g2 = s_bp2[g.a / chunk] + __ldcg(C.segpre + sv);
          const uint32_t nn_pre = (uint32_t)(g2 & 0xFFFFFFFFull), nl_pre = (uint32_t)(g2 >> 32);
          const uint32_t a = g.a, b = g.b, mid = g.mid;
          const uint32_t ln = mid - a, rn = b - mid + 1;
          const uint32_t nd = __ldcg(snode + sv);
          const uint32_t me = C.N2 + nd;
          Bounds bb = dec_bounds_cg(sacc + (size_t)sv * kSegWords);
          Bounds cb = dec_bounds_cg(sacc + (size_t)sv * kSegWords + 6);
          C.sah_axis[nd] = (uint32_t)bmax_extent(cb);
          C.sah_rng[2 * nd] = a;
          C.sah_rng[2 * nd + 1] = b + 1;
          const uint32_t ldm = __ldcg(C.sld[par] + sv);
          C.sah_ld[nd] = ldm;
          C.nb_lo[me] = make_float4(bb.lo.x, bb.lo.y, bb.lo.z, 0.0f);
          C.nb_hi[me] = make_float4(bb.hi.x, bb.hi.y, bb.hi.z, 0.0f);
          uint32_t node = node_base + nn_pre, segn = nl_pre;
          uint32_t cseg[2] = {kNone, kNone};
          const uint32_t ca[2] = {a, mid}, cb_[2] = {mid - 1, b}, cn[2] = {ln, rn};
          for (int q = 0; q < 2; ++q) {
            if (cn[q] < 2) continue;  // a single root: linked in phase E
            const uint32_t id = node++;
            // large children stay in the levels; medium and small ones are
            // queued (in any order: each is finished on its own)
            const bool large = cn[q] > kMedSeg, med = !large && cn[q] > kSmallSeg;
            const uint32_t z = large ? segn++ : atomicAdd(C.counters + (med ? 3 : 2), 1u);
            if (id >= T || z >= (large || med ? C.maxseg : T)) {
              atomicOr(C.err, kErrBuild);
              continue;
            }
            (q ? C.child1 : C.child0)[me] = C.N2 + id;
            C.parent[C.N2 + id] = (me << 1) | (uint32_t)q;
            if (large) {
              cseg[q] = z;
              C.sa[nx][z] = ca[q];
              C.sb[nx][z] = cb_[q];
              C.snode[nx][z] = id;
              C.sld[nx][z] = ld_child(ldm, q);
              init_segment(C.sacc[nx] + (size_t)z * kSegWords, C.sbk[nx] + (size_t)z * kBucketWords);
            } else {
              (med ? C.med_start : C.small_start)[z] = ca[q];
              (med ? C.med_end : C.small_end)[z] = cb_[q];
              (med ? C.med_node : C.small_node)[z] = id;
              (med ? C.med_ld : C.small_ld)[z] = ld_child(ldm, q);
            }
          }
          C.sdec[sv].z = cseg[0];
          C.sdec[sv].w = cseg[1];
        }
        __syncthreads();
      }
    }
    if (!coop_sync(C.bar, C.err)) return;

    // ---- E: swap pairs, next level's position arrays, single-root children ----
    {
      const uint32_t* item = C.item[par];
      uint32_t* item_n = C.item[nx];
      uint32_t* seg_n = C.seg_of[nx];
      for (uint32_t base = c0; base < c1; base += kBatch) {
        batch_segments(seg_of, base, c1, nseg, p, s, sl);
        if (threadIdx.x < kSlots) {
          SlotSeg& g = sl[threadIdx.x];
          if (g.s != kNone) {
            g.a = __ldcg(sa + g.s);
            g.b = __ldcg(sb + g.s);
            const uint4 dec = __ldcg(&C.sdec[g.s]);  // spt, mid, left segment, right segment
            g.spt = dec.x;
            g.mid = dec.y;
            g.cl = dec.z;
            g.cr = dec.w;
            g.best = __ldcg(C.sbest + g.s);
            g.node = __ldcg(snode + g.s);
            g.ld = __ldcg(C.sld[par] + g.s);
            if (!(g.a <= g.b && g.b < T)) {
              atomicOr(C.err, kErrBuild);
              g.s = kNone;
            }
          }
        }
        for (uint32_t k = threadIdx.x; k < 2 * kSlots * kSegWords; k += blockDim.x)
          s_nacc[k] = (((k % kSegWords) / 3) % 2 == 0) ? 0xFFFFFFFFu : 0u;
        if (threadIdx.x < 2 * kSlots) s_nid[threadIdx.x] = kNone;
        __syncthreads();
        uint32_t it[kBatchTiles];
#pragma unroll
        for (int k = 0; k < kBatchTiles; ++k) it[k] = p[k] < c1 ? __ldcg(item + p[k]) : 0u;
#pragma unroll 1
        for (int k = 0; k < kBatchTiles; ++k) {
          const uint32_t pk = p[k];
          uint32_t cs = kNone;  // the large child segment the root lands in
          float4 lv = make_float4(0.0f, 0.0f, 0.0f, 0.0f), hv = lv;
          if (pk < c1 && s[k] == kNone) {
            item_n[pk] = it[k];
            seg_n[pk] = kNone;
          } else if (pk < c1 && sl[s[k] & (kSlots - 1)].s != kNone) {
            const SlotSeg& g = sl[s[k] & (kSlots - 1)];
            const bool pred = __ldcg(C.bucket + pk) <= g.best;
            const bool fF = pk < g.spt && !pred, fT = pk >= g.spt && pred;
            uint32_t dst = pk;
            const uint32_t n = g.b - g.a + 1;
            if (fF || fT) {  // the r-th false (from the left) and the r-th true (from the right) trade places
              const uint32_t r = __ldcg(C.rnk + pk);
              dst = r < n ? __ldcg((fF ? C.posT : C.posF) + g.a + r) : kNone;
            }
            if (dst < g.a || dst > g.b) {
              atomicOr(C.err, kErrBuild);
            } else {
              item_n[dst] = it[k];
              lv = __ldcg(plo + pk);
              hv = __ldcg(phi + pk);
              C.plo[nx][dst] = lv;
              C.phi[nx][dst] = hv;
              cs = dst < g.mid ? g.cl : g.cr;
              seg_n[dst] = cs;
              const uint32_t me = C.N2 + g.node;
              if (dst == g.a && g.mid - g.a == 1) {
                uint32_t r = C.troot[it[k]];
                C.child0[me] = r;
                C.parent[r] = (me << 1) | 0u;
                C.t_ld[it[k]] = ld_child(g.ld, 0);
              }
              if (dst == g.b && g.b - g.mid + 1 == 1) {
                uint32_t r = C.troot[it[k]];
                C.child1[me] = r;
                C.parent[r] = (me << 1) | 1u;
                C.t_ld[it[k]] = ld_child(g.ld, 1);
              }
            }
          }
          // the next level's bounds and centroid bounds of the child segment:
          // the lanes of one child reduce together, their first lane adds
          // to the batch's slot (children of a batch's segments have
          // consecutive ids, at most 2 * kSlots of them)
          if (__any_sync(FULL, cs != kNone)) {
            const uint32_t peers = __match_any_sync(FULL, cs);
            if (cs != kNone) {
              const V3 lo{lv.x, lv.y, lv.z}, hi{hv.x, hv.y, hv.z};
              const V3 c = mul(add(lo, hi), 0.5f);
              uint32_t e[12];
              e[0] = fenc(lo.x); e[1] = fenc(lo.y); e[2] = fenc(lo.z);
              e[3] = fenc(hi.x); e[4] = fenc(hi.y); e[5] = fenc(hi.z);
              e[6] = fenc(c.x); e[7] = fenc(c.y); e[8] = fenc(c.z);
              e[9] = e[6]; e[10] = e[7]; e[11] = e[8];
#pragma unroll
              for (int q = 0; q < 12; ++q)
                e[q] = ((q / 3) % 2 == 0) ? __reduce_min_sync(peers, e[q]) : __reduce_max_sync(peers, e[q]);
              if (lane == (uint32_t)(__ffs(peers) - 1)) {
                const uint32_t z = cs & (2 * kSlots - 1);
                s_nid[z] = cs;
                uint32_t* r = s_nacc + z * kSegWords;
                for (int q = 0; q < 12; ++q) {
                  if ((q / 3) % 2 == 0)
                    atomicMin(r + q, e[q]);
                  else
                    atomicMax(r + q, e[q]);
                }
              }
            }
          }
        }
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < 2 * kSlots * kSegWords; k += blockDim.x) {
          const uint32_t cs = s_nid[k / kSegWords];
          if (cs == kNone) continue;
          const uint32_t v = s_nacc[k];
          const bool mn = ((k % kSegWords) / 3) % 2 == 0;
          if (v == (mn ? 0xFFFFFFFFu : 0u)) continue;
          uint32_t* dst = C.sacc[nx] + (size_t)cs * kSegWords + (k % kSegWords);
          if (mn)
            atomicMin(dst, v);
          else
            atomicMax(dst, v);
        }
        __syncthreads();
      }
    }
    if (!coop_sync(C.bar, C.err)) return;
    par = nx;
    if (__ldcg(C.lvl + 8 * par) == 0u) break;
  }
  // the positions end in buffer 0 (the warp-local SAH reads them there)
  if (par == 1u)
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < T; p += gridDim.x * blockDim.x)
      C.item[0][p] = __ldcg(C.item[1] + p);
  if (blockIdx.x == 0 && threadIdx.x == 0) C.counters[0] = __ldcg(C.lvl + 8 * par + 1);
}

// ---------------------------------------------------------------------------
// A8, segments of 33..kMedSeg treelet roots: all their SAH levels in one
// block, with the segment's positions, bounds and buckets in shared memory and
// block barriers between the phases. Each level runs the cooperative kernel's
// phases over every sub-segment of more than 32 roots at once: bounds and
// centroid bounds (order-preserving encodings, warp-reduced where a warp's
// positions share a sub-segment), buckets with per-sub-segment bucket counts
// and bounds, one warp_sah_split per sub-segment, the two-pointer partition
// of std::partition (the r-th "false" root from the left trades places with
// the r-th "true" one from the right, ranks from a block scan of the flags),
// and the children: single roots are linked, sub-segments of 2..32 roots go
// to the warp-local queue (as global positions), larger ones to the next
// level. New SAH node ids come from the shared counter; queue order does not
// matter. The positions are written back for the warp-local pass.
// ---------------------------------------------------------------------------
constexpr int kMedBlock = (int)kMedSeg / 4;
constexpr uint32_t kMedSlots = kMedSeg / 32;  // sub-segments of more than 32 roots in one level
constexpr int kMedPerSM = 4096 / (int)kMedSeg;  // resident blocks per SM (shared memory)
static_assert(kMedSeg / (kSmallSeg + 1) <= kMedSlots, "a level of a medium segment fits the slots");
static_assert(kMedSeg == 4 * kMedBlock, "the flag scan takes four positions per thread");
constexpr uint16_t kNoSub = 0xFFFFu;
// dynamic shared memory layout (bytes)
constexpr size_t kMedOffIt = 0;                                       // u32 item per position
constexpr size_t kMedOffPre = kMedOffIt + 4 * kMedSeg;                // u32 flag prefix per position (+1)
constexpr size_t kMedOffBnd = kMedOffPre + 4 * (kMedSeg + 32);        // f32 lo xyz, hi xyz per position
constexpr size_t kMedOffAcc = kMedOffBnd + 24 * (size_t)kMedSeg;     // u32 kSegWords per slot
constexpr size_t kMedOffBk = kMedOffAcc + 4 * kMedSlots * kSegWords;  // u32 kBucketWords per slot
constexpr size_t kMedOffTab = kMedOffBk + 4 * kMedSlots * kBucketWords;  // u32 slot tables
constexpr int kMedTabs = 14;
constexpr size_t kMedOffPos = kMedOffTab + 4 * kMedTabs * kMedSlots;  // u16 posF, posT
constexpr size_t kMedOffSid = kMedOffPos + 4 * (size_t)kMedSeg;      // u16 sub-segment per position
constexpr size_t kMedOffBkt = kMedOffSid + 2 * (size_t)kMedSeg;      // u8 bucket per position
constexpr size_t kMedOffMisc = kMedOffBkt + kMedSeg;                   // u32 warp sums, counters
constexpr size_t kMedSmem = kMedOffMisc + 4 * 64;
static_assert(kMedPerSM * (kMedSmem + 1024) <= 228 * 1024, "the medium SAH blocks fit one SM");

struct MedArgs {
  uint32_t N, N2;
  const uint32_t* troot;
  float4* nb_lo;
  float4* nb_hi;
  uint32_t* child0;
  uint32_t* child1;
  uint32_t* parent;
  uint32_t* sah_axis;
  uint32_t* sah_rng;
  uint32_t* cur;  // positions after the cooperative levels
  const uint32_t* med_start;
  const uint32_t* med_end;
  const uint32_t* med_node;
  const uint32_t* med_ld;
  uint32_t* small_start;
  uint32_t* small_end;
  uint32_t* small_node;
  uint32_t* small_ld;
  uint32_t* sah_ld;
  uint32_t* t_ld;
  uint32_t* counters;  // [0] SAH nodes allocated, [2] small segments queued, [3] medium segments queued,
                       // [4], [7] medium segments taken (two passes), [5], [1] small segments taken
  uint32_t* err;
};

__global__ void __launch_bounds__(kMedBlock, kMedPerSM) k_medium_sah(MedArgs M) {
  extern __shared__ __align__(16) unsigned char s_med[];
  uint32_t* s_it = (uint32_t*)(s_med + kMedOffIt);
  uint32_t* s_pre = (uint32_t*)(s_med + kMedOffPre);
  float* s_bnd = (float*)(s_med + kMedOffBnd);  // [6][kMedSeg]
  uint32_t* s_acc = (uint32_t*)(s_med + kMedOffAcc);
  uint32_t* s_bkc = (uint32_t*)(s_med + kMedOffBk);
  uint32_t* tab = (uint32_t*)(s_med + kMedOffTab);
  uint32_t* s_sa = tab;
  uint32_t* s_sb = tab + kMedSlots;
  uint32_t* s_snode = tab + 2 * kMedSlots;
  uint32_t* s_best = tab + 3 * kMedSlots;
  uint32_t* s_spt = tab + 4 * kMedSlots;
  uint32_t* s_mid = tab + 5 * kMedSlots;
  uint32_t* s_nsw = tab + 6 * kMedSlots;  // pairs that trade places
  uint32_t* s_cl = tab + 7 * kMedSlots;   // next-level slot of each child (kNone: not large)
  uint32_t* s_cr = tab + 8 * kMedSlots;
  uint32_t* s_na = tab + 9 * kMedSlots;   // next level's slots
  uint32_t* s_nb = tab + 10 * kMedSlots;
  uint32_t* s_nnode = tab + 11 * kMedSlots;
  uint32_t* s_ld = tab + 12 * kMedSlots;  // packed depth and child-0 steps of the slot's node
  uint32_t* s_nld = tab + 13 * kMedSlots;
  uint16_t* s_posF = (uint16_t*)(s_med + kMedOffPos);
  uint16_t* s_posT = s_posF + kMedSeg;
  uint16_t* s_sid = (uint16_t*)(s_med + kMedOffSid);
  uint8_t* s_bkt = (uint8_t*)(s_med + kMedOffBkt);
  uint32_t* s_misc = (uint32_t*)(s_med + kMedOffMisc);  // [0..31] warp sums, [32] active, [33] next active
  const uint32_t FULL = 0xFFFFFFFFu;
  const uint32_t t = threadIdx.x, lane = lane_id(), wid = t >> 5;
  const uint32_t nmed = M.counters[3];
  for (uint32_t pass = 0; pass < 2;) {
    // segments taken in turn from a counter, so that blocks that drew small
    // segments take more; the first pass takes those of more than kMedSeg / 2
    // roots and the second the others, so the last to run are the shorter
    // ones (the barrier first: every thread has read the last number)
    __syncthreads();
    if (t == 0) s_misc[38] = atomicAdd(M.counters + (pass == 0 ? 4 : 7), 1u);
    __syncthreads();
    const uint32_t seg = s_misc[38];
    if (seg >= nmed) {  // block-uniform
      ++pass;
      continue;
    }
    const uint32_t start = M.med_start[seg], end = M.med_end[seg];
    const uint32_t n = end - start + 1;
    if ((n > kMedSeg / 2) != (pass == 0)) continue;  // the other pass's segment
    if (end < start || end >= M.N || n <= kSmallSeg || n > kMedSeg) {  // block-uniform
      if (t == 0) atomicOr(M.err, kErrBuild);
      continue;
    }
    for (uint32_t i = t; i < n; i += kMedBlock) {
      const uint32_t it = M.cur[start + i];
      const uint32_t r = M.troot[it];
      const float4 l = M.nb_lo[r], h = M.nb_hi[r];
      s_it[i] = it;
      s_bnd[i] = l.x;
      s_bnd[kMedSeg + i] = l.y;
      s_bnd[2 * kMedSeg + i] = l.z;
      s_bnd[3 * kMedSeg + i] = h.x;
      s_bnd[4 * kMedSeg + i] = h.y;
      s_bnd[5 * kMedSeg + i] = h.z;
      s_sid[i] = 0;
    }
    if (t == 0) {
      s_sa[0] = 0;
      s_sb[0] = n - 1;
      s_snode[0] = M.med_node[seg];
      s_ld[0] = M.med_ld[seg];
      s_misc[32] = 1;
    }
    // the accumulators of a level's slots are reset by the phase before it
    for (uint32_t k = t; k < kSegWords; k += kMedBlock) s_acc[k] = (((k % kSegWords) / 3) % 2 == 0) ? 0xFFFFFFFFu : 0u;
    for (uint32_t k = t; k < kBucketWords; k += kMedBlock)
      s_bkc[k] = (k % 7 == 0) ? 0u : ((k % 7) <= 3 ? 0xFFFFFFFFu : 0u);
    __syncthreads();
    const uint32_t nw = div_up_d(n, 32) * 32;  // positions rounded up to whole warps
    for (uint32_t level = 0;; ++level) {
      const uint32_t nact = s_misc[32];
      if (nact == 0) break;
      if (level > kMedSeg || nact > kMedSlots) {  // block-uniform
        if (t == 0) atomicOr(M.err, level > kMedSeg ? kErrLoopLimit : kErrBuild);
        break;
      }
      // A: bounds and centroid bounds of every sub-segment
      for (uint32_t i = t; i < nw; i += kMedBlock) {
        const uint32_t sk = i < n ? (uint32_t)s_sid[i] : (uint32_t)kNoSub;
        uint32_t e[12];
        if (sk != kNoSub) {
          const V3 lo{s_bnd[i], s_bnd[kMedSeg + i], s_bnd[2 * kMedSeg + i]};
          const V3 hi{s_bnd[3 * kMedSeg + i], s_bnd[4 * kMedSeg + i], s_bnd[5 * kMedSeg + i]};
          const V3 c = mul(add(lo, hi), 0.5f);
          e[0] = fenc(lo.x); e[1] = fenc(lo.y); e[2] = fenc(lo.z);
          e[3] = fenc(hi.x); e[4] = fenc(hi.y); e[5] = fenc(hi.z);
          e[6] = fenc(c.x); e[7] = fenc(c.y); e[8] = fenc(c.z);
          e[9] = e[6]; e[10] = e[7]; e[11] = e[8];
        } else {
#pragma unroll
          for (int q = 0; q < 12; ++q) e[q] = ((q / 3) % 2 == 0) ? 0xFFFFFFFFu : 0u;
        }
        const uint32_t s0 = __shfl_sync(FULL, sk, 0);
        if (s0 != kNoSub && __all_sync(FULL, sk == s0)) {  // one sub-segment across the warp
#pragma unroll
          for (int q = 0; q < 12; ++q)
            e[q] = ((q / 3) % 2 == 0) ? __reduce_min_sync(FULL, e[q]) : __reduce_max_sync(FULL, e[q]);
          if (lane == 0) {
            uint32_t* r = s_acc + s0 * kSegWords;
            for (int q = 0; q < 12; ++q) {
              if ((q / 3) % 2 == 0)
                atomicMin(r + q, e[q]);
              else
                atomicMax(r + q, e[q]);
            }
          }
        } else if (sk != kNoSub) {
          uint32_t* r = s_acc + sk * kSegWords;
          for (int q = 0; q < 12; ++q) {
            if ((q / 3) % 2 == 0)
              atomicMin(r + q, e[q]);
            else
              atomicMax(r + q, e[q]);
          }
        }
      }
      __syncthreads();
      // B: buckets, bucket counts and bounds
      for (uint32_t i = t; i < n; i += kMedBlock) {
        const uint32_t sk = s_sid[i];
        if (sk == kNoSub) continue;
        const V3 lo{s_bnd[i], s_bnd[kMedSeg + i], s_bnd[2 * kMedSeg + i]};
        const V3 hi{s_bnd[3 * kMedSeg + i], s_bnd[4 * kMedSeg + i], s_bnd[5 * kMedSeg + i]};
        const Bounds cb = dec_bounds(s_acc + sk * kSegWords + 6);
        const uint32_t ib = sah_bucket(lo, hi, cb, bmax_extent(cb));
        s_bkt[i] = (uint8_t)ib;
        uint32_t* d = s_bkc + sk * kBucketWords + ib * 7;
        atomicAdd(d, 1u);
        atomicMin(d + 1, fenc(lo.x));
        atomicMin(d + 2, fenc(lo.y));
        atomicMin(d + 3, fenc(lo.z));
        atomicMax(d + 4, fenc(hi.x));
        atomicMax(d + 5, fenc(hi.y));
        atomicMax(d + 6, fenc(hi.z));
      }
      __syncthreads();
      // C: one decision per sub-segment, one warp each
      if (t == 0) s_misc[33] = 0;  // the next level's slots (counted by the children phase)
      for (uint32_t j = wid; j < nact; j += kMedBlock / 32) {
        const uint32_t* bk = s_bkc + j * kBucketWords;
        uint32_t cj = 0;
        Bounds bj = bempty();
        if (lane < 12) {
          cj = bk[lane * 7];
          if (cj) bj = dec_bounds(bk + lane * 7 + 1);
        }
        const Bounds bb = dec_bounds(s_acc + j * kSegWords);
        uint32_t kv;
        const int bv = warp_sah_split(cj, bj, barea(bb), &kv);
        if (lane == 0) {
          const uint32_t a = s_sa[j], b = s_sb[j], cnt = b - a + 1;
          s_best[j] = (uint32_t)bv;
          s_spt[j] = a + kv;
          s_mid[j] = (kv == cnt) ? a + cnt / 2 : a + kv;
        }
      }
      __syncthreads();
      // partition flags, block scan of (true << 16 | false) over positions
      // 4t .. 4t + 3
      {
        uint32_t v[4], sum = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint32_t i = 4 * t + q;
          v[q] = 0;
          if (i < n) {
            const uint32_t sk = s_sid[i];
            if (sk != kNoSub) {
              const bool pred = s_bkt[i] <= s_best[sk];
              const uint32_t spt = s_spt[sk];
              v[q] = (i < spt && !pred) ? 1u : ((i >= spt && pred) ? (1u << 16) : 0u);
            }
          }
          sum += v[q];
        }
        uint32_t x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(FULL, x, o);
          if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) s_misc[wid] = x;
        __syncthreads();
        if (wid == 0) {
          const uint32_t ws = s_misc[lane];
          uint32_t y = ws;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const uint32_t z = __shfl_up_sync(FULL, y, o);
            if (lane >= (uint32_t)o) y += z;
          }
          s_misc[lane] = y - ws;
        }
        __syncthreads();
        uint32_t run = s_misc[wid] + x - sum;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint32_t i = 4 * t + q;
          if (i <= n) s_pre[i] = run;  // s_pre[n]: the total
          run += v[q];
        }
        if (t == kMedBlock - 1) s_pre[4 * kMedBlock] = run;  // the total when n = 4 * kMedBlock
      }
      __syncthreads();
      // select tables: the r-th false from the left and the r-th true from
      // the right of each sub-segment
      for (uint32_t i = t; i < n; i += kMedBlock) {
        const uint32_t sk = s_sid[i];
        if (sk == kNoSub) continue;
        const uint32_t a = s_sa[sk], b = s_sb[sk], spt = s_spt[sk];
        const bool pred = s_bkt[i] <= s_best[sk];
        if (i < spt && !pred) {
          const uint32_t r = (s_pre[i] & 0xFFFFu) - (s_pre[a] & 0xFFFFu);
          if (a + r <= b) s_posF[a + r] = (uint16_t)i;
        } else if (i >= spt && pred) {
          const uint32_t r = (s_pre[b + 1] >> 16) - (s_pre[i] >> 16) - 1u;
          if (a + r <= b) s_posT[a + r] = (uint16_t)i;
        }
      }
      for (uint32_t j = t; j < nact; j += kMedBlock) {
        const uint32_t a = s_sa[j], b = s_sb[j];
        const uint32_t nf = (s_pre[b + 1] & 0xFFFFu) - (s_pre[a] & 0xFFFFu);
        const uint32_t nt = (s_pre[b + 1] >> 16) - (s_pre[a] >> 16);
        if (nf != nt) atomicOr(M.err, kErrBuild);
        s_nsw[j] = min(nf, nt);
      }
      __syncthreads();
      // E: the pairs trade places
      for (uint32_t k = t; k < n; k += kMedBlock) {
        const uint32_t sk = s_sid[k];
        if (sk == kNoSub) continue;
        const uint32_t r = k - s_sa[sk];
        if (r >= s_nsw[sk]) continue;
        const uint32_t pf = s_posF[k], pt = s_posT[k];
        if (pf >= n || pt >= n) {
          atomicOr(M.err, kErrBuild);
          continue;
        }
        const uint32_t ti = s_it[pf];
        s_it[pf] = s_it[pt];
        s_it[pt] = ti;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
          const float f = s_bnd[q * kMedSeg + pf];
          s_bnd[q * kMedSeg + pf] = s_bnd[q * kMedSeg + pt];
          s_bnd[q * kMedSeg + pt] = f;
        }
      }
      __syncthreads();
      // the sub-segments' SAH nodes and their children (one reservation of
      // SAH node ids and one of warp-local queue entries per sub-segment)
      for (uint32_t j = t; j < nact; j += kMedBlock) {
        const uint32_t a = s_sa[j], b = s_sb[j], mid = s_mid[j];
        const uint32_t nd = s_snode[j], me = M.N2 + nd;
        const Bounds bb = dec_bounds(s_acc + j * kSegWords);
        M.sah_axis[nd] = (uint32_t)bmax_extent(dec_bounds(s_acc + j * kSegWords + 6));
        M.sah_rng[2 * nd] = start + a;
        M.sah_rng[2 * nd + 1] = start + b + 1;
        const uint32_t ldm = s_ld[j];
        M.sah_ld[nd] = ldm;
        M.nb_lo[me] = make_float4(bb.lo.x, bb.lo.y, bb.lo.z, 0.0f);
        M.nb_hi[me] = make_float4(bb.hi.x, bb.hi.y, bb.hi.z, 0.0f);
        const uint32_t ca[2] = {a, mid}, ce[2] = {mid - 1, b}, cn[2] = {mid - a, b - mid + 1};
        const uint32_t nids = (uint32_t)(cn[0] >= 2) + (uint32_t)(cn[1] >= 2);
        const uint32_t nsm = (uint32_t)(cn[0] >= 2 && cn[0] <= kSmallSeg) + (uint32_t)(cn[1] >= 2 && cn[1] <= kSmallSeg);
        const uint32_t id0 = nids ? atomicAdd(M.counters, nids) : 0u;
        const uint32_t q0 = nsm ? atomicAdd(M.counters + 2, nsm) : 0u;
        uint32_t nid = 0, nq = 0, slot[2] = {kNone, kNone};
        for (int q = 0; q < 2; ++q) {
          uint32_t* cref = q ? M.child1 : M.child0;
          if (cn[q] == 1) {
            const uint32_t r = M.troot[s_it[ca[q]]];
            cref[me] = r;
            M.parent[r] = (me << 1) | (uint32_t)q;
            M.t_ld[s_it[ca[q]]] = ld_child(ldm, q);
            continue;
          }
          const uint32_t id = id0 + nid++;
          const bool large = cn[q] > kSmallSeg;
          const uint32_t z = large ? atomicAdd(s_misc + 33, 1u) : q0 + nq++;
          if (id >= M.N || z >= (large ? kMedSlots : M.N)) {
            atomicOr(M.err, kErrBuild);
            continue;
          }
          cref[me] = M.N2 + id;
          M.parent[M.N2 + id] = (me << 1) | (uint32_t)q;
          if (large) {
            s_na[z] = ca[q];
            s_nb[z] = ce[q];
            s_nnode[z] = id;
            s_nld[z] = ld_child(ldm, q);
            slot[q] = z;
          } else {
            M.small_start[z] = start + ca[q];
            M.small_end[z] = start + ce[q];
            M.small_node[z] = id;
            M.small_ld[z] = ld_child(ldm, q);
          }
        }
        s_cl[j] = slot[0];
        s_cr[j] = slot[1];
      }
      __syncthreads();
      const uint32_t nnext = min(s_misc[33], kMedSlots);
      // the next level's accumulators
      for (uint32_t k = t; k < nnext * kSegWords; k += kMedBlock)
        s_acc[k] = (((k % kSegWords) / 3) % 2 == 0) ? 0xFFFFFFFFu : 0u;
      for (uint32_t k = t; k < nnext * kBucketWords; k += kMedBlock)
        s_bkc[k] = (k % 7 == 0) ? 0u : ((k % 7) <= 3 ? 0xFFFFFFFFu : 0u);
      // the next level's sub-segment of every position, and its slots
      for (uint32_t k = t; k < n; k += kMedBlock) {
        const uint32_t sk = s_sid[k];
        if (sk == kNoSub) continue;
        const uint32_t z = k < s_mid[sk] ? s_cl[sk] : s_cr[sk];
        s_sid[k] = z < kMedSlots ? (uint16_t)z : kNoSub;
      }
      for (uint32_t j = t; j < nnext; j += kMedBlock) {
        s_sa[j] = s_na[j];
        s_sb[j] = s_nb[j];
        s_snode[j] = s_nnode[j];
        s_ld[j] = s_nld[j];
      }
      if (t == 0) s_misc[32] = nnext;
      __syncthreads();
    }
    for (uint32_t i = t; i < n; i += kMedBlock) M.cur[start + i] = s_it[i];
    __syncthreads();
  }
}

// An SAH node over the two roots in lanes p and p + 1 (warp-uniform call).
// The centroid bounds' minimum along their longest axis is one root's
// centroid, which falls in bucket 0, and the other lies at t = 1, bucket 11
// (both in bucket 0 when the centroids coincide along that axis, or the
// extent is not finite): every split then has the same two sides, so every
// cost is the same float and the sequential first-minimum picks split 0 —
// the root in bucket 0 goes left, which std::partition reaches by swapping
// the pair when the first root is the one in bucket 11. The bounds, centroid
// bounds, axis and buckets are computed exactly as the general step does;
// any other bucket pair returns false and is left to the general step.
__device__ bool sah_pair(const SahArgs& A, uint32_t base, uint32_t p, uint32_t nd, uint32_t ld, uint32_t N2, uint32_t& item, V3& lo, V3& hi,
                         uint32_t* sah_axis, float4* nb_lo, float4* nb_hi, uint32_t* child0, uint32_t* child1,
                         uint32_t* parent) {
  const uint32_t FULL = 0xFFFFFFFFu, lane = lane_id();
  const uint32_t it0 = __shfl_sync(FULL, item, p), it1 = __shfl_sync(FULL, item, p + 1);
  const V3 lo0{__shfl_sync(FULL, lo.x, p), __shfl_sync(FULL, lo.y, p), __shfl_sync(FULL, lo.z, p)};
  const V3 hi0{__shfl_sync(FULL, hi.x, p), __shfl_sync(FULL, hi.y, p), __shfl_sync(FULL, hi.z, p)};
  const V3 lo1{__shfl_sync(FULL, lo.x, p + 1), __shfl_sync(FULL, lo.y, p + 1), __shfl_sync(FULL, lo.z, p + 1)};
  const V3 hi1{__shfl_sync(FULL, hi.x, p + 1), __shfl_sync(FULL, hi.y, p + 1), __shfl_sync(FULL, hi.z, p + 1)};
  auto emin = [](float a, float b) { return fdec(min(fenc(a), fenc(b))); };
  auto emax = [](float a, float b) { return fdec(max(fenc(a), fenc(b))); };
  const Bounds bb{V3{emin(lo0.x, lo1.x), emin(lo0.y, lo1.y), emin(lo0.z, lo1.z)},
                  V3{emax(hi0.x, hi1.x), emax(hi0.y, hi1.y), emax(hi0.z, hi1.z)}};
  const V3 c0 = mul(add(lo0, hi0), 0.5f), c1 = mul(add(lo1, hi1), 0.5f);
  const Bounds cb{V3{emin(c0.x, c1.x), emin(c0.y, c1.y), emin(c0.z, c1.z)},
                  V3{emax(c0.x, c1.x), emax(c0.y, c1.y), emax(c0.z, c1.z)}};
  const int dim = bmax_extent(cb);
  const uint32_t b0 = sah_bucket(lo0, hi0, cb, dim), b1 = sah_bucket(lo1, hi1, cb, dim);
  bool swap;
  if (b0 == 0u && (b1 == 11u || b1 == 0u))
    swap = false;
  else if (b0 == 11u && b1 == 0u)
    swap = true;
  else
    return false;
  if (swap) {
    if (lane == p) {
      item = it1;
      lo = lo1;
      hi = hi1;
    } else if (lane == p + 1) {
      item = it0;
      lo = lo0;
      hi = hi0;
    }
  }
  if (lane == 0) {
    const uint32_t me = N2 + nd;
    sah_axis[nd] = (uint32_t)dim;
    A.sah_rng[2 * nd] = base + p;
    A.sah_rng[2 * nd + 1] = base + p + 2;
    A.sah_ld[nd] = ld;
    A.t_ld[swap ? it1 : it0] = ld_child(ld, 0);
    A.t_ld[swap ? it0 : it1] = ld_child(ld, 1);
    nb_lo[me] = make_float4(bb.lo.x, bb.lo.y, bb.lo.z, 0.0f);
    nb_hi[me] = make_float4(bb.hi.x, bb.hi.y, bb.hi.z, 0.0f);
    const uint32_t r0 = A.troot[swap ? it1 : it0], r1 = A.troot[swap ? it0 : it1];
    child0[me] = r0;
    parent[r0] = (me << 1) | 0u;
    child1[me] = r1;
    parent[r1] = (me << 1) | 1u;
  }
  return true;
}

// Segments of 2..32 roots: the whole SAH recursion inside one warp. Bounds
// by warp reductions, buckets by shared-memory atomics, the split decision by
// warp_sah_split, the two-pointer partition by ballots. Each segment's n - 2
// new SAH node ids are reserved with one atomic. Nodes over two roots (about
// half of them) are finished by sah_pair within the step that creates them
// instead of a step of their own. A persistent grid of warps walks the
// queue, whose length it reads from *nsmall_p (the cooperative and
// block-local levels fill the queue on the device), each warp taking the
// next segment from counters[5] (then counters[1]).
__global__ void k_small_sah(SahArgs A, const uint32_t* nsmall_p, const uint32_t* sm_start, const uint32_t* sm_end,
                            const uint32_t* sm_node, const uint32_t* sm_ld, uint32_t* cur, uint32_t* counters, uint32_t* sah_axis,
                            float4* nb_lo, float4* nb_hi, uint32_t* child0, uint32_t* child1, uint32_t* parent,
                            uint32_t N2, uint32_t* err) {
  __shared__ uint32_t sh_bcnt[kB / 32][12];
  __shared__ uint32_t sh_benc[kB / 32][12 * 6];
  __shared__ uint32_t sh_stack[kB / 32][4 * 64];
  const uint32_t FULL = 0xFFFFFFFFu;
  const uint32_t w = threadIdx.x >> 5, lane = lane_id();
  const uint32_t nsmall = *nsmall_p;
  for (uint32_t pass = 0; pass < 2;) {
    // segments (2 to 32 roots) taken in turn from a counter, which keeps the
    // warps' loads even; those of more than 16 roots first (pass 0), so the
    // last to run are the shorter ones
    uint32_t seg = 0;
    if (lane == 0) seg = atomicAdd(counters + (pass == 0 ? 5 : 1), 1u);
    seg = __shfl_sync(FULL, seg, 0);
    if (seg >= nsmall) {
      ++pass;
      continue;
    }
    if ((sm_end[seg] - sm_start[seg] + 1 > kSmallSeg / 2) != (pass == 0)) continue;
    const uint32_t base = sm_start[seg];
    const uint32_t n = sm_end[seg] - base + 1;
    if (n < 2 || n > kSmallSeg || sm_end[seg] >= A.N) {
      if (lane == 0) atomicOr(err, kErrBuild);
      continue;
    }
    uint32_t item = lane < n ? cur[base + lane] : 0u;
    V3 lo{0, 0, 0}, hi{0, 0, 0};
    if (lane < n) item_bounds(A, item, &lo, &hi);
    uint32_t id_base = 0, id_next = 0;
    if (lane == 0 && n > 2) id_base = atomicAdd(&counters[0], n - 2);
    id_base = __shfl_sync(FULL, id_base, 0);
    uint32_t* stk = sh_stack[w];
    __syncwarp();
    int sp = 1;
    const uint32_t ld0 = sm_ld[seg];
    if (n == 2 &&
        sah_pair(A, base, 0, sm_node[seg], ld0, N2, item, lo, hi, sah_axis, nb_lo, nb_hi, child0, child1, parent)) {
      sp = 0;
    } else if (lane == 0) {
      stk[0] = 0;
      stk[1] = n - 1;
      stk[2] = sm_node[seg];
      stk[3] = ld0;
    }
    __syncwarp();
    uint32_t guard = 0;
    while (sp > 0) {
      if (++guard > 64) {
        if (lane == 0) atomicOr(err, kErrLoopLimit);
        break;
      }
      --sp;
      uint32_t a = stk[4 * sp], b = stk[4 * sp + 1], nd = stk[4 * sp + 2], ld = stk[4 * sp + 3];
      __syncwarp();
      bool act = lane >= a && lane <= b;
      uint32_t cnt = b - a + 1;
      V3 c = mul(add(lo, hi), 0.5f);
      Bounds bb{V3{fdec(__reduce_min_sync(FULL, act ? fenc(lo.x) : 0xFFFFFFFFu)),
                   fdec(__reduce_min_sync(FULL, act ? fenc(lo.y) : 0xFFFFFFFFu)),
                   fdec(__reduce_min_sync(FULL, act ? fenc(lo.z) : 0xFFFFFFFFu))},
                V3{fdec(__reduce_max_sync(FULL, act ? fenc(hi.x) : 0u)),
                   fdec(__reduce_max_sync(FULL, act ? fenc(hi.y) : 0u)),
                   fdec(__reduce_max_sync(FULL, act ? fenc(hi.z) : 0u))}};
      Bounds cb{V3{fdec(__reduce_min_sync(FULL, act ? fenc(c.x) : 0xFFFFFFFFu)),
                   fdec(__reduce_min_sync(FULL, act ? fenc(c.y) : 0xFFFFFFFFu)),
                   fdec(__reduce_min_sync(FULL, act ? fenc(c.z) : 0xFFFFFFFFu))},
                V3{fdec(__reduce_max_sync(FULL, act ? fenc(c.x) : 0u)),
                   fdec(__reduce_max_sync(FULL, act ? fenc(c.y) : 0u)),
                   fdec(__reduce_max_sync(FULL, act ? fenc(c.z) : 0u))}};
      int dim = bmax_extent(cb);
      uint32_t ib = act ? sah_bucket(lo, hi, cb, dim) : 0u;
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
      uint32_t cj = lane < 12 ? bcnt[lane] : 0u;
      Bounds bj = (lane < 12 && cj) ? dec_bounds(benc + lane * 6) : bempty();
      uint32_t k;
      int best = warp_sah_split(cj, bj, barea(bb), &k);
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
        A.sah_rng[2 * nd] = base + a;
        A.sah_rng[2 * nd + 1] = base + b + 1;
        A.sah_ld[nd] = ld;
        nb_lo[me] = make_float4(bb.lo.x, bb.lo.y, bb.lo.z, 0.0f);
        nb_hi[me] = make_float4(bb.hi.x, bb.hi.y, bb.hi.z, 0.0f);
      }
      uint32_t ln = mid - a, rn = b - mid + 1;
      uint32_t litem = __shfl_sync(FULL, item, a);
      uint32_t ritem = __shfl_sync(FULL, item, b);
      // the children's node ids (lane 0 keeps the running count); children of
      // two roots are finished here
      uint32_t cl = 0, cr = 0;
      if (lane == 0) {
        if (ln > 1) cl = id_base + id_next++;
        if (rn > 1) cr = id_base + id_next++;
      }
      cl = __shfl_sync(FULL, cl, 0);
      cr = __shfl_sync(FULL, cr, 0);
      const bool lpair =
          ln == 2 && sah_pair(A, base, a, cl, ld_child(ld, 0), N2, item, lo, hi, sah_axis, nb_lo, nb_hi, child0, child1, parent);
      const bool rpair =
          rn == 2 && sah_pair(A, base, mid, cr, ld_child(ld, 1), N2, item, lo, hi, sah_axis, nb_lo, nb_hi, child0, child1, parent);
      if (lane == 0) {
        if (ln == 1) {
          uint32_t r = A.troot[litem];
          child0[me] = r;
          parent[r] = (me << 1) | 0u;
          A.t_ld[litem] = ld_child(ld, 0);
        } else {
          child0[me] = N2 + cl;
          parent[N2 + cl] = (me << 1) | 0u;
          if (!lpair) {
            stk[4 * sp] = a; stk[4 * sp + 1] = mid - 1; stk[4 * sp + 2] = cl; stk[4 * sp + 3] = ld_child(ld, 0);
            ++sp;
          }
        }
        if (rn == 1) {
          uint32_t r = A.troot[ritem];
          child1[me] = r;
          parent[r] = (me << 1) | 1u;
          A.t_ld[ritem] = ld_child(ld, 1);
        } else {
          child1[me] = N2 + cr;
          parent[N2 + cr] = (me << 1) | 1u;
          if (!rpair) {
            stk[4 * sp] = mid; stk[4 * sp + 1] = b; stk[4 * sp + 2] = cr; stk[4 * sp + 3] = ld_child(ld, 1);
            ++sp;
          }
        }
      }
      sp = __shfl_sync(FULL, sp, 0);
      __syncwarp();
    }
    if (lane < n) cur[base + lane] = item;
    __syncwarp();
  }
}

// Subtree node counts of SAH nodes. The roots under an SAH node fill the
// range of final positions its segment had when it was made (the levels only
// permute roots within a segment), so its count is its cnt - 1 SAH nodes
// plus the treelet sizes over that range: per position the treelet size of
// its root (zero past T), scanned, then one difference per SAH node.
struct PosTsizeIn {
  const uint32_t* info;
  const uint32_t* cur;
  const uint32_t* troot;
  const uint32_t* size;
  uint32_t* tinv;  // the final position of each treelet, written on the way
  __device__ __forceinline__ uint32_t operator()(uint32_t p) const {
    const uint32_t T = info[kInfoT];
    if (p < T && T > 1) {
      const uint32_t t = cur[p];
      if (t < T) {
        tinv[t] = p;
        return size[troot[t]];
      }
    }
    return 0u;
  }
};
__global__ void k_sah_sizes(const uint32_t* info, const uint32_t* rng, const uint32_t* tpre, uint32_t* size,
                            uint32_t N2, uint32_t* err) {
  const uint32_t nd = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t T = info[kInfoT];
  if (T < 2 || nd >= T - 1) return;
  const uint32_t a = rng[2 * nd], e = rng[2 * nd + 1];
  if (a + 2 > e || e > T) {
    atomicOr(err, kErrBuild);
    return;
  }
  size[N2 + nd] = (e - a - 1u) + (tpre[e] - tpre[a]);
}

// ---------------------------------------------------------------------------
// A9: flattenBVHTree — depth-first preorder index of every reference node
// ---------------------------------------------------------------------------
__global__ void k_flatten(uint32_t N, uint32_t* info, const uint32_t* skey, const uint32_t* tid,
                          const uint32_t* tstart, const uint32_t* rng_lo,
                          const uint32_t* rng_hi, const uint32_t* child0, const uint32_t* parent,
                          const uint32_t* size, const uint32_t* sah_axis, const float4* nb_lo, const float4* nb_hi,
                          const uint32_t* sah_ld, const uint32_t* sah_rng, const uint32_t* t_ld,
                          const uint32_t* tinv, const uint32_t* tpre, const uint8_t* role, uint32_t* lin_node,
                          float* lin_bounds, uint32_t* is_int, uint32_t* depth_max, uint32_t* err) {
  uint32_t X = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t N2 = 2 * N;
  const uint32_t T = info[kInfoT];
  const uint32_t nsah = T - 1u, root = info[kInfoRoot];
  const uint32_t M = root < N2 + N ? size[root] : kNone;
  if (M > N2) {  // a flattened tree has at most 2N - 1 nodes
    if (X == 0) {
      info[kInfoM] = 0u;
      atomicOr(err, kErrBuild);
    }
    return;
  }
  if (X == 0) info[kInfoM] = M;
  if (X >= N2 + nsah) return;
  uint32_t kind;  // 0 radix interior, 1 leaf, 2 SAH
  uint32_t lo = 0, hi = 0, t = 0, troot_ = 0;
  if (X >= N2) {
    kind = 2;
  } else {
    const uint32_t r = role[X];  // as the refit classified X
    if (r == 0u) return;
    if (X < N) {
      t = tid[X];
      lo = rng_lo[X];
      hi = rng_hi[X];
    } else {
      lo = hi = X - N;
      t = tid[lo];
    }
    troot_ = treelet_root(t, tstart, info, N);
    kind = r == 2u ? 0u : 1u;
  }
  // the preorder index: an SAH node or a treelet root takes it from its
  // recorded child-0 steps and depth (ld_child), its first position and the
  // treelet nodes before that position; a treelet's other nodes walk up to
  // their treelet root
  uint32_t idx = 0, depth = 0;
  if (kind == 2) {
    const uint32_t nd = X - N2, ld = sah_ld[nd], a = sah_rng[2 * nd];
    if (a >= T) {
      atomicOr(err, kErrBuild);
      return;
    }
    idx = (ld & 0xFFFFu) + a + tpre[a];
    depth = ld >> 16;
  } else {
    uint32_t cur = X;
    while (cur != troot_) {
      if (++depth > (1u << 22)) {
        atomicOr(err, kErrLoopLimit);
        return;
      }
      uint32_t pw = parent[cur];
      uint32_t p = pw >> 1;
      idx += (pw & 1u) ? 1u + size[child0[p]] : 1u;
      cur = p;
    }
    if (T > 1) {  // one treelet: its root is the tree's root
      const uint32_t pos = tinv[t], ld = t_ld[t];
      if (pos >= T) {
        atomicOr(err, kErrBuild);
        return;
      }
      idx += (ld & 0xFFFFu) + pos + tpre[pos];
      depth += ld >> 16;
    }
  }
  if (idx >= M) {
    atomicOr(err, kErrBuild);
    return;
  }
  {  // the tree depth: one atomic per warp's flattened nodes
    const uint32_t act = __activemask();
    const uint32_t dmax = __reduce_max_sync(act, depth);
    if ((threadIdx.x & 31u) == (uint32_t)(__ffs(act) - 1)) atomicMax(depth_max, dmax);
  }
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
// Interior nodes of the flattened tree (the last prefix of the flags).
__device__ __forceinline__ uint32_t n_int_of(const uint32_t* info, const uint32_t* is_int, const uint32_t* int_index) {
  const uint32_t M = info[kInfoM];
  return M ? int_index[M - 1] + is_int[M - 1] : 0u;
}

__global__ void k_int_kids(const uint32_t* info, const uint32_t* lin_node, const uint32_t* is_int,
                           const uint32_t* int_index, uint32_t* kids) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t M = info[kInfoM];
  if (i >= M || !is_int[i]) return;
  uint32_t c1 = lin_node[(size_t)i * 3];
  uint32_t k = (i + 1 < M ? is_int[i + 1] : 0u) + (c1 < M ? is_int[c1] : 0u);
  kids[int_index[i]] = k;
}
// slot[rank] = the node's index in the traversal layout; off = exclusive scan of kids
__global__ void k_int_slots(const uint32_t* info, const uint32_t* lin_node, const uint32_t* is_int,
                            const uint32_t* int_index, const uint32_t* off, uint32_t* slot) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t M = info[kInfoM];
  if (i >= M || !is_int[i]) return;
  uint32_t r = int_index[i];
  if (r == 0) slot[0] = 0;
  uint32_t s = 1 + off[r];
  uint32_t c0 = i + 1, c1 = lin_node[(size_t)i * 3];
  if (c0 < M && is_int[c0]) slot[int_index[c0]] = s++;
  if (c1 < M && is_int[c1]) slot[int_index[c1]] = s;
}

// Child-pair traversal layout.
// The record is written twice: into the reference layout and into the
// leaf-split layout's copy of it (k_split_emit then redirects split slots).
__global__ void k_node2(const uint32_t* info, const uint32_t* lin_node, const float* lin_bounds, const uint32_t* is_int,
                        const uint32_t* int_index, const uint32_t* slot, Node2* out, Node2* out_split) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t M = info[kInfoM];
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
  const uint32_t at = slot[int_index[i]];
  out[at] = nd;
  out_split[at] = nd;
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
// Slots past the tree's 2 * n_int (up to n_slots, the scanned length) count 0.
// Range-tree records of the last child slot of n_int interior records.
__device__ __forceinline__ uint32_t last_slot_split_count(const Node2* nodes, uint32_t n_int) {
  const int4 ml = nodes[n_int - 1].meta;
  const uint32_t dl = ml.y < 0 ? split_depth((uint32_t)ml.w & 0x3FFFFFFFu) : 0u;
  return dl ? (1u << dl) - 1u : 0u;
}

// Range-tree records of child slot s (0 for an interior child or a leaf too
// small or too large to split), and the deepest range tree in *max_d: the
// input of the scan that places the records (made inside the scan).
struct SplitCountIn {
  const uint32_t* info;
  const uint32_t* is_int;
  const uint32_t* int_index;
  const Node2* nodes;
  uint32_t* max_d;
  __device__ __forceinline__ uint32_t operator()(uint32_t s) const {
    const uint32_t n_int = n_int_of(info, is_int, int_index);
    if (s >= 2 * n_int) return 0u;
    int4 m = nodes[s >> 1].meta;
    int ref = (s & 1) ? m.y : m.x;
    uint32_t c = (s & 1) ? ((uint32_t)m.w & 0x3FFFFFFFu) : (uint32_t)m.z;
    uint32_t d = ref < 0 ? split_depth(c) : 0u;
    if (d) atomicMax(max_d, d);
    return d ? (1u << d) - 1u : 0u;
  }
};

// One thread per child slot: redirects the slot to its range tree and writes
// the tree's records (boxes = union of the primitive bounds of each range).
// out holds a copy of the reference layout's n_int records on entry and has
// room for n_cap records.
__global__ void k_split_emit(const uint32_t* info, const uint32_t* is_int, const uint32_t* int_index,
                             const Node2* nodes, const uint32_t* off, const uint32_t* sprim,
                             const float4* pb_lo, const float4* pb_hi, uint32_t n_prims, Node2* out, uint32_t n_cap,
                             uint32_t* err) {
  uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t n_int = n_int_of(info, is_int, int_index);
  if (s >= 2 * n_int) return;
  const uint32_t n_split = off[2 * n_int - 1] + last_slot_split_count(nodes, n_int);
  const uint32_t n_out = (uint64_t)n_int + n_split <= n_cap ? n_int + n_split : 0u;
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

// What the host needs once the tree is built, gathered for one copy:
// treelets, flattened nodes, interior nodes, leaf-split records and depth,
// tree depth, SAH nodes, the error word, the root's record and bounds.
constexpr uint32_t kSumWords = 17;
__global__ void k_build_summary(uint32_t* info, const uint32_t* is_int, const uint32_t* int_index,
                                const Node2* nodes, const uint32_t* split_off, const uint32_t* counters,
                                const uint32_t* depth_max, const uint32_t* lin_node, const float* lin_bounds,
                                const uint32_t* err) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  uint32_t* o = info + kInfoSum;
  const uint32_t n_int = n_int_of(info, is_int, int_index);
  o[0] = info[kInfoT];
  o[1] = info[kInfoM];
  o[2] = n_int;
  o[3] = n_int ? split_off[2 * n_int - 1] + last_slot_split_count(nodes, n_int) : 0u;
  o[4] = counters[6];
  o[5] = *depth_max;
  o[6] = counters[0];
  o[7] = *err;
  for (int k = 0; k < 3; ++k) o[8 + k] = lin_node[k];
  for (int k = 0; k < 6; ++k) o[11 + k] = __float_as_uint(lin_bounds[k]);
}
static_assert(kInfoSum + kSumWords <= kInfoWords, "summary block fits the info words");

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
// pair that holds the result. index_values: the values are the keys' input
// positions, made by the first pass (v0 is then only a ping-pong buffer).
cudaError_t radix_sort_pairs(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, uint32_t n, int bits,
                             DevBuf<uint32_t>& hist, DevBuf<uint32_t>& scan_tmp, cudaStream_t st, uint32_t** kres,
                             uint32_t** vres, bool first_hist, bool index_values) {
  uint32_t nblk = div_up(n, kRadixTile);
  *kres = k0;
  *vres = v0;
  if (n <= 1) return index_values && n == 1 ? cudaMemsetAsync(v0, 0, sizeof(uint32_t), st) : cudaSuccess;
  cudaError_t e = hist.ensure((size_t)256 * nblk);
  if (e != cudaSuccess) return e;
  uint32_t *kin = k0, *vin = v0, *kout = k1, *vout = v1;
  for (int shift = 0; shift < bits; shift += 8) {
    int w = bits - shift < 8 ? bits - shift : 8;
    uint32_t dmask = (1u << w) - 1u;
    if (shift > 0 || !first_hist) k_radix_hist<<<nblk, kB, 0, st>>>(kin, n, shift, dmask, hist.p, nblk);
    e = scan_exclusive(hist.p, hist.p, 256 * nblk, scan_tmp, st);
    if (e != cudaSuccess) return e;
    k_radix_scatter<<<nblk, kB, 0, st>>>(kin, (shift == 0 && index_values) ? nullptr : vin, kout, vout, n, shift,
                                         dmask, hist.p, nblk);
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
  // Sizes found on the device are bounded by N, so every buffer is sized
  // before the first kernel and the build reads back from the device only
  // once, at the end: treelets T <= N, flattened nodes M <= 2N - 1, interior
  // nodes < N, leaf-split records < N / 4 + 1 (a leaf of c primitives adds
  // fewer than c / 4).
  const uint32_t N2 = 2 * N;
  const uint32_t NU = 3 * N;  // unified id space [0, 2N + T)
  const uint32_t maxseg = N / (kSmallSeg + 1) + 2;
  const size_t split_cap = (size_t)N + N / 4 + 2;
  WPBR_CUDA(B.pb_lo.ensure(N));
  WPBR_CUDA(B.pb_hi.ensure(N));
  WPBR_CUDA(B.centroid.ensure(N));
  WPBR_CUDA(B.codes.ensure(N));
  WPBR_CUDA(B.cb_enc.ensure(8));
  WPBR_CUDA(B.k0.ensure(N));
  WPBR_CUDA(B.k1.ensure(N));
  WPBR_CUDA(B.v0.ensure(N));
  WPBR_CUDA(B.v1.ensure(N));
  const uint32_t nblk = div_up(N, kRadixTile);
  WPBR_CUDA(B.hist.ensure((size_t)256 * nblk));
  WPBR_CUDA(B.tid.ensure(N));
  WPBR_CUDA(B.tstart.ensure(N));
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
  WPBR_CUDA(B.cur.ensure(N));
  WPBR_CUDA(B.nxt.ensure(N));
  WPBR_CUDA(B.seg_of.ensure(N2));
  WPBR_CUDA(B.pos_lo.ensure(N2));
  WPBR_CUDA(B.pos_hi.ensure(N2));
  WPBR_CUDA(B.posF.ensure(N));
  WPBR_CUDA(B.posT.ensure(N));
  WPBR_CUDA(B.bucket.ensure(N));
  WPBR_CUDA(B.ftl.ensure(N));
  WPBR_CUDA(B.rnk.ensure(N));
  WPBR_CUDA(B.seg_start.ensure(2 * (size_t)maxseg));
  WPBR_CUDA(B.seg_end.ensure(2 * (size_t)maxseg));
  WPBR_CUDA(B.seg_node.ensure(2 * (size_t)maxseg));
  WPBR_CUDA(B.seg_acc.ensure(2 * (size_t)maxseg * kSegWords));
  WPBR_CUDA(B.seg_bk.ensure(2 * (size_t)maxseg * kBucketWords));
  WPBR_CUDA(B.seg_best.ensure(maxseg));
  WPBR_CUDA(B.seg_dec.ensure(maxseg));
  WPBR_CUDA(B.seg_pre.ensure(maxseg));
  WPBR_CUDA(B.chunk_tot.ensure(2 * (size_t)kMaxCoopGrid));
  WPBR_CUDA(B.lvl.ensure(16));
  WPBR_CUDA(B.bar.ensure(4));
  WPBR_CUDA(B.sah_rng.ensure(2 * (size_t)N));
  WPBR_CUDA(B.role.ensure(2 * (size_t)N));
  WPBR_CUDA(B.sah_ld.ensure(N));
  WPBR_CUDA(B.t_ld.ensure(N));
  WPBR_CUDA(B.tinv.ensure(N));
  WPBR_CUDA(B.seg_ld.ensure(2 * (size_t)maxseg));
  WPBR_CUDA(B.med_ld.ensure(maxseg));
  WPBR_CUDA(B.small_ld.ensure(N));
  WPBR_CUDA(B.tpos.ensure((size_t)N + 1));
  WPBR_CUDA(B.med_start.ensure(maxseg));
  WPBR_CUDA(B.med_end.ensure(maxseg));
  WPBR_CUDA(B.med_node.ensure(maxseg));
  WPBR_CUDA(B.small_start.ensure(N));
  WPBR_CUDA(B.small_end.ensure(N));
  WPBR_CUDA(B.small_node.ensure(N));
  WPBR_CUDA(B.sah_axis.ensure(N));
  WPBR_CUDA(B.counters.ensure(8));
  WPBR_CUDA(B.dinfo.ensure(kInfoWords));
  WPBR_CUDA(B.lin_node.ensure((size_t)3 * N2));
  WPBR_CUDA(B.lin_bounds.ensure((size_t)6 * N2));
  WPBR_CUDA(B.is_int.ensure(N2));
  WPBR_CUDA(B.int_index.ensure(N2));
  WPBR_CUDA(B.depth_max.ensure(1));
  WPBR_CUDA(B.int_kids.ensure(N));
  WPBR_CUDA(B.int_slot.ensure(N));
  WPBR_CUDA(B.nodes2.ensure(N));
  WPBR_CUDA(B.nodes_split.ensure(split_cap));
  WPBR_CUDA(B.prims.ensure((size_t)3 * N));
  WPBR_CUDA(B.split_off.ensure(N2));
  if (!B.h_info) WPBR_CUDA(cudaMallocHost((void**)&B.h_info, sizeof(uint32_t) * kInfoWords));

  const unsigned g = div_up(N, kB);
  // A3/A4: centroid bounds start empty (min words all ones, max words zero)
  WPBR_CUDA(cudaMemsetAsync(B.cb_enc.p, 0xFF, 12, st));
  WPBR_CUDA(cudaMemsetAsync(B.cb_enc.p + 3, 0, 12, st));
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
  WPBR_CUDA(scan_exclusive_in(TreeletFlagIn{B.skey}, B.tid.p, N, B.scan_tmp, st));
  k_treelet_ids<<<g, kB, 0, st>>>(B.skey, B.tid.p, B.tstart.p, N, B.dinfo.p);
  // A7
  WPBR_CUDA(cudaMemsetAsync(B.visits.p, 0, sizeof(uint32_t) * NU, st));
  WPBR_CUDA(cudaMemsetAsync(B.parent.p, 0xFF, sizeof(uint32_t) * NU, st));
  if (N > 1)
    k_karras<<<div_up(N - 1, kB), kB, 0, st>>>(B.skey, B.tid.p, B.tstart.p, B.dinfo.p, N, B.rng_lo.p, B.rng_hi.p,
                                               B.child0.p, B.child1.p, B.parent.p);
  k_refit<<<div_up(2 * N, kB), kB, 0, st>>>(N, B.skey, B.sprim, B.tid.p, B.tstart.p, B.dinfo.p, B.rng_lo.p,
                                            B.rng_hi.p, B.child0.p, B.child1.p, B.parent.p, B.visits.p, B.size.p,
                                            B.nb_lo.p, B.nb_hi.p, B.pb_lo.p, B.pb_hi.p, B.troot.p, B.role.p,
                                            ctx->d_err.p);
  // A8: the large segments' levels in one cooperative launch, then the
  // warp-local SAH of the small segments
  {
    int dev = 0, sms = 0, coop = 0, per_sm = 0;
    WPBR_CUDA(cudaGetDevice(&dev));
    WPBR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    WPBR_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    WPBR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sah_levels, kCoopBlock, 0));
    if (!coop || per_sm < 1) return set_err(ctx, WPBR_ERR_CUDA, "bvh_build: cooperative launch unavailable");
    if (per_sm > kCoopPerSM) per_sm = kCoopPerSM;
    if ((uint32_t)(per_sm * sms) > kMaxCoopGrid) per_sm = (int)(kMaxCoopGrid / (uint32_t)sms);
    if (per_sm < 1) return set_err(ctx, WPBR_ERR_CUDA, "bvh_build: too many SMs for the cooperative grid");
    WPBR_CUDA(cudaMemsetAsync(B.bar.p, 0, sizeof(uint32_t) * 4, st));
    CoopSah C{};
    C.N = N;
    C.N2 = N2;
    C.maxseg = maxseg;
    C.T_p = B.dinfo.p + kInfoT;
    C.troot = B.troot.p;
    C.nb_lo = B.nb_lo.p;
    C.nb_hi = B.nb_hi.p;
    C.child0 = B.child0.p;
    C.child1 = B.child1.p;
    C.parent = B.parent.p;
    C.sah_axis = B.sah_axis.p;
    C.sah_rng = B.sah_rng.p;
    C.sah_ld = B.sah_ld.p;
    C.t_ld = B.t_ld.p;
    C.med_ld = B.med_ld.p;
    C.small_ld = B.small_ld.p;
    C.item[0] = B.cur.p;
    C.item[1] = B.nxt.p;
    C.seg_of[0] = B.seg_of.p;
    C.seg_of[1] = B.seg_of.p + N;
    C.plo[0] = B.pos_lo.p;
    C.plo[1] = B.pos_lo.p + N;
    C.phi[0] = B.pos_hi.p;
    C.phi[1] = B.pos_hi.p + N;
    C.bucket = B.bucket.p;
    C.ftl = B.ftl.p;
    C.rnk = B.rnk.p;
    C.posF = B.posF.p;
    C.posT = B.posT.p;
    for (int q = 0; q < 2; ++q) {
      C.sa[q] = B.seg_start.p + (size_t)q * maxseg;
      C.sb[q] = B.seg_end.p + (size_t)q * maxseg;
      C.snode[q] = B.seg_node.p + (size_t)q * maxseg;
      C.sld[q] = B.seg_ld.p + (size_t)q * maxseg;
      C.sacc[q] = B.seg_acc.p + (size_t)q * maxseg * kSegWords;
      C.sbk[q] = B.seg_bk.p + (size_t)q * maxseg * kBucketWords;
    }
    C.sdec = B.seg_dec.p;
    C.sbest = B.seg_best.p;
    C.segpre = B.seg_pre.p;
    C.btot = B.chunk_tot.p;
    C.lvl = B.lvl.p;
    C.small_start = B.small_start.p;
    C.small_end = B.small_end.p;
    C.small_node = B.small_node.p;
    C.med_start = B.med_start.p;
    C.med_end = B.med_end.p;
    C.med_node = B.med_node.p;
    C.counters = B.counters.p;
    C.root_out = B.dinfo.p + kInfoRoot;
    C.bar = B.bar.p;
    C.err = ctx->d_err.p;
    void* args[] = {&C};
    WPBR_CUDA(cudaLaunchCooperativeKernel((const void*)k_sah_levels, dim3((unsigned)(per_sm * sms)),
                                          dim3(kCoopBlock), args, 0, st));
    WPBR_CUDA(cudaFuncSetAttribute((const void*)k_medium_sah, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)kMedSmem));
    MedArgs Md{N, N2, B.troot.p, B.nb_lo.p, B.nb_hi.p, B.child0.p, B.child1.p, B.parent.p, B.sah_axis.p, B.sah_rng.p, B.cur.p,
               B.med_start.p, B.med_end.p, B.med_node.p, B.med_ld.p, B.small_start.p, B.small_end.p, B.small_node.p,
               B.small_ld.p, B.sah_ld.p, B.t_ld.p, B.counters.p, ctx->d_err.p};
    k_medium_sah<<<kMedPerSM * (unsigned)sms, kMedBlock, kMedSmem, st>>>(Md);
    SahArgs A{N, B.troot.p, B.nb_lo.p, B.nb_hi.p, B.sah_rng.p, B.sah_ld.p, B.t_ld.p};
    k_small_sah<<<persistent_grid((const void*)k_small_sah, kB), kB, 0, st>>>(
        A, B.counters.p + 2, B.small_start.p, B.small_end.p, B.small_node.p, B.small_ld.p, B.cur.p, B.counters.p,
        B.sah_axis.p,
        B.nb_lo.p, B.nb_hi.p, B.child0.p, B.child1.p, B.parent.p, N2, ctx->d_err.p);
    WPBR_CUDA(scan_exclusive_in(PosTsizeIn{B.dinfo.p, B.cur.p, B.troot.p, B.size.p, B.tinv.p}, B.tpos.p, N + 1,
                                B.scan_tmp, st));
    k_sah_sizes<<<g, kB, 0, st>>>(B.dinfo.p, B.sah_rng.p, B.tpos.p, B.size.p, N2, ctx->d_err.p);
  }
  // A9
  WPBR_CUDA(cudaMemsetAsync(B.is_int.p, 0, sizeof(uint32_t) * N2, st));
  WPBR_CUDA(cudaMemsetAsync(B.depth_max.p, 0, 4, st));
  k_flatten<<<div_up((uint64_t)N2 + N, kB), kB, 0, st>>>(N, B.dinfo.p, B.skey, B.tid.p, B.tstart.p,
                                                          B.rng_lo.p, B.rng_hi.p, B.child0.p, B.parent.p, B.size.p,
                                                          B.sah_axis.p, B.nb_lo.p, B.nb_hi.p, B.sah_ld.p,
                                                          B.sah_rng.p, B.t_ld.p, B.tinv.p, B.tpos.p, B.role.p, B.lin_node.p,
                                                          B.lin_bounds.p, B.is_int.p, B.depth_max.p, ctx->d_err.p);
  WPBR_CUDA(scan_exclusive(B.is_int.p, B.int_index.p, N2, B.scan_tmp, st));
  WPBR_CUDA(cudaMemsetAsync(B.int_kids.p, 0, sizeof(uint32_t) * N, st));
  const unsigned g2 = div_up(N2, kB);
  k_int_kids<<<g2, kB, 0, st>>>(B.dinfo.p, B.lin_node.p, B.is_int.p, B.int_index.p, B.int_kids.p);
  WPBR_CUDA(scan_exclusive(B.int_kids.p, B.int_kids.p, N, B.scan_tmp, st));
  k_int_slots<<<g2, kB, 0, st>>>(B.dinfo.p, B.lin_node.p, B.is_int.p, B.int_index.p, B.int_kids.p, B.int_slot.p);
  k_node2<<<g2, kB, 0, st>>>(B.dinfo.p, B.lin_node.p, B.lin_bounds.p, B.is_int.p, B.int_index.p, B.int_slot.p,
                             B.nodes2.p, B.nodes_split.p);
  k_prims<<<g, kB, 0, st>>>(S, B.sprim, B.prims.p);
  // leaf-split layout (the default binary traversal); a tree whose root is a
  // leaf keeps the reference layout
  WPBR_CUDA(cudaMemsetAsync(B.counters.p + 6, 0, 4, st));
  WPBR_CUDA(scan_exclusive_in(SplitCountIn{B.dinfo.p, B.is_int.p, B.int_index.p, B.nodes2.p, B.counters.p + 6},
                              B.split_off.p, N2, B.scan_tmp, st));
  k_split_emit<<<g2, kB, 0, st>>>(B.dinfo.p, B.is_int.p, B.int_index.p, B.nodes2.p, B.split_off.p,
                                  B.sprim, B.pb_lo.p, B.pb_hi.p, N, B.nodes_split.p, (uint32_t)split_cap,
                                  ctx->d_err.p);
  k_build_summary<<<1, 32, 0, st>>>(B.dinfo.p, B.is_int.p, B.int_index.p, B.nodes2.p, B.split_off.p,
                                    B.counters.p, B.depth_max.p, B.lin_node.p, B.lin_bounds.p, ctx->d_err.p);
  WPBR_CUDA(cudaGetLastError());
  WPBR_CUDA(cudaMemcpyAsync(B.h_info, B.dinfo.p + kInfoSum, sizeof(uint32_t) * kSumWords, cudaMemcpyDeviceToHost,
                            st));
  WPBR_CUDA(cudaStreamSynchronize(st));
  const uint32_t* o = B.h_info;
  const uint32_t T = o[0], M = o[1], n_int = o[2], nsah = o[6], derr = o[7];
  uint32_t n_split = o[3], split_d = o[4];
  const uint32_t depth = o[5];
  if (derr) return set_err(ctx, WPBR_ERR_CUDA, "bvh_build: device invariant violated");
  if (T == 0 || nsah != T - 1) return set_err(ctx, WPBR_ERR_CUDA, "bvh_build: SAH node count mismatch");
  if ((uint64_t)n_int + n_split > split_cap || M == 0 || M >= N2)
    return set_err(ctx, WPBR_ERR_CUDA, "bvh_build: tree sizes out of range");
  B.T = T;
  B.M = M;
  B.n_int = n_int;
  B.max_depth = depth;
  if (!n_int || !n_split) {
    n_split = 0;
    split_d = 0;
  }
  BvhView v{};
  v.nodes = n_split ? B.nodes_split.p : B.nodes2.p;
  v.nodes_ref = B.nodes2.p;
  v.n_ref_int = n_int;
  v.ref_depth = depth;
  v.prims = B.prims.p;
  v.empty = 0;
  const uint32_t* node0 = o + 8;
  bool root_leaf = node0[1] > 0;
  v.root_ref = root_leaf ? ~(int)node0[0] : 0;
  v.root_count = root_leaf ? node0[1] : 0;
  for (int k = 0; k < 3; ++k) {
    memcpy(&v.root_lo[k], o + 11 + k, 4);
    memcpy(&v.root_hi[k], o + 14 + k, 4);
  }
  v.max_depth = depth + split_d;
  v.stack_cap = kDefaultStackCap;
  v.step_cap = kDefaultStepCap;
  v.n_prims = N;
  v.n_int = n_int + n_split;
  B.view = v;
  B.built = true;
  return WPBR_OK;
}

}  // namespace wpbr
