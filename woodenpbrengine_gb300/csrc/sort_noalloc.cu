// sort_noalloc.cu — wpbr_sort_morton_noalloc: the Morton-code sort of the
// LBVH build (stable LSD radix, 8-bit digits) for callers that cannot
// allocate device memory.
//
// Who needs it: hosts that own every byte of device memory through their own
// arena and forbid allocation inside a job (the reference engine hands each
// ECS job a linear temp allocator and resets it after the job), and real-time
// loops that must not take cudaMalloc's device-wide synchronisation. They pass their own input and output buffers
// and the sort keeps its temporaries in one file-scope device array.
//
// The array (g_scratch, about 8.5 MB) is part of the library image: every
// GPU that loads the library holds it until the process exits. Host code
// cannot use the array's name as a device address, so each call made outside
// stream capture looks the address up (cudaGetSymbolAddress, with the
// caller's device and context current) and remembers it per device; a call
// made while its stream is being captured uses the remembered address, which
// is why the first call on a device must come before any stream capture (such
// a call is refused otherwise). Looking the address up again on every
// uncaptured call keeps it right after a cudaDeviceReset or when the caller
// switches to another context of the same device. Every call shares the one
// array and leaves its last contents behind; calls whose GPU work overlaps
// (two streams, or two host threads) race on it and must be serialised by the
// caller.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "common.cuh"
#include "wpbr_gpu.h"

namespace {

constexpr uint32_t kMaxKeys = WPBR_SORT_NOALLOC_MAX_KEYS;
constexpr int kBlk = 256;
constexpr int kItems = 8;
constexpr int kTileKeys = kBlk * kItems;                       // 2048 keys per block
constexpr uint32_t kMaxBlocks = kMaxKeys / kTileKeys;          // 512
constexpr uint32_t kHist = 256 * kMaxBlocks;                   // 131072 counters
constexpr uint32_t kScanTiles = kHist / kTileKeys;             // 64 tile sums

struct Scratch {
  uint32_t keys[kMaxKeys];
  uint32_t vals[kMaxKeys];
  uint32_t hist[kHist];
  uint32_t tile_sums[kScanTiles];
};

static __device__ __align__(256) Scratch g_scratch;

// Per-device address of g_scratch last looked up outside stream capture.
constexpr int kMaxDevices = 64;
Scratch* g_addr[kMaxDevices] = {};
std::mutex g_mu;
thread_local char g_msg[256] = "";

__global__ void k_hist(const uint32_t* keys, uint32_t n, int shift, uint32_t dmask, uint32_t* hist, uint32_t nblk) {
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  uint32_t base = blockIdx.x * kTileKeys;
  for (int k = 0; k < kItems; ++k) {
    uint32_t i = base + threadIdx.x + k * kBlk;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & dmask], 1u);
  }
  __syncthreads();
  hist[threadIdx.x * nblk + blockIdx.x] = cnt[threadIdx.x];
}

// exclusive scan of one 2048-entry tile per block; optional tile totals
__global__ void k_scan(uint32_t* data, uint32_t n, uint32_t* sums) {
  __shared__ uint32_t sh[kTileKeys];
  __shared__ uint32_t ws[kBlk / 32];
  uint32_t base = blockIdx.x * kTileKeys;
  for (int k = 0; k < kItems; ++k) {
    uint32_t i = base + threadIdx.x + k * kBlk;
    sh[threadIdx.x + k * kBlk] = i < n ? data[i] : 0u;
  }
  __syncthreads();
  uint32_t v[kItems], sum = 0;
  for (int k = 0; k < kItems; ++k) {
    v[k] = sh[threadIdx.x * kItems + k];
    sum += v[k];
  }
  uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5, x = sum;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t a = lane < kBlk / 32 ? ws[lane] : 0u, inc = a;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
      if (lane >= (uint32_t)o) inc += y;
    }
    if (lane < kBlk / 32) ws[lane] = inc - a;
  }
  __syncthreads();
  uint32_t run = (x - sum) + ws[w], start = run;
  for (int k = 0; k < kItems; ++k) {
    sh[threadIdx.x * kItems + k] = run;
    run += v[k];
  }
  __syncthreads();
  for (int k = 0; k < kItems; ++k) {
    uint32_t i = base + threadIdx.x + k * kBlk;
    if (i < n) data[i] = sh[threadIdx.x + k * kBlk];
  }
  if (sums && threadIdx.x == kBlk - 1) sums[blockIdx.x] = start + sum;
}

__global__ void k_add(uint32_t* data, uint32_t n, const uint32_t* sums) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) data[i] += sums[i / kTileKeys];
}

// Stable scatter; vin == nullptr means the identity permutation (first pass).
__global__ void k_scatter(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t n,
                          int shift, uint32_t dmask, const uint32_t* offs, uint32_t nblk) {
  __shared__ uint32_t s_off[256];
  __shared__ uint32_t s_w[kBlk / 32][256];
  __shared__ uint32_t s_round[256];
  s_off[threadIdx.x] = offs[threadIdx.x * nblk + blockIdx.x];
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5, lt = (1u << lane) - 1u;
  uint32_t base = blockIdx.x * kTileKeys;
  for (int r = 0; r < kItems; ++r) {
    for (int q = 0; q < kBlk / 32; ++q) s_w[q][threadIdx.x] = 0;
    __syncthreads();
    uint32_t i = base + r * kBlk + threadIdx.x;
    bool valid = i < n;
    uint32_t key = valid ? kin[i] : 0u;
    uint32_t val = valid ? (vin ? vin[i] : i) : 0u;
    uint32_t d = valid ? ((key >> shift) & dmask) : (256u + lane);
    uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
    uint32_t rank = __popc(peers & lt);
    if (valid && rank == 0) s_w[w][d] = __popc(peers);
    __syncthreads();
    uint32_t acc = 0;
    for (int q = 0; q < kBlk / 32; ++q) {
      uint32_t c = s_w[q][threadIdx.x];
      s_w[q][threadIdx.x] = acc;
      acc += c;
    }
    s_round[threadIdx.x] = acc;
    __syncthreads();
    if (valid) {
      uint32_t pos = s_off[d] + s_w[w][d] + rank;
      kout[pos] = key;
      vout[pos] = val;
    }
    __syncthreads();
    s_off[threadIdx.x] += s_round[threadIdx.x];
    __syncthreads();
  }
}

wpbr_status fail(wpbr_status st, const char* msg) {
  snprintf(g_msg, sizeof(g_msg), "%s", msg);
  return st;
}

}  // namespace

extern "C" {

WPBR_API const char* wpbr_sort_morton_noalloc_error(void) { return g_msg; }

WPBR_API wpbr_status wpbr_sort_morton_noalloc(const uint32_t* d_codes, uint32_t n, uint32_t key_bits,
                                              uint32_t* d_sorted_codes, uint32_t* d_perm, void* stream) {
  g_msg[0] = '\0';
  if (n > kMaxKeys) {
    char b[160];
    snprintf(b, sizeof(b), "sort_morton_noalloc: n = %u exceeds the fixed scratch capacity of %u keys", n, kMaxKeys);
    return fail(WPBR_ERR_INVALID_ARG, b);
  }
  if (key_bits != 24 && key_bits != 30) return fail(WPBR_ERR_INVALID_ARG, "sort_morton_noalloc: key_bits must be 24 or 30");
  if (n == 0) return WPBR_OK;
  if (!d_codes || !d_sorted_codes || !d_perm)
    return fail(WPBR_ERR_INVALID_ARG, "sort_morton_noalloc: null buffer");
  if (d_sorted_codes == d_codes || d_perm == d_codes || d_perm == d_sorted_codes)
    return fail(WPBR_ERR_INVALID_ARG, "sort_morton_noalloc: buffers must not alias");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return fail(WPBR_ERR_NO_DEVICE, "sort_morton_noalloc: no current CUDA device");
  }
  cudaStream_t st = (cudaStream_t)stream;
  // A stream whose capture status cannot be read (the legacy stream while
  // another stream captures in global mode) counts as capturing.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
    cudaGetLastError();
    cap = cudaStreamCaptureStatusActive;
  }
  Scratch* S;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (cap == cudaStreamCaptureStatusNone) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
      if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return fail(WPBR_ERR_CUDA, "sort_morton_noalloc: cudaGetSymbolAddress(g_scratch) failed");
      }
      g_addr[dev] = (Scratch*)p;
    } else if (!g_addr[dev]) {
      return fail(WPBR_ERR_INVALID_ARG,
                  "sort_morton_noalloc: the first call on a device must come before any stream capture");
    }
    S = g_addr[dev];
  }
  const uint32_t nblk = (n + kTileKeys - 1) / kTileKeys;
  const uint32_t nh = 256 * nblk;
  const uint32_t ntiles = (nh + kTileKeys - 1) / kTileKeys;
  const int passes = key_bits == 24 ? 3 : 4;
  // ping-pong between the caller's output buffers and the scratch pair so the
  // last pass lands in the output: 3 passes in->out->S->out, 4 in->S->out->S->out
  const uint32_t* kin = d_codes;
  const uint32_t* vin = nullptr;
  for (int ps = 0; ps < passes; ++ps) {
    bool to_out = ((passes - 1 - ps) % 2) == 0;
    uint32_t* kout = to_out ? d_sorted_codes : S->keys;
    uint32_t* vout = to_out ? d_perm : S->vals;
    int shift = 8 * ps;
    uint32_t dmask = (ps == 3) ? 0x3Fu : 0xFFu;
    k_hist<<<nblk, kBlk, 0, st>>>(kin, n, shift, dmask, S->hist, nblk);
    k_scan<<<ntiles, kBlk, 0, st>>>(S->hist, nh, ntiles > 1 ? S->tile_sums : nullptr);
    if (ntiles > 1) {
      k_scan<<<1, kBlk, 0, st>>>(S->tile_sums, ntiles, nullptr);
      k_add<<<(nh + 255) / 256, 256, 0, st>>>(S->hist, nh, S->tile_sums);
    }
    k_scatter<<<nblk, kBlk, 0, st>>>(kin, vin, kout, vout, n, shift, dmask, S->hist, nblk);
    kin = kout;
    vin = vout;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(WPBR_ERR_CUDA, "sort_morton_noalloc: kernel launch failed");
  return WPBR_OK;
}

}  // extern "C"
