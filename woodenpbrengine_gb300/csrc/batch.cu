// batch.cu — batched scenes (wpbr_batch_*, include/wpbr_gpu.h).
//
// A batch owns one wpbr_ctx per scene (scene buffers, per-pixel render state,
// film) and one pooled device arena holding every scene's traversal layout
// (Node2 array and primitive records, each block 256-byte aligned). A sample pass of all scenes is one CUDA graph: a fork event on the
// batch stream, one branch per scene with the five kernels of the fused pass
// (render_pass_launch) on that scene's stream, and a join back. All branches
// read the pass index from one device word, so a pass costs one 4-byte copy and
// one graph launch whatever the number of scenes.
//
// The persistent traversal grid of each scene is either one full wave of
// resident blocks or ceil(pixels / rays_per_block) blocks; the autotuner times
// the graph for each candidate depth and keeps the fastest, remembering the
// choice in a text cache keyed by device, scene count and a hash of the
// scenes' film sizes and primitive counts.
#include <cuda_runtime.h>

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "common.cuh"
#include "ctx.hpp"
#include "wpbr_gpu.h"

struct wpbr_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  std::vector<wpbr_ctx*> scenes;
  bool built = false, ready = false;
  uint32_t spp = 0;
  uint64_t arena_bytes = 0, total_prims = 0;
  wpbr::DevBuf<unsigned char> arena;
  wpbr::DevBuf<uint32_t> pass_dev;
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  uint32_t rays_per_block = 0;
  uint32_t tune_source = 0;
};

namespace {

using namespace wpbr;

constexpr uint32_t kCandidates[4] = {0u, 4096u, 1024u, 256u};

wpbr_status berr(wpbr_batch* b, wpbr_status st, const std::string& msg) {
  if (b) b->err = msg;
  return st;
}
wpbr_status bcuda(wpbr_batch* b, cudaError_t e, const char* what) {
  cudaGetLastError();
  return berr(b, e == cudaErrorMemoryAllocation ? WPBR_ERR_OOM : WPBR_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}
wpbr_status from_scene(wpbr_batch* b, size_t k, wpbr_status st) {
  if (st != WPBR_OK) b->err = "scene " + std::to_string(k) + ": " + b->scenes[k]->err;
  return st;
}

#define BATCH_CUDA(call)                              \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return bcuda(b, e_, #call); \
  } while (0)

void drop_graph(wpbr_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
}

// Per-scene persistent grid for a queue depth: 0 keeps one full wave.
void apply_depth(wpbr_batch* b, uint32_t rpb) {
  for (wpbr_ctx* c : b->scenes) {
    uint64_t n = (uint64_t)c->rs.W * c->rs.H;
    c->rs.trace_grid = rpb ? (uint32_t)((n + rpb - 1) / rpb) : 0u;
    if (rpb && c->rs.trace_grid == 0) c->rs.trace_grid = 1;
  }
}

// Captures one pass of every scene as a fork/join graph on the batch stream.
wpbr_status capture_graph(wpbr_batch* b) {
  drop_graph(b);
  cudaGraph_t g = nullptr;
  BATCH_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  wpbr_status st = WPBR_OK;
  cudaError_t e = cudaEventRecord(b->fork, b->stream);
  for (size_t k = 0; k < b->scenes.size() && e == cudaSuccess && st == WPBR_OK; ++k) {
    wpbr_ctx* c = b->scenes[k];
    e = cudaStreamWaitEvent(c->stream, b->fork, 0);
    if (e != cudaSuccess) break;
    st = render_pass_launch(c);
    if (st != WPBR_OK) {
      from_scene(b, k, st);
      break;
    }
    e = cudaEventRecord(b->join[k], c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->join[k], 0);
  }
  cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
  if (st == WPBR_OK && e == cudaSuccess && e2 == cudaSuccess && g) e = cudaGraphInstantiate(&b->graph, g, 0);
  if (g) cudaGraphDestroy(g);
  if (st != WPBR_OK) {
    cudaGetLastError();
    return st;
  }
  if (e != cudaSuccess) return bcuda(b, e, "batch graph capture");
  if (e2 != cudaSuccess) return bcuda(b, e2, "batch graph capture");
  if (!b->graph) return berr(b, WPBR_ERR_CUDA, "batch graph capture produced no graph");
  return WPBR_OK;
}

// A failed capture leaves no graph, so the batch stops being ready: later
// render calls return WPBR_ERR_NOT_BUILT until wpbr_batch_render_setup
// succeeds again, instead of launching a null graph.
wpbr_status capture(wpbr_batch* b) {
  wpbr_status st = capture_graph(b);
  if (st != WPBR_OK) b->ready = false;
  return st;
}

wpbr_status launch_pass(wpbr_batch* b, uint32_t pass) {
  BATCH_CUDA(cudaMemcpyAsync(b->pass_dev.p, &pass, 4, cudaMemcpyHostToDevice, b->stream));
  BATCH_CUDA(cudaGraphLaunch(b->graph, b->stream));
  return WPBR_OK;
}

uint64_t fnv1a(uint64_t h, uint64_t v) {
  for (int i = 0; i < 8; ++i) {
    h ^= (v >> (8 * i)) & 0xFFu;
    h *= 0x100000001B3ull;
  }
  return h;
}

std::string tune_key(wpbr_batch* b) {
  cudaDeviceProp p{};
  cudaGetDeviceProperties(&p, b->device);
  uint64_t h = 0xCBF29CE484222325ull;
  for (wpbr_ctx* c : b->scenes) {
    h = fnv1a(h, ((uint64_t)c->rs.W << 32) | c->rs.H);
    h = fnv1a(h, c->N);
  }
  std::string name(p.name);
  for (char& ch : name)
    if (ch == ' ') ch = '_';
  char buf[256];
  snprintf(buf, sizeof(buf), "%s|sm%d|%d|n%zu|%016llx", name.c_str(), p.major * 10 + p.minor,
           p.multiProcessorCount, b->scenes.size(), (unsigned long long)h);
  return buf;
}

std::string cache_path() {
  const char* env = getenv("WPBR_AUTOTUNE_CACHE");
  if (env && *env) return env;
  const char* home = getenv("HOME");
  if (!home || !*home) return "";
  std::string dir = std::string(home) + "/.cache";
  mkdir(dir.c_str(), 0755);  // may exist already
  return dir + "/wpbr_autotune.txt";
}

bool cache_lookup(const std::string& key, uint32_t* rpb) {
  std::string path = cache_path();
  if (path.empty()) return false;
  FILE* f = fopen(path.c_str(), "r");
  if (!f) return false;
  char line[512];
  bool found = false;
  while (fgets(line, sizeof(line), f)) {
    char k[400];
    unsigned v = 0;
    if (sscanf(line, "%399s %u", k, &v) == 2 && key == k) {
      bool valid = false;
      for (uint32_t c : kCandidates) valid |= (c == v);
      if (valid) {
        *rpb = v;
        found = true;  // the last entry for a key wins
      }
    }
  }
  fclose(f);
  return found;
}

void cache_store(const std::string& key, uint32_t rpb, float ms) {
  std::string path = cache_path();
  if (path.empty()) return;
  FILE* f = fopen(path.c_str(), "a");
  if (!f) return;
  fprintf(f, "%s %u %.4f\n", key.c_str(), rpb, ms);
  fclose(f);
}

wpbr_status clear_films(wpbr_batch* b) {
  for (wpbr_ctx* c : b->scenes) {
    size_t n = (size_t)c->rs.W * c->rs.H;
    BATCH_CUDA(cudaMemsetAsync(c->rs.acc.p, 0, n * 4 * sizeof(float), b->stream));
  }
  BATCH_CUDA(cudaStreamSynchronize(b->stream));
  return WPBR_OK;
}

}  // namespace

extern "C" {

WPBR_API wpbr_status wpbr_batch_create(int device, wpbr_batch** out) {
  if (!out) return WPBR_ERR_INVALID_ARG;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return WPBR_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return WPBR_ERR_INVALID_ARG;
  wpbr_batch* b = new (std::nothrow) wpbr_batch();
  if (!b) return WPBR_ERR_OOM;
  b->device = device;
  e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = b->pass_dev.ensure(1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->stream) cudaStreamDestroy(b->stream);
    b->pass_dev.release();
    delete b;
    return e == cudaErrorMemoryAllocation ? WPBR_ERR_OOM : WPBR_ERR_CUDA;
  }
  b->own_stream = true;
  *out = b;
  return WPBR_OK;
}

WPBR_API void wpbr_batch_destroy(wpbr_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  for (wpbr_ctx* c : b->scenes) wpbr_destroy(c);  // traversal blocks live in the arena
  for (cudaEvent_t ev : b->join) cudaEventDestroy(ev);
  if (b->fork) cudaEventDestroy(b->fork);
  b->arena.release();
  b->pass_dev.release();
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

WPBR_API const char* wpbr_batch_last_error(const wpbr_batch* b) { return b ? b->err.c_str() : "null batch"; }

WPBR_API wpbr_status wpbr_batch_add_scene(wpbr_batch* b, const wpbr_scene_desc* scene, uint32_t quirks,
                                          uint32_t* index) {
  if (!b || !scene) return WPBR_ERR_INVALID_ARG;
  if (b->built) return berr(b, WPBR_ERR_INVALID_ARG, "batch_add_scene: batch already built");
  cudaSetDevice(b->device);
  wpbr_ctx* c = nullptr;
  wpbr_status st = wpbr_create(b->device, &c);
  if (st != WPBR_OK) return berr(b, st, "batch_add_scene: context creation failed");
  st = wpbr_set_quirks(c, quirks);
  if (st == WPBR_OK) st = wpbr_scene_upload(c, scene);
  if (st != WPBR_OK) {
    b->err = std::string("batch_add_scene: ") + c->err;
    wpbr_destroy(c);
    return st;
  }
  cudaEvent_t ev = nullptr;
  cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    wpbr_destroy(c);
    return bcuda(b, e, "batch_add_scene: event");
  }
  if (index) *index = (uint32_t)b->scenes.size();
  b->scenes.push_back(c);
  b->join.push_back(ev);
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_batch_build(wpbr_batch* b) {
  if (!b) return WPBR_ERR_INVALID_ARG;
  if (b->built) return berr(b, WPBR_ERR_INVALID_ARG, "batch_build: already built");
  if (b->scenes.empty()) return berr(b, WPBR_ERR_INVALID_ARG, "batch_build: no scenes");
  cudaSetDevice(b->device);
  // build one scene at a time; each frees its build scratch before the next
  std::vector<uint64_t> off_nodes(b->scenes.size()), off_prims(b->scenes.size());
  uint64_t total = 0, prims = 0;
  auto block = [&total](uint64_t bytes) {
    uint64_t at = total;
    total += (bytes + 255) & ~(uint64_t)255;
    return at;
  };
  for (size_t k = 0; k < b->scenes.size(); ++k) {
    wpbr_ctx* c = b->scenes[k];
    wpbr_status st = bvh_build(c);
    if (st != WPBR_OK) return from_scene(b, k, st);
    bvh_release(c, true);
    const BvhView& v = c->bvh.view;
    off_nodes[k] = block(v.empty ? 0 : (uint64_t)v.n_int * sizeof(Node2));
    off_prims[k] = block(v.empty ? 0 : (uint64_t)3 * v.n_prims * sizeof(float4));
    prims += c->N;
  }
  // one arena for every traversal layout
  BATCH_CUDA(b->arena.ensure(total ? total : 256));
  for (size_t k = 0; k < b->scenes.size(); ++k) {
    wpbr_ctx* c = b->scenes[k];
    BvhView& v = c->bvh.view;
    Node2* nd = (Node2*)(b->arena.p + off_nodes[k]);
    float4* pd = (float4*)(b->arena.p + off_prims[k]);
    if (!v.empty) {
      if (v.n_int)
        BATCH_CUDA(cudaMemcpyAsync(nd, v.nodes, (size_t)v.n_int * sizeof(Node2), cudaMemcpyDeviceToDevice,
                                   c->stream));
      BATCH_CUDA(cudaMemcpyAsync(pd, v.prims, (size_t)3 * v.n_prims * sizeof(float4), cudaMemcpyDeviceToDevice,
                                 c->stream));
    }
    BATCH_CUDA(cudaStreamSynchronize(c->stream));
    c->bvh.nodes2.release();
    c->bvh.nodes_split.release();
    c->bvh.prims.release();
    v.nodes = nd;
    v.nodes_ref = nullptr;  // the arena keeps the layout traversed only
    v.n_ref_int = 0;
    v.prims = pd;
  }
  b->arena_bytes = total;
  b->total_prims = prims;
  b->built = true;
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_batch_render_setup(wpbr_batch* b, uint32_t spp, uint32_t seed, uint32_t first_stream) {
  if (!b) return WPBR_ERR_INVALID_ARG;
  if (!b->built) return berr(b, WPBR_ERR_NOT_BUILT, "batch_render_setup: batch not built");
  if (spp == 0) return berr(b, WPBR_ERR_INVALID_ARG, "batch_render_setup: spp must be > 0");
  cudaSetDevice(b->device);
  BATCH_CUDA(cudaStreamSynchronize(b->stream));
  b->ready = false;
  for (size_t k = 0; k < b->scenes.size(); ++k) {
    wpbr_ctx* c = b->scenes[k];
    wpbr_status st = render_setup(c, spp, seed, first_stream + (uint32_t)k);
    if (st != WPBR_OK) return from_scene(b, k, st);
    c->rs.pass_ptr = b->pass_dev.p;
    BATCH_CUDA(cudaStreamSynchronize(c->stream));  // film clears done before the graph runs
  }
  b->spp = spp;
  apply_depth(b, b->rays_per_block);
  wpbr_status st = capture(b);
  if (st != WPBR_OK) return st;
  b->ready = true;
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_batch_set_rays_per_block(wpbr_batch* b, uint32_t rays_per_block) {
  if (!b) return WPBR_ERR_INVALID_ARG;
  b->rays_per_block = rays_per_block;
  b->tune_source = 3;
  if (!b->ready) return WPBR_OK;
  cudaSetDevice(b->device);
  BATCH_CUDA(cudaStreamSynchronize(b->stream));
  apply_depth(b, rays_per_block);
  return capture(b);
}

WPBR_API wpbr_status wpbr_batch_autotune(wpbr_batch* b, int use_cache) {
  if (!b) return WPBR_ERR_INVALID_ARG;
  if (!b->ready) return berr(b, WPBR_ERR_NOT_BUILT, "batch_autotune: no pass graph (render_setup not called, or the last graph capture failed)");
  cudaSetDevice(b->device);
  std::string key = tune_key(b);
  uint32_t rpb = 0;
  if (use_cache && cache_lookup(key, &rpb)) {
    b->rays_per_block = rpb;
    b->tune_source = 2;
    BATCH_CUDA(cudaStreamSynchronize(b->stream));
    apply_depth(b, rpb);
    return capture(b);
  }
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  BATCH_CUDA(cudaEventCreate(&t0));
  BATCH_CUDA(cudaEventCreate(&t1));
  float best_ms = 0.0f;
  uint32_t best = 0;
  bool have = false;
  wpbr_status st = WPBR_OK;
  for (uint32_t cand : kCandidates) {
    apply_depth(b, cand);
    st = capture(b);
    if (st != WPBR_OK) break;
    st = launch_pass(b, 0);  // warm-up
    for (uint32_t i = 0; i < 3 && st == WPBR_OK; ++i) {
      if (i == 0 && cudaEventRecord(t0, b->stream) != cudaSuccess) st = WPBR_ERR_CUDA;
      if (st == WPBR_OK) st = launch_pass(b, (i + 1) % b->spp);
    }
    if (st != WPBR_OK) break;
    cudaError_t e = cudaEventRecord(t1, b->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(t1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
    if (e != cudaSuccess) {
      st = bcuda(b, e, "batch_autotune timing");
      break;
    }
    if (!have || ms < best_ms) {
      best_ms = ms;
      best = cand;
      have = true;
    }
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (st != WPBR_OK) return st;
  cache_store(key, best, best_ms / 3.0f);
  b->rays_per_block = best;
  b->tune_source = 1;
  apply_depth(b, best);
  st = capture(b);
  if (st != WPBR_OK) return st;
  return clear_films(b);
}

WPBR_API wpbr_status wpbr_batch_render_pass(wpbr_batch* b, uint32_t pass) {
  if (!b) return WPBR_ERR_INVALID_ARG;
  if (!b->ready) return berr(b, WPBR_ERR_NOT_BUILT, "batch_render_pass: no pass graph (render_setup not called, or the last graph capture failed)");
  if (pass >= b->spp) return berr(b, WPBR_ERR_INVALID_ARG, "batch_render_pass: pass >= spp");
  cudaSetDevice(b->device);
  return launch_pass(b, pass);
}

WPBR_API wpbr_status wpbr_batch_render(wpbr_batch* b) {
  if (!b) return WPBR_ERR_INVALID_ARG;
  if (!b->ready) return berr(b, WPBR_ERR_NOT_BUILT, "batch_render: no pass graph (render_setup not called, or the last graph capture failed)");
  cudaSetDevice(b->device);
  for (uint32_t p = 0; p < b->spp; ++p) {
    wpbr_status st = launch_pass(b, p);
    if (st != WPBR_OK) return st;
  }
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_batch_synchronize(wpbr_batch* b) {
  if (!b) return WPBR_ERR_INVALID_ARG;
  cudaSetDevice(b->device);
  BATCH_CUDA(cudaStreamSynchronize(b->stream));
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_batch_info_get(const wpbr_batch* b, wpbr_batch_info* out) {
  if (!b || !out) return WPBR_ERR_INVALID_ARG;
  memset(out, 0, sizeof(*out));
  out->n_scenes = (uint32_t)b->scenes.size();
  out->spp = b->spp;
  for (const wpbr_ctx* c : b->scenes) out->total_pixels += (uint64_t)c->cam.W * c->cam.H;
  out->total_prims = b->total_prims;
  out->arena_bytes = b->arena_bytes;
  out->rays_per_block = b->rays_per_block;
  out->autotune_source = b->tune_source;
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_batch_film_size(const wpbr_batch* b, uint32_t scene, uint32_t* w, uint32_t* h) {
  if (!b || scene >= b->scenes.size()) return WPBR_ERR_INVALID_ARG;
  if (w) *w = b->scenes[scene]->cam.W;
  if (h) *h = b->scenes[scene]->cam.H;
  return WPBR_OK;
}

WPBR_API wpbr_status wpbr_batch_film_read(wpbr_batch* b, uint32_t scene, float* acc_L, float* acc_w) {
  if (!b || scene >= b->scenes.size()) return WPBR_ERR_INVALID_ARG;
  if (!b->ready) return berr(b, WPBR_ERR_NOT_BUILT, "batch_film_read: no pass graph (render_setup not called, or the last graph capture failed)");
  cudaSetDevice(b->device);
  BATCH_CUDA(cudaStreamSynchronize(b->stream));
  return from_scene(b, scene, wpbr_film_read(b->scenes[scene], acc_L, acc_w));
}

WPBR_API wpbr_status wpbr_batch_set_stream(wpbr_batch* b, void* stream) {
  if (!b) return WPBR_ERR_INVALID_ARG;
  if (!stream) return berr(b, WPBR_ERR_INVALID_ARG, "batch_set_stream: the legacy default stream cannot be captured");
  cudaSetDevice(b->device);
  BATCH_CUDA(cudaStreamSynchronize(b->stream));
  if (b->own_stream) cudaStreamDestroy(b->stream);
  b->stream = (cudaStream_t)stream;
  b->own_stream = false;
  if (!b->ready) return WPBR_OK;
  return capture(b);
}

WPBR_API wpbr_status wpbr_batch_check_device_errors(wpbr_batch* b) {
  if (!b) return WPBR_ERR_INVALID_ARG;
  cudaSetDevice(b->device);
  BATCH_CUDA(cudaStreamSynchronize(b->stream));
  for (size_t k = 0; k < b->scenes.size(); ++k) {
    wpbr_status st = wpbr_check_device_errors(b->scenes[k]);
    if (st != WPBR_OK) return from_scene(b, k, st);
  }
  return WPBR_OK;
}

}  // extern "C"
