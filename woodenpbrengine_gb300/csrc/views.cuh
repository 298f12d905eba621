// views.cuh — POD views of device-resident scene and BVH data, passed to
// kernels by value.
#pragma once

#include <cuda_runtime.h>

#include "camera.cuh"
#include "geom.cuh"
#include "shade.cuh"
#include "texture.cuh"
#include "wpbr_scene.h"

namespace wpbr {

struct SceneView {
  uint32_t ns, nt, N;
  const Xf* sph_o2w;
  const Xf* sph_w2o;
  const float* sph_r;
  const uint32_t* sph_mat;
  const float* pos;        // nv*3
  const uint32_t* idx;     // nt*3
  const float* nrm;        // nv*3 or null
  const float* tan;        // nv*3 or null
  const float* uv;         // nv*2 or null
  const uint32_t* tri_mat;
  const uint32_t* tri_flags;
  const wpbr_material* mats;
  const wpbr_light* lights;
  uint32_t nlights;
  int has_env;
  EnvView env;
  CameraParams cam;
  uint32_t quirks;
  TexView tex;  // textures of the textured-metal materials
};

// Child-pair BVH node: the bounds of both children of one interior node of
// the flattened CSceneTreeLBVH, so one 64-byte fetch tests two boxes.
// ref >= 0: interior node index; ref < 0: leaf whose primitives start at
// sorted position ~ref, count in cnt0 / (cnt1 & 0x3FFFFFFF). axis in the
// top two bits of cnt1 (the parent's split axis, for near-first order);
// axis code 3 marks the records of the leaf-split layout that subdivide one
// large leaf of the reference's tree: child 0 (the lower positions) first.
struct __align__(16) Node2 {
  float4 b0;   // c0 lo.x hi.x lo.y hi.y
  float4 b1;   // c1 lo.x hi.x lo.y hi.y
  float4 bz;   // c0 lo.z hi.z, c1 lo.z hi.z
  int4 meta;   // ref0, ref1, cnt0, (axis<<30)|cnt1
};

struct BvhView {
  const Node2* nodes;    // the layout traversed (leaf-split by default)
  const Node2* nodes_ref;  // the reference's leaves as they are (null once moved into a batch arena)
  const float4* prims;   // 3 float4 per sorted primitive
  int empty;
  int root_ref;          // >=0 interior index, <0 leaf (~first)
  uint32_t root_count;
  float root_lo[3], root_hi[3];
  uint32_t max_depth;
  uint32_t n_prims, n_int;  // bounds for the index guards in traversal
  uint32_t n_ref_int;       // records of nodes_ref
  uint32_t ref_depth;       // depth of the reference's tree (max_depth adds the split levels)
  uint32_t stack_cap;       // stack entries a lane may use (launches clamp it to the kernel's array)
  uint32_t step_cap;        // iterations of a traversal loop before the traversal gives up
};

// Bounds of a well-formed traversal: the stack never holds more entries than
// the tree is deep (the kernels' arrays are sized for that), and no loop
// comes near 2^26 iterations. wpbr_set_traversal_limits lowers them to
// exercise the limit paths.
constexpr uint32_t kDefaultStackCap = 0xFFFFFFFFu;
constexpr uint32_t kDefaultStepCap = 1u << 26;

// The same tree traversed over the reference's leaves as they are (the
// statistics kernel counts box and primitive tests of this layout).
inline BvhView reference_leaves_view(BvhView v) {
  if (v.nodes_ref) {
    v.nodes = v.nodes_ref;
    v.n_int = v.n_ref_int;
    v.max_depth = v.ref_depth;
  }
  return v;
}

}  // namespace wpbr
