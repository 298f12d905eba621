/*
 * oracle.cpp — TEST INFRASTRUCTURE (the oracle). CPU restatement of
 * WoodenPBREngine's per-sample ray pipeline: LBVH build (SLBVH.cpp), collision
 * (SLBVH.cpp, CSSphere.cpp, CSTriangle.cpp), camera (CSCameraPerspective.*),
 * direct-lighting MIS (SScattering.cpp), BSDFs (CBSDF*.cpp, MicrofaceDistr.h,
 * CBXDF.h), lights (CSSphere.*, CLightInfiniteArea.cpp) and the film splat
 * (CSFilm.cpp). Used only by tests/, the package smoke check and bench.py's
 * CPU-baseline leg, always as the checker, never as the product.
 *
 * Parity status: UNPINNED (see oracle_math.hpp). The reference publishes no
 * golden vectors and cannot be built here.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <vector>

#include "oracle_math.hpp"
#include "wpbr_record.h"
#include "wpbr_spectrum_data.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

/* ------------------------------------------------------------------------ */
/* Scene                                                                      */
/* ------------------------------------------------------------------------ */
struct Distrib1D {
  std::vector<float> func, cdf;
  float func_int = 0.0f;
  int count() const { return (int)func.size(); }
};

/* [wml] DDistributionbPieceWise2D — pbrt Distribution1D/2D semantics. */
static Distrib1D make_distrib1d(const float* f, int n) {
  Distrib1D d;
  d.func.assign(f, f + n);
  d.cdf.assign(n + 1, 0.0f);
  d.cdf[0] = 0.0f;
  for (int i = 1; i < n + 1; ++i) d.cdf[i] = d.cdf[i - 1] + d.func[i - 1] / (float)n;
  d.func_int = d.cdf[n];
  if (d.func_int == 0.0f) {
    for (int i = 1; i < n + 1; ++i) d.cdf[i] = (float)i / (float)n;
  } else {
    for (int i = 1; i < n + 1; ++i) d.cdf[i] = d.cdf[i] / d.func_int;
  }
  return d;
}
static int find_interval(const Distrib1D& d, float u) {
  int size = (int)d.cdf.size();
  int first = 0, len = size;
  while (len > 0) {
    int half = len >> 1, middle = first + half;
    if (d.cdf[middle] <= u) {
      first = middle + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  int r = first - 1;
  return r < 0 ? 0 : (r > size - 2 ? size - 2 : r);
}
static float sample_cont1d(const Distrib1D& d, float u, float* pdf, int* off) {
  int offset = find_interval(d, u);
  if (off) *off = offset;
  float du = u - d.cdf[offset];
  if ((d.cdf[offset + 1] - d.cdf[offset]) > 0.0f) du = du / (d.cdf[offset + 1] - d.cdf[offset]);
  if (pdf) *pdf = (d.func_int > 0.0f) ? d.func[offset] / d.func_int : 0.0f;
  return ((float)offset + du) / (float)d.count();
}

struct Env {
  int W = 0, H = 0;
  std::vector<float> rgb;
  M4 l2w, w2l;
  RGB le;
  std::vector<Distrib1D> cond;
  Distrib1D marg;
};

/* STexture2DSampler::triangle on mip 0 (R/CSTextureProcess.h:58-82); the
 * lower-index clamp keeps the reference's extrapolating weights, the upper
 * index is clamped to the last texel (the reference reads past the row when
 * s >= width - 0.5, which its blocked layout maps to an unrelated texel). */
static RGB env_texel(const Env& e, int x, int y) {
  const float* p = &e.rgb[((size_t)y * e.W + x) * 3];
  return RGB{p[0], p[1], p[2]};
}
static RGB env_bilerp(const Env& e, float s_in, float t_in) {
  float s = s_in * (float)e.W - 0.5f;
  float t = t_in * (float)e.H - 0.5f;
  int s0 = (int)std::floor(s), t0 = (int)std::floor(t);
  s0 = s0 > 0 ? s0 : 0;
  t0 = t0 > 0 ? t0 : 0;
  float ds = s - (float)s0, dt = t - (float)t0;
  int s0n = s0 + 1 < e.W - 1 ? s0 + 1 : e.W - 1;
  int t0n = t0 + 1 < e.H - 1 ? t0 + 1 : e.H - 1;
  s0n = s0n > 0 ? s0n : 0;
  t0n = t0n > 0 ? t0n : 0;
  s0 = s0 < e.W - 1 ? s0 : e.W - 1;
  t0 = t0 < e.H - 1 ? t0 : e.H - 1;
  RGB a = (env_texel(e, s0, t0) * (1.0f - ds)) * (1.0f - dt);
  RGB b = (env_texel(e, s0, t0n) * (1.0f - ds)) * dt;
  RGB c = (env_texel(e, s0n, t0) * ds) * (1.0f - dt);
  RGB d = (env_texel(e, s0n, t0n) * ds) * dt;
  return ((a + b) + c) + d;
}

/* JobLightInfiniteAreaPreprocessSampling (R/CLightInfiniteArea.cpp:113-139):
 * green channel (the .y() of the DVector3f the lookup returns) times sin(theta). */
static void env_preprocess(Env& e, uint32_t quirks) {
  int W = e.W, H = e.H;
  std::vector<float> data((size_t)W * H, 0.0f);
  for (int y = 0; y < H; ++y) {
    float yN = (float)y / (float)H;
    float sin_t = (float)sin_d((PI_D * (double)(float)((float)y + 0.5f)) / (double)(float)H);
    for (int x = 0; x < W; ++x) {
      float xN = (float)x / (float)W;
      size_t idx = (quirks & WPBR_Q_ENV_DISTRIB_INDEX_BUG) ? (size_t)x + (size_t)y * H : (size_t)x + (size_t)y * W;
      data[idx] = env_bilerp(e, xN, yN).g;
      data[idx] = data[idx] * sin_t;
    }
  }
  e.cond.clear();
  for (int v = 0; v < H; ++v) e.cond.push_back(make_distrib1d(&data[(size_t)v * W], W));
  std::vector<float> m(H);
  for (int v = 0; v < H; ++v) m[v] = e.cond[v].func_int;
  e.marg = make_distrib1d(m.data(), H);
}
static void env_sample_uv(const Env& e, float u0, float u1, float* uv0, float* uv1, float* pdf) {
  float pdfs[2];
  int v;
  float d1 = sample_cont1d(e.marg, u1, &pdfs[1], &v);
  float d0 = sample_cont1d(e.cond[v], u0, &pdfs[0], nullptr);
  *pdf = pdfs[0] * pdfs[1];
  *uv0 = d0;
  *uv1 = d1;
}
static float env_pdf_uv(const Env& e, float u, float v) {
  int nu = e.W, nv = e.H;
  int iu = (int)(u * (float)nu), iv = (int)(v * (float)nv);
  iu = iu < 0 ? 0 : (iu > nu - 1 ? nu - 1 : iu);
  iv = iv < 0 ? 0 : (iv > nv - 1 ? nv - 1 : iv);
  return e.cond[iv].func[iu] / e.marg.func_int;
}

struct Mat {
  uint32_t type;
  float ax, ay;
  RGB R;
  float eta_i[3], eta_t[3], k[3];
  uint32_t tex[2];
};

struct TexLevelO {
  uint32_t w = 0, h = 0;
  std::vector<RGB> t;
};

struct Light {
  uint32_t type, sphere;
  RGB le;
};

struct Camera {
  M4 c2w, raster_camera;
  V3 dx, dy;
  uint32_t W, H;
};

struct LinearNode {
  uint32_t offset, n_shapes;
  uint8_t axis;
};

struct Scene {
  uint32_t quirks = 0;
  uint32_t ns = 0, nt = 0;
  std::vector<M4> s_o2w, s_w2o;
  std::vector<float> s_r;
  std::vector<uint32_t> s_mat;
  std::vector<V3> pos, nrm, tan_;
  std::vector<V2> uvs;
  std::vector<uint32_t> idx, t_mat, t_flags;
  std::vector<Mat> mats;
  std::vector<Light> lights;
  bool has_env = false;
  Env env;
  Camera cam;
  std::vector<std::vector<TexLevelO>> textures;  /* MIP levels per texture */
  float gauss[64];
  /* BVH (CSceneTreeLBVH, R/SLBVH.h:28-40) */
  std::vector<LinearNode> nodes;
  std::vector<Bounds> node_bounds;
  std::vector<uint32_t> shapes; /* shapesEntities: primitive ids in leaf order */
  uint32_t max_depth = 0;
  /* build intermediates kept for parity checks */
  std::vector<Bounds> prim_bounds;
  std::vector<V3> prim_centroids;
  Bounds cbounds;
  std::vector<uint32_t> codes;         /* per primitive, input order */
  std::vector<uint32_t> sorted_codes;  /* the array the tree is built over */
  std::vector<uint32_t> sorted_prims;
  std::vector<uint32_t> treelet_start;
};

/* ------------------------------------------------------------------------ */
/* Camera — SCameraProjective::create / SCameraPerspective::create            */
/* (R/CSCameraProjective.h:19-53, R/CSCameraPerspective.h:17-39)              */
/* ------------------------------------------------------------------------ */
static void camera_setup(const wpbr_camera& c, Camera* out) {
  M4 camera_screen = perspective(c.fov_deg, c.near_z, c.far_z);
  float sx0 = c.screen[0], sy0 = c.screen[1], sx1 = c.screen[2], sy1 = c.screen[3];
  M4 t = translate(-sx0, -sy0, 0.0f);
  M4 s1 = scale((float)(1.0 / (double)(sx1 - sx0)), (float)(1.0 / (double)(sy1 - sy0)), 1.0f);
  M4 s2 = scale((float)((int)c.res_x - 1), (float)((int)c.res_y - 1), 1.0f);
  M4 screen_raster = compose(compose(t, s1), s2);
  M4 raster_screen = inverse(screen_raster);
  M4 screen_camera = inverse(camera_screen);
  out->raster_camera = compose(raster_screen, screen_camera);
  /* rasterCamera(DVector3f(...)): vector transform */
  out->dx = xf_vector(out->raster_camera, V3{1, 0, 0}) - xf_vector(out->raster_camera, V3{0, 0, 0});
  out->dy = xf_vector(out->raster_camera, V3{0, 1, 0}) - xf_vector(out->raster_camera, V3{0, 0, 0});
  out->c2w = m4(c.camera_to_world);
  out->W = c.res_x;
  out->H = c.res_y;
}

struct RayDiff {
  Ray r, rx, ry;
};
/* JobCameraPerspGenerateRaysDifferential (R/CSCameraPerspective.cpp:9-54) and
 * CTransform::operator()(DRayDifferentialf) (R/CTransform.h:68-76). */
static RayDiff camera_ray(const Camera& c, float fx, float fy) {
  V3 pcam = xf_point(c.raster_camera, V3{fx, fy, 0.0f});
  RayDiff rd;
  Ray r{V3{0, 0, 0}, normalize(pcam)};
  Ray rx{r.o, normalize(pcam + c.dx)};
  Ray ry{r.o, normalize(pcam + c.dy)};
  rd.r = Ray{xf_point(c.c2w, r.o), normalize(xf_vector(c.c2w, r.d))};
  rd.rx = xf_ray(c.c2w, rx);
  rd.ry = xf_ray(c.c2w, ry);
  return rd;
}

/* ------------------------------------------------------------------------ */
/* LBVH build — buildLBVH (R/MEngine.cpp:341-350)                              */
/* ------------------------------------------------------------------------ */
static uint32_t left_shift3(uint32_t x) { /* R/SLBVH.cpp:219-227 */
  if (x == (1u << 10)) --x;
  x = (x | (x << 16)) & 0b00000011000000000000000011111111u;
  x = (x | (x << 8)) & 0b00000011000000001111000000001111u;
  x = (x | (x << 4)) & 0b00000011000011000011000011000011u;
  x = (x | (x << 2)) & 0b00001001001001001001001001001001u;
  return x;
}
/* float -> uint32 truncation; NaN (a degenerate centroid axis, 0/0) gives 0 as
 * on x86-64 MSVC (cvttss2si into a 64-bit register). */
static uint32_t f2u_trunc(float v) {
  if (!(v >= 0.0f)) return 0u;
  return (uint32_t)v;
}

struct BNode {
  uint32_t start = 0, n = 0;
  Bounds b;
  int child[2] = {-1, -1};
  uint8_t axis = 0;
  bool leaf = true;
};

struct Builder {
  const Scene* sc;
  std::vector<BNode> nodes;
  std::vector<uint32_t> codes; /* tree-order codes */
  std::vector<Bounds> sbounds; /* tree-order bounds */
};

/* emitLBVH (R/SLBVH.cpp:353-406), maxPrimitiveInNode = 30. */
static int emit_lbvh(Builder& B, uint32_t start, uint32_t n, int bit) {
  if (bit == -1 || n < 30) {
    BNode nd;
    nd.start = start;
    nd.n = n;
    for (uint32_t i = 0; i < n; ++i) nd.b = bunion(nd.b, B.sbounds[start + i]);
    nd.leaf = true;
    B.nodes.push_back(nd);
    return (int)B.nodes.size() - 1;
  }
  uint32_t mask = 1u << bit;
  if ((B.codes[start] & mask) == (B.codes[start + n - 1] & mask)) return emit_lbvh(B, start, n, bit - 1);
  uint32_t lo = start, hi = start + n - 1;
  while (lo + 1 != hi) {
    uint32_t mid = (lo + hi) / 2;
    if ((B.codes[lo] & mask) == (B.codes[mid] & mask))
      lo = mid;
    else
      hi = mid;
  }
  uint32_t split = hi;
  B.nodes.push_back(BNode{});
  int me = (int)B.nodes.size() - 1;
  int c0 = emit_lbvh(B, start, split - start, bit - 1);
  int c1 = emit_lbvh(B, split, n - (split - start), bit - 1);
  BNode& nd = B.nodes[me];
  nd.leaf = false;
  nd.child[0] = c0;
  nd.child[1] = c1;
  nd.axis = (uint8_t)(bit % 3);
  nd.b = bunion(B.nodes[c0].b, B.nodes[c1].b);
  nd.n = 0;
  return me;
}

struct SubTree {
  int root;
  uint8_t bucket;
};

/* JobBuildUpperSAH::buildUpperSAH (R/SLBVH.cpp:457-563). std::partition is
 * the standard library's two-pointer swap partition (libstdc++ and MSVC's STL
 * implement the same scheme for bidirectional iterators). */
static int build_upper_sah(Builder& B, std::vector<SubTree>& st, uint32_t i0, uint32_t i1) {
  if (i0 == i1) return st[i0].root;
  Bounds bounds, cb;
  for (uint32_t i = i0; i <= i1; ++i) {
    const Bounds& rb = B.nodes[st[i].root].b;
    bounds = bunion(bounds, rb);
    V3 c = (rb.pmin + rb.pmax) * 0.5f;
    cb = bunion(cb, c);
  }
  int dim = max_extent(cb);
  const int NB = 12;
  Bounds bb[NB];
  uint32_t bc[NB] = {0};
  for (uint32_t i = i0; i <= i1; ++i) {
    float dist = comp(cb.pmax, dim) - comp(cb.pmin, dim);
    const Bounds& rb = B.nodes[st[i].root].b;
    float c = (comp(rb.pmin, dim) + comp(rb.pmax, dim)) * 0.5f;
    float t = (c - comp(cb.pmin, dim)) / dist;
    float bt = (float)NB * t;
    uint32_t ib = (bt >= 0.0f) ? (uint32_t)bt : 0u; /* NaN -> 0 (see f2u_trunc) */
    if (ib == (uint32_t)NB) ib = NB - 1;
    st[i].bucket = (uint8_t)ib;
    bc[ib]++;
    bb[ib] = bunion(bb[ib], rb);
  }
  float costs[NB - 1];
  float barea = area(bounds);
  for (int i = 0; i < NB - 1; ++i) {
    Bounds b0, b1;
    uint32_t n0 = 0, n1 = 0;
    for (int j = 0; j <= i; ++j) {
      b0 = bunion(b0, bb[j]);
      n0 += bc[j];
    }
    for (int j = i + 1; j < NB; ++j) {
      b1 = bunion(b1, bb[j]);
      n1 += bc[j];
    }
    float l = (n0 == 0) ? 0.0f : (float)n0 * area(b0);
    float r = (n1 == 0) ? 0.0f : (float)n1 * area(b1);
    costs[i] = (float)(0.125 + (double)((l + r) / barea));
  }
  float cmin = costs[0];
  int best = 0;
  for (int i = 1; i < NB - 1; ++i)
    if (costs[i] < cmin) {
      best = i;
      cmin = costs[i];
    }
  SubTree* split = std::partition(st.data() + i0, st.data() + i1 + 1,
                                  [best](const SubTree& s) { return s.bucket <= best; });
  uint32_t mid = (uint32_t)(split - st.data());
  if (mid == i1 + 1) mid = (i1 - i0 + 1) / 2 + i0;
  B.nodes.push_back(BNode{});
  int me = (int)B.nodes.size() - 1;
  int c0 = build_upper_sah(B, st, i0, mid - 1);
  int c1 = build_upper_sah(B, st, mid, i1);
  BNode& nd = B.nodes[me];
  nd.leaf = false;
  nd.child[0] = c0;
  nd.child[1] = c1;
  nd.axis = (uint8_t)dim;
  nd.b = bunion(B.nodes[c0].b, B.nodes[c1].b);
  return me;
}

/* flattenBVHTree (R/SLBVH.cpp:432-455): depth-first preorder. */
static uint32_t flatten(const Builder& B, int ni, Scene& sc, uint32_t& off, uint32_t depth) {
  const BNode& nd = B.nodes[ni];
  uint32_t me = off++;
  if (depth > sc.max_depth) sc.max_depth = depth;
  sc.node_bounds[me] = nd.b;
  if (nd.leaf) {
    sc.nodes[me] = LinearNode{nd.start, nd.n, 0};
  } else {
    sc.nodes[me].axis = nd.axis;
    sc.nodes[me].n_shapes = 0;
    flatten(B, nd.child[0], sc, off, depth + 1);
    sc.nodes[me].offset = flatten(B, nd.child[1], sc, off, depth + 1);
  }
  return me;
}

static void build_bvh(Scene& sc) {
  uint32_t N = sc.ns + sc.nt;
  sc.prim_bounds.assign(N, Bounds{});
  sc.prim_centroids.assign(N, V3{0, 0, 0});
  /* JobUpdateBoundsAndCentroidSphere (R/CSSphere.h:126-153): transform of the
   * local cube = union of its 8 transformed corners. */
  for (uint32_t i = 0; i < sc.ns; ++i) {
    float r = sc.s_r[i];
    Bounds b;
    bool first = true;
    for (int c = 0; c < 8; ++c) {
      V3 p{(c & 1) ? r : -r, (c & 2) ? r : -r, (c & 4) ? r : -r};
      V3 q = xf_point(sc.s_o2w[i], p);
      b = first ? bpoint(q) : bunion(b, q);
      first = false;
    }
    sc.prim_bounds[i] = b;
  }
  /* JobUpdateBoundsAndCentroidTriangle (R/CSTriangle.cpp:116-142) */
  for (uint32_t t = 0; t < sc.nt; ++t) {
    V3 a = sc.pos[sc.idx[3 * t]], b = sc.pos[sc.idx[3 * t + 1]], c = sc.pos[sc.idx[3 * t + 2]];
    Bounds bb{vmin(a, b), vmax(a, b)};
    sc.prim_bounds[sc.ns + t] = bunion(bb, c);
  }
  for (uint32_t i = 0; i < N; ++i) sc.prim_centroids[i] = centroid(sc.prim_bounds[i]);
  /* JobGenerateShapesCentroidBound (R/SLBVH.cpp:164-181) */
  Bounds cb;
  for (uint32_t i = 0; i < N; ++i) cb = bunion(cb, sc.prim_centroids[i]);
  sc.cbounds = cb;
  /* JobGenerateShapesMortonCode (R/SLBVH.cpp:186-217) */
  sc.codes.assign(N, 0);
  for (uint32_t i = 0; i < N; ++i) {
    V3 c = sc.prim_centroids[i];
    V3 nrm{(c.x - cb.pmin.x) / (cb.pmax.x - cb.pmin.x), (c.y - cb.pmin.y) / (cb.pmax.y - cb.pmin.y),
           (c.z - cb.pmin.z) / (cb.pmax.z - cb.pmin.z)};
    uint32_t code = (left_shift3(f2u_trunc(nrm.z * 1024.0f)) << 2) | (left_shift3(f2u_trunc(nrm.y * 1024.0f)) << 1) |
                    left_shift3(f2u_trunc(nrm.x * 1024.0f));
    sc.codes[i] = code;
  }
  /* JobSortsShapesByMortonCode (R/SLBVH.cpp:231-324): 6-bit LSD radix sort,
   * five passes ping-ponging between the code array and a temporary buffer. */
  std::vector<uint32_t> a_val(N), a_idx(N), t_val(N), t_idx(N);
  for (uint32_t i = 0; i < N; ++i) {
    a_val[i] = sc.codes[i];
    a_idx[i] = i;
  }
  if (N > 1) {
    for (int pass = 0; pass < 5; ++pass) {
      std::vector<uint32_t>& in_v = (pass & 1) ? t_val : a_val;
      std::vector<uint32_t>& in_i = (pass & 1) ? t_idx : a_idx;
      std::vector<uint32_t>& out_v = (pass & 1) ? a_val : t_val;
      std::vector<uint32_t>& out_i = (pass & 1) ? a_idx : t_idx;
      int low = pass * 6;
      uint32_t cnt[64] = {0};
      for (uint32_t i = 0; i < N; ++i) cnt[(in_v[i] >> low) & 63]++;
      uint32_t total = 0;
      for (int b = 0; b < 64; ++b) {
        uint32_t tmp = cnt[b];
        cnt[b] = total;
        total += tmp;
      }
      for (uint32_t i = 0; i < N; ++i) {
        uint32_t b = (in_v[i] >> low) & 63;
        uint32_t pos = cnt[b]++;
        out_v[pos] = in_v[i];
        out_i[pos] = in_i[i];
      }
    }
  }
  /* the reference keeps reading the code array (pass-4 result); the fully
   * sorted fifth pass sits in the temporary buffer */
  bool full = (sc.quirks & WPBR_Q_FULL_MORTON_SORT) != 0;
  const std::vector<uint32_t>& use_v = (full && N > 1) ? t_val : a_val;
  const std::vector<uint32_t>& use_i = (full && N > 1) ? t_idx : a_idx;
  sc.sorted_codes = use_v;
  sc.sorted_prims = use_i;
  Builder B;
  B.sc = &sc;
  B.codes = use_v;
  B.sbounds.resize(N);
  for (uint32_t i = 0; i < N; ++i) B.sbounds[i] = sc.prim_bounds[use_i[i]];
  /* treelets: top 12 bits (mask bits 29..18) */
  const uint32_t mask = 0b00111111111111000000000000000000u;
  std::vector<std::pair<uint32_t, uint32_t>> treelets;
  sc.treelet_start.clear();
  for (uint32_t s = 0, e = 1; e <= N; ++e) {
    if (e == N || (use_v[s] & mask) != (use_v[e] & mask)) {
      treelets.push_back({s, e - s});
      sc.treelet_start.push_back(s);
      s = e;
    }
  }
  /* JobEmitLBVH (R/SLBVH.cpp:328-351): every treelet once, from bit 17 */
  std::vector<SubTree> st;
  for (auto& tl : treelets) st.push_back(SubTree{emit_lbvh(B, tl.first, tl.second, 30 - 12 - 1), 0});
  int root = st.empty() ? -1 : build_upper_sah(B, st, 0, (uint32_t)st.size() - 1);
  sc.nodes.assign(B.nodes.size(), LinearNode{0, 0, 0});
  sc.node_bounds.assign(B.nodes.size(), Bounds{});
  sc.max_depth = 0;
  uint32_t off = 0;
  if (root >= 0) flatten(B, root, sc, off, 0);
  sc.nodes.resize(off);
  sc.node_bounds.resize(off);
  sc.shapes = use_i;
}

/* ------------------------------------------------------------------------ */
/* Collision — runCollisionSystem (R/MEngine.cpp:352-361)                      */
/* ------------------------------------------------------------------------ */
struct Hit {
  float t = 0.0f;          /* +inf on miss */
  uint32_t prim = 0xFFFFFFFFu;
  float b[3] = {0, 0, 0};  /* triangle barycentrics */
  Ray rl;                  /* sphere object-space ray */
  V3 phl{0, 0, 0};         /* sphere object-space hit */
};

static float prim_test(const Scene& sc, uint32_t prim, const Ray& r, Hit* h) {
  if (prim < sc.ns) {
    Ray rl;
    V3 ph;
    float t = sphere_intersect(sc.s_w2o[prim], sc.s_r[prim], r, &rl, &ph);
    if (h && t != 0.0f) {
      h->rl = rl;
      h->phl = ph;
    }
    return t;
  }
  uint32_t tri = prim - sc.ns;
  float bary[3];
  float t = triangle_intersect(sc.pos[sc.idx[3 * tri]], sc.pos[sc.idx[3 * tri + 1]], sc.pos[sc.idx[3 * tri + 2]], r,
                               sc.quirks, bary);
  if (h && t != 0.0f) {
    h->b[0] = bary[0];
    h->b[1] = bary[1];
    h->b[2] = bary[2];
  }
  return t;
}

/* JobProcessRayCasts (R/SLBVH.cpp:85-162) + JobProcessRayCastsResults
 * (R/SLBVH.cpp:9-66): every primitive of every leaf whose box the ray
 * pierces becomes a candidate, in near-first order; the closest non-zero t
 * wins and the first candidate wins ties (strict >). */
static Hit trace_faithful(const Scene& sc, const Ray& r) {
  Hit best;
  float tmin_best = INFINITY;
  if (sc.nodes.empty()) {
    best.t = INFINITY;
    return best;
  }
  V3 inv{1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z};
  int neg[3] = {inv.x < 0, inv.y < 0, inv.z < 0};
  int stack[256];
  int sp = 0, cur = 0;
  while (true) {
    const LinearNode& nd = sc.nodes[cur];
    float te;
    if (slab(sc.node_bounds[cur], r, inv, neg, INFINITY, &te)) {
      if (nd.n_shapes > 0) {
        for (uint32_t i = 0; i < nd.n_shapes; ++i) {
          uint32_t prim = sc.shapes[nd.offset + i];
          Hit h;
          float t = prim_test(sc, prim, r, &h);
          if (t == 0.0f) continue;
          if (tmin_best > t) {
            tmin_best = t;
            best = h;
            best.prim = prim;
          }
        }
        if (sp == 0) break;
        cur = stack[--sp];
      } else {
        if (neg[nd.axis]) {
          stack[sp++] = cur + 1;
          cur = (int)nd.offset;
        } else {
          stack[sp++] = (int)nd.offset;
          cur = cur + 1;
        }
      }
    } else {
      if (sp == 0) break;
      cur = stack[--sp];
    }
  }
  best.t = tmin_best;
  if (tmin_best == INFINITY) best.prim = 0xFFFFFFFFu;
  return best;
}

/* Same result with closest-t pruning: a box is skipped only when its entry
 * distance exceeds the best t by more than 2^-10 relative, which no
 * primitive inside it can undercut (ties never replace the earlier
 * candidate). Counts node visits and primitive tests for the byte model. */
static const float kPruneScale = 1.0f + 0x1p-10f;
static Hit trace_pruned(const Scene& sc, const Ray& r, bool any_hit, uint32_t* visits, uint32_t* tests) {
  Hit best;
  float tb = INFINITY;
  uint32_t nv = 0, np = 0;
  if (!sc.nodes.empty()) {
    V3 inv{1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z};
    int neg[3] = {inv.x < 0, inv.y < 0, inv.z < 0};
    int stack[256];
    int sp = 0, cur = 0;
    while (true) {
      const LinearNode& nd = sc.nodes[cur];
      float te;
      ++nv;
      bool hit = slab(sc.node_bounds[cur], r, inv, neg, INFINITY, &te) && !(te > tb * kPruneScale);
      bool done = false;
      if (hit) {
        if (nd.n_shapes > 0) {
          for (uint32_t i = 0; i < nd.n_shapes; ++i) {
            uint32_t prim = sc.shapes[nd.offset + i];
            Hit h;
            ++np;
            float t = prim_test(sc, prim, r, &h);
            if (t == 0.0f) continue;
            if (tb > t) {
              tb = t;
              best = h;
              best.prim = prim;
              if (any_hit) {
                done = true;
                break;
              }
            }
          }
          if (done || sp == 0) break;
          cur = stack[--sp];
        } else {
          if (neg[nd.axis]) {
            stack[sp++] = cur + 1;
            cur = (int)nd.offset;
          } else {
            stack[sp++] = (int)nd.offset;
            cur = cur + 1;
          }
        }
      } else {
        if (sp == 0) break;
        cur = stack[--sp];
      }
    }
  }
  best.t = tb;
  if (tb == INFINITY) best.prim = 0xFFFFFFFFu;
  if (visits) *visits = nv;
  if (tests) *tests = np;
  return best;
}

static SI make_si(const Scene& sc, const Ray& r, const Hit& h) {
  if (h.prim < sc.ns) {
    uint32_t s = h.prim;
    return sphere_si(sc.s_o2w[s], sc.s_w2o[s], sc.s_r[s], h.rl, h.phl, h.t, h.prim);
  }
  uint32_t t = h.prim - sc.ns;
  TriVerts tv;
  for (int k = 0; k < 3; ++k) {
    uint32_t vi = sc.idx[3 * t + k];
    tv.p[k] = sc.pos[vi];
    tv.n[k] = sc.nrm.empty() ? V3{0, 0, 0} : sc.nrm[vi];
    tv.s[k] = sc.tan_.empty() ? V3{0, 0, 0} : sc.tan_[vi];
    tv.uv[k] = sc.uvs.empty() ? V2{0, 0} : sc.uvs[vi];
  }
  tv.has_ns = (sc.t_flags[t] & WPBR_MESH_NORMALS_TANGENTS) != 0;
  tv.has_uv = (sc.t_flags[t] & WPBR_MESH_UVS) != 0;
  return triangle_si(tv, r, h.b, h.t, h.prim);
}

static uint32_t prim_material(const Scene& sc, uint32_t prim) {
  return prim < sc.ns ? sc.s_mat[prim] : sc.t_mat[prim - sc.ns];
}

/* ------------------------------------------------------------------------ */
/* Lights                                                                     */
/* ------------------------------------------------------------------------ */
/* SSphere::sample (R/CSSphere.cpp:248-281) + JobSphereLightProcessSamplingRequests
 * (R/CSSphere.h:187-230). */
static void sphere_light_sample(const Scene& sc, uint32_t s, V3 p, float u0, float u1, V3* wi, float* pdf) {
  V3 pc = xf_point(sc.s_o2w[s], V3{0, 0, 0});
  V3 wc = normalize(pc - p);
  V3 wcx, wcy;
  make_basis(wc, &wcx, &wcy);
  float r = sc.s_r[s];
  float s2 = (r * r) / length2(p - pc);
  double a = 1.0 - (double)s2;
  float cos_max = (float)sqrt_d(0.0 > a ? 0.0 : a);
  float cos_t = (float)((double)u0 * (1.0 - (double)cos_max) + (double)cos_max);
  double b = 1.0 - (double)(cos_t * cos_t);
  float sin_t = (float)sqrt_d(0.0 > b ? 0.0 : b);
  float phi = (float)((double)(u1 * 2.0f) * PI_D);
  float dc = length(p - pc);
  float q = r * r - ((dc * dc) * sin_t) * sin_t;
  float ds = dc * cos_t - sqrt_(0.0f > q ? 0.0f : q);
  float cos_a = ((dc * dc + r * r) - ds * ds) / ((2.0f * dc) * r);
  float w = 1.0f - cos_a * cos_a;
  float sin_a = sqrt_(0.0f > w ? 0.0f : w);
  V3 nl = spherical_dir(sin_a, cos_a, phi, -wcx, -wcy, -wc);
  V3 pl = nl * r;
  V3 sp = xf_point(sc.s_o2w[s], pl);
  *pdf = cone_pdf(cos_max);
  *wi = normalize(sp - p);
}
/* SSphere::pdf (R/CSSphere.cpp:221-246): the comma operator makes the cone
 * subtend from the world origin unless WPBR_Q_SPHERE_PDF_FIX. */
static float sphere_light_pdf(const Scene& sc, uint32_t s, V3 p) {
  V3 pc = xf_point(sc.s_o2w[s], V3{0, 0, 0});
  float r = sc.s_r[s];
  V3 d = (sc.quirks & WPBR_Q_SPHERE_PDF_FIX) ? (p - pc) : pc;
  float s2 = (r * r) / length2(d);
  float v = 1.0f - s2;
  float cos_max = sqrt_(0.0f > v ? 0.0f : v);
  return cone_pdf(cos_max);
}
/* JobLightInfiniteAreaLeCompute (R/CLightInfiniteArea.cpp:141-160) */
static RGB env_le(const Env& e, V3 d) {
  V3 dl = xf_vector(e.w2l, d);
  float s = (float)((double)spherical_phi(dl) / (2.0 * PI_D));
  float t = (float)((double)spherical_theta(dl) / PI_D);
  return env_bilerp(e, s, t) * e.le;
}
/* JobLightInfiniteAreaLiSample (R/CLightInfiniteArea.cpp:163-204) */
static void env_li_sample(const Env& e, uint32_t quirks, float u0, float u1, V3* wi, RGB* li, float* pdf, bool* ok) {
  float uv0, uv1, map_pdf;
  env_sample_uv(e, u0, u1, &uv0, &uv1, &map_pdf);
  *li = rgb(0.0f);
  *ok = false;
  if (map_pdf != 0.0f) {
    float theta = (float)((double)uv1 * PI_D);
    float phi = (float)((double)(uv0 * 2.0f) * PI_D);
    float ct = cosf_(theta), st = sinf_(theta);
    *wi = xf_vector(e.l2w, spherical_dir(st, ct, phi));
    *pdf = (st != 0.0f) ? (float)((double)map_pdf / (((2.0 * PI_D) * PI_D) * (double)st)) : 0.0f;
    *ok = true;
  }
  if (quirks & WPBR_Q_ENV_LI_SAMPLE_FIX) *li = env_bilerp(e, uv0, uv1) * e.le;
}
/* JobLightInfiniteAreaLiCompute (R/CLightInfiniteArea.cpp:206-237) */
static void env_li_compute(const Env& e, V3 wi, RGB* li, float* pdf) {
  V3 wl = xf_vector(e.w2l, wi);
  float theta = spherical_theta(wl);
  float phi = spherical_phi(wl);
  float u = (float)((double)phi / (2.0 * PI_D));
  float v = (float)((double)theta / PI_D);
  float st = sinf_(theta);
  *li = rgb(0.0f);
  *pdf = 0.0f;
  if (st != 0.0f) {
    *pdf = (float)((double)env_pdf_uv(e, u, v) / (((2.0 * PI_D) * PI_D) * (double)st));
    *li = env_bilerp(e, u, v) * e.le;
  }
}

#include "oracle_texture.inc"

/* ------------------------------------------------------------------------ */
/* BSDF Compute / Sample jobs                                                  */
/* ------------------------------------------------------------------------ */
static RGB mf_f_impl(const Mat& m, float d_wh, V3 wh, V3 wo, V3 wi) {
  float co = abs_cos(wo), ci = abs_cos(wi);
  if (ci == 0.0f || co == 0.0f) return rgb(0.0f);
  if (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) return rgb(0.0f);
  float c = dot(wi, wh);
  if (m.type == WPBR_MAT_CONDUCTOR) {
    RGB fr{fresnel_conductor1(c, m.eta_i[0], m.eta_t[0], m.k[0]), fresnel_conductor1(c, m.eta_i[1], m.eta_t[1], m.k[1]),
           fresnel_conductor1(c, m.eta_i[2], m.eta_t[2], m.k[2])};
    return (fr * m.R) * (d_wh / ((4.0f * ci) * co));
  }
  float fr = fresnel_dielectric(c, m.eta_i[0], m.eta_t[0]);
  return m.R * ((fr * d_wh) / ((4.0f * ci) * co));
}
/* SBSDF{Conductor,Dielectric}Microface::f + Job...Compute
 * (R/CBSDFConductorMicroface.cpp:44-58,84-97; R/CBSDFDielectricMicroface.cpp:
 * 44-58,84-97); SBXDFSpecularReflectance::f (R/CBSDFSpecularReflectance.cpp:42-48). */
static RGB bsdf_eval(const Mat& m, V3 wo, V3 wi, float* pdf) {
  if (m.type == WPBR_MAT_SPECULAR) {
    *pdf = 0.0f;
    return rgb(0.0f) * abs_cos(wi);
  }
  V3 wh = normalize(wo + wi);
  float d = tr_d(m.ax, m.ay, wh);
  *pdf = tr_pdf(d, wh) / (4.0f * dot(wo, wh));
  return mf_f_impl(m, d, wh, wo, wi) * abs_cos(wi);
}
/* sample_f + Job...Sample (R/CBSDFConductorMicroface.cpp:61-82,99-115;
 * R/CBSDFDielectricMicroface.cpp:61-82,99-115; R/CBSDFSpecularReflectance.cpp:
 * 51-61,75-93). A microfacet sample that lands in the other hemisphere leaves
 * the reference's pdf uninitialised; here it is marked invalid and contributes
 * nothing. */
static RGB bsdf_sample(const Mat& m, V3 wo, float u0, float u1, V3* wi, float* pdf, bool* valid) {
  if (m.type == WPBR_MAT_SPECULAR) {
    *wi = V3{-wo.x, -wo.y, wo.z};
    *pdf = 1.0f;
    *valid = true;
    float ci = abs_cos(*wi);
    RGB f = rgb(0.0f);
    if (ci != 0.0f) {
      float fr = fresnel_dielectric(wi->z, m.eta_i[0], m.eta_t[0]);
      f = m.R * (fr / abs_cos(*wi));
    }
    return f * abs_cos(*wi);
  }
  float d;
  V3 wh = tr_sample(m.ax, m.ay, wo, u0, u1, &d);
  *wi = reflect(wo, wh);
  if (!same_hemi(*wi, wo)) {
    *valid = false;
    *pdf = 0.0f;
    return rgb(0.0f);
  }
  *valid = true;
  *pdf = tr_pdf(d, wh) / (4.0f * dot(wo, wh));
  return mf_f_impl(m, d, wh, wo, *wi) * abs_cos(*wi);
}

static float power_heuristic(float f, float g) { /* R/SScattering.cpp:162-166 */
  float a = 1.0f * f, b = 1.0f * g;
  return (a * a) / (a * a + b * b);
}

/* ------------------------------------------------------------------------ */
/* One sample of one pixel — MEngine::render's per-spp job list               */
/* (R/MEngine.cpp:393-442)                                                    */
/* ------------------------------------------------------------------------ */
struct SampleOut {
  RGB L;
  float fx, fy;
};

static SampleOut shade_sample(const Scene& sc, const wpbr_rng::Stream& rs, uint32_t px, uint32_t py, uint32_t pass,
                              wpbr_pass_record* rec, size_t ri) {
  using namespace wpbr_rng;
  uint32_t pix = py * sc.cam.W + px;
  float u0, u1;
  sample2d(rs, pix, pass, DIM_CAMERA, &u0, &u1);
  /* JobSamplerUpdateCameraSamples (R/CSSampler.cpp:7-23) */
  float fx = (float)px + u0, fy = (float)py + u1;
  RayDiff rd = camera_ray(sc.cam, fx, fy);
  SampleOut out;
  out.fx = fx;
  out.fy = fy;
  RGB L = rgb(0.0f);
  Hit h = trace_pruned(sc, rd.r, false, nullptr, nullptr);
#define REC3(f, v)                      \
  if (rec && rec->f) {                  \
    rec->f[3 * ri + 0] = (v).x;         \
    rec->f[3 * ri + 1] = (v).y;         \
    rec->f[3 * ri + 2] = (v).z;         \
  }
#define RECC(f, c)                      \
  if (rec && rec->f) {                  \
    rec->f[3 * ri + 0] = (c).r;         \
    rec->f[3 * ri + 1] = (c).g;         \
    rec->f[3 * ri + 2] = (c).b;         \
  }
#define REC1(f, v) \
  if (rec && rec->f) rec->f[ri] = (v);
  if (rec && rec->pfilm) {
    rec->pfilm[2 * ri] = fx;
    rec->pfilm[2 * ri + 1] = fy;
  }
  REC3(ray_o, rd.r.o);
  REC3(ray_d, rd.r.d);
  REC3(ray_dx_d, rd.rx.d);
  REC3(ray_dy_d, rd.ry.d);
  REC1(hit_prim, h.prim);
  REC1(hit_t, h.t);
  if (h.prim == 0xFFFFFFFFu) {
    /* JobScatteringRequestEmittedLight / JobLightInfiniteAreaLeCompute /
     * JobScatteringAccumulateEmittedLight (R/SScattering.cpp:20-80): only
     * camera misses collect the environment. */
    if (sc.has_env) {
      RGB le = env_le(sc.env, rd.r.d);
      RECC(le, le);
      L = L + le;
    }
    RECC(L, L);
    out.L = L;
    return out;
  }
  SI si = make_si(sc, rd.r, h);
  REC3(si_p, si.p);
  REC3(si_n, si.n);
  REC3(si_wo, si.wo);
  REC3(si_sn, si.sn);
  REC3(si_sdpdu, si.sdpdu);
  REC3(si_dpdu, si.dpdu);
  REC3(si_dpdv, si.dpdv);
  REC3(si_dndu, si.dndu);
  REC3(si_dndv, si.dndv);
  Frame fr = bsdf_frame(si);
  if (rec && rec->frame) {
    float* f = rec->frame + 9 * ri;
    f[0] = fr.ss.x; f[1] = fr.ss.y; f[2] = fr.ss.z;
    f[3] = fr.ts.x; f[4] = fr.ts.y; f[5] = fr.ts.z;
    f[6] = fr.ns.x; f[7] = fr.ns.y; f[8] = fr.ns.z;
  }
  const Mat mat = hit_mat(sc, h.prim, si, rd);
  V3 wo_l = to_local(fr, si.wo);
  uint32_t nl = (uint32_t)sc.lights.size();
  if (nl == 0) {
    RECC(L, L);
    out.L = L;
    return out;
  }
  /* JobScatteringSampleLight (R/SScattering.cpp:82-88) */
  float ul = sample1d(rs, pix, pass, DIM_LIGHT_PICK);
  float fl = (ul + 0.5f) * (float)(nl - 1);
  uint32_t li_idx = (uint32_t)fl;
  if (li_idx > nl - 1) li_idx = nl - 1;
  REC1(light_idx, li_idx);
  const Light& lt = sc.lights[li_idx];
  uint32_t light_prim = (lt.type == WPBR_LIGHT_SPHERE) ? lt.sphere : 0xFFFFFFFEu;
  /* ---- light-sampling branch ---- */
  float lu0, lu1;
  sample2d(rs, pix, pass, DIM_LIGHT, &lu0, &lu1);
  V3 wi{0, 0, 0};
  RGB li = rgb(0.0f);
  float lpdf = 0.0f;
  bool lok = true;
  if (lt.type == WPBR_LIGHT_SPHERE) {
    sphere_light_sample(sc, lt.sphere, si.p, lu0, lu1, &wi, &lpdf);
    li = lt.le;
  } else {
    env_li_sample(sc.env, sc.quirks, lu0, lu1, &wi, &li, &lpdf, &lok);
  }
  REC3(l_wi, wi);
  RECC(l_li, li);
  REC1(l_pdf, lpdf);
  uint32_t lflags = 0;
  if (lok && !is_black(li)) {
    /* JobScatteringCastShadowRays / ProcessShadowRay (R/SScattering.cpp:99-125) */
    Ray sr{si.p + wi * (float)0.1, wi};
    Hit sh = trace_pruned(sc, sr, false, nullptr, nullptr);
    lflags |= 1u;
    if (sh.prim == 0xFFFFFFFFu || sh.prim == light_prim) {
      lflags |= 2u;
      float bpdf;
      RGB f = bsdf_eval(mat, wo_l, to_local(fr, wi), &bpdf);
      RECC(l_f, f);
      REC1(l_fpdf, bpdf);
      /* JobScatteringIntegrateImportanceLight (R/SScattering.cpp:127-150) */
      if (bpdf != 0.0f) {
        float w = power_heuristic(lpdf, bpdf);
        L = L + (li * f) * (w / lpdf);
      }
    }
  }
  REC1(l_flags, lflags);
  /* ---- BSDF-sampling branch ---- */
  float bu0, bu1;
  sample2d(rs, pix, pass, DIM_BSDF, &bu0, &bu1);
  V3 wi_l;
  float bpdf;
  bool valid;
  RGB bf = bsdf_sample(mat, wo_l, bu0, bu1, &wi_l, &bpdf, &valid);
  V3 wi_w = to_world(fr, wi_l);
  REC3(b_wi, wi_w);
  RECC(b_f, bf);
  REC1(b_pdf, bpdf);
  uint32_t bflags = valid ? 1u : 0u;
  if (valid) {
    /* JobScatteringCastShadowRaysWithInteraction / ProcessShadowRayWithInteraction
     * (R/SScattering.cpp:171-206) */
    Ray sr{si.p + wi_w * (float)0.01, wi_w};
    Hit sh = trace_pruned(sc, sr, false, nullptr, nullptr);
    bflags |= 2u;
    if (sh.prim == 0xFFFFFFFFu || sh.prim == light_prim) {
      bflags |= 4u;
      RGB bli;
      float blpdf;
      if (lt.type == WPBR_LIGHT_SPHERE) {
        blpdf = sphere_light_pdf(sc, lt.sphere, si.p);
        bli = lt.le;
      } else {
        env_li_compute(sc.env, wi_w, &bli, &blpdf);
      }
      RECC(b_li, bli);
      REC1(b_lpdf, blpdf);
      /* JobScatteringIntegrateImportanceBSDF (R/SScattering.cpp:209-254) */
      if (!is_black(bli)) {
        float w = (bpdf == 1.0f) ? 1.0f : power_heuristic(bpdf, blpdf);
        L = L + (bli * bf) * (w / bpdf);
      }
    }
  }
  REC1(b_flags, bflags);
  RECC(L, L);
#undef REC1
#undef REC3
#undef RECC
  out.L = L;
  return out;
}

/* MitchellFilter (R/CSFilm.h:20-44), radius 2, B = C = 1/3 */
static float mitchell1(float x) {
  const float B = (float)(1.0 / 3.0f), C = (float)(1.0 / 3.0f);
  x = fabs_(2.0f * x);
  if (x > 1.0f)
    return ((((((-B - 6.0f * C) * x) * x) * x + (((6.0f * B + 30.0f * C) * x) * x)) + ((-12.0f * B - 48.0f * C) * x)) +
            (8.0f * B + 24.0f * C)) *
           (1.0f / 6.0f);
  return (((((12.0f - 9.0f * B - 6.0f * C) * x) * x) * x + (((-18.0f + 12.0f * B + 6.0f * C) * x) * x)) +
          (6.0f - 2.0f * B)) *
         (1.0f / 6.0f);
}

/* JobAccumalateLIFromSamples (R/CSFilm.cpp:70-122): splat clipped to the
 * sample's 32x32 tile; weight evaluated at (x, y) - pFilm. */
static void film_splat(const Scene& sc, const std::vector<SampleOut>& smp, float* acc_L, float* acc_w) {
  uint32_t W = sc.cam.W, H = sc.cam.H;
  /* per pixel in any order: contributions arrive in row-major sample order */
#pragma omp parallel for schedule(dynamic, 16)
  for (long long y = 0; y < (long long)H; ++y) {
    for (uint32_t x = 0; x < W; ++x) {
      uint32_t tx0 = (x / 32) * 32, ty0 = ((uint32_t)y / 32) * 32;
      uint32_t tx1 = std::min(tx0 + 31, W - 1), ty1 = std::min(ty0 + 31, H - 1);
      RGB a = RGB{acc_L[3 * (y * W + x)], acc_L[3 * (y * W + x) + 1], acc_L[3 * (y * W + x) + 2]};
      float wsum = acc_w[y * W + x];
      int sy0 = std::max((int)ty0, (int)y - 3), sy1 = std::min((int)ty1, (int)y + 3);
      int sx0 = std::max((int)tx0, (int)x - 3), sx1 = std::min((int)tx1, (int)x + 3);
      for (int sy = sy0; sy <= sy1; ++sy)
        for (int sx = sx0; sx <= sx1; ++sx) {
          const SampleOut& s = smp[(size_t)sy * W + sx];
          float dx0 = s.fx - 0.5f, dy0 = s.fy - 0.5f;
          int pminx = (int)std::ceil(dx0 - 2.0f), pmaxx = (int)std::floor(dx0 + 2.0f);
          int pminy = (int)std::ceil(dy0 - 2.0f), pmaxy = (int)std::floor(dy0 + 2.0f);
          pminx = std::max(pminx, (int)tx0);
          pminy = std::max(pminy, (int)ty0);
          pmaxx = std::min(pmaxx, (int)tx1);
          pmaxy = std::min(pmaxy, (int)ty1);
          if ((int)x < pminx || (int)x > pmaxx || (int)y < pminy || (int)y > pmaxy) continue;
          float w = mitchell1(((float)x - s.fx) / 2.0f) * mitchell1(((float)y - s.fy) / 2.0f);
          if (!is_black(s.L)) a = a + s.L * w;
          wsum = wsum + w;
        }
      acc_L[3 * (y * W + x)] = a.r;
      acc_L[3 * (y * W + x) + 1] = a.g;
      acc_L[3 * (y * W + x) + 2] = a.b;
      acc_w[y * W + x] = wsum;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Scene ingest                                                               */
/* ------------------------------------------------------------------------ */
static Scene* scene_from_desc(const wpbr_scene_desc* d, uint32_t quirks) {
  Scene* sc = new Scene();
  sc->quirks = quirks;
  sc->ns = d->n_spheres;
  sc->nt = d->n_triangles;
  for (uint32_t i = 0; i < d->n_spheres; ++i) {
    sc->s_o2w.push_back(m4(d->spheres[i].object_to_world));
    sc->s_w2o.push_back(m4(d->spheres[i].world_to_object));
    sc->s_r.push_back(d->spheres[i].radius);
    sc->s_mat.push_back(d->spheres[i].material);
  }
  for (uint32_t i = 0; i < d->n_vertices; ++i) {
    sc->pos.push_back(V3{d->positions[3 * i], d->positions[3 * i + 1], d->positions[3 * i + 2]});
    if (d->normals) sc->nrm.push_back(V3{d->normals[3 * i], d->normals[3 * i + 1], d->normals[3 * i + 2]});
    if (d->tangents) sc->tan_.push_back(V3{d->tangents[3 * i], d->tangents[3 * i + 1], d->tangents[3 * i + 2]});
    if (d->uvs) sc->uvs.push_back(V2{d->uvs[2 * i], d->uvs[2 * i + 1]});
  }
  sc->idx.assign(d->indices, d->indices + 3 * (size_t)d->n_triangles);
  sc->t_mat.assign(d->n_triangles, 0);
  sc->t_flags.assign(d->n_triangles, 0);
  for (uint32_t m = 0; m < d->n_meshes; ++m)
    for (uint32_t t = d->meshes[m].tri_begin; t < d->meshes[m].tri_begin + d->meshes[m].tri_count; ++t) {
      sc->t_mat[t] = d->meshes[m].material;
      uint32_t fl = d->meshes[m].flags;
      if (!d->normals || !d->tangents) fl &= ~WPBR_MESH_NORMALS_TANGENTS;
      if (!d->uvs) fl &= ~WPBR_MESH_UVS;
      sc->t_flags[t] = fl;
    }
  for (uint32_t i = 0; i < d->n_materials; ++i) {
    const wpbr_material& m = d->materials[i];
    Mat o;
    o.type = m.type;
    o.ax = m.alpha_x;
    o.ay = m.alpha_y;
    o.R = RGB{m.R[0], m.R[1], m.R[2]};
    for (int c = 0; c < 3; ++c) {
      o.eta_i[c] = m.eta_i[c];
      o.eta_t[c] = m.eta_t[c];
      o.k[c] = m.k[c];
    }
    o.tex[0] = m.tex[0];
    o.tex[1] = m.tex[1];
    sc->mats.push_back(o);
  }
  for (uint32_t i = 0; i < d->n_lights; ++i)
    sc->lights.push_back(Light{d->lights[i].type, d->lights[i].sphere_index,
                               RGB{d->lights[i].Le[0], d->lights[i].Le[1], d->lights[i].Le[2]}});
  if (d->envmap) {
    sc->has_env = true;
    Env& e = sc->env;
    e.W = (int)d->envmap->width;
    e.H = (int)d->envmap->height;
    e.rgb.assign(d->envmap->rgb, d->envmap->rgb + (size_t)e.W * e.H * 3);
    e.l2w = m4(d->envmap->light_to_world);
    e.w2l = m4(d->envmap->world_to_light);
    e.le = rgb(1.0f);
    for (uint32_t i = 0; i < d->n_lights; ++i)
      if (d->lights[i].type == WPBR_LIGHT_ENV) e.le = RGB{d->lights[i].Le[0], d->lights[i].Le[1], d->lights[i].Le[2]};
    env_preprocess(e, quirks);
  }
  for (uint32_t i = 0; i < d->n_textures; ++i) {
    sc->textures.emplace_back();
    build_texture(d->textures[i], sc->textures.back());
  }
  build_gauss(sc->gauss);
  camera_setup(d->camera, &sc->cam);
  build_bvh(*sc);
  return sc;
}

#include "oracle_adjoint.inc"
#include "oracle_spectral.inc"

}  // namespace orc

/* ------------------------------------------------------------------------ */
/* C API for the test suite (ctypes)                                          */
/* ------------------------------------------------------------------------ */
using namespace orc;
extern "C" {

void* orc_scene_create(const wpbr_scene_desc* d, uint32_t quirks) { return scene_from_desc(d, quirks); }
void orc_scene_destroy(void* h) { delete (Scene*)h; }
int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* sizes: [n_prims, n_nodes, n_treelets, max_depth] */
void orc_bvh_sizes(void* h, uint32_t* out4) {
  Scene* s = (Scene*)h;
  out4[0] = s->ns + s->nt;
  out4[1] = (uint32_t)s->nodes.size();
  out4[2] = (uint32_t)s->treelet_start.size();
  out4[3] = s->max_depth;
}
/* prim_bounds[n*6], centroids[n*3], cbounds[6], codes[n], sorted_codes[n],
 * sorted_prims[n], treelet_start[T], nodes[M*3] (offset, n_shapes, axis),
 * node_bounds[M*6], shapes[n]; any pointer may be NULL */
void orc_bvh_export(void* h, float* prim_bounds, float* centroids, float* cbounds, uint32_t* codes,
                    uint32_t* sorted_codes, uint32_t* sorted_prims, uint32_t* treelet_start, uint32_t* nodes,
                    float* node_bounds, uint32_t* shapes) {
  Scene* s = (Scene*)h;
  uint32_t N = s->ns + s->nt;
  for (uint32_t i = 0; i < N; ++i) {
    if (prim_bounds) {
      const Bounds& b = s->prim_bounds[i];
      float v[6] = {b.pmin.x, b.pmin.y, b.pmin.z, b.pmax.x, b.pmax.y, b.pmax.z};
      memcpy(prim_bounds + 6 * i, v, sizeof(v));
    }
    if (centroids) {
      centroids[3 * i] = s->prim_centroids[i].x;
      centroids[3 * i + 1] = s->prim_centroids[i].y;
      centroids[3 * i + 2] = s->prim_centroids[i].z;
    }
    if (codes) codes[i] = s->codes[i];
    if (sorted_codes) sorted_codes[i] = s->sorted_codes[i];
    if (sorted_prims) sorted_prims[i] = s->sorted_prims[i];
    if (shapes) shapes[i] = s->shapes[i];
  }
  if (cbounds) {
    float v[6] = {s->cbounds.pmin.x, s->cbounds.pmin.y, s->cbounds.pmin.z,
                  s->cbounds.pmax.x, s->cbounds.pmax.y, s->cbounds.pmax.z};
    memcpy(cbounds, v, sizeof(v));
  }
  if (treelet_start)
    for (size_t i = 0; i < s->treelet_start.size(); ++i) treelet_start[i] = s->treelet_start[i];
  for (size_t i = 0; i < s->nodes.size(); ++i) {
    if (nodes) {
      nodes[3 * i] = s->nodes[i].offset;
      nodes[3 * i + 1] = s->nodes[i].n_shapes;
      nodes[3 * i + 2] = s->nodes[i].axis;
    }
    if (node_bounds) {
      const Bounds& b = s->node_bounds[i];
      float v[6] = {b.pmin.x, b.pmin.y, b.pmin.z, b.pmax.x, b.pmax.y, b.pmax.z};
      memcpy(node_bounds + 6 * i, v, sizeof(v));
    }
  }
}

/* rays: n*8 floats (o.xyz, 0, d.xyz, 0). mode 0 = faithful closest,
 * 1 = pruned closest, 2 = any hit. hits: n*4 (t, prim bits, b1, b2).
 * stats (optional): n*2 u32 (node visits, primitive tests) for modes 1, 2. */
void orc_trace(void* h, const float* rays, uint64_t n, int mode, float* hits, uint32_t* stats) {
  Scene* s = (Scene*)h;
#pragma omp parallel for schedule(dynamic, 64)
  for (long long i = 0; i < (long long)n; ++i) {
    Ray r{V3{rays[8 * i], rays[8 * i + 1], rays[8 * i + 2]}, V3{rays[8 * i + 4], rays[8 * i + 5], rays[8 * i + 6]}};
    Hit hh;
    uint32_t v = 0, p = 0;
    if (mode == 0)
      hh = trace_faithful(*s, r);
    else
      hh = trace_pruned(*s, r, mode == 2, &v, &p);
    hits[4 * i] = hh.t;
    uint32_t prim = hh.prim;
    memcpy(&hits[4 * i + 1], &prim, 4);
    hits[4 * i + 2] = hh.b[1];
    hits[4 * i + 3] = hh.b[2];
    if (stats) {
      stats[2 * i] = v;
      stats[2 * i + 1] = p;
    }
  }
}

/* camera: raster_camera[16], dx[3], dy[3] */
void orc_camera(void* h, float* raster_camera, float* dx, float* dy) {
  Scene* s = (Scene*)h;
  memcpy(raster_camera, s->cam.raster_camera.m, 64);
  dx[0] = s->cam.dx.x; dx[1] = s->cam.dx.y; dx[2] = s->cam.dx.z;
  dy[0] = s->cam.dy.x; dy[1] = s->cam.dy.y; dy[2] = s->cam.dy.z;
}

/* environment distribution: cond_func/cdf [H*W], [H*(W+1)], cond_int[H],
 * marg_cdf[H+1], marg_int[1] */
void orc_env_distribution(void* h, float* cond_cdf, float* cond_int, float* marg_cdf, float* marg_int) {
  Scene* s = (Scene*)h;
  if (!s->has_env) return;
  const Env& e = s->env;
  for (int v = 0; v < e.H; ++v) {
    if (cond_cdf) memcpy(cond_cdf + (size_t)v * (e.W + 1), e.cond[v].cdf.data(), sizeof(float) * (e.W + 1));
    if (cond_int) cond_int[v] = e.cond[v].func_int;
  }
  if (marg_cdf) memcpy(marg_cdf, e.marg.cdf.data(), sizeof(float) * (e.H + 1));
  if (marg_int) *marg_int = e.marg.func_int;
}

/* One sample pass over a pixel rectangle [x0,x1)x[y0,y1); rec arrays are
 * indexed by the rectangle's row-major pixel index. */
void orc_render_pass(void* h, uint32_t pass, uint32_t spp, uint32_t seed, uint32_t stream, uint32_t x0, uint32_t y0,
                     uint32_t x1, uint32_t y1, wpbr_pass_record* rec) {
  Scene* s = (Scene*)h;
  wpbr_rng::Stream rs{seed, stream, spp, (s->quirks & WPBR_Q_REF_SAMPLER_ARRAYS) ? 1u : 0u};
  uint32_t w = x1 - x0;
  long long n = (long long)w * (y1 - y0);
#pragma omp parallel for schedule(dynamic, 64)
  for (long long i = 0; i < n; ++i) {
    uint32_t px = x0 + (uint32_t)(i % w), py = y0 + (uint32_t)(i / w);
    shade_sample(*s, rs, px, py, pass, rec, (size_t)i);
  }
}

/* Full render: spp passes over the whole film, film accumulators out
 * (acc_L [W*H*3], acc_w [W*H], zero-initialised by the caller). */
void orc_render(void* h, uint32_t spp, uint32_t seed, uint32_t stream, float* acc_L, float* acc_w) {
  Scene* s = (Scene*)h;
  wpbr_rng::Stream rs{seed, stream, spp, (s->quirks & WPBR_Q_REF_SAMPLER_ARRAYS) ? 1u : 0u};
  uint32_t W = s->cam.W, H = s->cam.H;
  std::vector<SampleOut> smp((size_t)W * H);
  for (uint32_t pass = 0; pass < spp; ++pass) {
#pragma omp parallel for schedule(dynamic, 64)
    for (long long i = 0; i < (long long)W * H; ++i)
      smp[i] = shade_sample(*s, rs, (uint32_t)(i % W), (uint32_t)(i / W), pass, nullptr, 0);
    film_splat(*s, smp, acc_L, acc_w);
  }
}

/* The passes listed in `passes` (in that order) of an spp-pass render,
 * accumulated into the film arrays as orc_render accumulates every pass. */
void orc_render_passes(void* h, uint32_t spp, uint32_t seed, uint32_t stream, uint32_t n_passes,
                       const uint32_t* passes, float* acc_L, float* acc_w) {
  Scene* s = (Scene*)h;
  wpbr_rng::Stream rs{seed, stream, spp, (s->quirks & WPBR_Q_REF_SAMPLER_ARRAYS) ? 1u : 0u};
  uint32_t W = s->cam.W, H = s->cam.H;
  std::vector<SampleOut> smp((size_t)W * H);
  for (uint32_t k = 0; k < n_passes; ++k) {
    uint32_t pass = passes[k];
#pragma omp parallel for schedule(dynamic, 64)
    for (long long i = 0; i < (long long)W * H; ++i)
      smp[i] = shade_sample(*s, rs, (uint32_t)(i % W), (uint32_t)(i / W), pass, nullptr, 0);
    film_splat(*s, smp, acc_L, acc_w);
  }
}

/* Per-function known-answer hooks. */
float orc_fresnel_dielectric(float c, float ei, float et) { return fresnel_dielectric(c, ei, et); }
float orc_fresnel_conductor(float c, float ei, float et, float k) { return fresnel_conductor1(c, ei, et, k); }
float orc_tr_d(float ax, float ay, float x, float y, float z) { return tr_d(ax, ay, V3{x, y, z}); }
float orc_power_heuristic(float f, float g) { return power_heuristic(f, g); }
float orc_mitchell(float x) { return mitchell1(x); }
uint32_t orc_left_shift3(uint32_t x) { return left_shift3(x); }
float orc_roughness_to_alpha(float r) { return roughness_to_alpha(r); }
void orc_sample2d(uint32_t seed, uint32_t stream, uint32_t spp, uint32_t pixel, uint32_t pass, uint32_t dim,
                  uint32_t arrays, float* u) {
  wpbr_rng::Stream rs{seed, stream, spp, arrays};
  wpbr_rng::sample2d(rs, pixel, pass, dim, &u[0], &u[1]);
}
void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) { wpbr_rng::philox4x32_10(ctr, key, out); }
/* fn: 0 sin, 1 cos, 2 atan2(x, y), 3 acos, 4 exp, 5 log, 6 tan; 7 sin_d, 8 cos_d (double in/out) */
void orc_fmath(int fn, const float* x, const float* y, float* out, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) {
    float a = x[i];
    switch (fn) {
      case 0: out[i] = sinf_(a); break;
      case 1: out[i] = cosf_(a); break;
      case 2: out[i] = atan2f_(a, y[i]); break;
      case 3: out[i] = acosf_(a); break;
      case 4: out[i] = expf_(a); break;
      case 5: out[i] = logf_(a); break;
      default: out[i] = tanf_(a); break;
    }
  }
}
void orc_fmath_d(int fn, const double* x, double* out, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) out[i] = fn == 0 ? sin_d(x[i]) : cos_d(x[i]);
}
float orc_sample1d(uint32_t seed, uint32_t stream, uint32_t spp, uint32_t pixel, uint32_t pass, uint32_t dim,
                   uint32_t arrays) {
  wpbr_rng::Stream rs{seed, stream, spp, arrays};
  return wpbr_rng::sample1d(rs, pixel, pass, dim);
}
/* The FP64 frozen-direction estimator: sampling parameters are the scene's
 * own; mat (nmat*10) and env (W*H*3) are the evaluation parameters. Returns
 * the loss against target (0 without); image (W*H*3) optional; grad receives
 * dLoss/dparam for the n_sel parameter indices in sel (materials first, then
 * texels), by dual numbers. */
double orc_adjoint_eval(void* h, uint32_t spp, uint32_t seed, uint32_t stream, const double* mat, const double* env,
                        const float* target, double* image, uint32_t n_sel, const uint32_t* sel, double* grad) {
  const Scene& sc = *(const Scene*)h;
  std::vector<Frozen> fz = freeze_all(sc, spp, seed, stream);
  EvalParams<double> P;
  load_params(sc, mat, env, P);
  if (sc.has_env) eval_env_distribution(sc.env, sc.quirks, P);
  double loss = eval_loss(sc, fz, spp, P, target, image);
  const size_t nm = sc.mats.size() * 10;
  constexpr int K = 8;
  for (uint32_t b = 0; b < n_sel; b += K) {
    EvalParams<Dual<K>> D;
    load_params(sc, mat, env, D);
    for (int k = 0; k < K && b + k < n_sel; ++k) {
      uint32_t idx = sel[b + k];
      if (idx < nm)
        D.mat[idx].d[k] = 1.0;
      else
        D.env[idx - nm].d[k] = 1.0;
    }
    if (sc.has_env) eval_env_distribution(sc.env, sc.quirks, D);
    Dual<K> l = eval_loss(sc, fz, spp, D, target, nullptr);
    for (int k = 0; k < K && b + k < n_sel; ++k) grad[b + k] = l.d[k];
  }
  return loss;
}
/* FP64 central differences of the frozen-direction estimator's loss: for
 * each parameter index in sel (materials first, then texels), the loss at
 * the parameter + h and - h (the other parameters at mat / env, the frozen
 * state computed once), fd[k] = (loss(+h) - loss(-h)) / (2h). */
void orc_adjoint_fd(void* h, uint32_t spp, uint32_t seed, uint32_t stream, const double* mat, const double* env,
                    const float* target, uint32_t n_sel, const uint32_t* sel, double step, double* fd) {
  const Scene& sc = *(const Scene*)h;
  std::vector<Frozen> fz = freeze_all(sc, spp, seed, stream);
  const size_t nm = sc.mats.size() * 10;
  EvalParams<double> P;
  load_params(sc, mat, env, P);
  for (uint32_t k = 0; k < n_sel; ++k) {
    uint32_t idx = sel[k];
    double* slot = idx < nm ? &P.mat[idx] : &P.env[idx - nm];
    const double v0 = *slot;
    double l[2];
    for (int side = 0; side < 2; ++side) {
      *slot = v0 + (side == 0 ? step : -step);
      if (sc.has_env) eval_env_distribution(sc.env, sc.quirks, P);
      l[side] = eval_loss(sc, fz, spp, P, target, nullptr);
    }
    *slot = v0;
    fd[k] = (l[0] - l[1]) / (2.0 * step);
  }
}
/* Sampled64 render: spp passes of the spectral per-sample job list; the
 * film's spectra resolved with toRGB (acc_L[W*H*3]) and the weights. */
void orc_render_spectral(void* h, uint32_t spp, uint32_t seed, uint32_t stream, float* acc_L, float* acc_w) {
  spec_render(*(const Scene*)h, spp, seed, stream, acc_L, acc_w);
}
/* The binned spectral tables (64 floats each): X, Y, Z, 7 reflectance and
 * 7 illuminant bases, in that order (17 * 64 floats). */
void orc_spectral_tables(float* out) {
  const SpecTab& T = spec_tables();
  memcpy(out, &T, sizeof(T));
}
/* The MIP pyramid of one texture (SLoadTexture::generateMIPS): returns the
 * level count; with out != NULL copies level `level` (w*h*3 floats) and
 * writes its size to wh[2]. */
uint32_t orc_texture_level(const wpbr_texture* t, uint32_t level, float* out, uint32_t* wh) {
  std::vector<TexLevelO> lv;
  build_texture(*t, lv);
  if (out && level < lv.size()) {
    const TexLevelO& L = lv[level];
    for (size_t i = 0; i < L.t.size(); ++i) {
      out[3 * i] = L.t[i].r;
      out[3 * i + 1] = L.t[i].g;
      out[3 * i + 2] = L.t[i].b;
    }
    wh[0] = L.w;
    wh[1] = L.h;
  }
  return (uint32_t)lv.size();
}
/* STexture2DSamplerAnisotropic::eval (isotropic = 0) or
 * STexture2DSamplerIsotropic::eval (isotropic = 1) of one texture at the
 * footprint fp = (s, t, ds/dx, dt/dx, ds/dy, dt/dy); rgb to out[3]. */
void orc_texture_eval(const wpbr_texture* t, const float* fp, uint32_t isotropic, float* out) {
  std::vector<TexLevelO> lv;
  build_texture(*t, lv);
  float gauss[64];
  build_gauss(gauss);
  Footprint f;
  f.p = V2{fp[0], fp[1]};
  f.dx = V2{fp[2], fp[3]};
  f.dy = V2{fp[4], fp[5]};
  RGB c = isotropic ? tx_iso(lv, f) : tx_aniso(lv, gauss, f);
  out[0] = c.r;
  out[1] = c.g;
  out[2] = c.b;
}
}
