// scene_gen.cpp — seeded synthetic scenes and ray sets for the benchmark
// configurations (the reference publishes no benchmark data; these stand in
// for it with the stated shapes, sizes and value distributions).
//
//   config 0  plain render: 64 spheres r~U[0.2,1], centres~U[-10,10]^3, a
//             2-triangle ground quad (MeshTools::createQuad layout, with
//             normals/tangents/uvs), one sphere light r=1 Le=(10,10,10);
//             sphere materials alternate conductor / dielectric microfacet.
//   config 1  LBVH microbench: icosphere subdivided L times (20*4^L
//             triangles; L=8 gives 1,310,720), vertices displaced radially by
//             0.1 x 3-octave value noise; ray set = one coherent primary ray per
//             pixel centre of a res_x*res_y pinhole camera, then as many
//             incoherent rays from area-weighted surface points (offset 1e-4
//             along n) with cosine-weighted directions.
//   config 2  full frame: the config-1 mesh scaled x3 + 256 spheres
//             r~U[0.1,0.8], a procedural 1024x512 environment light (sky
//             gradient + 8 Gaussian lobes, peak U[5,50]); materials cycle
//             conductor / dielectric microfacet / perfect glass.
//
// All arithmetic is deterministic (portable math, no contraction) so the same
// scene is produced on any host.
#include <cstdlib>
#include <cstring>
#include <new>
#include <unordered_map>
#include <vector>

#include "camera.cuh"
#include "geom.cuh"
#include "host_xf.hpp"
#include "wpbr_gpu.h"
#include "wpbr_sampling.h"
#include "wpbr_scene.h"

using namespace wpbr;

namespace {

struct Rng {
  uint32_t k0, k1;
  uint32_t ctr = 0;
  uint32_t buf[4];
  int avail = 0;
  Rng(uint32_t seed, uint32_t purpose) : k0(seed), k1(purpose) {}
  uint32_t next_u32() {
    if (avail == 0) {
      uint32_t c[4] = {ctr++, 0x5CE7E5u, 0u, 0u};
      uint32_t k[2] = {k0, k1};
      wpbr_rng::philox4x32_10(c, k, buf);
      avail = 4;
    }
    return buf[--avail];
  }
  float u01() { return wpbr_rng::bits_to_u01(next_u32()); }
  float uni(float a, float b) { return a + (b - a) * u01(); }
};

void set_mat(wpbr_mat4* out, const Xf& x) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) out->m[4 * i + j] = x.m[i][j];
}

uint32_t hash3(int32_t x, int32_t y, int32_t z, uint32_t seed) {
  uint32_t h = seed * 0x9E3779B1u;
  h ^= (uint32_t)x * 0x8DA6B343u;
  h ^= (uint32_t)y * 0xD8163841u;
  h ^= (uint32_t)z * 0xCB1AB31Fu;
  h ^= h >> 16;
  h *= 0x85EBCA6Bu;
  h ^= h >> 13;
  h *= 0xC2B2AE35u;
  h ^= h >> 16;
  return h;
}
double lattice(int32_t x, int32_t y, int32_t z, uint32_t seed) {
  return (double)(hash3(x, y, z, seed) >> 8) * (2.0 / 16777216.0) - 1.0;  // [-1, 1)
}
double smooth(double t) { return t * t * (3.0 - 2.0 * t); }
// Trilinearly interpolated lattice value noise with smoothstep weights.
double value_noise(double x, double y, double z, uint32_t seed) {
  double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
  int32_t ix = (int32_t)fx, iy = (int32_t)fy, iz = (int32_t)fz;
  double tx = smooth(x - fx), ty = smooth(y - fy), tz = smooth(z - fz);
  double c[2][2][2];
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int d = 0; d < 2; ++d) c[a][b][d] = lattice(ix + a, iy + b, iz + d, seed);
  double x00 = c[0][0][0] + (c[1][0][0] - c[0][0][0]) * tx;
  double x10 = c[0][1][0] + (c[1][1][0] - c[0][1][0]) * tx;
  double x01 = c[0][0][1] + (c[1][0][1] - c[0][0][1]) * tx;
  double x11 = c[0][1][1] + (c[1][1][1] - c[0][1][1]) * tx;
  double y0 = x00 + (x10 - x00) * ty;
  double y1 = x01 + (x11 - x01) * ty;
  return y0 + (y1 - y0) * tz;
}

}  // namespace

struct wpbr_scenegen {
  std::vector<wpbr_sphere> spheres;
  std::vector<float> pos, nrm, tan_, uv;
  bool has_nrm = false, has_uv = false;
  std::vector<uint32_t> idx;
  std::vector<wpbr_mesh> meshes;
  std::vector<wpbr_material> mats;
  std::vector<wpbr_light> lights;
  std::vector<float> env_rgb;
  wpbr_envmap env;
  bool has_env = false;
  wpbr_camera cam;
  std::vector<std::vector<float>> tex_rgb;  // one rgb array per texture
  std::vector<uint32_t> tex_wh;             // width, height per texture
  std::vector<wpbr_texture> texs;
  wpbr_scene_desc desc;
  std::vector<float> rays;  // n * 8

  void add_sphere(V3 c, float r, uint32_t mat) {
    wpbr_sphere s;
    memset(&s, 0, sizeof(s));
    set_mat(&s.object_to_world, xf_translate(c.x, c.y, c.z));
    set_mat(&s.world_to_object, xf_translate(-c.x, -c.y, -c.z));
    s.radius = r;
    s.material = mat;
    spheres.push_back(s);
  }
  uint32_t add_material(uint32_t type, float alpha, const float eta_t[3], const float k[3], float eta_i = 1.0f) {
    wpbr_material m;
    memset(&m, 0, sizeof(m));
    m.type = type;
    m.alpha_x = alpha;
    m.alpha_y = alpha;
    for (int c = 0; c < 3; ++c) {
      m.R[c] = 1.0f;
      m.eta_i[c] = eta_i;
      m.eta_t[c] = eta_t[c];
      m.k[c] = k[c];
    }
    mats.push_back(m);
    return (uint32_t)mats.size() - 1;
  }
  void set_camera(V3 eye, V3 target, float fov, uint32_t W, uint32_t H) {
    memset(&cam, 0, sizeof(cam));
    Xf c2w = xf_look_at(eye, target, V3{0.0f, 1.0f, 0.0f});
    set_mat(&cam.camera_to_world, c2w);
    set_mat(&cam.world_to_camera, xf_inverse(c2w));
    cam.fov_deg = fov;
    cam.near_z = 0.1f;
    cam.far_z = 10000.0f;
    float aspect = (float)W / (float)H;
    cam.screen[0] = aspect >= 1.0f ? -aspect : -1.0f;
    cam.screen[1] = aspect >= 1.0f ? -1.0f : -1.0f / aspect;
    cam.screen[2] = -cam.screen[0];
    cam.screen[3] = -cam.screen[1];
    cam.res_x = W;
    cam.res_y = H;
  }
  // Icosphere with 20*4^level faces, radius r, displaced radially by
  // disp * (3-octave value noise), appended as one mesh.
  void add_icosphere(uint32_t level, double r, double disp, uint32_t seed, V3 center, uint32_t material) {
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<double> P = {-1, t, 0, 1, t, 0, -1, -t, 0, 1, -t, 0, 0, -1, t, 0, 1, t,
                             0, -1, -t, 0, 1, -t, t, 0, -1, t, 0, 1, -t, 0, -1, -t, 0, 1};
    for (size_t i = 0; i < P.size(); i += 3) {
      double l = std::sqrt(P[i] * P[i] + P[i + 1] * P[i + 1] + P[i + 2] * P[i + 2]);
      P[i] /= l;
      P[i + 1] /= l;
      P[i + 2] /= l;
    }
    std::vector<uint32_t> F = {0, 11, 5, 0, 5,  1,  0,  1, 7, 0, 7,  10, 0, 10, 11, 1, 5, 9, 5, 11,
                               4, 11, 10, 2, 10, 7,  6,  7, 1, 8, 3,  9,  4, 3,  4,  2, 3, 2, 6, 3,
                               6, 8,  3,  8, 9,  4,  9,  5, 2, 4, 11, 6,  2, 10, 8,  6, 7, 9, 8, 1};
    // orient every face outward
    for (size_t f = 0; f < F.size(); f += 3) {
      const double* a = &P[3 * F[f]];
      const double* b = &P[3 * F[f + 1]];
      const double* c = &P[3 * F[f + 2]];
      double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
      double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
      if (n[0] * a[0] + n[1] * a[1] + n[2] * a[2] < 0) std::swap(F[f + 1], F[f + 2]);
    }
    for (uint32_t l = 0; l < level; ++l) {
      std::unordered_map<uint64_t, uint32_t> mid;
      mid.reserve(F.size());
      std::vector<uint32_t> NF;
      NF.reserve(F.size() * 4);
      auto midpoint = [&](uint32_t a, uint32_t b) -> uint32_t {
        uint64_t key = a < b ? ((uint64_t)a << 32) | b : ((uint64_t)b << 32) | a;
        auto it = mid.find(key);
        if (it != mid.end()) return it->second;
        double m[3] = {(P[3 * a] + P[3 * b]) * 0.5, (P[3 * a + 1] + P[3 * b + 1]) * 0.5,
                       (P[3 * a + 2] + P[3 * b + 2]) * 0.5};
        double ln = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
        uint32_t id = (uint32_t)(P.size() / 3);
        P.push_back(m[0] / ln);
        P.push_back(m[1] / ln);
        P.push_back(m[2] / ln);
        mid.emplace(key, id);
        return id;
      };
      for (size_t f = 0; f < F.size(); f += 3) {
        uint32_t a = F[f], b = F[f + 1], c = F[f + 2];
        uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
        uint32_t q[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
        NF.insert(NF.end(), q, q + 12);
      }
      F.swap(NF);
    }
    uint32_t vbase = (uint32_t)(pos.size() / 3);
    uint32_t nv = (uint32_t)(P.size() / 3);
    for (uint32_t i = 0; i < nv; ++i) {
      double x = P[3 * i], y = P[3 * i + 1], z = P[3 * i + 2];
      double n = 0.0, amp = 1.0, freq = 4.0, norm = 0.0;
      for (int o = 0; o < 3; ++o) {
        n += amp * value_noise(x * freq, y * freq, z * freq, seed + (uint32_t)o);
        norm += amp;
        amp *= 0.5;
        freq *= 2.0;
      }
      double s = r * (1.0 + disp * (n / norm));
      pos.push_back((float)(x * s + (double)center.x));
      pos.push_back((float)(y * s + (double)center.y));
      pos.push_back((float)(z * s + (double)center.z));
    }
    wpbr_mesh m;
    m.tri_begin = (uint32_t)(idx.size() / 3);
    m.tri_count = (uint32_t)(F.size() / 3);
    m.material = material;
    m.flags = 0;
    for (uint32_t v : F) idx.push_back(vbase + v);
    meshes.push_back(m);
  }
  // MeshTools::createQuad (WoodenPBREngine/MeshTools.h:101-154) translated by c.
  void add_quad(float W, float D, V3 c, uint32_t material) {
    uint32_t vbase = (uint32_t)(pos.size() / 3);
    float wh = W / 2.0f, dh = D / 2.0f;
    float p[12] = {-wh, 0, dh, wh, 0, dh, -wh, 0, -dh, wh, 0, -dh};
    float u[8] = {0, 1, 1, 1, 0, 0, 1, 0};
    for (int i = 0; i < 4; ++i) {
      pos.push_back(p[3 * i] + c.x);
      pos.push_back(p[3 * i + 1] + c.y);
      pos.push_back(p[3 * i + 2] + c.z);
    }
    while (nrm.size() < pos.size() - 12) nrm.push_back(0.0f);
    while (tan_.size() < pos.size() - 12) tan_.push_back(0.0f);
    while (uv.size() < (pos.size() - 12) / 3 * 2) uv.push_back(0.0f);
    for (int i = 0; i < 4; ++i) {
      nrm.push_back(0.0f); nrm.push_back(1.0f); nrm.push_back(0.0f);
      tan_.push_back(1.0f); tan_.push_back(0.0f); tan_.push_back(0.0f);
      uv.push_back(u[2 * i]); uv.push_back(u[2 * i + 1]);
    }
    has_nrm = true;
    has_uv = true;
    wpbr_mesh m;
    m.tri_begin = (uint32_t)(idx.size() / 3);
    m.tri_count = 2;
    m.material = material;
    m.flags = WPBR_MESH_NORMALS_TANGENTS | WPBR_MESH_UVS;
    uint32_t q[6] = {0, 1, 2, 1, 2, 3};
    for (uint32_t v : q) idx.push_back(vbase + v);
    meshes.push_back(m);
  }
  void finish() {
    if (has_nrm) {
      nrm.resize(pos.size(), 0.0f);
      tan_.resize(pos.size(), 0.0f);
    }
    if (has_uv) uv.resize(pos.size() / 3 * 2, 0.0f);
    memset(&desc, 0, sizeof(desc));
    desc.spheres = spheres.data();
    desc.n_spheres = (uint32_t)spheres.size();
    desc.n_vertices = (uint32_t)(pos.size() / 3);
    desc.positions = pos.data();
    desc.normals = has_nrm ? nrm.data() : nullptr;
    desc.tangents = has_nrm ? tan_.data() : nullptr;
    desc.uvs = has_uv ? uv.data() : nullptr;
    desc.n_triangles = (uint32_t)(idx.size() / 3);
    desc.indices = idx.data();
    desc.meshes = meshes.data();
    desc.n_meshes = (uint32_t)meshes.size();
    desc.materials = mats.data();
    desc.n_materials = (uint32_t)mats.size();
    desc.lights = lights.data();
    desc.n_lights = (uint32_t)lights.size();
    desc.envmap = has_env ? &env : nullptr;
    desc.camera = cam;
    texs.clear();
    for (size_t i = 0; i < tex_rgb.size(); ++i) texs.push_back(wpbr_texture{tex_wh[2 * i], tex_wh[2 * i + 1], tex_rgb[i].data()});
    desc.textures = texs.empty() ? nullptr : texs.data();
    desc.n_textures = (uint32_t)texs.size();
  }
  // A procedural texture: `fn(x, y, rgb)` fills texel (x, y).
  template <typename F>
  uint16_t add_texture(uint32_t W, uint32_t H, F fn) {
    std::vector<float> t((size_t)W * H * 3);
    for (uint32_t y = 0; y < H; ++y)
      for (uint32_t x = 0; x < W; ++x) fn(x, y, &t[3 * ((size_t)y * W + x)]);
    tex_rgb.push_back(std::move(t));
    tex_wh.push_back(W);
    tex_wh.push_back(H);
    return (uint16_t)(tex_rgb.size() - 1);
  }
  uint32_t add_metal(uint16_t metallic, uint16_t roughness, uint32_t type = WPBR_MAT_METAL) {
    wpbr_material m;
    memset(&m, 0, sizeof(m));
    m.type = type;
    m.tex[0] = metallic;
    m.tex[1] = roughness;
    mats.push_back(m);
    return (uint32_t)mats.size() - 1;
  }
  void make_env(uint32_t W, uint32_t H, uint32_t seed) {
    Rng rng(seed, 0xE417u);
    V3 lobe_dir[8], lobe_col[8];
    float lobe_sig[8], lobe_peak[8];
    for (int i = 0; i < 8; ++i) {
      float z = 2.0f * rng.u01() - 1.0f, ph = 2.0f * kMathPi * rng.u01();
      float s = sqrt_(fmax_(0.0f, 1.0f - z * z));
      lobe_dir[i] = V3{s * cosf_(ph), s * sinf_(ph), z};
      lobe_sig[i] = rng.uni(0.02f, 0.2f);
      lobe_peak[i] = rng.uni(5.0f, 50.0f);
      lobe_col[i] = V3{rng.uni(0.7f, 1.0f), rng.uni(0.7f, 1.0f), rng.uni(0.7f, 1.0f)};
    }
    env_rgb.assign((size_t)W * H * 3, 0.0f);
    for (uint32_t y = 0; y < H; ++y) {
      float th = kMathPi * ((float)y + 0.5f) / (float)H;
      float ct = cosf_(th), st = sinf_(th);
      for (uint32_t x = 0; x < W; ++x) {
        float ph = 2.0f * kMathPi * ((float)x + 0.5f) / (float)W;
        V3 d{st * cosf_(ph), st * sinf_(ph), ct};
        V3 c;
        if (ct > 0.0f) {
          V3 zen{0.5f, 0.9f, 2.0f}, hor{2.0f, 1.9f, 1.7f};
          c = add(mul(hor, 1.0f - ct), mul(zen, ct));
        } else {
          c = V3{0.15f, 0.13f, 0.10f};
        }
        for (int i = 0; i < 8; ++i) {
          float a = acosf_(clampf(dot(d, lobe_dir[i]), -1.0f, 1.0f));
          float g = lobe_peak[i] * expf_(-(a * a) / (2.0f * lobe_sig[i] * lobe_sig[i]));
          c = add(c, mul(lobe_col[i], g));
        }
        float* o = &env_rgb[((size_t)y * W + x) * 3];
        o[0] = c.x;
        o[1] = c.y;
        o[2] = c.z;
      }
    }
    memset(&env, 0, sizeof(env));
    env.width = W;
    env.height = H;
    env.rgb = env_rgb.data();
    // light space +z (theta = 0) is world +y
    Xf l2w = xf_identity();
    l2w.m[1][1] = 0.0f; l2w.m[1][2] = 1.0f;
    l2w.m[2][1] = -1.0f; l2w.m[2][2] = 0.0f;
    Xf w2l = xf_identity();
    w2l.m[1][1] = 0.0f; w2l.m[1][2] = -1.0f;
    w2l.m[2][1] = 1.0f; w2l.m[2][2] = 0.0f;
    set_mat(&env.light_to_world, l2w);
    set_mat(&env.world_to_light, w2l);
    has_env = true;
    wpbr_light L;
    memset(&L, 0, sizeof(L));
    L.type = WPBR_LIGHT_ENV;
    L.Le[0] = L.Le[1] = L.Le[2] = 1.0f;
    lights.push_back(L);
  }
};

namespace {

void gen_config0(wpbr_scenegen* g, uint32_t seed, uint32_t W, uint32_t H) {
  Rng rng(seed, 0xC0u);
  for (int i = 0; i < 64; ++i) {
    V3 c{rng.uni(-10.0f, 10.0f), rng.uni(-10.0f, 10.0f), rng.uni(-10.0f, 10.0f)};
    float r = rng.uni(0.2f, 1.0f);
    float alpha = rng.uni(0.05f, 0.5f);
    uint32_t m;
    if ((i & 1) == 0) {
      float eta[3] = {rng.uni(0.2f, 3.0f), rng.uni(0.2f, 3.0f), rng.uni(0.2f, 3.0f)};
      float k[3] = {rng.uni(0.2f, 3.0f), rng.uni(0.2f, 3.0f), rng.uni(0.2f, 3.0f)};
      m = g->add_material(WPBR_MAT_CONDUCTOR, alpha, eta, k);
    } else {
      float e = rng.uni(1.3f, 1.7f);
      float eta[3] = {e, e, e}, k[3] = {0, 0, 0};
      m = g->add_material(WPBR_MAT_DIELECTRIC, alpha, eta, k);
    }
    g->add_sphere(c, r, m);
  }
  float qe[3] = {1.5f, 1.5f, 1.5f}, qk[3] = {0, 0, 0};
  uint32_t mq = g->add_material(WPBR_MAT_DIELECTRIC, 0.25f, qe, qk);
  float le[3] = {1.5f, 1.5f, 1.5f}, lk[3] = {1.0f, 1.0f, 1.0f};
  uint32_t ml = g->add_material(WPBR_MAT_CONDUCTOR, 0.3f, le, lk);
  g->add_sphere(V3{0.0f, 15.0f, 0.0f}, 1.0f, ml);
  wpbr_light L;
  memset(&L, 0, sizeof(L));
  L.type = WPBR_LIGHT_SPHERE;
  L.sphere_index = (uint32_t)g->spheres.size() - 1;
  L.Le[0] = L.Le[1] = L.Le[2] = 10.0f;
  g->lights.push_back(L);
  g->add_quad(40.0f, 40.0f, V3{0.0f, -11.0f, 0.0f}, mq);
  g->set_camera(V3{0.0f, 3.0f, -30.0f}, V3{0.0f, -2.0f, 0.0f}, 60.0f, W, H);
}

// Config 4, the differentiable-rendering scene: config 0's geometry (seed
// `seed`), one material per sphere (64; the ground quad and the light sphere
// share material 0) and a 256x128 environment light beside the sphere light.
// The material parameters and the environment come from `param_seed`:
// alternating conductor (alpha U[.05,.5], R U[.4,1]^3, eta, k U[.2,3]^3) and
// dielectric microfacet (alpha U[.05,.5], R U[.4,1]^3, eta U[1.3,1.7]).
void gen_config4(wpbr_scenegen* g, uint32_t seed, uint32_t param_seed, uint32_t W, uint32_t H) {
  Rng rng(seed, 0xC0u);
  Rng prm(param_seed, 0xC4u);
  for (int i = 0; i < 64; ++i) {
    V3 c{rng.uni(-10.0f, 10.0f), rng.uni(-10.0f, 10.0f), rng.uni(-10.0f, 10.0f)};
    float r = rng.uni(0.2f, 1.0f);
    float alpha = prm.uni(0.05f, 0.5f);
    float R[3] = {prm.uni(0.4f, 1.0f), prm.uni(0.4f, 1.0f), prm.uni(0.4f, 1.0f)};
    uint32_t m;
    if ((i & 1) == 0) {
      float eta[3] = {prm.uni(0.2f, 3.0f), prm.uni(0.2f, 3.0f), prm.uni(0.2f, 3.0f)};
      float k[3] = {prm.uni(0.2f, 3.0f), prm.uni(0.2f, 3.0f), prm.uni(0.2f, 3.0f)};
      m = g->add_material(WPBR_MAT_CONDUCTOR, alpha, eta, k);
    } else {
      float e = prm.uni(1.3f, 1.7f);
      float eta[3] = {e, e, e}, k[3] = {0, 0, 0};
      m = g->add_material(WPBR_MAT_DIELECTRIC, alpha, eta, k);
    }
    for (int ch = 0; ch < 3; ++ch) g->mats[m].R[ch] = R[ch];
    g->add_sphere(c, r, m);
  }
  g->add_sphere(V3{0.0f, 15.0f, 0.0f}, 1.0f, 0);
  wpbr_light L;
  memset(&L, 0, sizeof(L));
  L.type = WPBR_LIGHT_SPHERE;
  L.sphere_index = (uint32_t)g->spheres.size() - 1;
  L.Le[0] = L.Le[1] = L.Le[2] = 10.0f;
  g->lights.push_back(L);
  g->add_quad(40.0f, 40.0f, V3{0.0f, -11.0f, 0.0f}, 0);
  g->make_env(256, 128, 0xC4E0u + param_seed);
  g->set_camera(V3{0.0f, 3.0f, -30.0f}, V3{0.0f, -2.0f, 0.0f}, 60.0f, W, H);
}

// Config 5, the textured-metal scene: config 0's spheres and light with every
// third sphere and the ground quad made of CMaterialMetal (spheres 0, 6, 12,
// ... and the ground with the anisotropic sampler, spheres 3, 9, 15, ... with
// the isotropic one). Four procedural
// textures: a 256x256 checker of two metallic k colours with seeded texel
// noise (ground k), a 64x64 diagonal roughness ramp from 1e-5 to 1e-2 (log
// scale, with noise; roughnessToAlpha(90 r) then spans alpha ~0.04 to ~1.6)
// for the ground, a 100x60 striped metallic (sphere k; odd sizes exercise
// the MIP edge rules) and a 32x16 log-uniform roughness for the spheres. The camera looks
// along the ground at a grazing angle, so the footprints are anisotropic.
void gen_config5(wpbr_scenegen* g, uint32_t seed, uint32_t W, uint32_t H) {
  Rng tr(seed, 0xC5u);
  float ka[3] = {tr.uni(0.2f, 3.0f), tr.uni(0.2f, 3.0f), tr.uni(0.2f, 3.0f)};
  float kb[3] = {tr.uni(0.2f, 3.0f), tr.uni(0.2f, 3.0f), tr.uni(0.2f, 3.0f)};
  uint16_t t_km = g->add_texture(256, 256, [&](uint32_t x, uint32_t y, float* c) {
    const float* k = (((x >> 5) ^ (y >> 5)) & 1) ? ka : kb;
    for (int ch = 0; ch < 3; ++ch) c[ch] = k[ch] * tr.uni(0.9f, 1.1f);
  });
  uint16_t t_kr = g->add_texture(64, 64, [&](uint32_t x, uint32_t y, float* c) {
    c[0] = wpbr_fm::expf_(2.3025851f * (-5.0f + 3.0f * (float)((x + y) & 63) / 63.0f)) * tr.uni(0.5f, 1.0f);
    c[1] = tr.u01();
    c[2] = 0.0f;
  });
  uint16_t t_sm = g->add_texture(100, 60, [&](uint32_t x, uint32_t y, float* c) {
    const float* k = ((x / 7 + y / 11) & 1) ? ka : kb;
    for (int ch = 0; ch < 3; ++ch) c[ch] = k[ch] * tr.uni(0.8f, 1.2f);
  });
  uint16_t t_sr = g->add_texture(32, 16, [&](uint32_t, uint32_t, float* c) {
    c[0] = wpbr_fm::expf_(2.3025851f * tr.uni(-5.0f, -2.0f));
    c[1] = c[2] = 0.5f;
  });
  uint32_t m_ground = g->add_metal(t_km, t_kr);
  uint32_t m_sphere = g->add_metal(t_sm, t_sr);
  uint32_t m_sphere_iso = g->add_metal(t_sm, t_sr, WPBR_MAT_METAL_ISOTROPIC);
  Rng rng(seed, 0xC0u);
  for (int i = 0; i < 64; ++i) {
    V3 c{rng.uni(-10.0f, 10.0f), rng.uni(-10.0f, 10.0f), rng.uni(-10.0f, 10.0f)};
    float r = rng.uni(0.2f, 1.0f);
    float alpha = rng.uni(0.05f, 0.5f);
    uint32_t m;
    if ((i & 1) == 0) {
      float eta[3] = {rng.uni(0.2f, 3.0f), rng.uni(0.2f, 3.0f), rng.uni(0.2f, 3.0f)};
      float k[3] = {rng.uni(0.2f, 3.0f), rng.uni(0.2f, 3.0f), rng.uni(0.2f, 3.0f)};
      m = g->add_material(WPBR_MAT_CONDUCTOR, alpha, eta, k);
    } else {
      float e = rng.uni(1.3f, 1.7f);
      float eta[3] = {e, e, e}, k[3] = {0, 0, 0};
      m = g->add_material(WPBR_MAT_DIELECTRIC, alpha, eta, k);
    }
    g->add_sphere(c, r, i % 6 == 0 ? m_sphere : i % 6 == 3 ? m_sphere_iso : m);
  }
  float le[3] = {1.5f, 1.5f, 1.5f}, lk[3] = {1.0f, 1.0f, 1.0f};
  uint32_t ml = g->add_material(WPBR_MAT_CONDUCTOR, 0.3f, le, lk);
  g->add_sphere(V3{0.0f, 15.0f, 0.0f}, 1.0f, ml);
  wpbr_light L;
  memset(&L, 0, sizeof(L));
  L.type = WPBR_LIGHT_SPHERE;
  L.sphere_index = (uint32_t)g->spheres.size() - 1;
  L.Le[0] = L.Le[1] = L.Le[2] = 10.0f;
  g->lights.push_back(L);
  g->add_quad(40.0f, 40.0f, V3{0.0f, -11.0f, 0.0f}, m_ground);
  g->set_camera(V3{0.0f, -9.5f, -24.0f}, V3{0.0f, -10.5f, 0.0f}, 60.0f, W, H);
}

void gen_config1(wpbr_scenegen* g, uint32_t seed, uint32_t W, uint32_t H, uint32_t level, bool with_rays) {
  float e[3] = {1.5f, 1.5f, 1.5f}, k[3] = {1, 1, 1};
  uint32_t m = g->add_material(WPBR_MAT_CONDUCTOR, 0.2f, e, k);
  g->add_icosphere(level, 1.0, 0.1, seed, V3{0, 0, 0}, m);
  g->set_camera(V3{0.3f, 0.4f, -2.3f}, V3{0.0f, 0.0f, 0.0f}, 45.0f, W, H);
  g->finish();
  if (!with_rays) return;
  uint64_t n = (uint64_t)W * H;
  g->rays.assign(n * 2 * 8, 0.0f);
  CameraParams cp = camera_setup(g->cam);
  for (uint64_t i = 0; i < n; ++i) {
    uint32_t x = (uint32_t)(i % W), y = (uint32_t)(i / W);
    RayD r = camera_ray(cp, (float)x + 0.5f, (float)y + 0.5f);
    float* o = &g->rays[8 * i];
    o[0] = r.o.x; o[1] = r.o.y; o[2] = r.o.z; o[3] = 0.0f;
    o[4] = r.d.x; o[5] = r.d.y; o[6] = r.d.z; o[7] = INFINITY;
  }
  // incoherent: area-weighted surface points, cosine-weighted directions
  uint32_t nt = (uint32_t)(g->idx.size() / 3);
  std::vector<double> cdf(nt + 1, 0.0);
  for (uint32_t t = 0; t < nt; ++t) {
    const float* a = &g->pos[3 * g->idx[3 * t]];
    const float* b = &g->pos[3 * g->idx[3 * t + 1]];
    const float* c = &g->pos[3 * g->idx[3 * t + 2]];
    double e1[3] = {(double)b[0] - a[0], (double)b[1] - a[1], (double)b[2] - a[2]};
    double e2[3] = {(double)c[0] - a[0], (double)c[1] - a[1], (double)c[2] - a[2]};
    double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2], cz = e1[0] * e2[1] - e1[1] * e2[0];
    cdf[t + 1] = cdf[t] + 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
  }
  Rng rng(seed + 1u, 0x1C0u);
  for (uint64_t i = 0; i < n; ++i) {
    double u = (double)rng.u01() * cdf[nt];
    uint32_t lo = 0, hi = nt;
    while (lo + 1 < hi) {
      uint32_t mid = (lo + hi) / 2;
      if (cdf[mid] <= u) lo = mid; else hi = mid;
    }
    uint32_t t = lo;
    V3 a = V3{g->pos[3 * g->idx[3 * t]], g->pos[3 * g->idx[3 * t] + 1], g->pos[3 * g->idx[3 * t] + 2]};
    V3 b = V3{g->pos[3 * g->idx[3 * t + 1]], g->pos[3 * g->idx[3 * t + 1] + 1], g->pos[3 * g->idx[3 * t + 1] + 2]};
    V3 c = V3{g->pos[3 * g->idx[3 * t + 2]], g->pos[3 * g->idx[3 * t + 2] + 1], g->pos[3 * g->idx[3 * t + 2] + 2]};
    float su = sqrt_(rng.u01());
    float b0 = 1.0f - su, b1 = rng.u01() * su, b2 = 1.0f - b0 - b1;
    V3 p = add(add(mul(a, b0), mul(b, b1)), mul(c, b2));
    V3 nrm = normalize(cross(sub(b, a), sub(c, a)));
    V3 o = add(p, mul(nrm, 1e-4f));
    // concentric disk (Shirley-Chiu) -> cosine-weighted hemisphere
    float ux = 2.0f * rng.u01() - 1.0f, uy = 2.0f * rng.u01() - 1.0f;
    float dx = 0.0f, dy = 0.0f;
    if (ux != 0.0f || uy != 0.0f) {
      float rr, th;
      if (fabs_(ux) > fabs_(uy)) {
        rr = ux;
        th = (kMathPi / 4.0f) * (uy / ux);
      } else {
        rr = uy;
        th = kMathPi / 2.0f - (kMathPi / 4.0f) * (ux / uy);
      }
      dx = rr * cosf_(th);
      dy = rr * sinf_(th);
    }
    float dz = sqrt_(fmax_(0.0f, 1.0f - dx * dx - dy * dy));
    V3 s1, s2;
    if (fabs_(nrm.x) > fabs_(nrm.y))
      s1 = divs(V3{-nrm.z, 0.0f, nrm.x}, sqrt_(nrm.x * nrm.x + nrm.z * nrm.z));
    else
      s1 = divs(V3{0.0f, nrm.z, -nrm.y}, sqrt_(nrm.y * nrm.y + nrm.z * nrm.z));
    s2 = cross(nrm, s1);
    V3 d = normalize(add(add(mul(s1, dx), mul(s2, dy)), mul(nrm, dz)));
    float* ro = &g->rays[8 * (n + i)];
    ro[0] = o.x; ro[1] = o.y; ro[2] = o.z; ro[3] = 0.0f;
    ro[4] = d.x; ro[5] = d.y; ro[6] = d.z; ro[7] = INFINITY;
  }
}

void gen_config2(wpbr_scenegen* g, uint32_t seed, uint32_t W, uint32_t H, uint32_t level, uint32_t env_w,
                 uint32_t env_h) {
  float ce[3] = {0.27f, 0.42f, 1.5f}, ck[3] = {3.4f, 2.4f, 1.8f};
  uint32_t mesh_mat = g->add_material(WPBR_MAT_CONDUCTOR, 0.15f, ce, ck);
  Rng rng(seed, 0xC2u);
  for (int i = 0; i < 256; ++i) {
    V3 c{rng.uni(-10.0f, 10.0f), rng.uni(-10.0f, 10.0f), rng.uni(-10.0f, 10.0f)};
    float r = rng.uni(0.1f, 0.8f);
    float alpha = rng.uni(0.05f, 0.5f);
    uint32_t m;
    int kind = i % 3;
    if (kind == 0) {
      float eta[3] = {rng.uni(0.2f, 3.0f), rng.uni(0.2f, 3.0f), rng.uni(0.2f, 3.0f)};
      float k[3] = {rng.uni(0.2f, 3.0f), rng.uni(0.2f, 3.0f), rng.uni(0.2f, 3.0f)};
      m = g->add_material(WPBR_MAT_CONDUCTOR, alpha, eta, k);
    } else if (kind == 1) {
      float e = rng.uni(1.3f, 1.7f);
      float eta[3] = {e, e, e}, k[3] = {0, 0, 0};
      m = g->add_material(WPBR_MAT_DIELECTRIC, alpha, eta, k);
    } else {
      float eta[3] = {1.66f, 1.66f, 1.66f}, k[3] = {0, 0, 0};
      m = g->add_material(WPBR_MAT_SPECULAR, 0.0f, eta, k);
    }
    g->add_sphere(c, r, m);
  }
  g->add_icosphere(level, 3.0, 0.1, seed, V3{0, 0, 0}, mesh_mat);
  g->make_env(env_w, env_h, seed);
  g->set_camera(V3{0.0f, 4.0f, -16.0f}, V3{0.0f, 0.0f, 0.0f}, 60.0f, W, H);
}

// Config 3, scene k of the batched-scenes set: primitive counts log-uniform in
// [10k, 2M] (seed 3); even scenes and counts of at least 100k are displaced
// icospheres at the nearest subdivision level, the others random sphere sets;
// films uniform over {256, 512, 768, 1024}^2; one sphere light and a
// 256x128 procedural environment light. Film sides are scaled by
// film_scale/1024 and counts capped at max_count (1024 and 2M give the set as
// specified; smaller values give a quick test set of the same shape).
void gen_config3(wpbr_scenegen* g, uint32_t k, uint32_t seed, uint32_t film_scale, uint32_t max_count) {
  Rng pick(seed, 0xC3000u + k);
  double lo = std::log(10000.0), hi = std::log(2000000.0);
  double count = std::exp(lo + (hi - lo) * (double)pick.u01());
  if (count > (double)max_count) count = (double)max_count;
  static const uint32_t films[4] = {256, 512, 768, 1024};
  uint32_t res = (uint32_t)(((uint64_t)films[pick.next_u32() % 4] * film_scale) / 1024u);
  if (res < 8) res = 8;
  float ce[3] = {0.9f, 0.6f, 0.3f}, ck[3] = {2.0f, 2.5f, 3.0f};
  uint32_t m_cond = g->add_material(WPBR_MAT_CONDUCTOR, 0.2f, ce, ck);
  float de[3] = {1.5f, 1.5f, 1.5f}, dk[3] = {0, 0, 0};
  uint32_t m_diel = g->add_material(WPBR_MAT_DIELECTRIC, 0.3f, de, dk);
  bool mesh = (k % 2 == 0) || count >= 100000.0;
  if (mesh) {
    uint32_t level = 0;
    double best = 1e30;
    for (uint32_t L = 3; L <= 9; ++L) {
      double c = 20.0 * std::pow(4.0, (double)L);
      double dlog = std::fabs(std::log(c) - std::log(count));
      if (dlog < best) {
        best = dlog;
        level = L;
      }
    }
    if (level > 8) level = 8;
    g->add_icosphere(level, 3.0, 0.1, seed + k, V3{0, 0, 0}, m_cond);
  } else {
    uint32_t ns = (uint32_t)count;
    Rng rs(seed + k, 0x5F5u);
    float extent = 4.0f * std::cbrt((float)ns / 10000.0f);
    for (uint32_t i = 0; i < ns; ++i) {
      V3 c{rs.uni(-extent, extent), rs.uni(-extent, extent), rs.uni(-extent, extent)};
      g->add_sphere(c, rs.uni(0.02f, 0.12f), (i & 1) ? m_diel : m_cond);
    }
  }
  float le[3] = {1.5f, 1.5f, 1.5f}, lk[3] = {1.0f, 1.0f, 1.0f};
  uint32_t ml = g->add_material(WPBR_MAT_CONDUCTOR, 0.3f, le, lk);
  g->add_sphere(V3{0.0f, 9.0f, -3.0f}, 1.0f, ml);
  wpbr_light L;
  memset(&L, 0, sizeof(L));
  L.type = WPBR_LIGHT_SPHERE;
  L.sphere_index = (uint32_t)g->spheres.size() - 1;
  L.Le[0] = L.Le[1] = L.Le[2] = 40.0f;
  g->lights.push_back(L);
  g->make_env(256, 128, seed + k);
  float dist = mesh ? 9.0f : 3.2f * (4.0f * std::cbrt((float)count / 10000.0f));
  g->set_camera(V3{0.0f, 0.35f * dist, -dist}, V3{0.0f, 0.0f, 0.0f}, 50.0f, res, res);
}

}  // namespace

extern "C" {

WPBR_API wpbr_status wpbr_scenegen_create(uint32_t config, uint32_t seed, uint32_t res_x, uint32_t res_y,
                                          uint32_t level, uint32_t flags, wpbr_scenegen** out) {
  if (!out || res_x == 0 || res_y == 0) return WPBR_ERR_INVALID_ARG;
  *out = nullptr;
  wpbr_scenegen* g = new (std::nothrow) wpbr_scenegen();
  if (!g) return WPBR_ERR_OOM;
  try {
    if (config == 0) {
      gen_config0(g, seed, res_x, res_y);
      g->finish();
    } else if (config == 1) {
      gen_config1(g, seed, res_x, res_y, level ? level : 8, (flags & WPBR_SCENEGEN_RAYS) != 0);
    } else if (config == 2) {
      gen_config2(g, seed, res_x, res_y, level ? level : 8, 1024, 512);
      g->finish();
    } else if (config == 4) {
      gen_config4(g, seed, level, res_x, res_y);  // `level` is the parameter seed
      g->finish();
    } else if (config == 3) {
      // `level` selects the scene of the set; res_x scales the films, res_y caps the counts
      gen_config3(g, level, seed, res_x, res_y);
      g->finish();
    } else if (config == 5) {
      gen_config5(g, seed, res_x, res_y);
      g->finish();
    } else {
      delete g;
      return WPBR_ERR_INVALID_ARG;
    }
  } catch (const std::bad_alloc&) {
    delete g;
    return WPBR_ERR_OOM;
  }
  *out = g;
  return WPBR_OK;
}

WPBR_API const wpbr_scene_desc* wpbr_scenegen_desc(const wpbr_scenegen* g) { return g ? &g->desc : nullptr; }

WPBR_API uint64_t wpbr_scenegen_ray_count(const wpbr_scenegen* g) { return g ? g->rays.size() / 8 : 0; }

WPBR_API const float* wpbr_scenegen_rays(const wpbr_scenegen* g) {
  return (g && !g->rays.empty()) ? g->rays.data() : nullptr;
}

WPBR_API void wpbr_scenegen_destroy(wpbr_scenegen* g) { delete g; }

}  // extern "C"
