// wpbr_host.cpp — C++17 host runner over the C ABI (include/wpbr_gpu.h).
//
// Plays the role of MEngine (WoodenPBREngine/MEngine.cpp): builds a scene
// (a synthetic configuration, or an OBJ mesh with an optional PFM environment
// map), runs buildLBVH (:341-350) and, per sample pass, either the
// reference's job list one group at a time in MEngine::render's order
// (:393-442, --staged) or the fused graph-captured pass, then writes the
// filtered film (PFM radiance) and the tonemapped image (PPM, JobOutputFilm).
// Links libwpbr_gpu.so only: no CUDA, PyTorch or Python on this path.
//
//   wpbr_host --config 0 --res 256x256 --spp 4 --out film
//   wpbr_host --obj mesh.obj [--env sky.pfm] --res 512x512 --spp 16 --staged
//   wpbr_host --obj mesh.obj --dump-scene          (parse only, no GPU)
//   wpbr_host --obj mesh.obj --metal k.pfm rough.pfm --spectral   (textured
//       metal from two PFM textures, CMaterialMetal; Sampled64 spectra)
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "scene_io.hpp"
#include "wpbr_gpu.h"

namespace {

struct Args {
  int config = -1;
  uint32_t level = 0, seed = 0, render_seed = 0, spp = 4, quirks = 0, W = 256, H = 256;
  std::string obj, env, out, metal_k, metal_rough;
  bool staged = false, dump = false, spectral = false;
  float fov = 45.0f;
};

[[noreturn]] void usage(const char* msg) {
  fprintf(stderr, "wpbr_host: %s\n", msg);
  fprintf(stderr,
          "usage: wpbr_host (--config N [--level L] [--seed S] | --obj FILE [--env FILE.pfm] [--fov DEG]\n"
          "                  [--metal K.pfm ROUGHNESS.pfm])\n"
          "                 [--res WxH] [--spp N] [--render-seed S] [--quirks Q] [--staged | --spectral]\n"
          "                 [--out PREFIX] [--dump-scene]\n");
  exit(2);
}

Args parse(int argc, char** argv) {
  Args a;
  for (int i = 1; i < argc; ++i) {
    std::string k = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) usage(("missing value for " + k).c_str());
      return argv[++i];
    };
    if (k == "--config") a.config = std::stoi(next());
    else if (k == "--level") a.level = (uint32_t)std::stoul(next());
    else if (k == "--seed") a.seed = (uint32_t)std::stoul(next());
    else if (k == "--render-seed") a.render_seed = (uint32_t)std::stoul(next());
    else if (k == "--spp") a.spp = (uint32_t)std::stoul(next());
    else if (k == "--quirks") a.quirks = (uint32_t)std::stoul(next());
    else if (k == "--fov") a.fov = std::stof(next());
    else if (k == "--obj") a.obj = next();
    else if (k == "--env") a.env = next();
    else if (k == "--out") a.out = next();
    else if (k == "--staged") a.staged = true;
    else if (k == "--spectral") a.spectral = true;
    else if (k == "--metal") {
      a.metal_k = next();
      a.metal_rough = next();
    }
    else if (k == "--dump-scene") a.dump = true;
    else if (k == "--res") {
      std::string v = next();
      if (sscanf(v.c_str(), "%ux%u", &a.W, &a.H) != 2 || !a.W || !a.H) usage("bad --res");
    } else usage(("unknown option " + k).c_str());
  }
  if ((a.config < 0) == a.obj.empty()) usage("give exactly one of --config and --obj");
  if (a.staged && a.spectral) usage("the staged jobs run in RGB only");
  if (!a.metal_k.empty() && a.obj.empty()) usage("--metal applies to an --obj mesh");
  return a;
}

// Row-major 4x4, column vectors (the library's convention).
struct M4 {
  double m[4][4];
};
M4 look_at(const double eye[3], const double at[3], const double up[3]) {
  double d[3] = {at[0] - eye[0], at[1] - eye[1], at[2] - eye[2]};
  double dl = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  for (double& v : d) v /= dl;
  double r[3] = {up[1] * d[2] - up[2] * d[1], up[2] * d[0] - up[0] * d[2], up[0] * d[1] - up[1] * d[0]};
  double rl = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  for (double& v : r) v /= rl;
  double u[3] = {d[1] * r[2] - d[2] * r[1], d[2] * r[0] - d[0] * r[2], d[0] * r[1] - d[1] * r[0]};
  M4 c2w{};
  for (int i = 0; i < 3; ++i) {
    c2w.m[i][0] = r[i];
    c2w.m[i][1] = u[i];
    c2w.m[i][2] = d[i];
    c2w.m[i][3] = eye[i];
  }
  c2w.m[3][3] = 1.0;
  return c2w;
}
M4 rigid_inverse(const M4& a) {  // rotation + translation
  M4 r{};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[j][i];
  for (int i = 0; i < 3; ++i) r.m[i][3] = -(r.m[i][0] * a.m[0][3] + r.m[i][1] * a.m[1][3] + r.m[i][2] * a.m[2][3]);
  r.m[3][3] = 1.0;
  return r;
}
wpbr_mat4 to_mat4(const M4& a) {
  wpbr_mat4 o;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) o.m[4 * i + j] = (float)a.m[i][j];
  return o;
}

// A scene around an OBJ mesh: one conductor material, a sphere light above the
// mesh, an optional environment light, a camera framing the bounds.
struct ObjScene {
  wpbr_host::ObjMesh mesh;
  std::vector<float> env_rgb;
  uint32_t envW = 0, envH = 0;
  std::vector<float> tex_rgb[2];  // metallic, roughness
  wpbr_texture texs[2];
  wpbr_material mats[2];
  wpbr_mesh meshes[1];
  wpbr_sphere sphere;
  wpbr_light lights[2];
  wpbr_envmap envmap;
  wpbr_scene_desc desc;
};

void build_obj_scene(const Args& a, ObjScene& s) {
  s.mesh = wpbr_host::read_obj(a.obj);
  if (s.mesh.idx.empty()) throw std::runtime_error("OBJ has no faces");
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (size_t i = 0; i < s.mesh.pos.size(); i += 3)
    for (int c = 0; c < 3; ++c) {
      lo[c] = std::min(lo[c], (double)s.mesh.pos[i + c]);
      hi[c] = std::max(hi[c], (double)s.mesh.pos[i + c]);
    }
  double ctr[3], ext = 0.0;
  for (int c = 0; c < 3; ++c) {
    ctr[c] = 0.5 * (lo[c] + hi[c]);
    ext = std::max(ext, hi[c] - lo[c]);
  }
  memset(s.mats, 0, sizeof(s.mats));
  const float eta[3] = {0.2f, 0.92f, 1.1f}, kk[3] = {3.9f, 2.45f, 2.14f};
  for (wpbr_material& m : s.mats) {
    m.type = WPBR_MAT_CONDUCTOR;
    m.alpha_x = m.alpha_y = 0.25f;
    for (int c = 0; c < 3; ++c) {
      m.R[c] = 1.0f;
      m.eta_i[c] = 1.0f;
      m.eta_t[c] = eta[c];
      m.k[c] = kk[c];
    }
  }
  // OBJ normals come without tangents, and the shading-geometry branch needs
  // both: the mesh is shaded with its geometric normals.
  s.meshes[0] = wpbr_mesh{0, (uint32_t)(s.mesh.idx.size() / 3), 0, 0};
  if (s.mesh.has_uv) s.meshes[0].flags |= WPBR_MESH_UVS;
  memset(&s.desc, 0, sizeof(s.desc));
  if (!a.metal_k.empty()) {
    // CMaterialMetal with its two texture bindings (metallic k, roughness in
    // the red channel), looked up at the mesh's uvs
    if (!s.mesh.has_uv) throw std::runtime_error("--metal needs an OBJ with texture coordinates (vt)");
    const std::string* files[2] = {&a.metal_k, &a.metal_rough};
    for (int t = 0; t < 2; ++t) {
      uint32_t tw = 0, th = 0;
      s.tex_rgb[t] = wpbr_host::read_pfm(*files[t], &tw, &th);
      if (tw < 4 || th < 4) throw std::runtime_error("texture smaller than 4x4: " + *files[t]);
      s.texs[t] = wpbr_texture{tw, th, s.tex_rgb[t].data()};
    }
    s.mats[0].type = WPBR_MAT_METAL;
    s.mats[0].tex[0] = 0;
    s.mats[0].tex[1] = 1;
    s.desc.textures = s.texs;
    s.desc.n_textures = 2;
  }
  double lr = 0.1 * ext;
  double lp[3] = {ctr[0], hi[1] + 1.5 * ext, ctr[2]};
  M4 o2w{}, w2o{};
  for (int i = 0; i < 4; ++i) o2w.m[i][i] = w2o.m[i][i] = 1.0;
  for (int c = 0; c < 3; ++c) {
    o2w.m[c][3] = lp[c];
    w2o.m[c][3] = -lp[c];
  }
  memset(&s.sphere, 0, sizeof(s.sphere));
  s.sphere.object_to_world = to_mat4(o2w);
  s.sphere.world_to_object = to_mat4(w2o);
  s.sphere.radius = (float)lr;
  s.sphere.material = 1;
  uint32_t nl = 0;
  s.lights[nl++] = wpbr_light{WPBR_LIGHT_SPHERE, 0, {50.0f, 50.0f, 50.0f}};
  if (!a.env.empty()) {
    s.env_rgb = wpbr_host::read_pfm(a.env, &s.envW, &s.envH);
    memset(&s.envmap, 0, sizeof(s.envmap));
    s.envmap.width = s.envW;
    s.envmap.height = s.envH;
    s.envmap.rgb = s.env_rgb.data();
    // light-space +z (theta = 0) is world +y
    M4 l2w{}, w2l{};
    l2w.m[0][0] = w2l.m[0][0] = 1.0;
    l2w.m[1][2] = 1.0;
    l2w.m[2][1] = -1.0;
    w2l.m[1][2] = -1.0;
    w2l.m[2][1] = 1.0;
    l2w.m[3][3] = w2l.m[3][3] = 1.0;
    s.envmap.light_to_world = to_mat4(l2w);
    s.envmap.world_to_light = to_mat4(w2l);
    s.lights[nl++] = wpbr_light{WPBR_LIGHT_ENV, 0, {1.0f, 1.0f, 1.0f}};
    s.desc.envmap = &s.envmap;
  }
  s.desc.spheres = &s.sphere;
  s.desc.n_spheres = 1;
  s.desc.n_vertices = (uint32_t)(s.mesh.pos.size() / 3);
  s.desc.positions = s.mesh.pos.data();
  s.desc.uvs = s.mesh.has_uv ? s.mesh.uv.data() : nullptr;
  s.desc.n_triangles = (uint32_t)(s.mesh.idx.size() / 3);
  s.desc.indices = s.mesh.idx.data();
  s.desc.meshes = s.meshes;
  s.desc.n_meshes = 1;
  s.desc.materials = s.mats;
  s.desc.n_materials = 2;
  s.desc.lights = s.lights;
  s.desc.n_lights = nl;
  double eye[3] = {ctr[0] + 0.4 * ext, ctr[1] + 0.5 * ext, ctr[2] - 1.8 * ext};
  double up[3] = {0.0, 1.0, 0.0};
  M4 c2w = look_at(eye, ctr, up);
  wpbr_camera& cam = s.desc.camera;
  cam.camera_to_world = to_mat4(c2w);
  cam.world_to_camera = to_mat4(rigid_inverse(c2w));
  cam.fov_deg = a.fov;
  cam.near_z = 0.1f;
  cam.far_z = 10000.0f;
  float aspect = (float)a.W / (float)a.H;
  cam.screen[0] = aspect >= 1.0f ? -aspect : -1.0f;
  cam.screen[1] = aspect >= 1.0f ? -1.0f : -1.0f / aspect;
  cam.screen[2] = -cam.screen[0];
  cam.screen[3] = -cam.screen[1];
  cam.res_x = a.W;
  cam.res_y = a.H;
}

#define CHECK(call)                                                                          \
  do {                                                                                       \
    wpbr_status st_ = (call);                                                                \
    if (st_ != WPBR_OK) {                                                                    \
      fprintf(stderr, "wpbr_host: %s failed (%d): %s\n", #call, (int)st_, wpbr_last_error(gpu)); \
      return 1;                                                                              \
    }                                                                                        \
  } while (0)

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// MEngine::render's per-sample job groups in the reference's order.
const wpbr_job_id kJobOrder[] = {
    WPBR_JOB_CAMERA_RAYS,   WPBR_JOB_COLLIDE_PRIMARY, WPBR_JOB_EMITTED_LIGHT,   WPBR_JOB_BSDF_SETUP,
    WPBR_JOB_SAMPLE_LIGHT,  WPBR_JOB_SHADOW_LIGHT,    WPBR_JOB_BSDF_COMPUTE,    WPBR_JOB_INTEGRATE_LIGHT,
    WPBR_JOB_SAMPLE_BSDF,   WPBR_JOB_SHADOW_BSDF,     WPBR_JOB_LIGHT_COMPUTE,   WPBR_JOB_INTEGRATE_BSDF,
    WPBR_JOB_FILM_ACCUMULATE};

}  // namespace

int main(int argc, char** argv) {
  Args a = parse(argc, argv);
  ObjScene os;
  wpbr_scenegen* gen = nullptr;
  const wpbr_scene_desc* desc = nullptr;
  try {
    if (!a.obj.empty()) {
      build_obj_scene(a, os);
      desc = &os.desc;
    } else {
      if (wpbr_scenegen_create((uint32_t)a.config, a.seed, a.W, a.H, a.level, 0, &gen) != WPBR_OK) {
        fprintf(stderr, "wpbr_host: unknown configuration %d\n", a.config);
        return 2;
      }
      desc = wpbr_scenegen_desc(gen);
    }
  } catch (const std::exception& e) {
    fprintf(stderr, "wpbr_host: %s\n", e.what());
    return 2;
  }
  if (a.dump) {
    double psum = 0.0;
    uint64_t isum = 0;
    for (uint32_t i = 0; i < desc->n_vertices * 3; ++i) psum += desc->positions[i];
    for (uint32_t i = 0; i < desc->n_triangles * 3; ++i) isum += desc->indices[i];
    printf("{\"vertices\": %u, \"triangles\": %u, \"spheres\": %u, \"lights\": %u, \"uvs\": %d, "
           "\"position_sum\": %.9g, \"index_sum\": %llu, \"env\": [%u, %u], \"textures\": %u}\n",
           desc->n_vertices, desc->n_triangles, desc->n_spheres, desc->n_lights, desc->uvs != nullptr, psum,
           (unsigned long long)isum, desc->envmap ? desc->envmap->width : 0, desc->envmap ? desc->envmap->height : 0,
           desc->n_textures);
    if (gen) wpbr_scenegen_destroy(gen);
    return 0;
  }
  wpbr_ctx* gpu = nullptr;
  wpbr_status cs = wpbr_create(0, &gpu);
  if (cs != WPBR_OK) {
    fprintf(stderr, "wpbr_host: no usable CUDA device (%d)\n", (int)cs);
    return 3;
  }
  const uint32_t W = desc->camera.res_x, H = desc->camera.res_y;
  CHECK(wpbr_set_quirks(gpu, a.quirks));
  if (a.spectral) CHECK(wpbr_set_spectrum(gpu, WPBR_SPECTRUM_SAMPLED64));
  CHECK(wpbr_scene_upload(gpu, desc));
  double t0 = now_ms();
  CHECK(wpbr_bvh_build(gpu));
  CHECK(wpbr_synchronize(gpu));
  double t1 = now_ms();
  CHECK(wpbr_render_setup(gpu, a.spp, a.render_seed, 0));
  for (uint32_t p = 0; p < a.spp; ++p) {
    if (a.staged) {
      for (wpbr_job_id j : kJobOrder) CHECK(wpbr_job_run(gpu, j, p));
    } else {
      CHECK(wpbr_render_pass(gpu, p));
    }
  }
  CHECK(wpbr_synchronize(gpu));
  double t2 = now_ms();
  CHECK(wpbr_check_device_errors(gpu));
  std::vector<float> L((size_t)W * H * 3), w((size_t)W * H);
  CHECK(wpbr_film_read(gpu, L.data(), w.data()));
  std::vector<uint8_t> rgb((size_t)W * H * 3);
  CHECK(wpbr_film_tonemap(gpu, rgb.data()));
  if (!a.out.empty()) {
    std::vector<float> I(L.size());
    for (size_t i = 0; i < w.size(); ++i)
      for (int c = 0; c < 3; ++c) I[3 * i + c] = L[3 * i + c] / w[i];
    wpbr_host::write_pfm(a.out + ".pfm", I.data(), W, H);
    wpbr_host::write_pfm(a.out + ".weights.pfm", [&] {
      std::vector<float> ww(3 * w.size());
      for (size_t i = 0; i < w.size(); ++i) ww[3 * i] = ww[3 * i + 1] = ww[3 * i + 2] = w[i];
      return ww;
    }().data(), W, H);
    wpbr_host::write_ppm(a.out + ".ppm", rgb.data(), W, H);
  }
  printf("{\"film\": [%u, %u], \"spp\": %u, \"mode\": \"%s\", \"triangles\": %u, \"spheres\": %u, "
         "\"build_ms\": %.3f, \"render_ms\": %.3f, \"msamples_per_s\": %.3f}\n",
         W, H, a.spp, a.staged ? "staged" : (a.spectral ? "fused-sampled64" : "fused"), desc->n_triangles,
         desc->n_spheres, t1 - t0, t2 - t1,
         (double)W * H * a.spp / ((t2 - t1) * 1e3));
  wpbr_destroy(gpu);
  if (gen) wpbr_scenegen_destroy(gen);
  return 0;
}
