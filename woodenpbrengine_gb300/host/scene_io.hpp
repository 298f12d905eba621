// scene_io.hpp — scene ingestion and film output for the host runner: a
// Wavefront OBJ mesh reader (positions, normals, texture coordinates, polygon
// faces fanned into triangles), PFM read/write for environment maps and
// radiance films, and binary PPM output. The reference imports meshes with
// assimp (WoodenPBREngine/MeshTools.h:14-99) and images with lodepng
// (CSTextureProcess.h:304-527); these readers cover the formats the host needs
// without either library.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace wpbr_host {

struct ObjMesh {
  std::vector<float> pos, nrm, uv;  // per output vertex (3, 3, 2 floats)
  std::vector<uint32_t> idx;        // 3 per triangle
  bool has_nrm = false, has_uv = false;
};

// OBJ indices are 1-based, negative ones count from the end. A face corner
// "v", "v/vt", "v//vn" or "v/vt/vn" becomes its own output vertex unless the
// same corner tuple was seen before.
inline ObjMesh read_obj(const std::string& path) {
  std::ifstream in(path);
  if (!in) throw std::runtime_error("cannot open " + path);
  std::vector<float> P, N, T;
  ObjMesh m;
  struct Key {
    long v, t, n;
  };
  std::vector<Key> keys;
  std::vector<std::vector<std::pair<long, uint32_t>>> by_v;  // position -> (hash of t,n) -> output vertex
  auto resolve = [](long i, size_t count) -> long {
    if (i > 0) return i - 1;
    if (i < 0) return (long)count + i;
    throw std::runtime_error("OBJ index 0");
  };
  std::string line;
  bool any_t = false, any_n = false;
  std::vector<std::vector<Key>> faces;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    std::string tag;
    if (!(ls >> tag)) continue;
    if (tag == "v") {
      float x, y, z;
      ls >> x >> y >> z;
      P.insert(P.end(), {x, y, z});
    } else if (tag == "vn") {
      float x, y, z;
      ls >> x >> y >> z;
      N.insert(N.end(), {x, y, z});
    } else if (tag == "vt") {
      float u = 0, v = 0;
      ls >> u >> v;
      T.insert(T.end(), {u, v});
    } else if (tag == "f") {
      std::vector<Key> f;
      std::string c;
      while (ls >> c) {
        Key k{0, -1, -1};
        long a = 0, b = 0, d = 0;
        int got = 0;
        if (sscanf(c.c_str(), "%ld/%ld/%ld", &a, &b, &d) == 3) {
          got = 3;
        } else if (sscanf(c.c_str(), "%ld//%ld", &a, &d) == 2) {
          got = 4;
        } else if (sscanf(c.c_str(), "%ld/%ld", &a, &b) == 2) {
          got = 2;
        } else if (sscanf(c.c_str(), "%ld", &a) == 1) {
          got = 1;
        }
        if (!got) throw std::runtime_error("bad OBJ face corner: " + c);
        k.v = resolve(a, P.size() / 3);
        if (got == 2 || got == 3) k.t = resolve(b, T.size() / 2);
        if (got == 3 || got == 4) k.n = resolve(d, N.size() / 3);
        any_t |= k.t >= 0;
        any_n |= k.n >= 0;
        f.push_back(k);
      }
      if (f.size() < 3) throw std::runtime_error("OBJ face with fewer than 3 corners");
      faces.push_back(f);
    }
  }
  m.has_nrm = any_n;
  m.has_uv = any_t;
  by_v.resize(P.size() / 3);
  auto vertex_of = [&](const Key& k) -> uint32_t {
    if (k.v < 0 || (size_t)k.v >= P.size() / 3) throw std::runtime_error("OBJ position index out of range");
    long tag = (k.t + 1) * 1000003L + (k.n + 1);
    for (auto& e : by_v[k.v])
      if (e.first == tag) return e.second;
    uint32_t id = (uint32_t)(m.pos.size() / 3);
    m.pos.insert(m.pos.end(), {P[3 * k.v], P[3 * k.v + 1], P[3 * k.v + 2]});
    if (m.has_nrm) {
      if (k.n >= 0 && (size_t)k.n < N.size() / 3)
        m.nrm.insert(m.nrm.end(), {N[3 * k.n], N[3 * k.n + 1], N[3 * k.n + 2]});
      else
        m.nrm.insert(m.nrm.end(), {0.0f, 0.0f, 0.0f});
    }
    if (m.has_uv) {
      if (k.t >= 0 && (size_t)k.t < T.size() / 2)
        m.uv.insert(m.uv.end(), {T[2 * k.t], T[2 * k.t + 1]});
      else
        m.uv.insert(m.uv.end(), {0.0f, 0.0f});
    }
    by_v[k.v].push_back({tag, id});
    return id;
  };
  for (const auto& f : faces) {
    uint32_t a = vertex_of(f[0]);
    for (size_t i = 1; i + 1 < f.size(); ++i) {
      uint32_t b = vertex_of(f[i]), c = vertex_of(f[i + 1]);
      m.idx.insert(m.idx.end(), {a, b, c});
    }
  }
  return m;
}

// PFM ("PF" colour): rows stored bottom to top; a negative scale means
// little-endian data. Returned rows are top to bottom, 3 floats per pixel.
inline std::vector<float> read_pfm(const std::string& path, uint32_t* W, uint32_t* H) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) throw std::runtime_error("cannot open " + path);
  char magic[3] = {0, 0, 0};
  int w = 0, h = 0;
  double scale = 0.0;
  if (fscanf(f, "%2s %d %d %lf", magic, &w, &h, &scale) != 4 || strcmp(magic, "PF") != 0 || w <= 0 || h <= 0) {
    fclose(f);
    throw std::runtime_error("not a colour PFM: " + path);
  }
  fgetc(f);  // the single whitespace after the header
  std::vector<float> rows((size_t)w * h * 3);
  size_t got = fread(rows.data(), sizeof(float), rows.size(), f);
  fclose(f);
  if (got != rows.size()) throw std::runtime_error("truncated PFM: " + path);
  bool little = scale < 0.0;
  uint16_t probe = 1;
  bool host_little = *(uint8_t*)&probe == 1;
  if (little != host_little) {
    for (float& v : rows) {
      uint32_t u;
      memcpy(&u, &v, 4);
      u = (u >> 24) | ((u >> 8) & 0xFF00u) | ((u << 8) & 0xFF0000u) | (u << 24);
      memcpy(&v, &u, 4);
    }
  }
  std::vector<float> out(rows.size());
  for (int y = 0; y < h; ++y)
    memcpy(&out[(size_t)y * w * 3], &rows[(size_t)(h - 1 - y) * w * 3], sizeof(float) * 3 * w);
  *W = (uint32_t)w;
  *H = (uint32_t)h;
  return out;
}

inline void write_pfm(const std::string& path, const float* rgb, uint32_t W, uint32_t H) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  uint16_t probe = 1;
  bool host_little = *(uint8_t*)&probe == 1;
  fprintf(f, "PF\n%u %u\n%s\n", W, H, host_little ? "-1.0" : "1.0");
  for (uint32_t y = 0; y < H; ++y) fwrite(rgb + (size_t)(H - 1 - y) * W * 3, sizeof(float), 3 * (size_t)W, f);
  fclose(f);
}

inline void write_ppm(const std::string& path, const uint8_t* rgb, uint32_t W, uint32_t H) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  fprintf(f, "P6\n%u %u\n255\n", W, H);
  fwrite(rgb, 1, (size_t)W * H * 3, f);
  fclose(f);
}

}  // namespace wpbr_host
