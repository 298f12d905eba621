/*
 * wpbr_scene.h — plain-C scene description shared by every caller of the
 * ray-pipeline library (host arrays owned by the caller).
 *
 * It replaces the ECS entities WoodenPBREngine builds in MEngine::buildScene
 * (WoodenPBREngine/MEngine.cpp:82-339):
 *   spheres        SSphere::create (CSSphere.cpp:199-213): CTransform + CSphere
 *   triangle mesh  STriangleMesh::create (CSTriangleMesh.cpp:11-39): positions,
 *                  normals and tangents already baked to world space
 *   materials      CSMaterialMetal / CSMaterialDielectric / SMaterialPerfectGlass
 *                  parameter sets (CMaterialMetal.cpp:37-48,
 *                  CMaterialDieletric.cpp:24-32, CMaterialPerfectGlass.cpp:41-44)
 *   lights         CLight on a sphere entity (CSSphere.h:187-267) or the
 *                  infinite-area light (CLightInfiniteArea.cpp:82-103)
 *   camera         SCameraPerspective::create inputs (CSCameraPerspective.h:17-39)
 *
 * Primitive ids: spheres first (0 .. n_spheres-1), then triangles
 * (n_spheres .. n_spheres+n_triangles-1) — the order in which the reference
 * creates CCentroid components (spheres during buildScene, triangle entities
 * afterwards in JobTriangleMeshGenerateTriangles), which fixes the Morton-sort
 * tie order.
 *
 * Matrices are row-major and act on column vectors: p' = M * (p, 1).
 */
#ifndef WPBR_SCENE_H
#define WPBR_SCENE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct wpbr_mat4 {
  float m[16];
} wpbr_mat4;

enum wpbr_material_type {
  WPBR_MAT_CONDUCTOR = 0,  /* SBSDFConductorMicroface (Trowbridge-Reitz + conductor Fresnel) */
  WPBR_MAT_DIELECTRIC = 1, /* SBSDFDielectricMicroface (reflection lobe, dielectric Fresnel) */
  WPBR_MAT_SPECULAR = 2,   /* SBXDFSpecularReflectance (perfect glass material) */
  /* CMaterialMetal (CMaterialMetal.cpp:8-58): a conductor whose k is the
   * metallic texture and whose alpha is roughnessToAlpha(clamp(90 * r, 0, 90))
   * of the roughness texture's red channel, both looked up with anisotropic
   * EWA filtering at the hit's texture footprint; R = 1, eta_i = 1,
   * eta_t = 1.5. Texture indices in wpbr_material::tex. */
  WPBR_MAT_METAL = 3,
  /* The same material looked up with the isotropic trilinear sampler
   * (STexture2DSamplerIsotropic, CSTextureProcess.h:259-289), the
   * alternative left commented out in CMaterialMetal.cpp:34-35. */
  WPBR_MAT_METAL_ISOTROPIC = 4
};
#define WPBR_MAT_TEXTURED(type) ((type) == WPBR_MAT_METAL || (type) == WPBR_MAT_METAL_ISOTROPIC)

typedef struct wpbr_material {
  uint32_t type;     /* wpbr_material_type */
  float alpha_x;     /* CReflectDirSamplerMicroface::alphax */
  float alpha_y;     /* CReflectDirSamplerMicroface::alphay */
  float R[3];        /* CSpectrumScale */
  float eta_i[3];    /* conductor: per channel; dielectric/specular: [0] */
  float eta_t[3];
  float k[3];        /* conductor absorption */
  uint16_t tex[2];   /* textured metal: metallic and roughness texture indices */
} wpbr_material;     /* 64 bytes */

typedef struct wpbr_sphere {
  wpbr_mat4 object_to_world;
  wpbr_mat4 world_to_object;
  float radius;
  uint32_t material;
  uint32_t pad[2];
} wpbr_sphere;

enum wpbr_mesh_flags {
  WPBR_MESH_NORMALS_TANGENTS = 1u, /* both arrays present: shading-geometry branch */
  WPBR_MESH_UVS = 2u
};

typedef struct wpbr_mesh {
  uint32_t tri_begin;   /* first triangle (index into the triangle arrays) */
  uint32_t tri_count;
  uint32_t material;
  uint32_t flags;       /* wpbr_mesh_flags */
} wpbr_mesh;

enum wpbr_light_type { WPBR_LIGHT_SPHERE = 0, WPBR_LIGHT_ENV = 1 };

typedef struct wpbr_light {
  uint32_t type;          /* wpbr_light_type */
  uint32_t sphere_index;  /* WPBR_LIGHT_SPHERE: index into spheres (= its primitive id) */
  float Le[3];            /* CLight::LEmit (RGB) */
} wpbr_light;

typedef struct wpbr_envmap {
  uint32_t width, height;   /* texels; row 0 is theta = 0 */
  const float* rgb;         /* width*height*3 floats, row-major */
  wpbr_mat4 light_to_world;
  wpbr_mat4 world_to_light;
} wpbr_envmap;

/* An RGB texture (linear values, row 0 at t = 0), MIP-mapped at upload as
 * SLoadTexture::generateMIPS does (CSTextureProcess.h:352-400). At least 4x4. */
typedef struct wpbr_texture {
  uint32_t width, height;
  const float* rgb;          /* width*height*3 floats, row-major */
} wpbr_texture;

typedef struct wpbr_camera {
  wpbr_mat4 camera_to_world;
  wpbr_mat4 world_to_camera;
  float fov_deg;          /* makePerspective(fov, near, far) */
  float near_z, far_z;
  float screen[4];        /* screenWindow pMin.x, pMin.y, pMax.x, pMax.y */
  uint32_t res_x, res_y;  /* film resolution */
} wpbr_camera;

typedef struct wpbr_scene_desc {
  const wpbr_sphere* spheres;
  uint32_t n_spheres;
  uint32_t n_vertices;
  const float* positions;   /* n_vertices*3, world space */
  const float* normals;     /* n_vertices*3 or NULL */
  const float* tangents;    /* n_vertices*3 or NULL */
  const float* uvs;         /* n_vertices*2 or NULL */
  uint32_t n_triangles;
  const uint32_t* indices;  /* n_triangles*3 */
  const wpbr_mesh* meshes;
  uint32_t n_meshes;
  const wpbr_material* materials;
  uint32_t n_materials;
  const wpbr_light* lights;
  uint32_t n_lights;
  const wpbr_envmap* envmap; /* NULL when the scene has no infinite light */
  wpbr_camera camera;
  const wpbr_texture* textures; /* referenced by textured-metal materials */
  uint32_t n_textures;
} wpbr_scene_desc;

/* Behaviour switches shared by the GPU pipeline and the CPU oracle.
 * Default 0 keeps every deterministic behaviour of the reference and fixes
 * the ones that are undefined there. */
enum wpbr_quirk {
  /* Restore the triangle-test axis permutation bug (CSTriangle.cpp:34-35:
   * ky = kz + 2 selects a fourth SIMD lane when kz == 1); with the lane read
   * as 0, every ray whose largest direction component is y misses all
   * triangles. Default: pbrt's permutation (ky = 0 when kz == 1). */
  WPBR_Q_TRI_PERMUTATION_BUG = 1u << 0,
  /* JobLightInfiniteAreaLiSample discards the radiance it looks up and
   * returns black Li (CLightInfiniteArea.cpp:192-199). Set to return it. */
  WPBR_Q_ENV_LI_SAMPLE_FIX = 1u << 1,
  /* SSphere::pdf measures the cone from the world origin because of a comma
   * operator (CSSphere.cpp:228). Set to measure it from the shading point. */
  WPBR_Q_SPHERE_PDF_FIX = 1u << 2,
  /* Restore data[x + y*resY] when building the environment sampling
   * distribution (CLightInfiniteArea.cpp:130-131). Default indexes by resX. */
  WPBR_Q_ENV_DISTRIB_INDEX_BUG = 1u << 3,
  /* Build over the fully (30-bit) sorted Morton array. The reference's
   * five-pass radix sort ping-pongs between the code array and a temporary
   * buffer and leaves its last pass in the temporary buffer
   * (SLBVH.cpp:250-283), so the treelet split, the bounds gather and
   * emitLBVH all read the array after the fourth pass: codes sorted by their
   * low 24 bits. Default keeps that order. */
  WPBR_Q_FULL_MORTON_SORT = 1u << 4,
  /* Sampled64 mode only: xyzToRGB's stored matrix has 0.041556 where the
   * standard XYZ-to-sRGB matrix has 0.055648 (blue from X,
   * CoefficientSpectrum.h:17-19). Set to use the standard value. */
  WPBR_Q_XYZ_MATRIX_FIX = 1u << 5,
  /* Draw samples from the reference's per-pixel stratified arrays
   * (CSSamplerStratified.cpp:8-90 over the sizes of CSFilm.cpp:22-23): 80
   * shuffled 1D values stratified over [0, 1), and 272 shuffled 2D entries of
   * which 256 are stratified with the 1/data.size() scale of :79 (all inside
   * [0, 1/17)^2) and 16 are (0, 0). Pass p reads 1D position p and 2D
   * positions 3p, 3p+1, 3p+2 (camera, light, BSDF) of the pixel's arrays.
   * Default: stratification over the passes with the intended 1/n scale. */
  WPBR_Q_REF_SAMPLER_ARRAYS = 1u << 6
};
/* Every defined quirk bit; other bits are rejected. */
#define WPBR_QUIRK_MASK 0x7Fu

#ifdef __cplusplus
}
#endif

#endif /* WPBR_SCENE_H */
