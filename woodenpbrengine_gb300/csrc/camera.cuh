// camera.cuh — perspective camera (GB300 pipeline side).
//   A1 camera_setup: SCameraProjective::create + SCameraPerspective::create
//      (WoodenPBREngine/CSCameraProjective.h:19-53, CSCameraPerspective.h:17-39)
//   A2 camera_ray:   JobCameraPerspGenerateRaysDifferential::update
//      (WoodenPBREngine/CSCameraPerspective.cpp:9-54) and
//      CTransform::operator()(DRayDifferentialf) (CTransform.h:68-76)
#pragma once

#include "geom.cuh"
#include "wpbr_scene.h"

namespace wpbr {

struct CameraParams {
  Xf raster_camera;  // raster -> camera
  Xf c2w;            // camera -> world
  V3 dx, dy;         // dxCamera / dyCamera
  uint32_t W, H;
};

struct RayD {
  V3 o, d;            // main ray (dir normalised after the world transform)
  V3 dxo, dxd, dyo, dyd;  // differential rays (not renormalised)
};

// A2. pFilm in raster space (pixel + jitter).
WPBR_HD RayD camera_ray(const CameraParams& c, float fx, float fy) {
  V3 pcam = xpoint(c.raster_camera, V3{fx, fy, 0.0f});
  V3 d = normalize(pcam);
  V3 ddx = normalize(add(pcam, c.dx));
  V3 ddy = normalize(add(pcam, c.dy));
  RayD r;
  V3 o = V3{0.0f, 0.0f, 0.0f};
  r.o = xpoint(c.c2w, o);
  r.d = normalize(xvector(c.c2w, d));
  r.dxo = xpoint(c.c2w, o);
  r.dxd = xvector(c.c2w, ddx);
  r.dyo = xpoint(c.c2w, o);
  r.dyd = xvector(c.c2w, ddy);
  return r;
}

}  // namespace wpbr

#include "host_xf.hpp"
namespace wpbr {
// host-only (setup) part
inline Xf xf_from(const wpbr_mat4& a) {
  Xf r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) r.m[i][j] = a.m[4 * i + j];
  return r;
}
// A1. screenRaster = T(-pMin) then S(1/extent) then S(res-1); rasterCamera =
// inverse(screenRaster) then inverse(cameraScreen); dx/dyCamera from the
// vector transform of the unit axes (the reference passes DVector3f).
inline CameraParams camera_setup(const wpbr_camera& c) {
  Xf camera_screen = xf_perspective(c.fov_deg, c.near_z, c.far_z);
  float sx0 = c.screen[0], sy0 = c.screen[1], sx1 = c.screen[2], sy1 = c.screen[3];
  Xf t = xf_translate(-sx0, -sy0, 0.0f);
  Xf s1 = xf_scale((float)(1.0 / (double)(sx1 - sx0)), (float)(1.0 / (double)(sy1 - sy0)), 1.0f);
  Xf s2 = xf_scale((float)((int)c.res_x - 1), (float)((int)c.res_y - 1), 1.0f);
  Xf screen_raster = compose(compose(t, s1), s2);
  CameraParams p;
  p.raster_camera = compose(xf_inverse(screen_raster), xf_inverse(camera_screen));
  p.dx = sub(xvector(p.raster_camera, V3{1, 0, 0}), xvector(p.raster_camera, V3{0, 0, 0}));
  p.dy = sub(xvector(p.raster_camera, V3{0, 1, 0}), xvector(p.raster_camera, V3{0, 0, 0}));
  p.c2w = xf_from(c.camera_to_world);
  p.W = c.res_x;
  p.H = c.res_y;
  return p;
}
}  // namespace wpbr
