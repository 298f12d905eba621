/*
 * wpbr_record.h — per-pixel record of one sample pass, stage by stage.
 *
 * One entry per pixel of the recorded rectangle, in row-major order. Each
 * pointer may be NULL (that stage is not recorded). The GPU pipeline's
 * staged (job-by-job) pass and the CPU oracle fill the same layout, so every
 * row of the reference's per-spp job list can be compared in isolation:
 *
 *   pfilm, ray_*        JobSamplerUpdateCameraSamples + JobCameraPerspGenerateRaysDifferential
 *   hit_prim, hit_t     runCollisionSystem (primary rays)
 *   si_*                Job{Sphere,Triangle}ProcessFullInteractionRequests
 *   frame               JobBSDFComputeTransform (rows ss, ts, ns)
 *   le                  JobLightInfiniteAreaLeCompute (camera misses)
 *   light_idx           JobScatteringSampleLight
 *   l_wi, l_li, l_pdf   JobSphereLightProcessSamplingRequests / JobLightInfiniteAreaLiSample
 *   l_flags             bit0 shadow ray traced, bit1 unoccluded
 *   l_f, l_fpdf         JobBSDF*Compute (written when unoccluded)
 *   b_wi, b_f, b_pdf    JobBSDF*Sample (b_wi in world space)
 *   b_flags             bit0 sample valid, bit1 shadow ray traced, bit2 unoccluded
 *   b_li, b_lpdf        JobSphereLightProcessComputeRequests / JobLightInfiniteAreaLiCompute
 *   L                   the sample's radiance after both MIS integrations
 *
 * Entries of stages a pixel does not reach are left untouched (callers
 * pre-fill them).
 */
#ifndef WPBR_RECORD_H
#define WPBR_RECORD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct wpbr_pass_record {
  float* pfilm;     /* 2 */
  float* ray_o;     /* 3 */
  float* ray_d;     /* 3 */
  float* ray_dx_d;  /* 3 */
  float* ray_dy_d;  /* 3 */
  uint32_t* hit_prim;
  float* hit_t;
  float* si_p;      /* 3 */
  float* si_n;      /* 3 */
  float* si_wo;     /* 3 */
  float* si_sn;     /* 3 */
  float* si_sdpdu;  /* 3 */
  float* si_dpdu;   /* 3 */
  float* si_dpdv;   /* 3 */
  float* si_dndu;   /* 3 */
  float* si_dndv;   /* 3 */
  float* frame;     /* 9 */
  float* le;        /* 3 */
  uint32_t* light_idx;
  float* l_wi;      /* 3 */
  float* l_li;      /* 3 */
  float* l_pdf;
  uint32_t* l_flags;
  float* l_f;       /* 3 */
  float* l_fpdf;
  float* b_wi;      /* 3 */
  float* b_f;       /* 3 */
  float* b_pdf;
  uint32_t* b_flags;
  float* b_li;      /* 3 */
  float* b_lpdf;
  float* L;         /* 3 */
} wpbr_pass_record;

#ifdef __cplusplus
}
#endif

#endif /* WPBR_RECORD_H */
