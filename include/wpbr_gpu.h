/*
 * wpbr_gpu.h — C ABI of the GB300 ray-pipeline library (libwpbr_gpu.so).
 *
 * Drop-in for WoodenPBREngine's per-sample ray pipeline: the ECS jobs that
 * MEngine runs through JOB_RUN (WoodenPBREngine/MEngine.cpp:44-50) in the
 * order of MEngine::buildLBVH (:341-350), runCollisionSystem (:352-361) and
 * MEngine::render (:380-448). The reference exposes that surface as C++ job
 * classes over ECS components; this library exposes one context per GPU and
 * plain pointers and sizes, so any host (C++, Python ctypes, cgo, JNI) can bind
 * it. Reference interface replaced by each entry point is cited beside it.
 *
 * Conventions
 *  - Every call returns wpbr_status; wpbr_last_error() describes the last
 *    failure of a context. No exception crosses the ABI.
 *  - A context is externally synchronised (one host thread at a time). All its
 *    GPU work is issued on its stream (wpbr_set_stream; default: a stream the
 *    context creates). Calls taking HOST buffers synchronise before returning;
 *    calls taking DEVICE buffers (suffix _device) are asynchronous.
 *  - Rays are 8 floats: origin xyz, unused, direction xyz, tmax (+inf for the
 *    reference's unbounded rays). Hits are 4 floats: t (+inf on a miss), the
 *    primitive id's bits (0xFFFFFFFF on a miss), barycentric weights of the
 *    triangle's second and third vertex (0 for spheres).
 *  - Primitive ids: spheres first, then triangles (see wpbr_scene.h).
 *  - No CPU fallback: without a usable CUDA device the calls that need one
 *    return WPBR_ERR_NO_DEVICE.
 */
#ifndef WPBR_GPU_H
#define WPBR_GPU_H

#include <stdint.h>

#include "wpbr_record.h"
#include "wpbr_scene.h"

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define WPBR_API __attribute__((visibility("default")))
#else
#define WPBR_API
#endif

typedef enum wpbr_status {
  WPBR_OK = 0,
  WPBR_ERR_INVALID_ARG = 1,
  WPBR_ERR_OOM = 2,
  WPBR_ERR_CUDA = 3,
  WPBR_ERR_TRAVERSAL_LIMIT = 4, /* a traversal stack or loop bound was hit */
  WPBR_ERR_NOT_BUILT = 5,       /* scene / BVH / render setup missing */
  WPBR_ERR_NO_DEVICE = 6
} wpbr_status;

typedef struct wpbr_ctx wpbr_ctx;

/* ---- context --------------------------------------------------------- */
/* Replaces MEngine's singleton ECS (MEngine.h:9-36) for one GPU. */
WPBR_API wpbr_status wpbr_create(int device, wpbr_ctx** out);
WPBR_API void wpbr_destroy(wpbr_ctx* ctx);
WPBR_API const char* wpbr_last_error(const wpbr_ctx* ctx);
WPBR_API wpbr_status wpbr_set_stream(wpbr_ctx* ctx, void* cuda_stream);
WPBR_API void* wpbr_get_stream(const wpbr_ctx* ctx);
/* wpbr_quirk bits (wpbr_scene.h); applies to later builds and renders. */
WPBR_API wpbr_status wpbr_set_quirks(wpbr_ctx* ctx, uint32_t quirks);
WPBR_API wpbr_status wpbr_synchronize(wpbr_ctx* ctx);
/* Traversal layout (an implementation choice of this library; the results
 * are the same): BINARY (default) traverses the child-pair layout of the
 * reference's tree with every leaf of more than 8 (and at most 4096)
 * primitives subdivided into a small tree over ranges of its sorted
 * positions, visited in position order; BINARY_FULL_LEAVES the same layout
 * with the reference's leaves as they are. Value 1 (a four-wide collapse,
 * slower on this GPU) is no longer accepted. */
enum wpbr_traversal { WPBR_TRAVERSAL_BINARY = 0, WPBR_TRAVERSAL_BINARY_FULL_LEAVES = 2 };
WPBR_API wpbr_status wpbr_set_traversal(wpbr_ctx* ctx, uint32_t mode);
/* Spectral representation of the render passes. RGB (default) carries three
 * channels; SAMPLED64 is the reference's Spectrum (SampledSpectrum, 64 bins
 * over 400-700 nm, CSpectrum.h:8): scene RGB values become spectra (grey
 * values constant, others through the RGB-to-spectrum bases; environment
 * texels as illuminants), shading runs per bin, and the film accumulates
 * spectra that wpbr_film_read / wpbr_film_tonemap see through toRGB. Its
 * wavefront shares the RGB pass's traversals and replaces spawn, finish and
 * film with per-bin kernels; no staged jobs, no adjoint. Takes effect at the
 * next wpbr_render_setup. */
enum wpbr_spectrum { WPBR_SPECTRUM_RGB = 0, WPBR_SPECTRUM_SAMPLED64 = 1 };
WPBR_API wpbr_status wpbr_set_spectrum(wpbr_ctx* ctx, uint32_t mode);
/* Device error word (traversal limits etc.) since the last call; cleared. */
WPBR_API wpbr_status wpbr_check_device_errors(wpbr_ctx* ctx);

/* ---- scene ------------------------------------------------------------- */
/* MEngine::buildScene (MEngine.cpp:82-339) inputs + preprocess (:374-378):
 * copies the scene to the device, sets up the camera
 * (SCameraPerspective::create, CSCameraPerspective.h:17-39) and builds the
 * environment sampling distribution
 * (JobLightInfiniteAreaPreprocessSampling, CLightInfiniteArea.cpp:113-139). */
WPBR_API wpbr_status wpbr_scene_upload(wpbr_ctx* ctx, const wpbr_scene_desc* scene);
/* camera setup result: raster_camera[16] (row-major), dx[3], dy[3] */
WPBR_API wpbr_status wpbr_camera_info(wpbr_ctx* ctx, float* raster_camera, float* dx, float* dy);
/* The same setup without a context or GPU (host arithmetic only). */
WPBR_API wpbr_status wpbr_camera_setup(const wpbr_camera* camera, float* raster_camera, float* dx, float* dy);
/* environment distribution (A21): cond_cdf[H*(W+1)], cond_int[H],
 * marg_cdf[H+1], marg_int[1]; host pointers, any may be NULL */
WPBR_API wpbr_status wpbr_env_distribution(wpbr_ctx* ctx, float* cond_cdf, float* cond_int, float* marg_cdf,
                                           float* marg_int);

/* ---- BVH --------------------------------------------------------------- */
/* MEngine::buildLBVH (MEngine.cpp:341-350): JobUpdateBoundsAndCentroid*,
 * JobGenerateShapesCentroidBound, JobGenerateShapesMortonCode,
 * JobSortsShapesByMortonCode, JobEmitLBVH, JobBuildUpperSAH (SLBVH.cpp). */
WPBR_API wpbr_status wpbr_bvh_build(wpbr_ctx* ctx);
/* out[4] = n_prims, n_nodes, n_treelets, max_depth */
WPBR_API wpbr_status wpbr_bvh_info(wpbr_ctx* ctx, uint32_t* out4);
/* Copies the build products to host arrays (NULL skips): per primitive (input
 * order) bounds[6], centroids[3], Morton codes; cbounds[6]; the array the tree
 * is built over (sorted_codes, sorted_prims); treelet starts; the flattened
 * CSceneTreeLBVH (nodes[3] = offset, n_shapes, axis; node_bounds[6]; shapes). */
WPBR_API wpbr_status wpbr_bvh_export(wpbr_ctx* ctx, float* prim_bounds, float* centroids, float* cbounds,
                                     uint32_t* codes, uint32_t* sorted_codes, uint32_t* sorted_prims,
                                     uint32_t* treelet_start, uint32_t* nodes, float* node_bounds,
                                     uint32_t* shapes);

/* ---- collision ----------------------------------------------------------- */
/* runCollisionSystem (MEngine.cpp:352-361): JobProcessRayCasts,
 * Job{Sphere,Triangle}...InteractionRequests, JobProcessRayCastsResults.
 * CLOSEST returns the reference's hit (closest non-zero t, first candidate in
 * near-first order on ties); ANY stops at the first hit (occlusion only). */
enum wpbr_trace_mode { WPBR_TRACE_CLOSEST = 0, WPBR_TRACE_ANY = 1 };
/* Host buffers (rays: n x 8 floats o.xyz, 0, d.xyz, tmax; hits: n x 4 floats
 * t, prim id bits, b1, b2). Batches of 2^22 rays and more are copied and
 * traced in four chunks, the copies of one chunk overlapping the traversal
 * of its neighbours (page-locked host buffers let them overlap). */
WPBR_API wpbr_status wpbr_collide(wpbr_ctx* ctx, const float* rays, uint64_t n, float* hits, uint32_t mode);
WPBR_API wpbr_status wpbr_collide_device(wpbr_ctx* ctx, const void* d_rays, uint64_t n, void* d_hits,
                                         uint32_t mode);
/* Large batches (256k rays and more) are traced in the order of their
 * origins' Morton cells on a 2^b per axis grid over the scene bounds
 * (b = bits_per_axis, default 8, at most 10) and written back at their input
 * positions; the hits do not depend on the order. 0 traces in input order. */
WPBR_API wpbr_status wpbr_set_ray_sort(wpbr_ctx* ctx, uint32_t bits_per_axis);
/* Per-ray node visits and primitive tests (u32 pairs) of the near-first
 * traversal over the reference's leaves as they are, for the byte model. */
WPBR_API wpbr_status wpbr_collide_stats(wpbr_ctx* ctx, const float* rays, uint64_t n, float* hits,
                                        uint32_t* stats, uint32_t mode);
/* Number of kernels one wpbr_collide_device call of n rays launches with the
 * context's current settings (the traversal, plus the ray-order key and
 * radix-sort kernels for large batches). */
WPBR_API wpbr_status wpbr_collide_launches(const wpbr_ctx* ctx, uint64_t n, uint32_t* launches);
/* Instrumentation: with timing enabled, each collide call's traversal
 * launch is bracketed by CUDA events on the context's stream (the first 64
 * launches after enabling or after the last read); wpbr_kernel_timing
 * waits for them and returns their summed duration and count, then starts
 * a new series. */
WPBR_API wpbr_status wpbr_set_kernel_timing(wpbr_ctx* ctx, uint32_t enable);
WPBR_API wpbr_status wpbr_kernel_timing(wpbr_ctx* ctx, float* total_ms, uint32_t* launches);

/* ---- rendering -------------------------------------------------------------- */
/* Film + sample streams for spp passes (JobGenerateFilmTiles,
 * JobCreateCameraSamples, CSFilm.cpp:10-68); clears the film. */
WPBR_API wpbr_status wpbr_render_setup(wpbr_ctx* ctx, uint32_t spp, uint32_t seed, uint32_t stream);
/* One sample pass through the fused wavefront kernels (graph-captured):
 * the per-spp job list of MEngine::render (MEngine.cpp:393-442) plus
 * JobAccumalateLIFromSamples. */
WPBR_API wpbr_status wpbr_render_pass(wpbr_ctx* ctx, uint32_t pass);
/* All spp passes. */
WPBR_API wpbr_status wpbr_render(wpbr_ctx* ctx);
/* Film accumulators to host: acc_L[W*H*3], acc_w[W*H] (pre-tonemap). */
WPBR_API wpbr_status wpbr_film_read(wpbr_ctx* ctx, float* acc_L, float* acc_w);
/* JobOutputFilmTitles + JobOutputFilm (CSFilm.cpp:129-242): 8-bit RGB. */
WPBR_API wpbr_status wpbr_film_tonemap(wpbr_ctx* ctx, uint8_t* rgb8);

/* Staged path: the reference's jobs one by one (see wpbr_job_id), each a
 * separate kernel over per-pixel state buffers. */
typedef enum wpbr_job_id {
  WPBR_JOB_CAMERA_RAYS = 0,       /* JobSamplerUpdateCameraSamples + JobCameraPerspGenerateRaysDifferential */
  WPBR_JOB_COLLIDE_PRIMARY = 1,   /* runCollisionSystem on camera rays (full interactions) */
  WPBR_JOB_EMITTED_LIGHT = 2,     /* JobScatteringRequestEmittedLight..AccumulateEmittedLight */
  WPBR_JOB_BSDF_SETUP = 3,        /* JobGenerateBSDFRequests + material jobs + JobBSDFComputeTransform */
  WPBR_JOB_SAMPLE_LIGHT = 4,      /* JobScatteringSampleLight + SampleLightLI + light sampling jobs */
  WPBR_JOB_SHADOW_LIGHT = 5,      /* JobScatteringCastShadowRays + runCollisionSystem + ProcessShadowRay */
  WPBR_JOB_BSDF_COMPUTE = 6,      /* JobBSDF{Conductor,Specular,Dielectric}*Compute */
  WPBR_JOB_INTEGRATE_LIGHT = 7,   /* JobScatteringIntegrateImportanceLight */
  WPBR_JOB_SAMPLE_BSDF = 8,       /* JobScatteringSampleBSDF + JobBSDF*Sample */
  WPBR_JOB_SHADOW_BSDF = 9,       /* ...CastShadowRaysWithInteraction + runCollisionSystem + Process... */
  WPBR_JOB_LIGHT_COMPUTE = 10,    /* JobSphereLightProcessComputeRequests + JobLightInfiniteAreaLiCompute */
  WPBR_JOB_INTEGRATE_BSDF = 11,   /* JobScatteringIntegrateImportanceBSDF */
  WPBR_JOB_FILM_ACCUMULATE = 12,  /* JobAccumalateLIFromSamples */
  WPBR_JOB_COUNT = 13
} wpbr_job_id;
WPBR_API wpbr_status wpbr_job_run(wpbr_ctx* ctx, uint32_t job, uint32_t pass);
/* Copies the staged path's per-pixel state for the pixel rectangle
 * [x0,x1)x[y0,y1) into host arrays (NULL fields skipped). */
WPBR_API wpbr_status wpbr_job_record(wpbr_ctx* ctx, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                                     wpbr_pass_record* rec);

/* ---- synthetic scenes (benchmark and test inputs) -------------------------- */
typedef struct wpbr_scenegen wpbr_scenegen;
enum { WPBR_SCENEGEN_RAYS = 1u };
/* config 0 plain render, 1 LBVH microbench (level = icosphere subdivisions,
 * 0 -> 8; flag RAYS also builds res_x*res_y coherent + as many incoherent
 * rays), 2 full frame, 3 scene `level` of the batched set (films scaled by
 * res_x/1024, primitive counts capped at res_y; 1024 and 2000000 give the set
 * as specified), 4 the differentiable scene (config 0's geometry, 64
 * materials, sphere + 256x128 environment light; `level` seeds the material
 * parameters and the environment), 5 the textured-metal scene (config 0's
 * spheres, every third one and the ground CMaterialMetal with four procedural
 * textures, grazing camera). Host-only, no GPU needed. */
WPBR_API wpbr_status wpbr_scenegen_create(uint32_t config, uint32_t seed, uint32_t res_x, uint32_t res_y,
                                          uint32_t level, uint32_t flags, wpbr_scenegen** out);
WPBR_API const wpbr_scene_desc* wpbr_scenegen_desc(const wpbr_scenegen* g);
WPBR_API uint64_t wpbr_scenegen_ray_count(const wpbr_scenegen* g);
WPBR_API const float* wpbr_scenegen_rays(const wpbr_scenegen* g);
WPBR_API void wpbr_scenegen_destroy(wpbr_scenegen* g);

/* ---- allocation-free Morton sort ----------------------------------------------
 * No counterpart in the reference (its sort runs inside JobSortsShapesByMortonCode
 * on the engine's temp allocator). For callers that cannot allocate device
 * memory: hosts that hand out all device memory from their own arena and
 * forbid allocation inside a job, and loops that must not take cudaMalloc's
 * device-wide synchronisation. Stable LSD radix sort of n Morton codes by their
 * low key_bits bits (24: the order the reference builds over; 30: full), the
 * same permutation as wpbr_bvh_build. Device buffers in and out (no aliasing),
 * asynchronous on `stream`, no allocation: temporaries live in one file-scope
 * device array of WPBR_SORT_NOALLOC_MAX_KEYS keys (about 8.5 MB per GPU that
 * loads the library, held until exit). Every call made outside stream capture
 * looks up the array's address in the current device context (so a device
 * reset or a switch of context is picked up); a call on a capturing stream
 * reuses the address last looked up on that device, so the first call on a
 * device must come before any stream capture (it is refused otherwise). All calls share
 * the array; calls whose GPU work overlaps race. n above the maximum returns
 * WPBR_ERR_INVALID_ARG; wpbr_sort_morton_noalloc_error() says why. */
#define WPBR_SORT_NOALLOC_MAX_KEYS (1u << 20)
WPBR_API wpbr_status wpbr_sort_morton_noalloc(const uint32_t* d_codes, uint32_t n, uint32_t key_bits,
                                              uint32_t* d_sorted_codes, uint32_t* d_perm, void* stream);
WPBR_API const char* wpbr_sort_morton_noalloc_error(void);

/* ---- batched scenes ---------------------------------------------------------
 * No counterpart in the reference, which renders one scene per engine
 * (MEngine::render, MEngine.cpp:380-448). A batch holds many independent
 * scenes of uneven size and film resolution; their traversal layouts live in
 * one pooled device arena, and each sample pass of all scenes is one CUDA
 * graph with one branch per scene (the five kernels of wpbr_render_pass), so a
 * pass of every scene costs one graph launch. Each scene's film is bit-identical
 * to rendering it alone with a wpbr_ctx and the same spp, seed and stream id.
 * The persistent traversal grid per scene is picked by wpbr_batch_autotune. */
typedef struct wpbr_batch wpbr_batch;
typedef struct wpbr_batch_info {
  uint32_t n_scenes;
  uint32_t spp;
  uint64_t total_pixels;      /* sum over scenes of film width x height */
  uint64_t total_prims;
  uint64_t arena_bytes;       /* pooled traversal arena (Node2 + primitive records) */
  uint32_t rays_per_block;    /* traversal queue depth in effect (0 = one full wave) */
  uint32_t autotune_source;   /* 0 default, 1 measured, 2 cache file, 3 set by caller */
} wpbr_batch_info;
WPBR_API wpbr_status wpbr_batch_create(int device, wpbr_batch** out);
WPBR_API void wpbr_batch_destroy(wpbr_batch* b);
WPBR_API const char* wpbr_batch_last_error(const wpbr_batch* b);
/* Adds a scene (copied; same rules as wpbr_scene_upload) with its own quirk
 * bits; *index receives its position. Only before wpbr_batch_build. */
WPBR_API wpbr_status wpbr_batch_add_scene(wpbr_batch* b, const wpbr_scene_desc* scene, uint32_t quirks,
                                          uint32_t* index);
/* Builds every scene's BVH (one at a time, reusing one set of build scratch)
 * and moves the traversal layouts into the pooled arena. */
WPBR_API wpbr_status wpbr_batch_build(wpbr_batch* b);
/* wpbr_render_setup for all scenes (stream id = first_stream + scene index)
 * and captures the pass graph. */
WPBR_API wpbr_status wpbr_batch_render_setup(wpbr_batch* b, uint32_t spp, uint32_t seed, uint32_t first_stream);
/* Times the pass graph for each candidate traversal queue depth (rays per
 * persistent block: one full wave, 4096, 1024, 256), keeps the fastest and
 * records it in the cache file named by WPBR_AUTOTUNE_CACHE (default
 * $HOME/.cache/wpbr_autotune.txt) under a key of device, scene count and film
 * sizes; with use_cache a cached entry is taken without timing. Clears the
 * films afterwards. */
WPBR_API wpbr_status wpbr_batch_autotune(wpbr_batch* b, int use_cache);
/* Sets the queue depth directly (0 = one full wave) and recaptures. */
WPBR_API wpbr_status wpbr_batch_set_rays_per_block(wpbr_batch* b, uint32_t rays_per_block);
/* One sample pass of every scene (one graph launch, asynchronous). */
WPBR_API wpbr_status wpbr_batch_render_pass(wpbr_batch* b, uint32_t pass);
/* All spp passes, asynchronous. */
WPBR_API wpbr_status wpbr_batch_render(wpbr_batch* b);
WPBR_API wpbr_status wpbr_batch_synchronize(wpbr_batch* b);
WPBR_API wpbr_status wpbr_batch_info_get(const wpbr_batch* b, wpbr_batch_info* out);
/* Film size and accumulated film of one scene (as wpbr_film_read). */
WPBR_API wpbr_status wpbr_batch_film_size(const wpbr_batch* b, uint32_t scene, uint32_t* w, uint32_t* h);
WPBR_API wpbr_status wpbr_batch_film_read(wpbr_batch* b, uint32_t scene, float* acc_L, float* acc_w);
/* The stream the pass graph is launched on (default: one the batch creates). */
WPBR_API wpbr_status wpbr_batch_set_stream(wpbr_batch* b, void* stream);
WPBR_API wpbr_status wpbr_batch_check_device_errors(wpbr_batch* b);

/* ---- differentiable estimator (forward / backward) -----------------------------
 * No counterpart in the reference (it renders forward only). Gradients of the
 * image loss  sum_pixels sum_rgb (I - T)^2 / (3 W H),  I = filtered film
 * radiance of wpbr_adjoint_setup's spp passes, with respect to
 *  - per material m, 10 floats at mat_params[10 m]: alpha (sets alpha_x and
 *    alpha_y), albedo R[3], eta_t[3] (a dielectric uses eta_t[0]), k[3];
 *  - the environment texels, 3 floats per texel in row order (env_params).
 * The differentiated function is the frozen-direction estimator: directions,
 * hits and visibility come from the sampling parameters captured by
 * wpbr_adjoint_freeze; BSDF values, pdfs, MIS weights and emitted / incident
 * radiance are evaluated at the current parameters (wpbr_adjoint_set_params).
 * At equal parameters its image is MEngine::render's (MEngine.cpp:393-442)
 * up to rounding. wpbr_adjoint_backward replays the sample passes (no stored
 * paths) and needs a wpbr_adjoint_forward with a target at the current
 * parameters. Samples whose radiance is not finite contribute zero. */
WPBR_API wpbr_status wpbr_adjoint_setup(wpbr_ctx* ctx, uint32_t spp, uint32_t seed, uint32_t stream);
WPBR_API wpbr_status wpbr_adjoint_param_counts(wpbr_ctx* ctx, uint32_t* n_mat_params, uint32_t* n_env_params);
WPBR_API wpbr_status wpbr_adjoint_get_params(wpbr_ctx* ctx, float* mat_params, float* env_params);
/* NULL keeps the current values of that group. */
WPBR_API wpbr_status wpbr_adjoint_set_params(wpbr_ctx* ctx, const float* mat_params, const float* env_params);
WPBR_API wpbr_status wpbr_adjoint_set_params_device(wpbr_ctx* ctx, const float* d_mat_params,
                                                    const float* d_env_params);
WPBR_API wpbr_status wpbr_adjoint_freeze(wpbr_ctx* ctx);
/* target and image: W*H*3 floats (NULL: no loss / no image); *loss receives
 * the loss when a target is given. */
WPBR_API wpbr_status wpbr_adjoint_forward(wpbr_ctx* ctx, const float* target, float* image, double* loss);
WPBR_API wpbr_status wpbr_adjoint_forward_device(wpbr_ctx* ctx, const float* d_target, float* d_image, double* loss);
WPBR_API wpbr_status wpbr_adjoint_backward(wpbr_ctx* ctx, float* grad_mat, float* grad_env);
WPBR_API wpbr_status wpbr_adjoint_backward_device(wpbr_ctx* ctx, float* d_grad_mat, float* d_grad_env);

/* ---- testing aids ------------------------------------------------------------
 * No counterpart in the reference (its traversal stack, nodesToVisit[256] in
 * SLBVH.cpp:101, is unchecked, and its allocators abort on failure). */
/* Lowers the traversal's bounds so that their limit paths can be exercised:
 * at most max_stack_entries entries on a lane's traversal stack (at most
 * 256) and max_loop_steps iterations of a traversal loop (the persistent
 * kernels count a warp's rounds); 0 restores a default (the stack the tree's
 * depth needs, 2^26 steps). A traversal that reaches a bound gives up on the
 * rays it holds (their hits are not valid), records the bound in the device
 * error word and returns, so wpbr_check_device_errors returns
 * WPBR_ERR_TRAVERSAL_LIMIT; nothing traps and the context stays usable.
 * Applies to later launches (pass graphs are recaptured). */
WPBR_API wpbr_status wpbr_set_traversal_limits(wpbr_ctx* ctx, uint32_t max_stack_entries, uint32_t max_loop_steps);
/* The order wpbr_collide traces a batch of n rays in when it sorts them
 * (batches of 2^18 rays and more, wpbr_set_ray_sort > 0): keys[i] is the
 * Morton code of ray i's origin cell (3 x bits-per-axis bits over the scene
 * bounds) and perm[j] the input index of the j-th ray traced, a stable sort of
 * the keys. rays as for wpbr_collide (host); any n below 2^32 - 1. */
WPBR_API wpbr_status wpbr_debug_ray_order(wpbr_ctx* ctx, const float* rays, uint64_t n, uint32_t* keys,
                                          uint32_t* perm);
/* Process-wide device-allocation fault injection: with n >= 0 the library's
 * next n device allocations succeed and every later one fails (cudaMalloc is
 * not called), so the call that needed it returns WPBR_ERR_OOM; n < 0 (the
 * default) disables it. */
WPBR_API void wpbr_debug_fail_allocations(int64_t n);

/* Library build identification (host-only). */
WPBR_API const char* wpbr_version(void);

#ifdef __cplusplus
}
#endif

#endif /* WPBR_GPU_H */
